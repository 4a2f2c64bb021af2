"""Batched snapshots (many decks, one node launch + one work-list launch, CUDA graph).

Each deck's slice of a batch snapshot must equal that deck's own single-context snapshot
bit for bit (the same tile arithmetic over the same nodes), and the oracle within the
single-deck tolerances: 0.01 K for FP32 + Kahan, 1e-7 K for FP64."""
import numpy as np
import pytest

TOL_FP32 = 0.01     # K
TOL_FP64 = 1e-7     # K


@pytest.fixture(scope="module")
def sweep(tmp_path_factory, decks):
    base = tmp_path_factory.mktemp("sweep")
    return [d.write(str(base / d.name)) for d in decks.small_sweep()]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp32", TOL_FP32), ("fp64", TOL_FP64)])
def test_batch_matches_single_decks_and_oracle(built_library, thesis, oracle, sweep, precision, tol):
    with thesis.Batch(sweep, precision) as b:
        off = b.offsets
        for idx in range(2):
            T = b.snapshot(idx)
            for d, path in enumerate(sweep):
                part = T[off[d]:off[d + 1]]
                with thesis.Simulation(path, precision) as sim:
                    assert sim.pnum == off[d + 1] - off[d]
                    assert np.array_equal(part, sim.snapshot(idx)), f"deck {d} snapshot {idx}"
                ref = oracle(path).snapshot(idx)
                assert np.max(np.abs(part - ref)) <= tol, f"deck {d} snapshot {idx}"


@pytest.mark.gpu
def test_batch_graph_replay_and_tile_shapes(built_library, thesis, sweep):
    """Replaying a cached graph repeats the result exactly; every tile shape (and the one
    the tuner picks) agrees within the FP32 tolerance; pair counts add up."""
    with thesis.Batch(sweep, "fp32") as b:
        first = b.snapshot(1)
        assert np.array_equal(b.snapshot(1), first)
        for shape in [(4, 1), (4, 4), (2, 2), (2, 4), (8, 1), (8, 2)]:
            b.set_tile_shape(*shape)
            assert np.max(np.abs(b.snapshot(1) - first)) <= TOL_FP32, shape
        kp, kch = b.autotune(1)
        assert (kp, kch) in [(4, 2), (4, 1), (4, 4), (2, 2), (2, 4), (8, 1), (8, 2)]
        assert np.max(np.abs(b.snapshot(1) - first)) <= TOL_FP32
    with thesis.Batch(sweep, "fp32") as b:
        b.snapshot(1)
        expect = 0
        for path in sweep:
            with thesis.Simulation(path, "fp32") as sim:
                expect += sim.integrate(sim.snapshot_times[1])["xb"].size * sim.pnum
        assert b.pairs == expect


@pytest.mark.gpu
def test_batch_snapshot_device_on_torch_stream(built_library, thesis, sweep):
    torch = pytest.importorskip("torch")
    with thesis.Batch(sweep, "fp32") as b:
        ref = b.snapshot(0)
        out = torch.empty(b.pnum, dtype=torch.float64, device="cuda")
        s = torch.cuda.Stream()
        b.snapshot_device(0, out.data_ptr(), s.cuda_stream)
        s.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.gpu
def test_single_context_autotune(built_library, thesis, deck_dir):
    with thesis.Simulation(deck_dir("small_snapshot"), "fp32") as sim:
        base = sim.snapshot(2)
        shape = sim.autotune(2)
        assert shape in [(4, 2), (4, 1), (4, 4), (2, 2), (2, 4), (8, 1), (8, 2)]
        assert np.max(np.abs(sim.snapshot(2) - base)) <= TOL_FP32


def test_batch_rejects_bad_decks_before_touching_the_device(built_library, thesis, sweep, deck_dir):
    """Host-side validation: a Solidification deck or a missing file fails with
    TH_ERR_INVALID and a message naming the deck, with or without a GPU."""
    with pytest.raises(thesis.ThesisError) as e:
        thesis.Batch([sweep[0], deck_dir("small_surface")])
    assert e.value.status == 1 and "deck 1" in str(e.value)
    with pytest.raises(thesis.ThesisError) as e:
        thesis.Batch([sweep[0], sweep[1] + ".missing"])
    assert e.value.status == 1 and "deck 1" in str(e.value)
