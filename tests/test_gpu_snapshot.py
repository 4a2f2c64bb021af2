"""GPU parity of node generation and the point x node sums (CUDA path through the C ABI).

Tolerances: node fields are compared bit for bit (the device walk uses explicitly rounded
FP64); FP64 temperatures within 1e-7 K; FP32 + Kahan temperatures within 0.01 K of the
FP64 oracle (the target stated for the compensated form)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(HERE, "golden")
TOL_FP32 = 0.01     # K
TOL_FP64 = 1e-7     # K


@pytest.fixture(scope="module")
def lib(built_library, thesis):
    return thesis


@pytest.mark.parametrize("deck", sorted(make_golden.NODE_TIMES))
def test_device_nodes_bit_identical_to_reference(lib, deck, tmp_path):
    g = dict(np.load(os.path.join(GOLDEN, f"nodes_{deck}.npz")))
    path = make_golden.node_deck(deck).write(str(tmp_path / deck))
    with lib.Simulation(path, "fp64") as sim:
        for i in range(len(make_golden.NODE_TIMES[deck])):
            for sol in (False, True):
                ref = g[f"{'sol_' if sol else ''}nodes{i}"]
                got = sim.integrate(float(g[f"t{i}"]), sol)
                assert got["xb"].size == ref.shape[1]
                for c, f in enumerate(lib.NODE_FIELDS[:7]):
                    assert np.array_equal(got[f], ref[c]), f"{deck} t{i} sol={sol} field {f}"
                np.testing.assert_allclose(got["expmod"], ref[7], rtol=1e-14, atol=1e-13)


@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("fp32", TOL_FP32)])
def test_calc_T_matches_reference_golden(lib, deck_dir, precision, tol):
    g = dict(np.load(os.path.join(GOLDEN, "temp_snapshot_raster.npz")))
    with lib.Simulation(deck_dir("snapshot_raster"), precision) as sim:
        for i in range(3):
            T = sim.calc_T(float(g[f"t{i}"]), g["pts"])
            assert np.max(np.abs(T - g[f"T{i}"])) <= tol


@pytest.mark.parametrize("name", ["snapshot_raster", "small_spots", "small_snapshot"])
@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("fp32", TOL_FP32)])
def test_whole_grid_snapshot_matches_oracle(lib, oracle, deck_dir, name, precision, tol):
    path = deck_dir(name)
    o = oracle(path)
    with lib.Simulation(path, precision) as sim:
        for i in range(o.n_snapshots):
            ref = o.snapshot(i)
            got = sim.snapshot(i)
            err = np.max(np.abs(got - ref))
            assert err <= tol, f"{name} snapshot {i}: max |dT| = {err:.3e} K (Tmax {ref.max():.0f} K)"


def test_boundary_images_and_multibeam_snapshot(lib, oracle, tmp_path):
    for name in ("small_bcs", "small_multibeam"):
        d = make_golden.node_deck(name)
        d.mode, d.scan_fracs, d.tracking = "Snapshots", [40, 100], "None"
        path = d.write(str(tmp_path / name))
        o = oracle(path)
        with lib.Simulation(path, "fp32") as sim:
            for i in range(2):
                assert np.max(np.abs(sim.snapshot(i) - o.snapshot(i))) <= TOL_FP32


def test_list_and_grid_kernels_agree_at_full_size(lib, deck_dir):
    """Size-independent property at the full 800k-point grid: the tiled kernel (FP64 tile
    offsets) and the point-list kernel (split-float coordinates) agree everywhere."""
    with lib.Simulation(deck_dir("snapshot_raster"), "fp32") as sim:
        t = sim.snapshot_times[2]
        grid = sim.snapshot(2)
        lst = sim.calc_T(t, np.arange(sim.pnum, dtype=np.int64))
        assert np.max(np.abs(grid - lst)) <= TOL_FP32


@pytest.mark.parametrize("shape", [(4, 1), (4, 4), (2, 2), (2, 4), (8, 1), (8, 2)])
def test_tile_shapes_are_equivalent(lib, deck_dir, shape):
    with lib.Simulation(deck_dir("snapshot_raster"), "fp32") as sim:
        base = sim.snapshot(2)
        sim.set_tile_shape(*shape)
        assert np.max(np.abs(sim.snapshot(2) - base)) <= TOL_FP32


def test_temperature_rise_is_linear_in_power(lib, deck_dir, decks):
    """T - T0 is proportional to absorbed power: doubling P doubles the rise (full grid)."""
    def mut(d):
        d.beams[0].power *= 2
    with lib.Simulation(deck_dir("snapshot_raster"), "fp32") as a, \
            lib.Simulation(deck_dir("snapshot_raster", mutate=mut, tag="raster_2p"), "fp32") as b:
        ra = a.snapshot(2) - 300.0
        rb = b.snapshot(2) - 300.0
        assert np.max(np.abs(rb - 2 * ra)) <= 2 * TOL_FP32


def test_pair_count(lib, deck_dir, oracle):
    path = deck_dir("snapshot_raster")
    o = oracle(path)
    with lib.Simulation(path, "fp32") as sim:
        sim.snapshot(0)
        n = sim.integrate(sim.snapshot_times[0])["xb"].size
        assert sim.pairs == n * sim.pnum == 205 * 800000


def test_times_in_one_launch_match_single_snapshots(lib, deck_dir):
    """th_calc_T_times_device (all node lists in one launch) gives every snapshot's T bit
    for bit as the one-time path."""
    torch = pytest.importorskip("torch")
    with lib.Simulation(deck_dir("snapshot_raster"), "fp32") as sim:
        times = sim.snapshot_times
        out = torch.empty(len(times) * sim.pnum, dtype=torch.float64, device="cuda")
        sim.calc_T_times_device(times, 0, sim.pnum, out.data_ptr())
        sim.sync()
        got = out.cpu().numpy().reshape(len(times), sim.pnum)
        for i in range(len(times)):
            assert np.array_equal(got[i], sim.snapshot(i)), i


@pytest.mark.parametrize("name", ["comp_spots", "comp_lines", "comp_zigzag"])
@pytest.mark.parametrize("precision,tol", [("fp64", TOL_FP64), ("fp32", TOL_FP32)])
def test_path_compression_snapshots_and_batch(lib, oracle, tmp_path, name, precision, tol):
    """Decks with path compression (GaussCompressIntegrate, src/Calc.cpp:213-501): the
    device's lists are the reference's (test_device_nodes_bit_identical_to_reference covers
    these decks' goldens), the whole-grid snapshots match the oracle, and the same decks in
    one batch match their single-deck snapshots."""
    d = make_golden.node_deck(name)
    path = d.write(str(tmp_path / name))
    o = oracle(path)
    singles = []
    with lib.Simulation(path, precision) as sim:
        for i in range(o.n_snapshots):
            ref = o.snapshot(i)
            got = sim.snapshot(i)
            assert np.max(np.abs(got - ref)) <= tol, (name, i, np.max(np.abs(got - ref)))
            singles.append(got)
    with lib.Batch([path, path], precision) as b:
        T = b.snapshot(o.n_snapshots - 1)
    off = b.offsets
    assert np.array_equal(T[off[0]:off[1]], singles[-1]) and np.array_equal(T[off[1]:off[2]], singles[-1])
