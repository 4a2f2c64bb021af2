"""Stork tracking (Run::Stork, src/Run.cpp:711-1079) on the device against the oracle, and
the RRDF file of th_simulate against the reference's own (tests/golden/rrdf_small_stork.npz).

The rows follow from the liquid sets of consecutive steps alone, so the row set, its order
(step, then ascending cell index: the reference's single-thread order), the cell indices
and the step times are compared exactly; the 16 vertex temperatures within the
temperature tolerance of the precision (FP64 1e-7 K, FP32 0.01 K)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
import parity  # noqa: E402

pytestmark = pytest.mark.gpu
T_TOL = {"fp64": 1e-7, "fp32": 0.01}


@pytest.fixture(scope="module")
def stork_runs(oracle, tmp_path_factory):
    """Per deck: the deck's path and the oracle's rows."""
    out = {}
    for name in make_golden.RRDF_DECKS:
        path = make_golden.rrdf_deck(name).write(str(tmp_path_factory.mktemp("stork") / name))
        o = oracle(path)
        steps = o.solidify(threads=4)
        out[name] = (path, steps, o.rrdf())
    return out


def _compare(ref, got, prec, what):
    (ri, rt, rT), (gi, gt, gT) = ref, got
    assert gi.shape == ri.shape, f"{what}: {gi.shape[0]} rows, oracle {ri.shape[0]}"
    assert np.array_equal(gt, rt), f"{what}: step times differ"
    bad = np.flatnonzero(np.any(gi != ri, axis=1))
    assert bad.size == 0, f"{what}: cell {gi[bad[0]]} at row {bad[0]} (step t={gt[bad[0], 1]}), oracle {ri[bad[0]]}"
    err = np.abs(gT - rT)
    r, c = np.unravel_index(np.argmax(err), err.shape)
    assert err[r, c] <= T_TOL[prec], (f"{what}: vertex {c} of cell {gi[r]} at t={gt[r, 1]}: {gT[r, c]!r} K, "
                                     f"oracle {rT[r, c]!r} K")


@pytest.mark.parametrize("name", make_golden.RRDF_DECKS)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stork_rows_match_oracle(built_library, thesis, stork_runs, name, prec):
    path, steps, ref = stork_runs[name]
    with thesis.Simulation(path, prec) as sim:
        assert sim.solidify() == steps
        got = sim.rrdf()
        stats = sim.run_stats()
    _compare(ref, got, prec, f"{name} {prec}")
    assert stats["rrdf_rows"] == ref[0].shape[0]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stork_rows_across_calls_and_reset(built_library, thesis, stork_runs, prec):
    """A run split over several calls (each ends a tracking launch mid-window, the next one
    starts from the last step's liquid list) and a run after a reset give the same rows."""
    path, steps, ref = stork_runs["surface_stork"]
    with thesis.Simulation(path, prec) as sim:
        done = 0
        for cut in (37, 120, 300):
            done = sim.solidify(max_steps=cut)
            assert done == min(cut, steps)
        assert sim.solidify() == steps
        _compare(ref, sim.rrdf(), prec, f"split {prec}")
        sim.reset()
        assert sim.solidify() == steps
        _compare(ref, sim.rrdf(), prec, f"after reset {prec}")


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_simulate_writes_the_reference_rrdf_file(built_library, thesis, stork_runs, tmp_path, prec):
    """th_simulate writes Data/<name>.RRDF.csv (bin/Main.cpp:109-111, Grid::Output_RRDF_csv,
    src/Grid.cpp:203-238) and nothing else.  Indices and times print identically; a
    temperature's text may differ only where the tolerance reaches a rounding boundary of the
    exact value (the oracle's, bit-equal to the reference's): there the printed value lies
    within the tolerance, and half a printed unit, of the exact value."""
    deck = make_golden.rrdf_deck("small_stork")
    path = deck.write(str(tmp_path / "small_stork"))
    with thesis.Simulation(path, prec) as sim:
        sim.simulate()
    g = np.load(os.path.join(HERE, "golden", "rrdf_small_stork.npz"))
    names = [str(n) for n in g["names"]]
    data = os.path.join(os.path.dirname(path), "Data")
    assert sorted(os.listdir(data)) == names
    ref_lines = bytes(g["file0"]).decode().splitlines()
    with open(os.path.join(data, names[0])) as f:
        got_lines = f.read().splitlines()
    assert got_lines[0] == ref_lines[0]
    assert len(got_lines) == len(ref_lines)
    exact = stork_runs["small_stork"][2][2]
    for r, (a, b) in enumerate(zip(ref_lines[1:], got_lines[1:])):
        if a == b:
            continue
        ra, rb = a.split(","), b.split(",")
        assert ra[:5] == rb[:5], (r, a, b)
        for c in range(5, 21):
            if ra[c] == rb[c]:
                continue
            va, vb, v = float(ra[c]), float(rb[c]), exact[r, c - 5]
            unit = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb)))) - 5)
            assert abs(vb - v) <= T_TOL[prec] + 0.5 * unit, (r, c, ra[c], rb[c], v)
            assert abs(va - v) <= 0.5 * unit * (1 + 1e-9), (r, c, ra[c], rb[c], v)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_output_rrdf_binary_matches_the_reference_file(built_library, thesis, tmp_path, prec):
    """th_output_rrdf with binary 1 writes Data/<name>.<tag>.bin in the layout of
    Grid::Output_RRDF_bin (src/Grid.cpp:241-273): its header (row count, point counts,
    minima, x resolution, liquidus) is the reference's byte for byte, the indices and times
    are the reference's, the temperatures within the precision's tolerance; with binary 0 it
    writes the CSV that th_simulate writes, under the given tag."""
    deck = make_golden.rrdf_deck("small_stork")
    path = deck.write(str(tmp_path / "small_stork"))
    g = np.load(os.path.join(HERE, "golden", "rrdf_small_stork.npz"))
    ref_buf = g["bin_file"].tobytes()
    with thesis.Simulation(path, prec) as sim:
        sim.solidify()
        sim.output_rrdf("RRDF", binary=True)
        sim.output_rrdf("Copy", binary=False)
    data = os.path.join(os.path.dirname(path), "Data")
    assert sorted(os.listdir(data)) == [f"{deck.name}.Copy.csv", f"{deck.name}.RRDF.bin"]
    with open(os.path.join(data, f"{deck.name}.RRDF.bin"), "rb") as f:
        buf = f.read()
    assert buf[:56] == ref_buf[:56]
    got, ref = parity.read_rrdf_bin(buf), parity.read_rrdf_bin(ref_buf)
    assert np.array_equal(got["idx"], ref["idx"]) and np.array_equal(got["ts"], ref["ts"])
    err = float(np.max(np.abs(got["Ts"] - ref["Ts"])))
    assert err <= T_TOL[prec], err
    with open(os.path.join(data, f"{deck.name}.Copy.csv")) as f:
        lines = f.read().splitlines()
    assert lines[0] == bytes(g["file0"]).decode().splitlines()[0]
    assert len(lines) == 1 + ref["rows"]
