"""The CPU oracle against vectors produced by the unmodified reference (tests/golden)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
import parity  # noqa: E402

GOLDEN = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


@pytest.mark.parametrize("deck", sorted(make_golden.NODE_TIMES))
def test_oracle_nodes_match_reference(deck, oracle, tmp_path):
    g = _load(f"nodes_{deck}.npz")
    path = make_golden.node_deck(deck).write(str(tmp_path / deck))
    o = oracle(path)
    for i, t in enumerate(make_golden.NODE_TIMES[deck]):
        for sol in (False, True):
            ref = g[f"{'sol_' if sol else ''}nodes{i}"]
            got = o.nodes(float(g[f"t{i}"]), sol)
            assert got["xb"].size == ref.shape[1], (deck, t, sol)
            for c, f in enumerate(("xb", "yb", "zb", "phix", "phiy", "phiz", "dtau", "expmod")):
                np.testing.assert_allclose(got[f], ref[c], rtol=1e-13, atol=0, err_msg=f"{deck} t={t} {f}")


def test_oracle_temperature_matches_reference(oracle, tmp_path, decks):
    g = _load("temp_snapshot_raster.npz")
    o = oracle(decks.snapshot_raster().write(str(tmp_path / "raster")))
    for i in range(3):
        assert o.snapshot_time(i) == float(g[f"t{i}"])
        T = o.calc_T(o.snapshot_time(i), g["pts"])
        np.testing.assert_allclose(T, g[f"T{i}"], rtol=1e-13, atol=1e-10)


@pytest.mark.parametrize("tag", sorted(make_golden.RUNS))
def test_oracle_solidification_matches_reference(tag, oracle, tmp_path):
    g = _load(f"run_{tag}.npz")
    deck = make_golden.run_deck(tag)
    o = oracle(deck.write(str(tmp_path / tag)))
    o.solidify(threads=4)
    flag = o.field("output_flag") > 0
    assert np.array_equal(np.packbits(flag), g["mask"]), "molten-point set differs"
    sub = g["sample"]
    for key in g:
        if not key.endswith("_sample"):
            continue
        f = key[:-len("_sample")]
        v = o.field(f)
        np.testing.assert_allclose(v[sub], g[key], rtol=1e-12, atol=1e-12, err_msg=f)
        np.testing.assert_allclose(np.sum(v[flag]), g[f + "_sum"], rtol=1e-11, err_msg=f)
    if "rdf_counts" in g:                          # the reduced data format: every event
        counts, vals, _ = o.rdf()
        assert np.array_equal(counts.ravel(), g["rdf_counts"]), "RDF event counts differ"
        np.testing.assert_allclose(vals, g["rdf_vals"], rtol=1e-12, atol=0, err_msg="RDF values")


def test_oracle_solidification_time_budget(oracle, tmp_path):
    """The budgeted run (the bench's bounded CPU sample) stops after the first step that ends
    past the budget, returning the number of steps it ran, and otherwise runs exactly the
    unbudgeted loop."""
    deck = make_golden.run_deck("small_surface")
    path = deck.write(str(tmp_path / "budget"))
    full = oracle(path).solidify(threads=2)
    cut = oracle(path).solidify(threads=2, budget_s=1e-9)
    assert cut == 1 < full
    ample = oracle(path)
    assert ample.solidify(threads=2, budget_s=3600.0) == full
    ref = oracle(path)
    ref.solidify(threads=2)
    assert np.array_equal(ample.field("tSol"), ref.field("tSol"))


@pytest.mark.parametrize("name", make_golden.RRDF_DECKS)
def test_oracle_stork_rows_match_reference(name, oracle, tmp_path):
    """A whole Stork run (Run::Stork, src/Run.cpp:711-1079): the oracle's doubly reduced data
    equals the reference's bit for bit (same rows in the same order, same index, time and
    temperature words)."""
    g = _load(f"rrdf_{name}.npz")
    deck = make_golden.rrdf_deck(name)
    o = oracle(deck.write(str(tmp_path / name)))
    o.solidify(threads=4)
    idx, ts, Ts = o.rrdf()
    assert idx.shape[0] == int(g["rows"])
    assert np.unique(ts[:, 1]).size == int(g["steps"])
    assert make_golden.rrdf_digest(idx, ts, Ts) == str(g["digest"])
    if name == "small_stork":                      # the pool reaches the bottom cell layer
        assert idx[:, 2].min() == 0


def test_oracle_snapshots_print_as_the_reference_T_hist(oracle, tmp_path):
    """The reference's temperature-history file of a Snapshots deck (Output T_hist 1,
    Grid::Output_T_hist, src/Grid.cpp:101-136): its header holds the snapshot times and
    each row a point's temperature at every snapshot, all printed with 6 decimals; the
    oracle's snapshots print to the same text."""
    g = _load("thist_snapshot.npz")
    lines = bytes(g["file_bytes"]).decode().splitlines()
    deck = make_golden.thist_deck("thist_snapshot")
    o = oracle(deck.write(str(tmp_path / deck.name)))
    head = lines[0].split(",")
    assert head[:3] == ["x", "y", "z"] and len(head) == 3 + o.n_snapshots
    assert head[3:] == ["%f" % o.snapshot_time(i) for i in range(o.n_snapshots)]
    T = [o.snapshot(i, threads=2) for i in range(o.n_snapshots)]
    assert len(lines) == 1 + T[0].size
    for p in range(0, T[0].size, 97):
        assert lines[1 + p].split(",")[3:] == ["%f" % T[i][p] for i in range(len(T))], p


def test_reference_rrdf_binary_layout():
    """The reference's binary RRDF file of small_stork (Grid::Output_RRDF_bin,
    src/Grid.cpp:241-273) read with the layout the GPU test checks the library's file
    against: the header holds the row count, the deck's point counts, its minima, x
    resolution and liquidus, and the rows are the reference's own."""
    g = _load("rrdf_small_stork.npz")
    b = parity.read_rrdf_bin(g["bin_file"].tobytes())
    deck = make_golden.rrdf_deck("small_stork")
    assert b["rows"] == int(g["rows"])
    assert b["extent"].tolist() == [ax.num for ax in deck.axes]
    assert np.array_equal(b["geometry"][:3], [ax.vmin for ax in deck.axes])
    assert b["geometry"][4] == deck.material.TL
    assert make_golden.rrdf_digest(b["idx"], b["ts"], b["Ts"]) == str(g["digest"])


@pytest.mark.parametrize("name", make_golden.CUSTOM_DECKS)
def test_oracle_custom_points_match_reference(name, oracle, tmp_path):
    """Custom point files (Domain: Custom File, src/Init.cpp:686-703, 816-857): the oracle
    reads the same points and runs them without tracking as the reference does - every
    snapshot's T, or the solidification run's T, tSol, G, V and dTdt, bit for bit."""
    g = _load(f"{name}.npz")
    deck = make_golden.custom_deck(name)
    o = oracle(deck.write(str(tmp_path / name)))
    assert o.pnum == int(g["info"][3]) == len(deck.points)
    if deck.mode == "Snapshots":
        for i in range(o.n_snapshots):
            assert np.array_equal(o.snapshot(i, threads=2), g[f"T{i}"]), i
    else:
        o.solidify(threads=2)
        for f in ("T", "tSol", "G", "V", "dTdt"):
            assert np.array_equal(o.field(f), g[f]), f
