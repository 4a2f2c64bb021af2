"""Output files: th_simulate (the CLI path) writes the reference's own files for a small
Snapshots deck and a small four-beam Solidification deck - the same names, header and rows
(tests/golden/csv_*.npz hold the unmodified reference's files, Grid::Output,
src/Grid.cpp:72-99, named as bin/Main.cpp:104-118 and src/Run.cpp:117 name them).

Values are printed with 6 significant digits, as the reference's ostream prints them.  A
value's text must equal the reference's, except where the field's tolerance (the parity
tests': T 1e-7 K / 0.01 K, tSol 1e-15 / 1e-8 s, the other fields 1e-9 / 1e-4 relative)
reaches a rounding boundary of the exact value (the oracle's, which matches the
reference's in-memory doubles to 1e-12): there the printed value must be within the
tolerance, and half a printed unit, of the exact value."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _tol(col, v, prec):
    """Absolute tolerance of a value of column col (the parity tests' tolerances)."""
    fp64 = prec == "fp64"
    if col in ("x", "y", "z", "numMelt"):
        return 0.0
    if col == "T":
        return 1e-7 if fp64 else 0.01
    if col == "tSol":
        return 1e-15 if fp64 else 1e-8
    if col == "dTdt":                      # the reference's int-truncated rate: one unit
        return (1e-9 if fp64 else 1e-4) * abs(v) + 1.0
    return (1e-9 if fp64 else 1e-4) * abs(v)


def _exact(oracle, deck, path):
    """The oracle's values of every output row, per file name: {file: {column: array}}."""
    o = oracle(path)
    out = {}
    if deck.mode == "Snapshots":
        for i in range(o.n_snapshots):
            out[f"{deck.name}.Snapshot.{i:02d}.csv"] = {"T": o.snapshot(i)}
        flag = np.ones(o.pnum, dtype=bool)
    else:
        o.solidify()
        flag = o.field("output_flag") > 0
        out[f"{deck.name}.Solidification.Final.csv"] = {
            f: o.field(f) for f in ("T", "tSol", "G", "V", "dTdt", "numMelt")}
    return {k: {c: v[flag] for c, v in cols.items()} for k, cols in out.items()}


@pytest.mark.parametrize("name", make_golden.CSV_DECKS)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_simulate_writes_the_reference_files(built_library, thesis, oracle, tmp_path, name, prec):
    deck = make_golden.csv_deck(name)
    path = deck.write(str(tmp_path / name))
    with thesis.Simulation(path, prec) as sim:
        sim.simulate()
    g = np.load(os.path.join(HERE, "golden", f"csv_{name}.npz"))
    names = [str(n) for n in g["names"]]
    data = os.path.join(os.path.dirname(path), "Data")
    assert sorted(os.listdir(data)) == names
    exact = _exact(oracle, deck, path)
    for i, fname in enumerate(names):
        ref_lines = bytes(g[f"file{i}"]).decode().splitlines()
        with open(os.path.join(data, fname)) as f:
            got_lines = f.read().splitlines()
        assert got_lines[0] == ref_lines[0], fname                    # header
        assert len(got_lines) == len(ref_lines), fname                 # one row per output point
        cols = ref_lines[0].split(",")
        ref_rows = [r.split(",") for r in ref_lines[1:]]
        got_rows = [r.split(",") for r in got_lines[1:]]
        for c, col in enumerate(cols):
            for r, (a, b) in enumerate(zip(ref_rows, got_rows)):
                if a[c] == b[c]:
                    continue
                # texts differ only where the field's tolerance reaches a rounding boundary of
                # the exact value: the printed value is within the tolerance (and half a printed
                # unit) of the exact value, and so is the reference's
                assert col in exact.get(fname, {}), (fname, col, r, a[c], b[c])
                va, vb = float(a[c]), float(b[c])
                v = exact[fname][col][r]
                unit = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb)))) - 5)
                assert abs(vb - v) <= _tol(col, v, prec) + 0.5 * unit, (fname, col, r, a[c], b[c], v)
                assert abs(va - v) <= 1e-12 * abs(v) + 0.5 * unit, (fname, col, r, a[c], b[c], v)


def _rdf_rows(counts, vals, flag):
    """The reduced data's file rows (tm, tl, cr) from per-point counts and values, as
    Grid::Output_RDF walks them: output points in order, per melting time."""
    rows, at = [], 0
    for p in np.flatnonzero(counts.sum(axis=1)):
        a, b, c = counts[p]
        at = int(at)
        if flag[p]:
            for e in range(a):
                rows.append((vals[at + e], vals[at + a + e], vals[at + a + b + e]))
        at += a + b + c
    return rows


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_simulate_writes_the_reference_rdf_file(built_library, thesis, oracle, tmp_path, prec):
    """Output RDF 1 on the small Surface deck: th_simulate adds Data/<name>.RDF.Final.csv
    (Grid::Output_RDF, src/Grid.cpp:176-201, named by bin/Main.cpp:117) beside the
    Solidification.Final file; the reference's file is in tests/golden/run_small_surface_rdf.npz.
    Same header, rows, coordinates and melting times (text equal); where a solidification
    time's or cooling rate's text differs, each file prints its own run's value (the GPU's
    from th_rdf, the reference's = the oracle's) to half a printed unit - the two values are
    compared, event by event, by test_gpu_solidify.py::test_rdf_matches_oracle."""
    deck = make_golden.run_deck("small_surface_rdf")
    path = deck.write(str(tmp_path / deck.name))
    with thesis.Simulation(path, prec) as sim:
        sim.simulate()
        gcounts, gvals = sim.rdf()
        gflag = sim.field("output_flag") > 0
    data = os.path.join(os.path.dirname(path), "Data")
    assert sorted(os.listdir(data)) == [f"{deck.name}.RDF.Final.csv", f"{deck.name}.Solidification.Final.csv"]
    g = np.load(os.path.join(HERE, "golden", "run_small_surface_rdf.npz"))
    ref_lines = bytes(g["rdf_file"]).decode().splitlines()
    with open(os.path.join(data, f"{deck.name}.RDF.Final.csv")) as f:
        got_lines = f.read().splitlines()
    assert got_lines[0] == ref_lines[0]
    assert len(got_lines) == len(ref_lines)
    o = oracle(path)
    o.solidify()
    ocounts, ovals, _ = o.rdf()
    ref_rows = _rdf_rows(ocounts, ovals, o.field("output_flag") > 0)
    gpu_rows = _rdf_rows(gcounts, gvals, gflag)
    assert len(ref_rows) == len(gpu_rows) == len(ref_lines) - 1
    for r, (ra, rb) in enumerate(zip(ref_lines[1:], got_lines[1:])):
        if ra == rb:
            continue
        a, b = ra.split(","), rb.split(",")
        assert a[:4] == b[:4], (r, ra, rb)
        for c in (4, 5):
            if a[c] == b[c]:
                continue
            va, vb = float(a[c]), float(b[c])
            unit = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb)))) - 5)
            assert abs(vb - gpu_rows[r][c - 3]) <= 0.5 * unit * (1 + 1e-12), (r, c, b[c], gpu_rows[r][c - 3])
            assert abs(va - ref_rows[r][c - 3]) <= 0.5 * unit * (1 + 1e-12), (r, c, a[c], ref_rows[r][c - 3])


def _read_thist(text):
    """A temperature-history file: header fields, coordinate texts (n, 3), T texts (n, nt)."""
    lines = text.splitlines()
    rows = [ln.split(",") for ln in lines[1:]]
    return lines[0].split(","), [r[:3] for r in rows], np.array([[float(v) for v in r[3:]] for r in rows])


@pytest.mark.parametrize("name", make_golden.THIST_DECKS)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_simulate_writes_the_reference_T_hist(built_library, thesis, tmp_path, name, prec):
    """Output T_hist 1 without tracking (Grid::Output_T_hist, src/Grid.cpp:101-136, named as
    bin/Main.cpp:113-115 names it): th_simulate writes <name>T.hist.csv with the reference's
    header (x,y,z and the evaluation times, printed alike: the snapshot times, or every step
    the solidification loop ran) and rows (every point's coordinates as the reference prints
    them); each temperature, printed with 6 decimals, is within the temperature tolerance
    (1e-7 K / 0.01 K) and half a printed unit of the reference's.  th_T_hist returns the same
    history."""
    deck = make_golden.thist_deck(name)
    path = deck.write(str(tmp_path / name))
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    with thesis.Simulation(path, prec) as sim:
        sim.simulate()
        t, T = sim.T_hist()
    fname = str(g["file_name"])
    with open(os.path.join(os.path.dirname(path), "Data", fname)) as f:
        got = f.read()
    ref_head, ref_xyz, ref_T = _read_thist(bytes(g["file_bytes"]).decode())
    head, xyz, T_txt = _read_thist(got)
    assert head == ref_head
    assert xyz == ref_xyz
    tol = 1e-7 if prec == "fp64" else 0.01
    err = np.abs(T_txt - ref_T)
    assert float(err.max()) <= tol + 1e-6, (float(err.max()), np.unravel_index(np.argmax(err), err.shape))
    assert ["%f" % v for v in t] == ref_head[3:]
    assert T.shape == (len(t), len(ref_xyz))
    assert float(np.max(np.abs(T.T - T_txt))) <= 5e-7 + 1e-9


def _close_text(a, b, tol):
    """Two printed values: equal text, or within the tolerance and one printed unit."""
    if a == b:
        return True
    va, vb = float(a), float(b)
    unit = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb), 1e-300))) - 5)
    return abs(va - vb) <= tol + unit * (1 + 1e-9)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_custom_points_snapshots_match_the_reference(built_library, thesis, tmp_path, prec):
    """Domain: Custom File (src/Init.cpp:686-703, 816-857): the points file's points in place
    of a grid, evaluated like the grid (src/Run.cpp:61, 80-124).  Every snapshot's T at every
    point within 1e-7 K (FP64) / 0.01 K (FP32) of the reference's, and th_simulate writes the
    reference's Snapshot files: the same header, the points' coordinates as the reference
    prints them, each T within the tolerance and a printed unit."""
    deck = make_golden.custom_deck("custom_snapshot")
    path = deck.write(str(tmp_path / deck.name))
    g = np.load(os.path.join(HERE, "golden", "custom_snapshot.npz"))
    tol = 1e-7 if prec == "fp64" else 0.01
    with thesis.Simulation(path, prec) as sim:
        assert sim.pnum == len(deck.points)
        for i in range(3):
            T = sim.snapshot(i)
            err = float(np.max(np.abs(T - g[f"T{i}"])))
            assert err <= tol, (i, err)
        sim.simulate()
    data = os.path.join(os.path.dirname(path), "Data")
    names = [str(n) for n in g["names"]]
    assert sorted(os.listdir(data)) == names
    for i, nm in enumerate(names):
        ref = bytes(g[f"file{i}"]).decode().splitlines()
        with open(os.path.join(data, nm)) as f:
            got = f.read().splitlines()
        assert got[0] == ref[0] and len(got) == len(ref)
        for r, (a, b) in enumerate(zip(ref[1:], got[1:])):
            ra, rb = a.split(","), b.split(",")
            assert ra[:3] == rb[:3], (nm, r, a, b)
            assert _close_text(ra[3], rb[3], tol), (nm, r, a, b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_custom_points_solidify_without_tracking(built_library, thesis, tmp_path, prec):
    """A Solidification deck with custom points runs without tracking whatever its Tracking
    says (src/Run.cpp:391): every point every step (src/Run.cpp:409-467).  Its fields are the
    reference's within the parity tolerances (T 1e-7 / 0.01 K, tSol 1e-15 / 1e-8 s, G and V
    1e-9 / 1e-4 relative, the int-truncated dTdt within a unit beyond that), and the
    Solidification.Final file has the reference's header, rows and coordinates.  A point's
    G, V and dTdt may differ only where its two solidification times fall on different
    quadrature schedules: the node lists at the two times (th_nodes, bit for bit the
    reference's) differ, so the gradient sums run over different nodes (an ulp of t_sol
    can flip the schedule)."""
    deck = make_golden.custom_deck("custom_notrack")
    path = deck.write(str(tmp_path / deck.name))
    g = np.load(os.path.join(HERE, "golden", "custom_notrack.npz"))
    fp64 = prec == "fp64"
    rel = 1e-9 if fp64 else 1e-4
    with thesis.Simulation(path, prec) as sim:
        assert sim.info["tracking"] == 0                  # TH_TRACK_NONE
        sim.simulate()
        got = {f: sim.field(f) for f in ("T", "tSol", "G", "V", "dTdt")}
        off = np.zeros(len(deck.points), dtype=bool)
        for f in ("G", "V"):
            off |= np.abs(got[f] - g[f]) > rel * np.abs(g[f]) + 1e-300
        off |= np.abs(got["dTdt"] - g["dTdt"]) > rel * np.abs(g["dTdt"]) + 1.0
        unexplained = []
        for p in np.flatnonzero(off):
            a, b = sim.integrate(got["tSol"][p], True), sim.integrate(g["tSol"][p], True)
            if all(np.array_equal(a[k], b[k]) for k in a):
                unexplained.append(int(p))
    assert (g["tSol"] > 0).sum() > 30
    assert np.array_equal(got["tSol"] > 0, g["tSol"] > 0)
    assert float(np.max(np.abs(got["T"] - g["T"]))) <= (1e-7 if fp64 else 0.01)
    assert float(np.max(np.abs(got["tSol"] - g["tSol"]))) <= (1e-15 if fp64 else 1e-8)
    assert unexplained == [], (int(off.sum()), unexplained)
    ref = bytes(g["file0"]).decode().splitlines()
    with open(os.path.join(os.path.dirname(path), "Data", str(g["names"][0]))) as f:
        out = f.read().splitlines()
    assert out[0] == ref[0] and len(out) == len(ref)
    assert [r.split(",")[:3] for r in out[1:]] == [r.split(",")[:3] for r in ref[1:]]
