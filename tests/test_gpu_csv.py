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
