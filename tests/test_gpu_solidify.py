"""GPU Solidification mode (NoTracking / Volume / Surface, one and four beams, reflecting
planes) against the CPU oracle and the reference's golden runs, through the C ABI.

Every point is compared (tests/parity.py states the rules): identical molten and evaluated
sets, numMelt and step counts in both precisions; T within 1e-7 K (FP64) and 0.01 K (FP32);
tSol within the secant's sensitivity to the temperatures' error; G, V, dT/dt, the unit
gradient and eqFrac within 1e-9 (FP64) and 1e-4 (FP32) relative of the oracle at the GPU's
own t_sol, and of the oracle's run except where a point is excused by name (its two t_sol
values lie on different quadrature schedules, or the oracle's own fields change by more
than the tolerance between them)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402
import parity  # noqa: E402

pytestmark = pytest.mark.gpu
CASES = sorted(make_golden.RUNS)
# tolerances per precision: T (K), relative fields, the temperature error bound for tSol (K),
# depth (m)
TOL = {"fp64": dict(T_tol=1e-7, rel=1e-9, T_err=1e-9, depth_tol=1e-15),
       "fp32": dict(T_tol=0.01, rel=1e-4, T_err=1e-3, depth_tol=1e-8)}


def _fields(deck):
    return ["T", "output_flag"] + [f for f in ("tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac", "numMelt",
                                               "depth") if deck.outputs.get(f)]


def _gpu_run(thesis, path, prec, fields, max_steps=0, rdf=False):
    with thesis.Simulation(path, prec) as sim:
        steps = sim.solidify(max_steps=max_steps)
        out = {f: sim.field(f) for f in fields}
        if rdf:
            out["rdf"] = sim.rdf()
    out["steps"] = steps
    return out


@pytest.fixture(scope="module")
def runs(built_library, thesis, oracle, tmp_path_factory):
    """Every case run once on the oracle and on the GPU in both precisions."""
    out = {}
    base = tmp_path_factory.mktemp("sol")
    for tag in CASES:
        deck = make_golden.run_deck(tag)
        path = deck.write(str(base / tag))
        o = oracle(path)
        steps = o.solidify(threads=8)
        ref = {f: o.field(f) for f in _fields(deck)}
        ref["steps"] = steps
        rdf = bool(deck.outputs.get("RDF"))
        if rdf:
            ref["rdf"] = o.rdf()
        gpu = {prec: _gpu_run(thesis, path, prec, _fields(deck), rdf=rdf) for prec in ("fp64", "fp32")}
        out[tag] = (deck, o, ref, gpu)
    return out


@pytest.mark.parametrize("tag", CASES)
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_run_matches_oracle(runs, tag, prec):
    deck, o, ref, gpu = runs[tag]
    rep = parity.compare_solidification(o, ref, gpu[prec], dt=deck.timestep, **TOL[prec])
    assert rep["counts"]["molten"] > 1000
    assert rep["violations"] == [], rep


@pytest.mark.parametrize("tag", [t for t in CASES if t.endswith("_rdf")])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_rdf_matches_oracle(runs, tag, prec):
    """The reduced data (Output RDF 1): per point the same melting / solidification / cooling
    rate counts, melting times equal, and the solidification times and cooling rates of every
    melt event (not only the last) by the rules of the fields (tests/parity.py)."""
    deck, o, ref, gpu = runs[tag]
    tol = TOL[prec]
    rep = parity.compare_rdf(o, ref["rdf"], gpu[prec]["rdf"], rel=tol["rel"], T_err=tol["T_err"], dt=deck.timestep)
    assert rep["violations"] == [], rep
    assert rep["counts"]["solidifications"] > 1000
    if deck.tracking == "Surface":                 # only Surface tracking records melting times
        assert rep["counts"]["melts"] == rep["counts"]["solidifications"]
    else:
        assert rep["counts"]["melts"] == 0
    g = np.load(os.path.join(HERE, "golden", f"run_{tag}.npz"))     # and the reference's own counts
    assert np.array_equal(gpu[prec]["rdf"][0].ravel(), g["rdf_counts"])


@pytest.mark.parametrize("tag", CASES)
def test_fp64_run_matches_reference_golden(runs, tag):
    """The FP64 run against the unmodified reference's own run (golden fixture): the molten
    set bit for bit, T / tSol / numMelt / depth to 1e-12, and G / V / dT/dt to 1e-9 relative
    except at points whose GPU and reference t_sol lie on different quadrature schedules
    (where the GPU equals the oracle at the GPU's t_sol)."""
    g = dict(np.load(os.path.join(HERE, "golden", f"run_{tag}.npz")))
    deck, o, ref, gpu = runs[tag]
    run = gpu["fp64"]
    assert np.array_equal(np.packbits(run["output_flag"] > 0), g["mask"])
    sub = g["sample"]
    for f in ("T", "tSol", "numMelt", "depth"):
        if f + "_sample" in g:
            np.testing.assert_allclose(run[f][sub], g[f + "_sample"], rtol=1e-12, atol=1e-12, err_msg=f)
    if "tSol_sample" not in g:
        return
    ts_g, ts_ref = run["tSol"][sub], g["tSol_sample"]
    solid = (ts_ref != 0) & (g["G_sample"] != parity.TINY) if "G_sample" in g else ts_ref != 0
    off = np.zeros(sub.size, dtype=bool)
    for f in ("G", "V", "dTdt"):
        if f + "_sample" in g:
            r, v = g[f + "_sample"], run[f][sub]
            slack = 1.0 if f == "dTdt" else 0.0
            off |= solid & (np.abs(v - r) > 1e-9 * np.abs(r) + slack)
    idx = np.flatnonzero(off)
    if idx.size:
        assert np.all(o.schedule(ts_g[idx], True) != o.schedule(ts_ref[idx], True)), sub[idx]
        want = o.solid_fields_many(sub[idx], ts_g[idx])
        np.testing.assert_allclose(run["G"][sub[idx]], want["G"], rtol=1e-9)


@pytest.fixture(scope="module")
def bcs_run(built_library, oracle, tmp_path_factory):
    """The small Surface deck with four reflecting planes (two reflections): every node list
    carries its image copies, several hundred nodes."""
    d = make_golden.run_deck("small_surface")
    d.name = "small_surface_bcs"
    d.bcs = {"X_min": -0.1e-3, "X_max": 0.5e-3, "Y_min": -0.15e-3, "Z_min": -0.2e-3, "Reflections": 2}
    path = d.write(str(tmp_path_factory.mktemp("bcs") / d.name))
    o = oracle(path)
    steps = o.solidify(threads=8)
    ref = {f: o.field(f) for f in _fields(d)}
    ref["steps"] = steps
    n = max(len(o.nodes(i * 1e-4, True)["xb"]) for i in range(1, 40))
    return d, path, o, ref, n


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_lists_past_the_staged_copy(bcs_run, thesis, monkeypatch, prec):
    """With at most 128 nodes of each list staged in shared memory, the tracking passes read
    the rest of the list from the node window (the path of lists longer than the stage).
    FP64 lanes keep their summation order, so that run is bit-identical to the fully staged
    one; both precisions meet the oracle comparison above on a deck with image copies."""
    deck, path, o, ref, n_max = bcs_run
    assert n_max > 256, n_max
    runs = {}
    for cap in ("", "128"):
        monkeypatch.setenv("THESIS_GB300_STAGE_CAP", cap)
        runs[cap] = _gpu_run(thesis, path, prec, _fields(deck))
    if prec == "fp64":
        for f in runs["128"]:
            assert np.array_equal(runs["128"][f], runs[""][f]), f
    for cap in ("", "128"):
        rep = parity.compare_solidification(o, ref, runs[cap], dt=deck.timestep, **TOL[prec])
        assert rep["violations"] == [], (cap, rep)
