"""Parity at the benchmarked sizes, through the C ABI, against the CPU oracle run on all host
cores in the same process.

* the headline Surface deck (500 x 500 x 100, 25 M points, 31,769 timesteps) in FP64 and
  FP32: every point compared as in test_gpu_solidify (tests/parity.py);
* the four-beam Volume deck (400 x 400 x 80): its first 2,000 timesteps;
* the headline deck with Stork tracking: the doubly reduced data of its first 300
  timesteps (about 230,000 rows);
* eight decks of the 256-deck snapshot sweep, evaluated as part of the whole batch;
* the calibration deck (300 x 300 x 60, 4,096 probes x 3 times): the adjoint gradient
  against central differences of the oracle for P, efficiency, the widths, alpha and the ten
  path vertices with the largest gradients.

Each case runs the oracle's whole problem; together they take a few minutes on the GPU
box's host cores."""
import copy
import os

import numpy as np
import pytest

import parity

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 1
TOL = {"fp64": dict(T_tol=1e-7, rel=1e-9, T_err=1e-9, depth_tol=1e-15),
       "fp32": dict(T_tol=0.01, rel=1e-4, T_err=1e-3, depth_tol=1e-8)}
FIELDS = ("T", "output_flag", "tSol", "G", "V", "dTdt")


@pytest.fixture(scope="module")
def surface(built_library, decks, oracle, tmp_path_factory):
    deck = decks.surface_serpentine()
    path = deck.write(str(tmp_path_factory.mktemp("surf") / "surface"))
    o = oracle(path)
    steps = o.solidify(threads=THREADS)
    ref = {f: o.field(f) for f in FIELDS}
    ref["steps"] = steps
    return deck, path, o, ref


@pytest.fixture(scope="module")
def volume(built_library, decks, oracle, tmp_path_factory):
    deck = decks.volume_multibeam()
    path = deck.write(str(tmp_path_factory.mktemp("vol") / "volume"))
    o = oracle(path)
    steps = o.solidify(threads=THREADS, max_steps=2000)
    ref = {f: o.field(f) for f in FIELDS}
    ref["steps"] = steps
    return deck, path, o, ref


@pytest.fixture(scope="module")
def stork(built_library, decks, oracle, tmp_path_factory):
    deck = decks.surface_serpentine()
    deck.tracking, deck.name = "Stork", "surface_serpentine_stork"
    path = deck.write(str(tmp_path_factory.mktemp("stork") / "stork"))
    o = oracle(path)
    steps = o.solidify(threads=THREADS, max_steps=300)
    return path, steps, o.rrdf()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stork_prefix_full_size(stork, thesis, prec):
    """The same rows in the same order (cell indices and step times exactly), the 16 vertex
    temperatures within the temperature tolerance (1e-7 K / 0.01 K)."""
    path, steps, (ri, rt, rT) = stork
    with thesis.Simulation(path, prec) as sim:
        assert sim.solidify(max_steps=300) == steps
        gi, gt, gT = sim.rrdf()
    assert ri.shape[0] > 100000
    assert gi.shape == ri.shape
    assert np.array_equal(gi, ri) and np.array_equal(gt, rt)
    err = float(np.max(np.abs(gT - rT)))
    assert err <= TOL[prec]["T_tol"], err


def _gpu(thesis, path, prec, max_steps=0):
    with thesis.Simulation(path, prec) as sim:
        steps = sim.solidify(max_steps=max_steps)
        out = {f: sim.field(f) for f in FIELDS}
    out["steps"] = steps
    return out


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_surface_serpentine_full_run(surface, thesis, prec):
    deck, path, o, ref = surface
    assert ref["steps"] == 31769
    rep = parity.compare_solidification(o, ref, _gpu(thesis, path, prec), dt=deck.timestep, threads=THREADS,
                                        **TOL[prec])
    assert rep["counts"]["solidified"] > 1_000_000
    assert rep["violations"] == [], rep


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_volume_multibeam_first_2000_steps(volume, thesis, prec):
    deck, path, o, ref = volume
    assert ref["steps"] == 2000
    rep = parity.compare_solidification(o, ref, _gpu(thesis, path, prec, max_steps=2000), dt=deck.timestep,
                                        threads=THREADS, **TOL[prec])
    assert rep["counts"]["solidified"] > 50_000
    assert rep["violations"] == [], rep


def _stats_run(thesis, path, prec, max_steps):
    with thesis.Simulation(path, prec) as sim:
        steps = sim.solidify(max_steps=max_steps)
        out = {f: sim.field(f) for f in FIELDS}
        st = sim.run_stats()
    return steps, out, st


@pytest.mark.parametrize("which,max_steps", [("surface", 0), ("volume", 2000)])
def test_record_high_water_mark_ends_launches_early(surface, volume, thesis, monkeypatch, which, max_steps):
    """A record high-water mark of 100 records (THESIS_GB300_REC_HIGH_WATER; the buffers
    keep their size) ends tracking launches early, at the first blocks' record flushes -
    Surface: a block whose flush passes the mark asks the next step to end the launch,
    through the step word; Volume: the step's finisher reads the record count - and the host
    starts the next launch from the step reached.  The run does the same work either way: in
    FP64 (whose records are solidified alike in any buffer; FP32 runs pick a record's FP64
    path by the size of its buffer's queues) every field is the same bits as the run's with
    the normal mark."""
    path = (surface if which == "surface" else volume)[1]
    steps, ref, st0 = _stats_run(thesis, path, "fp64", max_steps)
    monkeypatch.setenv("THESIS_GB300_REC_HIGH_WATER", "100")
    got_steps, got, st = _stats_run(thesis, path, "fp64", max_steps)
    monkeypatch.delenv("THESIS_GB300_REC_HIGH_WATER")
    assert got_steps == steps
    assert st["records"] == st0["records"] > 100_000
    assert st["windows"] > st0["windows"] + 3, (st["windows"], st0["windows"])   # launches that ended early
    for f in FIELDS:
        assert np.array_equal(got[f], ref[f], equal_nan=True), f


@pytest.fixture(scope="module")
def sweep(built_library, decks, tmp_path_factory):
    base = tmp_path_factory.mktemp("sweep")
    ds = decks.snapshot_sweep()
    paths = [d.write(str(base / d.name)) for d in ds]
    sizes = [np.prod([ax.num for ax in d.axes]) for d in ds]
    # every 32nd deck and the largest one
    pick = sorted(set(list(range(0, len(ds), 32)) + [int(np.argmax(sizes))]))[:8]
    return ds, paths, pick


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-7), ("fp32", 0.01)])
def test_sweep_decks_in_the_whole_batch(sweep, thesis, oracle, prec, tol):
    ds, paths, pick = sweep
    with thesis.Batch(paths, prec) as b:
        if prec == "fp32":
            b.autotune(0)
        T = b.snapshot(0)
        off = b.offsets
    for i in pick:
        ref = oracle(paths[i]).snapshot(0, threads=THREADS)
        got = T[off[i]:off[i + 1]]
        assert got.size == ref.size
        assert np.max(np.abs(got - ref)) <= tol, (ds[i].name, np.max(np.abs(got - ref)))


# ------------------------------------------------------------------ adjoint (calibration)
def _deck_at(deck, theta):
    """The calibration deck with theta = (P, efficiency, Width_X, Width_Y, Depth_Z, alpha,
    then x, y of every path vertex after the origin, metres) written into its files."""
    d = copy.deepcopy(deck)
    b = d.beams[0]
    b.power, b.efficiency, b.width_x, b.width_y, b.depth_z = (float(v) for v in theta[:5])
    m = d.material
    m.k = float(theta[5]) * m.rho * m.c
    segs = []
    for j, s in enumerate(d.paths[0]):
        segs.append((s[0], float(theta[6 + 2 * j]) * 1e3, float(theta[7 + 2 * j]) * 1e3, s[3], s[4], s[5]))
    d.paths = [segs]
    return d


def test_adjoint_calibration_against_oracle_differences(built_library, thesis, decks, oracle, tmp_path):
    deck = decks.adjoint_calibration()
    path = deck.write(str(tmp_path / "calib"))
    probes, times = decks.adjoint_probes(deck)
    probes = np.asarray(probes, dtype=np.int64)
    n = [0]

    def oracle_T(theta):
        n[0] += 1
        o = oracle(_deck_at(deck, theta).write(str(tmp_path / f"fd{n[0]}")))
        return o, np.stack([o.calc_T(t, probes, threads=THREADS) for t in times])

    with thesis.Adjoint(path, probes, times, "fp64") as a64, thesis.Adjoint(path, probes, times, "fp32") as a32:
        theta = a64.params()
        assert theta.size == 6 + 2 * len(deck.paths[0])
        # the deck written back from its own theta is the deck
        o0, T0 = oracle_T(theta)
        np.testing.assert_allclose(a64.forward(theta), T0, rtol=0, atol=1e-7)
        tt = theta.copy()
        tt[0] *= 1.1
        tt[2] *= 0.9
        tt[5] *= 1.05
        target = oracle_T(tt)[1]
        grads = {}
        for prec, a in (("fp64", a64), ("fp32", a32)):
            T = a.forward(theta)
            grads[prec] = a.backward(2.0 * (T - target))
        # a vertex that ends or starts a zero-length segment (the serpentine's first move from
        # the origin to its start point) sits on a kink: moving it either way lengthens that
        # segment, so no central difference exists there
        xy = np.concatenate([[[0.0, 0.0]], theta[6:].reshape(-1, 2)])
        zero = np.flatnonzero(np.hypot(*np.diff(xy, axis=0).T) == 0.0)          # segment k ends at vertex k
        kinked = set(int(k) for k in zero) | set(int(k) - 1 for k in zero if k > 0)
        order = [int(v) for v in np.argsort(-np.abs(grads["fp64"][6:])) if int(v) // 2 not in kinked]
        verts = [6 + v for v in order[:10]]
        checked = []
        for j in list(range(6)) + verts:
            fd = None
            for h_rel in (1e-6, 1e-7, 1e-8):
                h = h_rel * max(abs(theta[j]), 1e-4)
                tp, tm = theta.copy(), theta.copy()
                tp[j] += h
                tm[j] -= h
                op, Tp = oracle_T(tp)
                om, Tm = oracle_T(tm)
                # a central difference is the derivative only if the quadrature schedule is the
                # same at both ends (the adjoint holds the walk's discrete choices fixed)
                if all(op.schedule(t)[0] == o0.schedule(t)[0] == om.schedule(t)[0] for t in times):
                    fd = (np.sum((Tp - target) ** 2) - np.sum((Tm - target) ** 2)) / (2 * h)
                    break
            assert fd is not None, f"parameter {j}: every step crosses a schedule change"
            for prec in ("fp64", "fp32"):
                g = grads[prec][j]
                assert abs(g - fd) <= 1e-4 * abs(fd), (prec, j, g, fd)
            checked.append(j)
        assert len(checked) == 16
