"""Per-point comparison of a GPU solidification run with the CPU oracle's run of the same
deck (test infrastructure).

Every difference is either within its stated tolerance or named by the reason it is
allowed; nothing is absorbed by a percentage.

* The molten-point set, the set of evaluated points, numMelt and the number of steps are
  identical.  The FP32 form takes each liquid decision within 1.5e-6 (T_L - T_0) of T_L on an
  FP64 sum, so its decisions are the FP64 form's, and the FP64 form's are the oracle's.
* T (at each point's last evaluation, the same step in both runs) within ``T_tol`` K.
* tSol within the secant's own sensitivity to its temperatures: the reference's secant
  (src/Grid.cpp:366-401) puts t_sol on the line through (t - dt, T_last) and (t, T), so
  errors e in the two temperatures move it by at most dt * 2 e / |T - T_last|.
* G, V, dT/dt, the unit gradient and eqFrac:
  - "matched": the GPU's value equals the oracle's evaluated at the GPU's own t_sol
    within ``rel`` (this isolates the gradient sums);
  - against the oracle's run within ``rel``, except at points named by one of two reasons,
    each excused only when the point's matched comparison passes (so the GPU's value is
    the oracle's at the GPU's t_sol, and the whole difference comes from t_sol):
    "schedule" - the two t_sol values lie on different quadrature schedules (the oracle's
    walk signature differs).  The reference's schedule changes discontinuously with t: its
    step-doubling test compares an accumulated interval sum with a threshold it equals in
    exact arithmetic, so the choice flips with the last bits of t_sol, and G jumps by the
    quadrature error (~1e-3);
    "t_sol" - on the same schedule, the oracle's own fields at the two t_sol values (which
    differ by less than the bound above) differ by more than ``rel``: a cooling rate that
    cancels strongly changes fast with t.
  - dT/dt is the reference's int-truncated cooling rate (src/Grid.cpp:535), so a relative
    error e in the untruncated rate moves it by at most e |dT/dt| + 1.
"""
from __future__ import annotations

import numpy as np

SOLID = ("G", "V", "dTdt", "Gx", "Gy", "Gz", "eqFrac")
TINY = np.finfo(np.float64).tiny        # the reference's DBL_MIN liquid marker


def _rel(a, b, floor=1e-300):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def _off(f, g, r, rel, dTdt_ref):
    """Mask of values g off from r by more than the field's tolerance."""
    if f == "dTdt":
        return np.abs(g - r) > rel * np.abs(r) + 1.0
    if f in ("Gx", "Gy", "Gz"):
        return np.abs(g - r) > rel
    if f == "eqFrac":
        return np.abs(g - r) > rel * np.maximum(np.abs(r), 1e-6)
    if f == "V":                # V = dTdt / G: the truncation unit of dTdt carries over
        return _rel(g, r) > 2 * rel + 1.0 / np.maximum(np.abs(dTdt_ref), 1.0)
    return _rel(g, r) > rel


def compare_solidification(o, ref: dict, gpu: dict, *, T_tol: float, rel: float, T_err: float, dt: float,
                           depth_tol: float = 0.0, threads: int = 0, max_listed: int = 8) -> dict:
    """ref / gpu: full per-point fields (the keys present in both are compared) plus "steps".
    T_err: the bound on each evaluated temperature's error used for the tSol sensitivity;
    depth_tol: absolute depth tolerance (m) on top of 1e-12 relative.
    Returns a report whose "violations" list is empty when the runs agree."""
    rep = {"violations": [], "counts": {}}
    bad = rep["violations"]

    def fail(what, idx=None, **extra):
        item = {"check": what}
        if idx is not None:
            idx = np.asarray(idx)
            item["n"] = int(idx.size)
            item["points"] = [int(i) for i in idx[:max_listed]]
        item.update(extra)
        bad.append(item)

    if ref.get("steps") is not None and gpu.get("steps") != ref["steps"]:
        fail("steps", steps_ref=int(ref["steps"]), steps_gpu=int(gpu["steps"]))
    a, b = ref["output_flag"] > 0, gpu["output_flag"] > 0
    d = np.flatnonzero(a != b)
    rep["counts"]["molten"] = int(a.sum())
    if d.size:
        band = o.field("band")
        fail("molten set", d, band_of_listed=[float(band[i]) for i in d[:max_listed]])
    ea, eb = ref["T"] != 0, gpu["T"] != 0
    d = np.flatnonzero(ea != eb)
    rep["counts"]["evaluated"] = int(ea.sum())
    if d.size:
        fail("evaluated set", d)
    common = ea & eb
    dT = np.abs(ref["T"][common] - gpu["T"][common])
    rep["max_dT"] = float(dT.max()) if dT.size else 0.0
    if dT.size and rep["max_dT"] > T_tol:
        fail("T", np.flatnonzero(common)[dT > T_tol], max_dT=rep["max_dT"], tol=T_tol)
    if "numMelt" in ref and "numMelt" in gpu:
        d = np.flatnonzero(ref["numMelt"] != gpu["numMelt"])
        if d.size:
            fail("numMelt", d)
    if "depth" in ref and "depth" in gpu:
        # depth = (layer + (T_L - T_l) / (T_s - T_l)) z spacing: an error e in either
        # temperature moves it by at most 2 e / |T_s - T_l| layers
        dd = np.abs(ref["depth"] - gpu["depth"])
        rep["max_ddepth"] = float(dd.max())
        d = np.flatnonzero(dd > 1e-12 * np.abs(ref["depth"]) + depth_tol)
        if d.size:
            fail("depth", d, max_ddepth=rep["max_ddepth"])
    if "tSol" not in ref or "tSol" not in gpu:
        return rep

    ts_r, ts_g = ref["tSol"], gpu["tSol"]
    solid = np.flatnonzero((ts_r != 0) | (ts_g != 0))
    d = solid[(ts_r[solid] == 0) != (ts_g[solid] == 0)]
    if d.size:
        fail("solidified set", d)
    solid = solid[(ts_r[solid] != 0) & (ts_g[solid] != 0)]
    # points liquid when the run stopped keep the reference's markers (G = V = DBL_MIN,
    # eqFrac = -1, src/Grid.cpp:300-311) over an earlier solidification's values
    if "G" in ref and "G" in gpu:
        mr, mg = ref["G"][solid] == TINY, gpu["G"][solid] == TINY
        if (mr != mg).any():
            fail("liquid markers", solid[mr != mg])
        rep["counts"]["liquid_at_end"] = int(mr.sum())
        solid = solid[~mr & ~mg]
    rep["counts"]["solidified"] = int(solid.size)
    sdT = np.abs(o.field("sol_dT")[solid])
    dts = np.abs(ts_r[solid] - ts_g[solid])
    bound = dt * 2.0 * T_err / np.maximum(sdT, 1e-300) + 4 * np.spacing(np.abs(ts_r[solid]))
    rep["max_dtSol"] = float(dts.max()) if dts.size else 0.0
    over = dts > bound
    if over.any():
        fail("tSol", solid[over], max_over_bound=float(np.max(dts[over] / bound[over])))

    # matched: the oracle's fields at the GPU's own t_sol
    want = o.solid_fields_many(solid, ts_g[solid], threads=threads)
    fields = [f for f in SOLID if f in gpu and f in ref]
    for f in fields:
        bad_f = _off(f, gpu[f][solid], want[f], rel, want["dTdt"])
        if bad_f.any():
            fail(f"{f} at the GPU's t_sol", solid[bad_f], max_rel=float(np.max(_rel(gpu[f][solid], want[f])[bad_f])))
    rep["matched_max_rel"] = {f: float(np.max(_rel(gpu[f][solid], want[f]))) if solid.size else 0.0
                              for f in fields if f in ("G", "V", "dTdt")}

    # against the oracle's run: points off by more than rel need a reason
    off = np.zeros(solid.size, dtype=bool)
    for f in ("G", "V", "dTdt"):
        if f in fields:
            off |= _off(f, gpu[f][solid], ref[f][solid], rel, ref["dTdt"][solid] if "dTdt" in ref else 1.0)
    idx = np.flatnonzero(off)
    rep["counts"]["off_by_schedule"] = rep["counts"]["off_by_tsol"] = 0
    if idx.size:
        pts = solid[idx]
        same = o.schedule(ts_r[pts], True, threads=threads) == o.schedule(ts_g[pts], True, threads=threads)
        rep["counts"]["off_by_schedule"] = int((~same).sum())
        j = idx[same]
        if j.size:
            # on the same schedule the oracle's own change between the two times must exceed
            # rel (the part the GPU's sums could add is <= rel, by the matched check)
            own = o.solid_fields_many(solid[j], ts_r[solid[j]], threads=threads)
            moved = np.zeros(j.size, dtype=bool)
            for f in ("G", "dTdt"):
                if f in fields:
                    moved |= _off(f, want[f][j], own[f], rel, own["dTdt"])
            rep["counts"]["off_by_tsol"] = int(moved.sum())
            if (~moved).any():
                k = j[~moved]
                fail("G/V/dTdt against the oracle's run, same schedule, not explained by t_sol", solid[k],
                     dtSol=[float(ts_g[solid[i]] - ts_r[solid[i]]) for i in k[:max_listed]])
    return rep


def compare_rdf(o, ref, gpu, *, rel: float, T_err: float, dt: float, threads: int = 0, max_listed: int = 8) -> dict:
    """The reduced data of a run (Output RDF 1): ref = the oracle's (counts, vals, dT), gpu =
    the library's (counts, vals).  Per point the same numbers of melting times, solidification
    times and cooling rates; melting times (step times) equal; each solidification time
    within the secant bound above; each cooling rate within ``rel`` (+ 1, its truncation) of
    the oracle's at the GPU's own solidification time, and of the oracle's own except where
    named by "schedule" or "t_sol" as for the fields."""
    rep = {"violations": [], "counts": {}}
    bad = rep["violations"]
    cr_, vr, dT = ref
    cg, vg = gpu
    d = np.flatnonzero(np.any(cr_ != cg, axis=1))
    if d.size:
        bad.append({"check": "RDF counts", "n": int(d.size), "points": [int(i) for i in d[:max_listed]]})
        return rep
    n = cr_.sum(axis=1)
    start = np.concatenate(([0], np.cumsum(n)[:-1]))
    pts = np.flatnonzero(n)
    tm_i = np.concatenate([start[p] + np.arange(cr_[p, 0]) for p in pts]) if pts.size else np.zeros(0, int)
    tl_i = np.concatenate([start[p] + cr_[p, 0] + np.arange(cr_[p, 1]) for p in pts]) if pts.size else np.zeros(0, int)
    cr_i = (np.concatenate([start[p] + cr_[p, 0] + cr_[p, 1] + np.arange(cr_[p, 2]) for p in pts]) if pts.size
            else np.zeros(0, int))
    sp = np.repeat(np.arange(cr_.shape[0]), cr_[:, 1])          # the point of each solidification
    rep["counts"].update(melts=int(tm_i.size), solidifications=int(tl_i.size))
    d = np.flatnonzero(vg[tm_i] != vr[tm_i])
    if d.size:
        bad.append({"check": "melting times", "n": int(d.size)})
    tl_r, tl_g, c_r, c_g = vr[tl_i], vg[tl_i], vr[cr_i], vg[cr_i]
    bound = dt * 2.0 * T_err / np.maximum(np.abs(dT), 1e-300) + 4 * np.spacing(np.abs(tl_r))
    over = np.abs(tl_g - tl_r) > bound
    if over.any():
        bad.append({"check": "solidification times", "n": int(over.sum()), "points": [int(i) for i in sp[over][:max_listed]]})
    want = o.solid_fields_many(sp, tl_g, threads=threads)["dTdt"] if sp.size else np.zeros(0)
    off = _off("dTdt", c_g, want, rel, want)
    if off.any():
        bad.append({"check": "cooling rate at the GPU's time", "n": int(off.sum()),
                    "points": [int(i) for i in sp[off][:max_listed]]})
    off = _off("dTdt", c_g, c_r, rel, c_r)
    rep["counts"]["off_by_schedule"] = rep["counts"]["off_by_tsol"] = 0
    j = np.flatnonzero(off)
    if j.size:
        same = o.schedule(tl_r[j], True, threads=threads) == o.schedule(tl_g[j], True, threads=threads)
        rep["counts"]["off_by_schedule"] = int((~same).sum())
        k = j[same]
        if k.size:
            own = o.solid_fields_many(sp[k], tl_r[k], threads=threads)["dTdt"]
            moved = _off("dTdt", want[k], own, rel, own)
            rep["counts"]["off_by_tsol"] = int(moved.sum())
            if (~moved).any():
                bad.append({"check": "cooling rate against the oracle's, not explained", "n": int((~moved).sum()),
                            "points": [int(i) for i in sp[k[~moved]][:max_listed]]})
    return rep


def read_rrdf_bin(buf: bytes) -> dict:
    """Stork's doubly reduced data in the reference's binary layout (Grid::Output_RRDF_bin,
    src/Grid.cpp:241-273), little-endian: the row count and the grid's three point counts
    (uint32), its x, y, z minima, x resolution and liquidus (double), then the rows' indices
    (3 x uint32), times (2 x double) and vertex temperatures (16 x double), block by block.
    Raises if the buffer is not exactly that long."""
    head = np.frombuffer(buf[:16], dtype="<u4")
    n = int(head[0])
    sizes = (16, 40, 12 * n, 16 * n, 128 * n)
    if len(buf) != sum(sizes):
        raise ValueError(f"{len(buf)} bytes for {n} rows, expected {sum(sizes)}")
    o = np.cumsum((0,) + sizes)
    return {"rows": n, "extent": head[1:4].copy(), "geometry": np.frombuffer(buf[o[1]:o[2]], dtype="<f8").copy(),
            "idx": np.frombuffer(buf[o[2]:o[3]], dtype="<u4").reshape(n, 3),
            "ts": np.frombuffer(buf[o[3]:o[4]], dtype="<f8").reshape(n, 2),
            "Ts": np.frombuffer(buf[o[4]:o[5]], dtype="<f8").reshape(n, 16)}
