"""Benchmark of the 3DThesis hot path on GB300: point x node pairs per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload surface_serpentine|volume_multibeam|snapshot_raster|snapshot_sweep|
                                adjoint_calibration]
                    [--precision fp32|fp64] [--tile KPxKCH]

Workloads (synthetic decks in the reference's own input format, 3dthesis_gb300/decks.py):
  surface_serpentine (default; the metric's configuration) - Solidification mode, Surface
      tracking: 50 x 5 mm serpentine, hatch 80 um, 0.8 m/s, 200 W, 500x500x100 grid at
      10 um (25 M points), dt = 1e-5 s, outputs tSol/G/V/dTdt.  One step = the whole run
      (31,769 timesteps to the finish test) from t = 0.
  volume_multibeam - Solidification mode, Volume tracking, four beams on seeded rotated
      serpentines over a 400x400x80 grid, dt = 5e-6 s.  One step = the whole run.
  snapshot_raster - Snapshots mode: 10 x 2 mm raster on a 200x100x40 grid, snapshots at
      25/50/100 %.  One step = the three snapshots.
  snapshot_sweep - 256 independent Snapshots decks of uneven sizes (a process-parameter
      sweep) evaluated as one batch: one step = one CUDA-graph replay of the batch snapshot.
  adjoint_calibration - probe temperatures of the Surface deck's path on a 300x300x60 grid
      and their gradient over all parameters: one step = forward + adjoint.

``value`` = point x node pairs of the step / the step's time with the deck resident in HBM
(inputs on the device before timing; L2 flushed with a 256 MiB write before each step,
outside the timed region; times from CUDA events on the library's stream).
``e2e`` times what a user calls through the C ABI with host buffers: context creation from
the deck files (parse + upload), the run, and the D2H copy of the output fields into
pinned memory.  ``cpu_baseline`` and ``--impl reference`` time the CPU oracle (the
reference's algorithm restated in C++, OpenMP over all host cores): for the Surface deck
the whole run (the same work as one GPU step, ~15 s), for the other solidification decks
the run from t = 0 until the timestep that ends past a 15 s budget, for snapshots whole
snapshots within ~15 s.  Solidification runs also time the plain FP64 form of the same run
(``detail.fp64_form``).  The roofline's peak uses the SM count and the MUFU ex2 / FP32
rates measured on the device by probe kernels (th_device_rates).

Under torchrun each rank runs the same per-GPU workload (weak scaling, no collective on
the data path), except the 256-deck sweep, whose decks are split across the ranks
(th.shard_decks; strong scaling); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "point-node pairs/s"
# FP32 lane-operations the tiled kernel issues per compensated pair: per node and thread
# 6 scalar ops shared by its 4 points, per packed pair of points 8 f32x2 ops (2 lanes each)
# -> (6 + 2 x 16) / 4 = 9.5
FP32_OPS_KAHAN = 9.5
OPS_PER_PAIR = 16           # algorithmic work of a pair: 15 floating-point operations + 1 exp
# DRAM bytes (read + write) of one launch of the dominant kernel, from one ncu capture of
# that kernel on that deck (dram__bytes_read.sum + dram__bytes_write.sum)
NCU_TRAFFIC = {"snapshot_raster": 21248, "surface_serpentine": 5916819, "volume_multibeam": 38883143}

DECK_TEXT = {
    "surface_serpentine": "Solidification/Surface; 50 tracks x 5 mm serpentine, hatch 80 um, 0.8 m/s, P=200 W, "
                          "eta=0.35, 50/50/1 um; grid 500x500x100 at 10 um; dt=1e-5 s; outputs tSol,G,V,dTdt",
    "volume_multibeam": "Solidification/Volume, 4 beams (seed 0), each a serpentine of 20 x 3 mm tracks rotated "
                        "by U[0,pi), v~U(0.5,1.5) m/s, P~U(150,400) W, widths~U(40,100) um; grid 400x400x80 at "
                        "10 um; dt=5e-6 s; outputs tSol,G,V,dTdt",
    "snapshot_raster": "Snapshots; 10 tracks x 2 mm, hatch 0.1 mm, 1.0 m/s, P=200 W, eta=0.35, 50/50/1 um; "
                       "grid 200x100x40 at 10 um; snapshots at 25/50/100 %",
    "snapshot_sweep": "256 independent Snapshots decks (seed 0): P~U(100,400) W, v~U(0.5,2) m/s, "
                      "width~U(40,120) um, U{1..30} x 2 mm tracks, grids U{50..400}^2 x U{10..60} at 10 um, "
                      "snapshot at 100 %",
    "adjoint_calibration": "serpentine path and material of the Surface deck on a 300x300x60 grid; loss = sum "
                           "(T - T_target)^2 over 4096 seeded probes x 3 times (0.05/0.15/0.30 s), target from "
                           "P x 1.1, Width_X x 0.9, alpha x 1.05; one step = forward + adjoint over all 208 "
                           "parameters",
}


# Solidification workloads whose whole run takes the CPU oracle under a minute on the GPU
# box's host cores: their CPU legs time the whole run (the same work as one GPU step);
# the others time the run from t = 0 up to a time budget.
CPU_WHOLE_RUN = {"surface_serpentine"}
_RATES = None


def device_rates(th):
    """SM count and measured MUFU ex2 / FP32 FMA rates per SM per clock (probe kernels)."""
    global _RATES
    if _RATES is None:
        _RATES = th.device_rates()
    return _RATES


def fp32_peak_pairs(th, clk_mhz):
    """The FP32 / MUFU issue bound of the FP32 pair arithmetic, pairs/s, and its basis."""
    r = device_rates(th)
    per_clk = min(r["fma_per_sm_clk"] / FP32_OPS_KAHAN, r["ex2_per_sm_clk"])
    basis = (f"{r['sm_count']} SMs (read from the device) x {clk_mhz:.0f} MHz x min({r['fma_per_sm_clk']:.1f} "
             f"FP32 lane-ops/{FP32_OPS_KAHAN}, {r['ex2_per_sm_clk']:.2f} MUFU ex2) pairs/clk, rates measured "
             f"with probe kernels")
    return r["sm_count"] * clk_mhz * 1e6 * per_clk, basis


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines, self.t = index, None, [], None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits", "-lms", "200"],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=lambda: [self.lines.append(l.strip()) for l in self.proc.stdout],
                                  daemon=True)
        self.t.start()

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_deck(name: str, tmp: str):
    decks = importlib.import_module("3dthesis_gb300.decks")
    deck = getattr(decks, name)()
    if isinstance(deck, list):
        return deck, [d.write(os.path.join(tmp, name, d.name)) for d in deck]
    return deck, deck.write(os.path.join(tmp, name))


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    """The slowest rank's time (every rank gets it); NCCL reduces on the GPU, gloo on the CPU."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ solidification workload
def run_solidification(args, th, torch, dev, path, deck, world):
    sim = th.Simulation(path, args.precision)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        sim.reset()
        sim.solidify()
    stats = []
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    wall = []
    for _ in range(args.steps):
        sim.reset()
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.solidify()
        torch.cuda.synchronize()
        wall.append(time.perf_counter() - t0)
        stats.append(sim.run_stats())
    clk = clocks.stop()
    barrier(world)
    dev_s = [s["ms_device"] / 1e3 for s in stats]
    total_s = allreduce_max(sum(dev_s), world)
    pairs = stats[-1]["pairs_total"]
    value = pairs * args.steps * world / total_s
    st = stats[-1]
    launches = int(st["windows"] * 2 + st["windows"] * 2 + 2)   # node window + tracking, latest-pass + solidify

    # end to end: deck files -> context -> run -> output fields in pinned host memory
    outs = [f for f in ("tSol", "G", "V", "dTdt") if deck.outputs.get(f)]
    pinned = torch.empty(sim.pnum, dtype=torch.float64, pin_memory=True).numpy()
    e2e_t = []
    for _ in range(max(1, min(args.steps, 2))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with th.Simulation(path, args.precision) as s2:
            s2.solidify()
            for f in outs:
                s2._check(s2._lib.th_field(s2._ctx, f.encode(), pinned.ctypes.data))
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = allreduce_max(statistics.median(e2e_t), world)
    e2e = {"value": pairs * world / e2e_s, "unit": "pairs/s",
           "h2d_bytes_per_step": int(sum(len(p) for p in deck.paths) * 64 + 8 * st["steps"]),
           "d2h_bytes_per_step": int(8 * sim.pnum * len(outs)),
           "ms_per_step": 1e3 * e2e_s,
           "includes": "deck parse + context creation + the whole run + D2H of " + ",".join(outs)}

    pk, src = peaks()
    clk_mhz = (clk or {}).get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    track_pairs = st["pairs_total"] - st["pairs_solidify"]
    peak_pairs, basis = fp32_peak_pairs(th, clk_mhz)
    achieved = track_pairs / (st["ms_track"] / 1e3)
    loop = "Volume" if args.workload == "volume_multibeam" else "Surface"
    roof = {"bound": "latency", "kernel": f"k_track (persistent {loop} loop)",
            "achieved": achieved / 1e9, "peak": peak_pairs / 1e9, "unit": "Gpairs/s", "frac": achieved / peak_pairs,
            "peak_basis": basis, "device_rates": device_rates(th),
            "note": (("each timestep runs ~26,600 work items (re-tests three to an item, claimed neighbours "
                      "evaluated by their claimer up to three to a pass: ~34,400 passes of ~1,465 nodes) over "
                      "twelve warps per SM; bound by the passes' latency at three warps per scheduler and the items' "
                      "L2 round trips, not by FP32/MUFU issue or HBM") if loop == "Volume" else
                     ("each timestep runs ~580 work items (~690 evaluation passes of ~400 nodes) as a chain of "
                      "dependent L2 round trips (claims, queue slots, step word); the loop is bound by per-step "
                      "latency, not by FP32/MUFU issue or HBM")),
            "traffic": NCU_TRAFFIC.get(args.workload) if args.precision == "fp32" else None,
            "traffic_unit": "DRAM bytes per tracking launch (~256 timesteps)", "peak_source": src}
    sim.close()
    # the plain FP64 form of the same deck, one warm run, for the FP32 / FP64 ratio
    fp64 = None
    if args.precision == "fp32" and not args.no_fp64:
        with th.Simulation(path, "fp64") as s64:
            s64.solidify(max_steps=300)
            s64.reset()
            flush.zero_()
            torch.cuda.synchronize()
            s64.solidify()
            st64 = s64.run_stats()
        v64 = st64["pairs_total"] / (st64["ms_device"] / 1e3)
        fp64 = {"value": v64, "unit": "pairs/s", "ms_per_step": st64["ms_device"], "fp32_over_fp64": value / v64,
                "ms_tracking": st64["ms_track"], "ms_solidify": st64["ms_solidify"],
                "note": "the same deck and run in the plain FP64 form (TH_FP64), one run after a 300-step warm-up"}
    detail = {"steps": int(st["steps"]), "pairs_per_step": pairs, "ms_node_windows": st["ms_nodes"],
              "ms_tracking": st["ms_track"], "ms_solidify": st["ms_solidify"], "records": int(st["records"]),
              "records_redone_fp64": int(st["records_redone_fp64"]),
              "records_fixed_fp64": int(st["records_fixed_fp64"]), "guarded_decisions": int(st["guarded_decisions"]),
              "fp64_form": fp64,
              "max_items_per_step": int(st["max_items"]), "wall_s_per_step": statistics.median(wall),
              "device_s_per_step": statistics.median(dev_s)}
    if st.get("loop_steps"):
        n = st["loop_steps"]
        detail["loop_profile"] = {
            "us_work_per_timestep": 1e3 * st["loop_ms_work"] / n, "us_barrier_per_timestep": 1e3 * st["loop_ms_barrier"] / n,
            "items_per_timestep": st["loop_items"] / n,
            "us_per_item": st["loop_item_clocks"] / max(1, st["loop_items"]) / clk_mhz,
            "us_waiting_per_warp_timestep": st["loop_wait_clocks"] / n / clk_mhz / (device_rates(th)["sm_count"] * 4),
            "chain_depth_per_timestep": st["loop_depth_sum"] / n,
            "evals_per_timestep": st["loop_evals"] / n,
            "us_per_eval": st["loop_eval_clocks"] / max(1, st["loop_evals"]) / clk_mhz,
            "nodes_per_eval": st["loop_eval_nodes"] / max(1, st["loop_evals"]),
            "us_latest_item_start_by_chain_depth": [1e3 * st[f"loop_ms_start{l}"] / n for l in range(4)],
            "us_latest_item_end_by_chain_depth": [1e3 * st[f"loop_ms_end{l}"] / n for l in range(4)]}
    return {"value": value, "ms_per_step": 1e3 * total_s / args.steps, "e2e": e2e, "roofline": roof,
            "clocks": clk, "gpu_launches": launches * args.steps, "detail": detail}


# ------------------------------------------------------------------ snapshot workload
def run_snapshot(args, th, torch, dev, path, deck, world):
    sim = th.Simulation(path, args.precision)
    if args.tile:
        sim.set_tile_shape(*[int(v) for v in args.tile.split("x")])
    pnum, times = sim.pnum, sim.snapshot_times
    counts = [sim.integrate(t)["xb"].size for t in times]
    pairs_per_step = sum(c * pnum for c in counts)
    d_T = torch.empty(pnum, dtype=torch.float64, device=dev)
    d_T_all = torch.empty(len(times) * pnum, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def step():          # the node lists of all snapshots in one launch, then one sum each
        sim.calc_T_times_device(times, 0, pnum, d_T_all.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    total_s = allreduce_max(sum(a.elapsed_time(b) for a, b in ev) / 1e3, world)
    sim.sync(stream.cuda_stream)
    value = pairs_per_step * args.steps * world / total_s
    # the last snapshot's node list and sum, timed alone on the same stream
    gen_ms, sum_ms = [], []
    pts = torch.zeros(1, dtype=torch.int64, device=dev)
    one = torch.empty(1, dtype=torch.float64, device=dev)
    for _ in range(5):
        a, b, c = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        flush.zero_()
        a.record(stream)
        sim.calc_T_device(times[-1], pts.data_ptr(), 1, one.data_ptr(), stream.cuda_stream)
        b.record(stream)
        sim.calc_T_device(times[-1], 0, pnum, d_T.data_ptr(), stream.cuda_stream)
        c.record(stream)
        torch.cuda.synchronize()
        gen_ms.append(a.elapsed_time(b))
        sum_ms.append(b.elapsed_time(c))
    kernel_ms = max(statistics.median(sum_ms) - statistics.median(gen_ms), 1e-6)

    pinned = torch.empty(pnum, dtype=torch.float64, pin_memory=True).numpy()
    e2e_t = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with th.Simulation(path, args.precision) as s2:
            for i in range(len(times)):
                s2.snapshot(i, out=pinned)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = allreduce_max(statistics.median(e2e_t), world)
    e2e = {"value": pairs_per_step * world / e2e_s, "unit": "pairs/s",
           "h2d_bytes_per_step": int(sum(len(p) for p in deck.paths) * 64),
           "d2h_bytes_per_step": int(8 * pnum * len(times)), "ms_per_step": 1e3 * e2e_s,
           "includes": "deck parse + context creation + per-snapshot D2H of T into pinned memory"}
    pk, src = peaks()
    clk_mhz = (clk or {}).get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    pairs_last = counts[-1] * pnum
    achieved = pairs_last / (kernel_ms / 1e3)
    peak_pairs, basis = fp32_peak_pairs(th, clk_mhz)
    roof = {"bound": "fp32_issue", "kernel": "k_grid_fp32" if args.precision == "fp32" else "k_grid_fp64",
            "achieved": achieved / 1e9, "peak": peak_pairs / 1e9, "unit": "Gpairs/s", "frac": achieved / peak_pairs,
            "achieved_tops": achieved * OPS_PER_PAIR / 1e12, "kernel_ms": kernel_ms, "pairs_per_launch": pairs_last,
            "peak_basis": basis, "device_rates": device_rates(th),
            "hbm": {"algorithmic_bytes": int(8 * pnum + counts[-1] * 104), "peak_gbs": pk.get("hbm_gbs"),
                    "achieved_gbs": (8 * pnum + counts[-1] * 104) / (kernel_ms / 1e3) / 1e9, "peak_source": src},
            "traffic": NCU_TRAFFIC.get(args.workload) if args.precision == "fp32" else None}
    sim.close()
    return {"value": value, "ms_per_step": 1e3 * total_s / args.steps, "e2e": e2e, "roofline": roof,
            "clocks": clk, "gpu_launches": (1 + len(times)) * args.steps,
            "detail": {"pairs_per_step": pairs_per_step, "node_counts": counts,
                       "node_gen_ms": statistics.median(gen_ms)}}


# ------------------------------------------------------------------ batched sweep workload
def allreduce_sum(x, world):
    """The sum over ranks (every rank gets it)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_sweep(args, th, torch, dev, paths, deck, world):
    """One step = the 100 % snapshot of all 256 decks: one graph replay (node lists for
    every deck, then the work-list kernel over every deck's tiles).  Under torchrun the decks
    are split across the ranks (th.shard_decks: heaviest first to the least-loaded rank; no
    exchange), each rank replays its own batch, and the job's pairs are summed."""
    if world > 1:
        import torch.distributed as dist
        mine = th.shard_decks(paths, dist.get_rank(), world)
        paths = [paths[i] for i in mine]
        deck = [deck[i] for i in mine]
    b = th.Batch(paths, args.precision)
    if args.tile:
        b.set_tile_shape(*[int(v) for v in args.tile.split("x")])
    else:
        b.autotune(0)
    pnum = b.pnum
    d_T = torch.empty(pnum, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    p0 = b.pairs
    b.snapshot(0)
    pairs_per_step = b.pairs - p0

    def step():
        b.snapshot_device(0, d_T.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(world)
    step_ms = [a.elapsed_time(c) for a, c in ev]
    total_s = allreduce_max(sum(step_ms) / 1e3, world)
    job_pairs = allreduce_sum(pairs_per_step, world)          # the decks are split, not replicated
    value = job_pairs * args.steps / total_s
    b.snapshot(0)                       # surfaces any node-list error of the timed replays

    pinned = torch.empty(pnum, dtype=torch.float64, pin_memory=True).numpy()
    e2e_t = []
    for _ in range(max(1, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with th.Batch(paths, args.precision) as b2:
            b2.snapshot(0, out=pinned)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = allreduce_max(statistics.median(e2e_t), world)
    e2e = {"value": job_pairs / e2e_s, "unit": "pairs/s",
           "h2d_bytes_per_step": int(sum(len(p) for d in deck for p in d.paths) * 64),
           "d2h_bytes_per_step": int(8 * pnum), "ms_per_step": 1e3 * e2e_s,
           "includes": "256 deck parses + batch creation (node sizing, graph capture) + D2H of T into pinned memory"}
    pk, src = peaks()
    clk_mhz = (clk or {}).get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    kernel_ms = statistics.median(step_ms)
    achieved = pairs_per_step / (kernel_ms / 1e3)
    peak_pairs, basis = fp32_peak_pairs(th, clk_mhz)
    roof = {"bound": "fp32_issue", "kernel": "k_batch_grid (step incl. k_batch_nodes)",
            "achieved": achieved / 1e9, "peak": peak_pairs / 1e9, "unit": "Gpairs/s", "frac": achieved / peak_pairs,
            "achieved_tops": achieved * OPS_PER_PAIR / 1e12, "kernel_ms": kernel_ms,
            "pairs_per_launch": pairs_per_step,
            "peak_basis": basis, "device_rates": device_rates(th),
            "hbm": {"algorithmic_bytes": int(8 * pnum), "peak_gbs": pk.get("hbm_gbs"),
                    "achieved_gbs": 8 * pnum / (kernel_ms / 1e3) / 1e9, "peak_source": src},
            "traffic": None}
    b.close()
    return {"value": value, "ms_per_step": 1e3 * total_s / args.steps, "e2e": e2e, "roofline": roof,
            "clocks": clk, "gpu_launches": 2 * args.steps,
            "detail": {"pairs_per_step": job_pairs, "points": pnum, "decks": len(paths),
                       "rank0_pairs_per_step": pairs_per_step}}


# ------------------------------------------------------------------ adjoint workload
def run_adjoint(args, th, torch, dev, path, deck, world):
    """One step = forward temperatures at the probes + the adjoint gradient (host dual walk
    with tangents, device per-node adjoint sums), through the public API."""
    decks = importlib.import_module("3dthesis_gb300.decks")
    probes, times = decks.adjoint_probes(deck)
    adj = th.Adjoint(path, np.asarray(probes, dtype=np.int64), times, args.precision)
    theta = adj.params()
    tt = theta.copy()
    tt[0] *= 1.1
    tt[2] *= 0.9
    tt[5] *= 1.05
    target = adj.forward(tt)
    nodes = [adj.host_nodes(theta, i)[0].shape[1] for i in range(len(times))]
    pairs_per_step = 2 * sum(nodes) * len(probes)          # forward sums + adjoint sums

    def step():
        T = adj.forward(theta)
        return adj.backward(2.0 * (T - target))

    for _ in range(args.warmup):
        step()
    barrier(world)
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    wall = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step()
        wall.append(time.perf_counter() - t0)
    clk = clocks.stop()
    barrier(world)
    total_s = allreduce_max(sum(wall), world)
    value = pairs_per_step * args.steps * world / total_s
    # the host walk alone (values, no recording), for the split of the step
    t0 = time.perf_counter()
    for i in range(len(times)):
        adj.host_nodes(theta, i)
    host_s = time.perf_counter() - t0
    e2e = {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": int(8 * 8 * sum(nodes) * 2 + 8 * len(probes) * 3),
           "d2h_bytes_per_step": int(8 * len(probes) * len(times) + 7 * 8 * sum(nodes)), "ms_per_step": 1e3 * total_s / args.steps,
           "includes": "host node walks (values, then tangents), node uploads, forward and adjoint kernels, D2H"}
    roof = {"bound": "host walk + launch latency", "note": "the node walks (forward values, backward recorded "
            "for the reverse sweep) run on the host; the device sums are ~1e7 pairs per step",
            "host_value_walk_ms": 1e3 * host_s,
            "achieved": value / 1e9, "unit": "Gpairs/s", "peak": None, "frac": None, "traffic": None}
    adj.close()
    return {"value": value, "ms_per_step": 1e3 * total_s / args.steps, "e2e": e2e, "roofline": roof,
            "clocks": clk, "gpu_launches": 2 * len(times) * args.steps * 2,
            "detail": {"pairs_per_step": pairs_per_step, "nodes_per_time": nodes, "params": int(theta.size)}}


# ------------------------------------------------------------------ CPU oracle legs
def cpu_sample(path, workload, threads, budget_s):
    """The CPU oracle on the same deck: solidification runs a prefix of the timesteps,
    snapshots run whole snapshots, until ~budget_s of work."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.load()
    if workload == "adjoint_calibration":
        decks = importlib.import_module("3dthesis_gb300.decks")
        deck = decks.adjoint_calibration()
        probes, times = decks.adjoint_probes(deck)
        o = oracle_lib.Oracle(path)
        pts = np.asarray(probes, dtype=np.int64)
        pairs, used, n = 0, 0.0, 0
        while used < budget_s and n < 20000:
            p0, t0 = o.pairs, time.perf_counter()
            o.calc_T(times[n % len(times)], pts, threads=threads)
            used += time.perf_counter() - t0
            pairs += o.pairs - p0
            n += 1
        return pairs / used, f"{n} probe-temperature evaluations (4096 probes) on the oracle ({used:.1f} s)"
    if workload == "snapshot_sweep":
        pairs, used, n = 0, 0.0, 0
        while used < budget_s and n < len(path):
            o = oracle_lib.Oracle(path[n])
            p0, t0 = o.pairs, time.perf_counter()
            o.snapshot(0, threads=threads)
            used += time.perf_counter() - t0
            pairs += o.pairs - p0
            n += 1
        return pairs / used, f"the 100 % snapshot of the first {n} decks of the sweep ({used:.1f} s)"
    if workload == "snapshot_raster":
        o = oracle_lib.Oracle(path)
        pairs, used, n = 0, 0.0, 0
        while used < budget_s and n < 9:
            p0, t0 = o.pairs, time.perf_counter()
            o.snapshot(n % o.n_snapshots, threads=threads)
            used += time.perf_counter() - t0
            pairs += o.pairs - p0
            n += 1
        return pairs / used, f"{n} whole snapshots of the deck ({used:.1f} s)"
    # solidification: the whole run, or the run from t = 0 until the step that ends past the
    # time budget (budget_s > 0)
    o = oracle_lib.Oracle(path)
    t0 = time.perf_counter()
    done = o.solidify(threads=threads, budget_s=budget_s)
    used = time.perf_counter() - t0
    what = f"all {done} timesteps of the run" if budget_s <= 0 else f"the first {done} timesteps of the run"
    return o.pairs / used, f"{what} ({used:.1f} s, {o.pairs:.3e} pairs)"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="surface_serpentine", choices=sorted(DECK_TEXT))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--tile", default="")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-form comparator run")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    config = {"workload": args.workload, "deck": DECK_TEXT[args.workload], "precision": args.precision,
              "l2": "flushed (256 MiB write) before each step; state arrays exceed L2",
              "scaling_mode": "replicas: every rank runs the full workload"}

    if args.impl == "reference":
        if rank != 0:
            return
        tmp = tempfile.mkdtemp(prefix="thesis_ref_")
        _, path = make_deck(args.workload, tmp)
        threads = os.cpu_count() or 1
        for _ in range(args.warmup):
            cpu_sample(path, args.workload, threads, budget_s=1.0)
        vals, sample = [], ""
        # each step is the same work as one step of the GPU arm where that fits (the whole
        # Surface run, ~15 s); otherwise a 15 s prefix of the run
        budget = 0.0 if args.workload in CPU_WHOLE_RUN else 15.0
        for _ in range(args.steps):
            v, sample = cpu_sample(path, args.workload, threads, budget_s=budget)
            vals.append(v)
        shutil.rmtree(tmp, ignore_errors=True)
        value = statistics.median(vals)
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "impl": "reference", "dtype": "f64",
            "data": "synthetic", "config": config, "scaling": "weak", "vs_baseline": None,
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    th = importlib.import_module("3dthesis_gb300")
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    tmp = tempfile.mkdtemp(prefix="thesis_bench_")
    deck, path = make_deck(args.workload, tmp)
    runner = {"surface_serpentine": run_solidification, "volume_multibeam": run_solidification,
              "snapshot_raster": run_snapshot,
              "snapshot_sweep": run_sweep, "adjoint_calibration": run_adjoint}[args.workload]
    r = runner(args, th, torch, dev, path, deck, world)
    if args.workload == "snapshot_sweep":
        config["scaling_mode"] = "decks split across ranks (th.shard_decks), no collective on the data path"
    line = {"metric": METRIC, "value": r["value"], "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "strong" if args.workload == "snapshot_sweep" else "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": config, "e2e": r["e2e"], "roofline": r["roofline"], "clocks": r["clocks"],
            "gpu_launches": r["gpu_launches"], "detail": r["detail"]}
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, sample = cpu_sample(path, args.workload, threads, budget_s=0.0 if args.workload in CPU_WHOLE_RUN else 15.0)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port", "sample": sample}
    shutil.rmtree(tmp, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
