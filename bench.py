"""Benchmark of the 3DThesis hot path on GB300: point x node pairs per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload snapshot_raster] [--precision fp32|fp64]

One step is one pass of the workload's hot path over its synthetic deck:
  snapshot_raster : the 10 x 2 mm raster on the 200x100x40 grid, snapshots at 25/50/100 %
                    (3 x (device node generation + whole-grid point x node sum)).
``value`` is device-timed with the deck already resident in HBM (CUDA events on the
launching stream, L2 flushed by a 256 MiB write before every step, outside the events).
``e2e`` goes through the public C-ABI calls a user makes - context creation from the deck
files, th_snapshot into pinned host memory per snapshot, context destruction - with the
host<->device copies inside the timed region.  ``cpu_baseline`` / ``--impl reference`` time
the CPU oracle (the reference's algorithm restated in C++, OpenMP over the host cores).

Under torchrun each rank runs the same per-GPU workload (weak scaling, no collective on
the data path); rank 0 prints the max-over-ranks time.
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
# per-pair algorithmic work of the temperature sum (15 floating-point operations + 1 exp)
OPS_PER_PAIR = 16
SM_COUNT = 152
FP32_LANES = 128            # FP32 lanes per SM per clock
MUFU_LANES = 16             # MUFU.EX2 results per SM per clock
FP32_OPS_KAHAN = 14         # minimum FP32-pipe instructions per compensated pair


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits", "-lms", "200"],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

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
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ workloads
def make_deck(name: str, tmp: str):
    decks = importlib.import_module("3dthesis_gb300.decks")
    deck = getattr(decks, name)()
    return deck, deck.write(os.path.join(tmp, name))


def run_ours(args, rank: int, world: int):
    import torch
    th = importlib.import_module("3dthesis_gb300")
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    tmp = tempfile.mkdtemp(prefix="thesis_bench_")
    deck, path = make_deck(args.workload, tmp)
    sim = th.Simulation(path, args.precision)
    if args.tile:
        sim.set_tile_shape(*[int(v) for v in args.tile.split("x")])
    pnum = sim.pnum
    times = sim.snapshot_times
    counts = [sim.integrate(t)["xb"].size for t in times]
    pairs_per_step = sum(c * pnum for c in counts)
    d_T = torch.empty(pnum, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    # a real stream: the library launches on the stream it is given, and the events, the
    # L2 flush and the kernels must all be ordered on that one stream
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    launches_per_step = 2 * len(times)

    def step():
        for t in times:
            sim.calc_T_device(t, 0, pnum, d_T.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # per-kernel time of the dominant kernel (the last snapshot's sum), same stream
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index if dev.index is not None else 0)
    clocks.start()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        for ti, t in enumerate(times):
            if ti == len(times) - 1:
                kev[k][0].record(stream)
            sim.calc_T_device(t, 0, pnum, d_T.data_ptr(), stream.cuda_stream)
            if ti == len(times) - 1:
                kev[k][1].record(stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier(world)
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_s = sum(step_ms) / 1e3
    total_s = allreduce_max(total_s, world)
    # the node generation is a single-warp kernel; time it separately to split the step
    gen_ms = time_node_generation(sim, times[-1], stream, torch)
    last_kernel_ms = [a.elapsed_time(b) for a, b in kev]
    sum_ms = max(statistics.median(last_kernel_ms) - gen_ms, 1e-6)
    value = pairs_per_step * args.steps * world / total_s

    # end to end through the public API with host buffers
    e2e = None
    if rank == 0 or world > 1:
        pinned = torch.empty(pnum, dtype=torch.float64, pin_memory=True)
        host = pinned.numpy()
        e2e_times = []
        for k in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2 = th.Simulation(path, args.precision)
            for i in range(len(times)):
                s2.snapshot(i, out=host)
            s2.close()
            e2e_times.append(time.perf_counter() - t0)
        e2e_s = allreduce_max(sum(e2e_times), world)
        e2e = {"value": pairs_per_step * len(e2e_times) * world / e2e_s, "unit": METRIC,
               "h2d_bytes_per_step": int(sum(len(p) for p in deck.paths) * 56),
               "d2h_bytes_per_step": int(8 * pnum * len(times)),
               "ms_per_step": 1e3 * e2e_s / len(e2e_times),
               "includes": "deck parse + context creation + per-snapshot D2H of T into pinned memory"}
    sim.close()
    shutil.rmtree(tmp, ignore_errors=True)

    pk, src = peaks()
    clk_mhz = (clk or {}).get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    n_last = counts[-1]
    pairs_last = n_last * pnum
    achieved_pairs = pairs_last / (sum_ms / 1e3)
    peak_pairs = SM_COUNT * clk_mhz * 1e6 * min(FP32_LANES / FP32_OPS_KAHAN, MUFU_LANES)
    roof = {"bound": "fp32_issue", "kernel": "k_grid_fp32<4,2>" if args.precision == "fp32" else "k_grid_fp64<4,2>",
            "achieved": achieved_pairs / 1e9, "peak": peak_pairs / 1e9, "unit": "Gpairs/s",
            "frac": achieved_pairs / peak_pairs,
            "achieved_tops": achieved_pairs * OPS_PER_PAIR / 1e12,
            "peak_basis": f"{SM_COUNT} SMs x {clk_mhz:.0f} MHz (median SM clock under load) x "
                          f"min({FP32_LANES}/{FP32_OPS_KAHAN} FP32 issue, {MUFU_LANES} MUFU) pairs/clk",
            "kernel_ms": sum_ms, "pairs_per_launch": pairs_last,
            "hbm": {"algorithmic_bytes": int(8 * pnum + n_last * 56), "peak_gbs": pk.get("hbm_gbs"),
                    "achieved_gbs": (8 * pnum + n_last * 56) / (sum_ms / 1e3) / 1e9, "peak_source": src},
            "traffic": None}
    return {
        "value": value, "ms_per_step": 1e3 * total_s / args.steps, "wall_s": wall, "e2e": e2e,
        "roofline": roof, "clocks": clk, "gpu_launches": launches_per_step * args.steps,
        "pairs_per_step": pairs_per_step, "node_counts": counts, "node_gen_ms": gen_ms,
    }


def time_node_generation(sim, t, stream, torch):
    """Device time of one node-list generation (a 1-point evaluation is negligible)."""
    pts = torch.zeros(1, dtype=torch.int64, device=torch.device("cuda", torch.cuda.current_device()))
    out = torch.empty(1, dtype=torch.float64, device=pts.device)
    ms = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        sim.calc_T_device(t, pts.data_ptr(), 1, out.data_ptr(), stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    return statistics.median(ms)


def cpu_pairs_per_s(path, threads, budget_s=20.0):
    """The CPU oracle on the same deck: whole snapshots until ~budget_s of work."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib
    oracle_lib.load()
    o = oracle_lib.Oracle(path)
    done_pairs, t_used, snaps = 0, 0.0, 0
    while t_used < budget_s and snaps < 3 * 3:
        i = snaps % o.n_snapshots
        p0 = o.pairs
        t0 = time.perf_counter()
        o.snapshot(i, threads=threads)
        t_used += time.perf_counter() - t0
        done_pairs += o.pairs - p0
        snaps += 1
    return done_pairs / t_used, snaps, t_used


def run_reference(args):
    tmp = tempfile.mkdtemp(prefix="thesis_ref_")
    _, path = make_deck(args.workload, tmp)
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_pairs_per_s(path, threads, budget_s=2.0)
    for _ in range(args.steps):
        v, snaps, used = cpu_pairs_per_s(path, threads, budget_s=max(2.0, 60.0 / max(1, args.steps)))
        vals.append(v)
    shutil.rmtree(tmp, ignore_errors=True)
    value = statistics.median(vals)
    return value, threads


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="snapshot_raster")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--tile", default="")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    config = {"workload": args.workload, "deck": "synthetic; 10 tracks x 2 mm, hatch 0.1 mm, 1.0 m/s, "
              "P=200 W, eta=0.35, 50/50/1 um; grid 200x100x40 at 10 um; snapshots at 25/50/100 %",
              "points": 800000, "precision": args.precision, "l2": "flushed (256 MiB write) before each step",
              "scaling_mode": "replicas: every rank runs the full workload"}

    if args.impl == "reference":
        if rank != 0:
            return
        value, threads = run_reference(args)
        line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "impl": "reference", "dtype": "f64",
                "data": "synthetic", "config": config, "scaling": "weak", "vs_baseline": None,
                "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                                 "sample": "whole snapshots of the deck (3 per pass) on all host threads"},
                "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    r = run_ours(args, rank, world)
    line = {"metric": METRIC, "value": r["value"], "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
            "config": config, "e2e": r["e2e"], "roofline": r["roofline"], "clocks": r["clocks"],
            "gpu_launches": r["gpu_launches"],
            "detail": {"pairs_per_step": r["pairs_per_step"], "node_counts": r["node_counts"],
                       "node_gen_ms": r["node_gen_ms"], "wall_s": r["wall_s"]}}
    if rank == 0 and not args.no_cpu_baseline:
        tmp = tempfile.mkdtemp(prefix="thesis_cpu_")
        _, path = make_deck(args.workload, tmp)
        threads = os.cpu_count() or 1
        v, snaps, used = cpu_pairs_per_s(path, threads, budget_s=15.0)
        line["cpu_baseline"] = {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port",
                                "sample": f"{snaps} whole snapshots of the same deck ({used:.1f} s of CPU work)"}
        shutil.rmtree(tmp, ignore_errors=True)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
