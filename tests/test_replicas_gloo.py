"""The multi-rank path of bench.py (replicas: every rank runs the whole workload, rank 0
reports the slowest rank's time) with two gloo ranks on the CPU, and bench.py's bounded
CPU-oracle sample."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, deck_path, out):
    import numpy as np
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import bench
    import oracle_lib
    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle_lib.load()
    # each replica evaluates the same deck (as each GPU would) and times itself
    T = oracle_lib.Oracle(deck_path).snapshot(1, threads=1)
    bench.barrier(world)
    slowest = bench.allreduce_max(float(rank + 1), world)
    out[rank] = (slowest, float(np.sum(T)))
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path, decks):
    mp = pytest.importorskip("torch.multiprocessing")
    path = decks.small_spots().write(str(tmp_path / "spots"))
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, path, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 2.0          # both ranks see the slowest rank's time
    assert res[0][1] == res[1][1]                 # replicas compute the same result


def test_bench_cpu_sample_is_bounded(tmp_path, decks):
    """The bench's CPU leg on a solidification deck stops near its time budget (the sample
    is the run from t = 0 up to the step that ends past the budget) and reports pairs/s."""
    import time
    sys.path.insert(0, ROOT)
    import bench
    path = decks.small_surface("Surface").write(str(tmp_path / "surface"))
    t0 = time.perf_counter()
    value, sample = bench.cpu_sample(path, "surface_serpentine", 2, budget_s=0.05)
    assert time.perf_counter() - t0 < 10.0
    assert value > 0 and "timesteps of the run" in sample
