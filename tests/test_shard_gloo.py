"""Splitting a parameter sweep's decks across GPUs (th.shard_decks, the multi-GPU path of
the 256-deck sweep): every deck runs on exactly one rank, the ranks agree on the split
without exchanging anything, and the load is balanced.  Two gloo ranks on the CPU call the
library's host path (th_deck_info parses each deck without a GPU) and bench.py's sum and
max over ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, paths, out):
    import importlib
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    th = importlib.import_module("3dthesis_gb300")
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = th.shard_decks(paths, rank, world)
    weights = [th.deck_weight(paths[i]) for i in mine]
    everyone = [None] * world
    dist.all_gather_object(everyone, mine)              # test only: the split itself exchanges nothing
    total = bench.allreduce_sum(sum(weights), world)
    slowest = bench.allreduce_max(sum(weights), world)
    out[rank] = (mine, everyone, total, slowest)
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_sweep(tmp_path, decks, built_library):
    mp = pytest.importorskip("torch.multiprocessing")
    import importlib
    th = importlib.import_module("3dthesis_gb300")
    sweep = decks.small_sweep(n=10)
    paths = [d.write(str(tmp_path / d.name)) for d in sweep]
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, paths, out), nprocs=2, join=True)
        res = dict(out)
    (m0, all0, tot0, slow0), (m1, all1, tot1, slow1) = res[0], res[1]
    assert all0 == all1 == [m0, m1]                     # both ranks computed the same split
    assert sorted(m0 + m1) == list(range(len(paths)))   # every deck exactly once
    w = [th.deck_weight(p) for p in paths]
    assert tot0 == tot1 == pytest.approx(sum(w))
    assert slow0 == slow1 <= sum(w) / 2 + max(w)       # greedy: within one deck of an even split
    info = th.deck_info(paths[0])
    assert info["pnum"] == info["nx"] * info["ny"] * info["nz"] and info["precision"] == -1


def test_shard_decks_partition():
    import importlib
    th = importlib.import_module("3dthesis_gb300")
    w = [5, 1, 1, 1, 3, 3, 2, 8, 1, 1, 4]
    for world in (1, 2, 3, 4, 16):
        parts = [th.shard_decks([None] * len(w), r, world, weights=w) for r in range(world)]
        assert sorted(sum(parts, [])) == list(range(len(w)))
        loads = [sum(w[i] for i in p) for p in parts]
        assert max(loads) <= sum(w) / world + max(w)
    with pytest.raises(ValueError):
        th.shard_decks([None], 2, 2, weights=[1])
