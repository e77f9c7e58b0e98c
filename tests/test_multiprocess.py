"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), no GPU.

Transforms are independent, so the multi-GPU path is replicas: each rank runs its own full
per-GPU batch (weak scaling) with no data-path collective; the only communication is the
barrier and the max over ranks of the timed interval, checked here.  With --shard the ranks
split one ragged batch by lfg.shard_ragged, each computing the same split on its own."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _shard_worker(rank, ws, port, q):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "lean-fftw_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import numpy as np
    import torch
    import torch.distributed as dist
    import lfg
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sizes = lfg.ragged_sizes(8192)
    shard, cost = lfg.shard_ragged(sizes, ws)
    mine = np.flatnonzero(shard == rank)
    # every rank computed the same split: gather each rank's indices and check the cover
    n = torch.tensor([mine.size])
    ns = [torch.zeros(1, dtype=torch.int64) for _ in range(ws)]
    dist.all_gather(ns, n)
    width = int(max(t.item() for t in ns))
    pad = torch.full((width,), -1, dtype=torch.int64)
    pad[: mine.size] = torch.from_numpy(mine)
    allp = [torch.zeros(width, dtype=torch.int64) for _ in range(ws)]
    dist.all_gather(allp, pad)
    q.put((rank, [p[p >= 0].tolist() for p in allp], float(cost.max() / cost.mean())))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_shards_cover_the_batch():
    """bench.py --shard: each rank computes the cost-balanced split of the one ragged batch on
    its own; the ranks' shares are disjoint and cover every transform."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res[0][1] == res[1][1]                        # the same split on both ranks
    a, b = set(res[0][1][0]), set(res[0][1][1])
    assert not (a & b) and len(a | b) == 8192
    assert res[0][2] <= 1.01


def _worker(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    dist.barrier()
    w, r, l = bench.dist_env()
    m = bench.max_over_ranks(1.5 + rank)
    q.put((rank, w, r, l, m, bench.rank_seed(rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [2, 2] and [r[2] for r in res] == [0, 1]
    assert all(r[4] == 2.5 for r in res)                 # max over ranks on every rank
    assert res[0][5] != res[1][5]                        # each rank its own batch


def test_single_process_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
