"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), no GPU.

Transforms are independent, so the multi-GPU path is replicas: each rank runs its own full
per-GPU batch (weak scaling) with no data-path collective; the only communication is the
barrier and the max over ranks of the timed interval, checked here."""
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
