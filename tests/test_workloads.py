"""The benchmark's synthetic workloads are fixed by their seeds (no GPU needed): the ragged
batch's size draw (log-uniform over the 13-smooth integers in [2, 16384], snapped in log
distance, ties to the smaller) and the configurations bench.py runs."""
import importlib.util
import os

import numpy as np

import lfg
from conftest import ROOT


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_ragged_batch_is_pinned():
    sizes = lfg.ragged_sizes(8192)
    assert sizes.size == 8192
    assert len(np.unique(sizes)) == 859
    assert int(sizes.sum()) == 14922904
    assert int(np.median(sizes)) == 182
    assert sizes.min() >= 2 and sizes.max() <= 16384
    for n in np.unique(sizes):
        m = int(n)
        for p in (2, 3, 5, 7, 11, 13):
            while m % p == 0:
                m //= p
        assert m == 1, n


def test_bench_workloads_match_the_configurations():
    b = _bench()
    W = b.WORKLOADS
    assert W["ragged"]["count"] == 8192
    for k in range(1, 19):                       # 2^k, batch moving 1 GiB (binary64)
        w = W[f"c2c_{1 << k}"]
        assert w["n"] * w["batch"] == 1 << 26
    assert W["small_1024"]["n"] == 1024 and W["small_1024"]["batch"] == 1
    assert (W["grad_4096"]["n"], W["grad_4096"]["batch"]) == (4096, 256)
    assert (W["large_262144"]["n"], W["large_262144"]["batch"]) == (1 << 18, 32)
    assert W["large_262144_f32"]["precision"] == "f32"
    assert (W["r2c_512x512"]["n0"], W["r2c_512x512"]["n1"], W["r2c_512x512"]["batch"]) == (512, 512, 64)
    assert np.array_equal(b.ragged_workload_sizes(W["ragged"]), np.sort(lfg.ragged_sizes(8192)))


def test_shard_ragged_balances_and_covers():
    """lfg.shard_ragged splits the benchmark's ragged batch over 2..8 devices: every transform
    exactly once, shard costs equal to the sum of their transforms' codelet operations, and the
    largest shard within 1 % of the mean (host only, no GPU)."""
    import lfg
    from lfg.codegen.plans import choose_radices
    from lfg.codegen.kernel import butterfly_k
    sizes = lfg.ragged_sizes(8192)
    ops = {}
    for n in set(sizes.tolist()):
        rs = choose_radices(n)
        ops[n] = sum((n // R) * sum(butterfly_k(True, R, t > 0).counts()) for t, R in enumerate(rs))
    for k in (2, 3, 4, 8):
        shard, cost = lfg.shard_ragged(sizes, k)
        assert shard.min() >= 0 and shard.max() < k
        for s in range(k):
            assert cost[s] == sum(ops[int(n)] for n in sizes[shard == s])
        assert cost.max() <= 1.01 * cost.mean(), (k, cost)
    again, _ = lfg.shard_ragged(sizes, 4)
    assert (again == lfg.shard_ragged(sizes, 4)[0]).all()
