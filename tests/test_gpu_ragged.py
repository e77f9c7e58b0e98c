"""GPU parity of ragged batches (one persistent, graph-replayed launch for many sizes).

Every transform of the batch must equal the oracle's refTransform for its size and the
radix sequence the plan picked, bit for bit, in every execution mode (persistent kernel
with and without graph replay, per-size launches), with scattered offsets whose gaps stay
untouched.  The full benchmark batch (8192 sizes drawn log-uniformly from the 13-smooth
integers in [2, 16384]) is checked completely.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

SENT = complex(-7.5e300, 3.25e299)


def _check(plan, sizes, x, y_np, in_off, out_off):
    bad = []
    by_size = {}
    for i, n in enumerate(sizes):
        by_size.setdefault(int(n), []).append(i)
    for n, idx in by_size.items():
        rs = plan.radices(n)
        xs = np.stack([x[in_off[i]: in_off[i] + n] for i in idx])
        ref = O.ref_transform(True, n, rs, xs, nthreads=8)
        got = np.stack([y_np[out_off[i]: out_off[i] + n] for i in idx])
        if not np.array_equal(got.view(np.uint64), ref.view(np.uint64)):
            bad.append((n, rs))
    return bad


@pytest.mark.parametrize("mode", ["graph", "direct", "per_size", "per_size_concurrent",
                                  "per_size_concurrent_direct"])
def test_ragged_small_scattered(mode):
    rng = np.random.default_rng(3)
    sizes = np.array([2, 3, 16, 60, 60, 60, 1000, 4096, 2310, 7, 13, 13, 8192, 10368, 16384,
                      15015, 243, 2, 1024, 1024] * 2, dtype=np.int64)
    rng.shuffle(sizes)
    gaps = rng.integers(0, 5, size=sizes.size)
    in_off = np.cumsum(np.concatenate([[3], sizes[:-1] + gaps[:-1]])).astype(np.int64)
    out_off = np.cumsum(np.concatenate([[1], sizes[:-1] + gaps[::-1][:-1]])).astype(np.int64)
    tin = int(in_off[-1] + sizes[-1] + 2)
    tout = int(out_off[-1] + sizes[-1] + 7)
    x = O.uniform_complex((tin,), seed=9)
    plan = lfg.plan_ragged(sizes, -1, in_off, out_off, per_size=mode.startswith("per_size"),
                           graph=not mode.endswith("direct"), concurrent="concurrent" in mode)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full((tout,), SENT, dtype=torch.complex128, device="cuda")
    for _ in range(2):        # a second execution reuses the graph and the zeroed queue
        plan.execute(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    assert not _check(plan, sizes, x, y, in_off, out_off)
    mask = np.ones(tout, bool)
    for o, n in zip(out_off, sizes):
        mask[o: o + n] = False
    assert np.all(y[mask] == SENT)


def test_ragged_benchmark_batch_full():
    sizes = lfg.ragged_sizes(8192)
    plan = lfg.plan_ragged(sizes, -1)
    info = plan.info()
    assert info.count == 8192 and info.launches == 1
    total = int(sizes.sum())
    x = O.uniform_complex((total,), seed=20261016)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plan.execute(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    assert not _check(plan, sizes, x, y, plan.in_offsets, plan.out_offsets)
    # per-size strategy gives the same bits, its launches in one chain or on 64 branches
    for conc in (False, True):
        ps = lfg.plan_ragged(sizes, -1, per_size=True, concurrent=conc)
        y2 = torch.empty_like(xd)
        ps.execute(xd, y2)
        torch.cuda.synchronize()
        assert torch.equal(y2.view(torch.float64), yd.view(torch.float64)), conc


def test_ragged_host_entry():
    sizes = np.array([12, 5000, 3, 720], dtype=np.int64)
    x = O.uniform_complex((int(sizes.sum()),), seed=1)
    plan = lfg.plan_ragged(sizes, 1)
    y = plan.execute_host(x, np.zeros_like(x))
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    for o, n in zip(off, sizes):
        ref = O.ref_transform(False, int(n), plan.radices(int(n)), x[o: o + n])
        assert np.array_equal(y[o: o + n].view(np.uint64), ref.view(np.uint64))


def test_ragged_measured_plan_bitexact():
    sizes = lfg.ragged_sizes(512, seed=11)
    plan = lfg.plan_ragged(sizes, -1, measure=True)
    x = O.uniform_complex((int(sizes.sum()),), seed=12)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plan.execute(xd, yd)
    torch.cuda.synchronize()
    assert not _check(plan, sizes, x, yd.cpu().numpy(), plan.in_offsets, plan.out_offsets)


def test_ragged_pinned_host_entry():
    """Pinned host buffers: the persistent kernel reads and writes host memory directly
    (asynchronous tile copies from host memory, two-group intermediates in device slabs)."""
    sizes = lfg.ragged_sizes(1024, seed=5)
    sizes[:3] = [16384, 15015, 4096]          # two-group items next to one-group ones
    plan = lfg.plan_ragged(sizes, -1)
    total = int(sizes.sum())
    x = O.uniform_complex((total,), seed=21)
    hin = torch.from_numpy(x).pin_memory()
    hout = torch.full((total,), SENT, dtype=torch.complex128).pin_memory()
    for _ in range(2):
        plan.execute_host(hin.numpy(), hout.numpy())
    assert not _check(plan, sizes, x, hout.numpy(), plan.in_offsets, plan.out_offsets)


def test_ragged_host_pageable_and_gapped():
    """Pageable host arrays (copied in and out around the launch); and pinned buffers whose
    inputs and outputs leave gaps (the kernel reads and writes host memory directly): the
    caller's values in the output gaps stay."""
    sizes = lfg.ragged_sizes(256, seed=8)
    plan = lfg.plan_ragged(sizes, -1)
    x = O.uniform_complex((int(sizes.sum()),), seed=9)
    y = plan.execute_host(x, np.zeros_like(x))
    assert not _check(plan, sizes, x, y, plan.in_offsets, plan.out_offsets)
    in_off = np.concatenate([[0], np.cumsum(sizes + 5)[:-1]]).astype(np.int64)
    out_off = np.concatenate([[0], np.cumsum(sizes + 3)[:-1]]).astype(np.int64)
    gapped = lfg.plan_ragged(sizes, -1, in_offsets=in_off, out_offsets=out_off)
    xg = O.uniform_complex((int(in_off[-1] + sizes[-1]),), seed=10)
    hin = torch.from_numpy(xg).pin_memory()
    hout = torch.full((int(out_off[-1] + sizes[-1]),), SENT, dtype=torch.complex128).pin_memory()
    gapped.execute_host(hin.numpy(), hout.numpy())
    y2 = hout.numpy()
    assert not _check(gapped, sizes, xg, y2, in_off, out_off)
    for o, n in zip(out_off, sizes):
        assert np.all(y2[o + n: o + n + 3] == SENT)     # (empty past the last output)


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("tile,single", [(2048, 2048), (4096, 4096), (1024, 1024)])
def test_ragged_block_shapes(shape, tile, single):
    """Every block shape of the persistent kernel, with the tile and single-group limits the
    autotuner chooses from (three tile buffers must fit the shared memory)."""
    sizes = lfg.ragged_sizes(384, seed=shape * 7 + tile // 1024)
    sizes[:2] = [4096, 3000]
    plan = lfg.plan_ragged(sizes, 1, block_shape=shape, tile_target=tile, single_max=single)
    assert plan.info().smem_bytes <= 232448 - 1024
    x = O.uniform_complex((int(sizes.sum()),), seed=shape)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    plan.execute(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    bad = []
    for i, (a, o, n) in enumerate(zip(plan.in_offsets, plan.out_offsets, sizes)):
        ref = O.ref_transform(False, int(n), plan.radices(int(n)), x[a: a + n])
        if not np.array_equal(y[o: o + n].view(np.uint64), ref.view(np.uint64)):
            bad.append(int(n))
    assert not bad


def test_ragged_rejects_misaligned_buffers():
    """Buffers must start on a complex element: an 8-byte offset is refused before launch."""
    import ctypes
    from lfg._lib import LFG_ERR_INVALID
    sizes = np.array([64, 12], dtype=np.int64)
    plan = lfg.plan_ragged(sizes, -1)
    buf = torch.zeros(200, dtype=torch.complex128, device="cuda")
    p = buf.data_ptr()
    st = lfg.lib().lfg_execute_ragged(plan._h, ctypes.c_void_p(p + 8), ctypes.c_void_p(p + 1600),
                                      None)
    assert st == LFG_ERR_INVALID
    p1 = lfg.plan_1d(64, -1, 2)
    st = lfg.lib().lfg_execute(p1._h, ctypes.c_void_p(p), ctypes.c_void_p(p + 2056), None)
    assert st == LFG_ERR_INVALID
    torch.cuda.synchronize()
