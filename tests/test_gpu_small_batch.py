"""Batched small sizes on the warp-tile kernel (csrc/small.cu).

A plan of N <= 16 points is one untwiddled codelet per transform; the warp-tile kernel runs
it with per-warp shared-memory chunks instead of the CTA-wide tile of the group kernels, and
it runs the two passes of binary32 plans of up to 32 points between two warp tiles.  Its
results must be the bits of the reference transform (binary64: the oracle's refTransform for
the plan's radix sequence; both precisions: the group kernels, LFG_GENERIC_KERNELS), for
batches that leave a partial last chunk, in place, scaled, and over gapped and transposed
line layouts (the kernel's general-stride load and store orders).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

SIZES = list(range(2, 17))


def _expect_small(n, precision):
    """The planner's choice for back-to-back lines: binary64 every N; binary32 all but the
    sizes the bulk-copy kernel runs faster (N = 2, 4, 12)."""
    if precision == "f64":
        return 1
    return int(n not in (2, 4, 12))


def _bits_equal(a, b):
    return torch.equal(a.view(torch.int64) if a.dtype == torch.complex128 else a.view(torch.int32),
                       b.view(torch.int64) if b.dtype == torch.complex128 else b.view(torch.int32))


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", SIZES)
def test_small_sizes_match_group_kernel_and_oracle(n, precision):
    B = 1237 + n                                   # a partial last chunk for every K
    x = O.uniform_complex((B, n), seed=100 + n)
    dt = torch.complex128 if precision == "f64" else torch.complex64
    xd = torch.from_numpy(x).to("cuda", dt)
    for sign in (-1, 1):
        plan = lfg.plan_1d(n, sign, B, precision=precision)
        assert plan.info().small_kernel == _expect_small(n, precision), n
        y = plan.execute(xd)
        generic = lfg.plan_1d(n, sign, B, precision=precision, generic_kernels=True)
        assert generic.info().small_kernel == 0
        assert _bits_equal(y, generic.execute(xd)), (n, sign)
        inplace = xd.clone()
        plan.execute(inplace, inplace)
        assert _bits_equal(inplace, y), (n, sign)
        if precision == "f64":
            ref = O.ref_transform(sign < 0, n, plan.radices, x)
            got = y.cpu().numpy()
            assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (n, sign)


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [3, 8, 13, 15, 16])
def test_small_sizes_scaled(n, precision):
    B = 999
    x = O.uniform_complex((B, n), seed=n)
    dt = torch.complex128 if precision == "f64" else torch.complex64
    xd = torch.from_numpy(x).to("cuda", dt)
    plan = lfg.plan_1d(n, 1, B, precision=precision).set_scale(1.0 / n)
    generic = lfg.plan_1d(n, 1, B, precision=precision, generic_kernels=True).set_scale(1.0 / n)
    assert plan.info().small_kernel == 1
    assert _bits_equal(plan.execute(xd), generic.execute(xd)), n


@pytest.mark.parametrize("n", [2, 5, 8, 15, 16])
def test_small_sizes_strided_layouts(n):
    """Lines dist = n + 3 apart (gapped: the element-contiguous order without the packed fast
    path) and lines interleaved (stride B, dist 1: the line-contiguous order), binary64,
    against the oracle."""
    B = 301
    x = O.uniform_complex((B, n), seed=7 * n)
    ref = O.ref_transform(True, n, lfg.plan_1d(n, -1, B).radices, x)
    # gapped: complex element j of line b at b*(n+3) + j (doubles: twice that)
    d = n + 3
    buf = np.zeros((B, d), dtype=np.complex128)
    buf[:, :n] = x
    spec = [0, -1, 1, 1, 0, 1, 0, 1, n, 2, 2, B, 2 * d, 2 * d]
    plan = lfg.plan_spec(spec)
    assert plan.info().small_kernel == 1
    xin = torch.from_numpy(buf.reshape(-1).view(np.float64).copy()).cuda()
    out = torch.zeros(2 * B * d, dtype=torch.float64, device="cuda")
    plan.execute(xin, out)
    got = out.cpu().numpy().view(np.complex128).reshape(B, d)[:, :n]
    assert np.array_equal(np.ascontiguousarray(got).view(np.uint64), ref.view(np.uint64)), n
    # transposed: element j of line b at j*B + b
    xt = np.ascontiguousarray(x.T)
    spec = [0, -1, 1, 1, 0, 1, 0, 1, n, 2 * B, 2 * B, B, 2, 2]
    plan = lfg.plan_spec(spec)
    assert plan.info().small_kernel == 1
    xin = torch.from_numpy(xt.reshape(-1).view(np.float64).copy()).cuda()
    out = torch.zeros(2 * B * n, dtype=torch.float64, device="cuda")
    plan.execute(xin, out)
    got = np.ascontiguousarray(out.cpu().numpy().view(np.complex128).reshape(n, B).T)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), n


@pytest.mark.parametrize("n", [2, 4, 12])
def test_small_sizes_f32_gapped_equal_bulk_copy(n):
    """The binary32 sizes that the bulk-copy kernel takes over back-to-back lines run on the
    warp-tile kernel over gapped lines: the same bits."""
    B = 777
    x = O.uniform_complex((B, n), seed=n).astype(np.complex64)
    d = n + 1
    buf = np.zeros((B, d), dtype=np.complex64)
    buf[:, :n] = x
    spec = [0, -1, 1, 1, 0, 1, 0, 1, n, 2, 2, B, 2 * d, 2 * d]
    plan = lfg.plan_spec(spec, precision="f32")
    assert plan.info().small_kernel == 1
    xin = torch.from_numpy(buf.reshape(-1).view(np.float32).copy()).cuda()
    out = torch.zeros(2 * B * d, dtype=torch.float32, device="cuda")
    plan.execute(xin, out)
    got = np.ascontiguousarray(out.cpu().numpy().view(np.complex64).reshape(B, d)[:, :n])
    packed = lfg.plan_1d(n, -1, B, precision="f32")
    assert packed.info().small_kernel == 0
    ref = packed.execute(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), n


@pytest.mark.parametrize("n", [18, 20, 21, 22, 24, 25, 26, 27, 28, 30, 32])
def test_two_pass_f32_sizes(n):
    """Binary32 two-pass sizes up to 32: odd sizes over back-to-back lines, and every size over
    gapped lines, run on the warp-tile kernel (even sizes over back-to-back lines take the
    bulk-copy kernel); all give the group kernels' bits, in place too, and scaled."""
    B = 1000 + n
    x = O.uniform_complex((B, n), seed=50 + n).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    d = n + 1
    buf = np.zeros((B, d), dtype=np.complex64)
    buf[:, :n] = x
    for sign in (-1, 1):
        ref = lfg.plan_1d(n, sign, B, precision="f32", generic_kernels=True).execute(xd)
        plan = lfg.plan_1d(n, sign, B, precision="f32")
        assert plan.info().small_kernel == n % 2, n
        assert _bits_equal(plan.execute(xd), ref), (n, sign)
        inplace = xd.clone()
        plan.execute(inplace, inplace)
        assert _bits_equal(inplace, ref), (n, sign)
        spec = [0, sign, 1, 1, 0, 1, 0, 1, n, 2, 2, B, 2 * d, 2 * d]
        gapped = lfg.plan_spec(spec, precision="f32")
        assert gapped.info().small_kernel == 1
        xin = torch.from_numpy(buf.reshape(-1).view(np.float32).copy()).cuda()
        out = torch.zeros(2 * B * d, dtype=torch.float32, device="cuda")
        gapped.execute(xin, out)
        got = np.ascontiguousarray(out.cpu().numpy().view(np.complex64).reshape(B, d)[:, :n])
        assert np.array_equal(got.view(np.uint32), ref.cpu().numpy().view(np.uint32)), (n, sign)
    scaled = lfg.plan_1d(n, 1, B, precision="f32").set_scale(1.0 / n)
    gen = lfg.plan_1d(n, 1, B, precision="f32", generic_kernels=True).set_scale(1.0 / n)
    assert _bits_equal(scaled.execute(xd), gen.execute(xd)), n


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("n", [2, 3, 8, 16])
def test_small_pipelined_equals_plain(n, precision, monkeypatch):
    """One-pass plans run the pipelined variant (asynchronous copies into two tiles per warp);
    the unpipelined one (LFG_SMALL_PIPE=0) gives the same bits."""
    B = 3001 + n
    dt = torch.complex128 if precision == "f64" else torch.complex64
    xd = torch.from_numpy(O.uniform_complex((B, n), seed=70 + n)).to("cuda", dt)
    piped = lfg.plan_1d(n, -1, B, precision=precision).execute(xd)
    monkeypatch.setenv("LFG_SMALL_PIPE", "0")
    plain = lfg.plan_1d(n, -1, B, precision=precision).execute(xd)
    assert _bits_equal(piped, plain), (n, precision)
