"""The binary32 variant: error against the extended-precision oracle, per size.

Twiddles come from the binary64 exact-integer tables (rounded to binary32); sizes >= 2^16
use compensated (hi, lo) twiddle products in their last passes.  The error is measured
against the double-double DFT of the same (binary32) input and must stay at the binary32
level (a few times 2^-24); compensated products must lower it at the largest sizes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

U32 = 2.0 ** -24


def _run(n, B, x, sign=-1, compensated=True):
    plan = lfg.plan_1d(n, sign, B, precision="f32", compensated=compensated)
    xd = torch.from_numpy(x.astype(np.complex64)).cuda()
    y = plan.execute(xd)
    torch.cuda.synchronize()
    assert lfg.lib().lfg_device_status(plan._h) == 0     # no bounded wait gave up
    return y.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("n", [2 ** k for k in range(1, 19)] + [6, 60, 360, 1000, 10368, 75600])
def test_fp32_error_per_size(n):
    B = max(1, min(8, (1 << 17) // n))
    x = O.uniform_complex((B, n), seed=n).astype(np.complex64).astype(np.complex128)
    for sign in (-1, 1):
        y = _run(n, B, x, sign)
        e = O.rel_l2(y, O.dd_dft(sign < 0, x, nthreads=8))
        assert e < 4 * U32 * max(1.0, np.sqrt(np.log2(n))), (n, sign, e)


def test_fp32_inplace_and_unaligned():
    """The persistent bulk-copy kernel runs in place; a buffer offset by one complex value
    (8 bytes, not 16-byte aligned) takes the other kernel; both agree."""
    n, B = 1024, 37
    x = O.uniform_complex((B + 1, n), seed=3).astype(np.complex64)
    plan = lfg.plan_1d(n, -1, B, precision="f32")
    a = torch.from_numpy(x[:B].copy()).cuda()
    ref = plan.execute(a.clone())
    plan.execute(a, a)                                   # in place
    buf = torch.from_numpy(x.reshape(-1)).cuda()
    un_in = buf[1: 1 + B * n]                            # 8-byte offset
    un_out = torch.empty(B * n + 1, dtype=torch.complex64, device="cuda")[1:]
    plan.execute(un_in, un_out)
    torch.cuda.synchronize()
    assert torch.equal(a, ref)
    shifted = torch.from_numpy(x.reshape(-1)[1: 1 + B * n].reshape(B, n)).cuda()
    assert torch.equal(un_out.view(B, n), plan.execute(shifted))


@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("n", [1 << k for k in range(4, 13)])
def test_power_of_two_variants_equal_generic_passes(n, sign):
    """One-group power-of-two plans run a kernel whose passes are compiled for the plan
    (shifts, masks and immediate offsets instead of runtime index arithmetic): the
    register-staged kernel for 2^9 .. 2^12 points (any 8-byte aligned buffer), else the
    persistent bulk-copy kernel, whose buffers offset by one complex value (not 16-byte
    aligned) take the generic kernel with runtime pass descriptors.  Every route, and the
    generic kernels (LFG_GENERIC_KERNELS), must give the same bits; a batch that is not a
    multiple of the tile leaves a partial last tile."""
    B = max(3, min(64, (1 << 16) // n)) + 1
    x = O.uniform_complex((B + 1, n), seed=n + sign).astype(np.complex64)
    plan = lfg.plan_1d(n, sign, B, precision="f32")
    assert plan.info().direct_groups == (1 if 512 <= n <= 4096 else 0)
    aligned = torch.from_numpy(x[:B].copy()).cuda()
    fast = plan.execute(aligned)
    generic = lfg.plan_1d(n, sign, B, precision="f32", generic_kernels=True)
    assert generic.info().direct_groups == 0
    assert torch.equal(generic.execute(aligned), fast), n
    inplace = aligned.clone()
    plan.execute(inplace, inplace)
    assert torch.equal(inplace, fast), n
    buf = torch.from_numpy(x.reshape(-1)).cuda()
    un_out = torch.empty(B * n + 1, dtype=torch.complex64, device="cuda")[1:]
    plan.execute(buf[1: 1 + B * n], un_out)                     # 8-byte offset: generic
    shifted = torch.from_numpy(x.reshape(-1)[1: 1 + B * n].reshape(B, n)).cuda()
    fast_shifted = plan.execute(shifted)                         # aligned copy: variant
    torch.cuda.synchronize()
    assert torch.equal(un_out.view(B, n), fast_shifted), n
    ref = O.dd_dft(sign < 0, x[:B].astype(np.complex128), nthreads=8)
    e = O.rel_l2(fast.cpu().numpy().astype(np.complex128), ref)
    assert e < 4 * U32 * max(1.0, np.sqrt(np.log2(n))), (n, e)


@pytest.mark.parametrize("comp", [True, False])
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("n", [1 << k for k in range(13, 19)])
def test_two_group_variants_equal_generic_kernels(n, sign, comp):
    """Two-group power-of-two plans (2^13 .. 2^18) run each group on the register-staged
    kernel compiled for its geometry (first pass from global memory, last pass to global
    memory, second-group tables in pass order); the generic kernels (LFG_GENERIC_KERNELS)
    must give the same bits, compensated or not, out of place (the intermediate in the
    output) and in place."""
    B = max(2, (1 << 20) // n)
    x = torch.from_numpy(O.uniform_complex((B, n), seed=n + sign).astype(np.complex64)).cuda()
    fast = lfg.plan_1d(n, sign, B, precision="f32", compensated=comp)
    slow = lfg.plan_1d(n, sign, B, precision="f32", compensated=comp, generic_kernels=True)
    assert fast.info().ngroups == 2
    assert fast.info().direct_groups == 2
    assert slow.info().direct_groups == 0
    a, b = fast.execute(x), slow.execute(x)
    torch.cuda.synchronize()
    assert torch.equal(a, b), n
    c = x.clone()
    fast.execute(c, c)                               # in place (through the plan's scratch)
    torch.cuda.synchronize()
    assert torch.equal(c, a)


@pytest.mark.parametrize("n,B", [(256, 37), (512, 64), (1024, 9), (2048, 5), (4096, 3), (600, 7)])
def test_real_rows_register_staged_equal_generic(n, B):
    """Binary32 r2c rows of a power-of-two size with a register-staged kernel (first pass from
    the rows, split epilogue from the last shared tile) give the generic kernel's bits; the
    batch leaves a partial last tile; a size without such a kernel (600) is unaffected."""
    x = torch.from_numpy(np.random.default_rng(n).random((B, n)).astype(np.float32) - 0.5).cuda()
    fast, slow = lfg.plan_r2c(n, B, precision="f32"), lfg.plan_r2c(n, B, precision="f32", generic_kernels=True)
    yf = torch.empty(B, n // 2 + 1, dtype=torch.complex64, device="cuda")
    ys = torch.empty_like(yf)
    fast.execute(x, yf)
    slow.execute(x, ys)
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(yf), torch.view_as_real(ys)), n


@pytest.mark.parametrize("n0,n1,B", [(512, 512, 3), (256, 256, 2), (64, 1024, 2), (128, 128, 5),
                                     (100, 512, 2), (512, 60, 2)])
def test_real_2d_register_staged_equal_generic(n0, n1, B):
    """Binary32 rank-2 r2c and c2r: the register-staged row kernel and column kernel (16
    columns per tile, tiles straddling images; power-of-two column lengths 64 .. 512) give
    the generic kernels' bits in both directions."""
    x = torch.from_numpy(np.random.default_rng(n0 + n1).random((B, n0, n1)).astype(np.float32)
                         - 0.5).cuda()
    h = n1 // 2 + 1
    fast = lfg.plan_r2c_2d(n0, n1, B, precision="f32")
    slow = lfg.plan_r2c_2d(n0, n1, B, precision="f32", generic_kernels=True)
    yf = torch.empty(B, n0, h, dtype=torch.complex64, device="cuda")
    ys = torch.empty_like(yf)
    fast.execute(x, yf)
    slow.execute(x, ys)
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(yf), torch.view_as_real(ys)), (n0, n1)
    cf = lfg.plan_c2r_2d(n0, n1, B, precision="f32")
    cs = lfg.plan_c2r_2d(n0, n1, B, precision="f32", generic_kernels=True)
    zf = torch.empty(B, n0, n1, dtype=torch.float32, device="cuda")
    zs = torch.empty_like(zf)
    cf.execute(yf.clone(), zf)
    cs.execute(yf.clone(), zs)
    torch.cuda.synchronize()
    assert torch.equal(zf, zs), (n0, n1)
    # and the round trip is the identity up to binary32 rounding (scale n0 * n1)
    e = float(torch.linalg.vector_norm(zf / (n0 * n1) - x) / torch.linalg.vector_norm(x))
    assert e < 1e-5, e


@pytest.mark.parametrize("n", [1 << 16, 1 << 17, 1 << 18])
def test_compensation_helps_large_sizes(n):
    """Compensated (hi, lo) twiddle products in the last passes remove the twiddles' own
    binary32 rounding from those passes: the error must drop, by at least 1 % (measured:
    2.2-2.5 % at 2^16-2^18; the rest of the binary32 error is the butterflies' rounding)."""
    B = 4
    x = O.uniform_complex((B, n), seed=7).astype(np.complex64).astype(np.complex128)
    ref = O.dd_dft(True, x, nthreads=8)
    e_comp = O.rel_l2(_run(n, B, x, compensated=True), ref)
    e_plain = O.rel_l2(_run(n, B, x, compensated=False), ref)
    assert e_comp < 0.99 * e_plain, (e_comp, e_plain)


def test_bounded_wait_recovery():
    """The persistent binary32 kernel waits on its bulk copies with an iteration limit.  A
    plan made with LFG_TEST_WAIT_GIVE_UP gives every tile wait up at once (the copies still
    land, and each CTA waits for its own before it exits): the call reports LFG_ERR_TIMEOUT
    through lfg_device_status, the status is then clear, and the next call of a normal plan
    on the same data is correct to the bit."""
    import ctypes
    from lfg._lib import LFG_ERR_TIMEOUT, LFG_OK, LFG_TEST_WAIT_GIVE_UP, lib
    n, B = 1024, 4096
    x = torch.from_numpy(O.uniform_complex((B, n), seed=11).astype(np.complex64)).cuda()
    h = ctypes.c_void_p()
    assert lib().lfg_plan_1d(n, -1, B, 1, LFG_TEST_WAIT_GIVE_UP, ctypes.byref(h)) == LFG_OK
    failing = lfg.Plan(h)
    y = torch.zeros_like(x)
    failing.execute(x, y)
    assert lib().lfg_device_status(failing.handle) == LFG_ERR_TIMEOUT
    assert lib().lfg_device_status(failing.handle) == LFG_OK        # cleared once read
    good = lfg.plan_1d(n, -1, B, precision="f32")
    ref = good.execute(x)
    torch.cuda.synchronize()
    assert lib().lfg_device_status(good.handle) == LFG_OK
    again = torch.empty_like(x)
    good.execute(x, again)
    torch.cuda.synchronize()
    assert torch.equal(again, ref)
    ref64 = O.ref_transform(True, n, good.radices, x.cpu().numpy().astype(np.complex128)[:8])
    e = O.rel_l2(ref[:8].cpu().numpy().astype(np.complex128), ref64)
    assert e < 4 * U32 * np.sqrt(np.log2(n)), e
