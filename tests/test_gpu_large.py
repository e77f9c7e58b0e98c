"""The largest sizes the planner accepts (n = 2^24, lfg_plan_1d's limit, as the libbench2
backend's `can_do` in bench/backends/bench-leanfftw.c:253-268), and 2^20 / 2^22 in between:
two pass groups of up to 4096 points, out of place and in place (the in-place intermediate in
the plan's scratch).  Binary64 results equal lean-fftw's reference transform bit for bit;
binary32 is held to a few binary32 ulps against the binary64 result."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


@pytest.mark.parametrize("k,batch", [(20, 2), (22, 1), (24, 1)])
def test_largest_sizes_bitexact(k, batch):
    n = 1 << k
    x = O.uniform_complex((batch, n), seed=k)
    plan = lfg.plan_1d(n, -1, batch)
    assert plan.info().ngroups == 2
    xd = torch.from_numpy(x).cuda()
    y = plan.execute(xd)
    torch.cuda.synchronize()
    ref = O.ref_transform(True, n, plan.radices, x, nthreads=batch)
    assert np.array_equal(y.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    # in place: same bits
    z = xd.clone()
    plan.execute(z, z)
    torch.cuda.synchronize()
    assert torch.equal(z.view(torch.float64), y.view(torch.float64))


def test_largest_size_backward_and_fp32():
    n = 1 << 24
    x = O.uniform_complex((n,), seed=3)
    xd = torch.from_numpy(x).cuda()
    bwd = lfg.plan_1d(n, 1, 1)
    y = bwd.execute(xd)
    torch.cuda.synchronize()
    ref = O.ref_transform(False, n, bwd.radices, x)
    assert np.array_equal(y.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    f32 = lfg.plan_1d(n, 1, 1, precision="f32")
    y32 = f32.execute(xd.to(torch.complex64))
    torch.cuda.synchronize()
    e = (torch.linalg.vector_norm(y32.to(torch.complex128) - y) / torch.linalg.vector_norm(y)).item()
    assert e < 4 * 2.0 ** -24 * math.sqrt(24), e


@pytest.mark.parametrize("n", [1024, 4096, 360])
def test_special_values_match_reference(n):
    """Signed zeros, subnormals, overflow to infinity, infinities and NaNs: the codelets'
    fused forms (a*1 + b, a*b + (-0)) must round and propagate exactly as the reference's
    separate adds and multiplies.  NaN payloads are not compared, only where NaNs appear."""
    B = 6
    x = O.uniform_complex((B, n), seed=n)
    x[0] = 0.0
    x[1] = -0.0 + 0.0j
    x[1].imag = -0.0
    x[2] *= 1e-310                      # subnormal inputs and results
    x[3, ::7] = 1.7e308                 # sums overflow to infinity
    x[4, 5] = complex(np.inf, -np.inf)
    x[5, 9] = complex(np.nan, 1.0)
    for sign in (-1, 1):
        plan = lfg.plan_1d(n, sign, B)
        y = plan.execute(torch.from_numpy(x).cuda()).cpu().numpy()
        ref = O.ref_transform(sign < 0, n, plan.radices, x)
        yv, rv = y.view(np.float64), ref.view(np.float64)
        nan_y, nan_r = np.isnan(yv), np.isnan(rv)
        assert np.array_equal(nan_y, nan_r)
        assert np.array_equal(yv[~nan_y].view(np.uint64), rv[~nan_r].view(np.uint64))
