"""GPU butterflies against lean-fftw's own generated kernels (LeanFFTW/Native/Kernels.lean).

The sixteen radix-2/4/8/16 kernels of the reference's Lean backend (tests/golden/
native_kernels.json, read by oracle/native_dag.py without the product's generator) run here
through the C ABI's explicit radix plans (lfg_plan_1d_radices):

* a plan [R] of size R is one untwiddled butterfly per line: every line's GPU output equals
  the reference kernel bfly{R}n{f,b} applied to it, bit for bit;
* a plan [m, R] ends with the twiddled kernel bfly{R}t{f,b} on the plan's twiddle table: the
  GPU output equals the oracle's refTransform, whose radix-2/4/8/16 butterflies are those
  kernels, bit for bit.

Inputs: uniform random lines, lines of wide dynamic range, and lines holding signed zeros,
subnormals, infinities, NaNs and values whose sums overflow.  NaN payloads are not compared,
only where NaNs appear.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

RADICES = (2, 4, 8, 16)
SPECIALS = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, -1e-310,
            1.7976931348623157e308, -1.7976931348623157e308, math.inf, -math.inf, math.nan, 1e300]


def _lines(n, count, seed):
    rng = np.random.default_rng(seed)
    x = np.empty((3 * count, 2 * n))
    x[:count] = rng.uniform(-0.5, 0.5, (count, 2 * n))
    x[count:2 * count] = rng.standard_normal((count, 2 * n)) * 10.0 ** rng.integers(-300, 300, (count, 2 * n))
    x[2 * count:] = rng.uniform(-1, 1, (count, 2 * n))
    for row in x[2 * count:]:
        idx = rng.choice(2 * n, size=min(2 * n, int(rng.integers(1, 5))), replace=False)
        row[idx] = rng.choice(SPECIALS, size=idx.size)
    return np.ascontiguousarray(x).view(np.complex128)


def _same(a, b) -> bool:
    a, b = np.asarray(a).view(np.float64), np.asarray(b).view(np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint64), b[~nb].view(np.uint64)))


def _gpu(n, rs, fwd, x):
    plan = lfg.plan_1d(n, -1 if fwd else 1, x.shape[0], radices=rs)
    assert list(plan.radices) == list(rs)
    y = plan.execute(torch.from_numpy(x).cuda())
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("fwd", [True, False])
@pytest.mark.parametrize("R", RADICES)
def test_untwiddled_kernel_per_line(R, fwd):
    x = _lines(R, 32, seed=R + 100 * fwd)
    y = _gpu(R, [R], fwd, x)
    for i in range(x.shape[0]):
        want = O.bfly(fwd, R, False, x[i].view(np.float64))
        assert _same(y[i], want), (R, fwd, i)


@pytest.mark.parametrize("fwd", [True, False])
@pytest.mark.parametrize("m", RADICES)
@pytest.mark.parametrize("R", RADICES)
def test_twiddled_kernel_in_a_plan(R, m, fwd):
    n = m * R
    x = _lines(n, 16, seed=1000 * R + 10 * m + fwd)
    y = _gpu(n, [m, R], fwd, x)
    ref = O.ref_transform(fwd, n, [m, R], x)
    assert _same(y, ref), (m, R, fwd)


@pytest.mark.parametrize("fwd", [True, False])
@pytest.mark.parametrize("rs", [[16, 16, 4], [8, 8, 8, 2], [4, 16, 16, 16], [2, 8, 16, 4, 16]])
def test_power_of_two_plans_of_reference_kernels(rs, fwd):
    """Longer plans of these radices: every pass is a reference kernel."""
    n = int(np.prod(rs))
    x = O.uniform_complex((8, n), seed=n + fwd)
    y = _gpu(n, rs, fwd, x)
    assert _same(y, O.ref_transform(fwd, n, rs, x))
