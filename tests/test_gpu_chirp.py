"""Sizes with a prime factor above 13.

lean-fftw's fast engine plans only 13-smooth sizes; its generic engine takes any size, with a
direct sum for each prime factor (Core/Alg.lean:31-105).  Up to 4096 points with factors up
to 1024 the GPU runs that same algorithm (generic.cu) and must match the oracle's restatement
of it bit for bit; larger sizes go through Bluestein's identity on the library's own
transforms and must be at least as accurate: relative L2 error against the
extended-precision DFT within 1.5x of the generic engine's, forward and backward, batched and
strided, and inside multi-axis and r2r plans."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


def _exec(plan, x, dtype=torch.complex128):
    xd = torch.from_numpy(np.ascontiguousarray(x)).to("cuda", dtype)
    y = torch.empty_like(xd)
    plan.execute(xd, y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("n", [17, 19, 23, 29, 31, 34, 37, 97, 101, 127, 289, 1009, 2 * 3 * 17 * 19,
                               4099, 2 * 2053, 17 * 1031])
def test_non_smooth_error_vs_generic(n):
    B = 3
    x = O.uniform_complex((B, n), seed=n)
    for sign in (-1, 1):
        y = _exec(lfg.plan_1d(n, sign, B), x)
        gen = O.generic_dft(sign < 0, x, nthreads=8)
        if n <= 4096 and _largest_prime(n) <= 1024:
            assert np.array_equal(y.view(np.uint64), gen.view(np.uint64)), (n, sign)
            continue
        ref = O.dd_dft(sign < 0, x, nthreads=8)
        e_gpu, e_gen = O.rel_l2(y, ref), O.rel_l2(gen, ref)
        assert e_gpu <= 1.5 * e_gen + 1e-16, (n, sign, e_gpu, e_gen)


def _largest_prime(n):
    best, d = 1, 2
    while d * d <= n:
        while n % d == 0:
            best, n = max(best, d), n // d
        d += 1
    return max(best, n) if n > 1 else best


def test_chirp_large_prime_roundtrip():
    n, B = 65537, 2
    x = O.uniform_complex((B, n), seed=3)
    y = _exec(lfg.plan_1d(n, -1, B), x)
    z = _exec(lfg.plan_1d(n, 1, B).set_scale(1.0 / n), y)
    assert np.max(np.abs(z - x)) < 1e-13
    # spot check against numpy's transform
    ref = np.fft.fft(x, axis=-1)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-14


def test_chirp_strided_spec_and_inplace():
    n, B = 101, 4
    istride, idist = 2, 2 * n + 5
    total = (n - 1) * istride + (B - 1) * idist + 1
    buf = O.uniform_complex((total,), seed=8)
    spec = [0, -1, 1, 1, 0, 1, 0, 1, n, 2 * istride, 2, B, 2 * idist, 2 * n]
    plan = lfg.plan_spec(spec)
    out = torch.zeros(B * n, dtype=torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(buf).cuda(), out)
    torch.cuda.synchronize()
    lines = np.stack([buf[b * idist + istride * np.arange(n)] for b in range(B)])
    ref = O.dd_dft(True, lines, nthreads=8)
    assert O.rel_l2(out.cpu().numpy().reshape(B, n), ref) < 1e-15
    p2 = lfg.plan_1d(n, -1, B)
    a = torch.from_numpy(lines.copy()).cuda()
    b = torch.empty_like(a)
    p2.execute(a, b)
    p2.execute(a, a)                              # in place
    torch.cuda.synchronize()
    assert torch.equal(a, b)


def test_chirp_in_multiaxis_and_fp32():
    shape = (17, 24)
    x = O.uniform_complex(shape, seed=5)
    spec = [0, -1, 2, 0, 0, 1, 0, 1, 17, 48, 48, 24, 2, 2]
    y = _exec(lfg.plan_spec(spec), x)
    ref = np.fft.fft2(x)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-15
    n = 1009
    x32 = O.uniform_complex((2, n), seed=6).astype(np.complex64)
    y32 = _exec(lfg.plan_1d(n, -1, 2, precision="f32"), x32, torch.complex64)
    e = O.rel_l2(y32.astype(np.complex128), O.dd_dft(True, x32.astype(np.complex128), nthreads=8))
    assert e < 8 * 2.0 ** -24, e
