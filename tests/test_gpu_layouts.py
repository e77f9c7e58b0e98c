"""Layouts the kernels do not take directly, through dense buffers (pack.cu): split real and
imaginary arrays and strides of either sign (lean-fftw's problem description allows both,
LeanFFTW/FFI.lean:13-21), and rdft2 problems of odd, non-smooth or rank >= 3 sizes or with a
split complex side, computed as the generic engine defines them (Core/Problem.lean:142-150,
222-236)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


def _exec_spec(spec, xbuf, out_len, dtype=torch.float64):
    plan = lfg.plan_spec(spec)
    xin = torch.from_numpy(np.ascontiguousarray(xbuf)).to("cuda", dtype)
    out = torch.zeros(out_len, dtype=dtype, device="cuda")
    plan.execute(xin, out)
    torch.cuda.synchronize()
    return plan, out.cpu().numpy()


@pytest.mark.parametrize("n,B", [(1024, 3), (360, 5), (17, 4)])
def test_split_arrays_c2c(n, B):
    """Re block then im block (libbench2's split layout), both sides: equal to the
    interleaved transform bit for bit (the same inner plan runs on the gathered data)."""
    x = O.uniform_complex((B, n), seed=n)
    buf = np.concatenate([x.real.reshape(-1), x.imag.reshape(-1)])
    spec = [0, -1, 1, 1, 0, n * B, 0, n * B, n, 1, 1, B, n, n]
    plan, o = _exec_spec(spec, buf, 2 * n * B)
    y = o[: n * B] + 1j * o[n * B:]
    ref = lfg.plan_1d(n, -1, B).execute(torch.from_numpy(x).cuda()).cpu().numpy()
    assert np.array_equal(y.view(np.uint64), ref.reshape(-1).view(np.uint64))


def test_negative_strides_c2c():
    """A line read backwards (negative stride) and written backwards."""
    n = 240
    x = O.uniform_complex((n,), seed=2)
    buf = x.view(np.float64)
    # element j at double offset 2(n-1-j): re at 2(n-1) - 2j, im one after
    spec = [0, -1, 1, 0, 2 * (n - 1), 2 * (n - 1) + 1, 2 * (n - 1), 2 * (n - 1) + 1, n, -2, -2]
    plan, o = _exec_spec(spec, buf, 2 * n)
    y = np.ascontiguousarray(o.view(np.complex128)[::-1])
    ref = O.ref_transform(True, n, plan.radices, x[::-1].copy()[None])[0]
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("n", [15, 45, 101, 1001])
def test_rdft2_odd_sizes(n):
    B = 3
    x = np.random.default_rng(n).random((B, n)) - 0.5
    h = n // 2 + 1
    spec = [1, -1, 1, 1, 0, 0, 0, 1, n, 1, 2, B, n, 2 * h]
    _, o = _exec_spec(spec, x.reshape(-1), 2 * h * B)
    X = o.view(np.complex128).reshape(B, h)
    ref = O.dd_r2c(x, nthreads=8)
    e_gpu, e_gen = O.rel_l2(X, ref), O.rel_l2(O.generic_r2c(x, nthreads=8), ref)
    assert e_gpu <= 1.5 * e_gen + 1e-16, (n, e_gpu, e_gen)
    # c2r back (imaginary parts of bin 0 ignored)
    spec_b = [1, 1, 1, 1, 0, 1, 0, 0, n, 2, 1, B, 2 * h, n]
    _, y = _exec_spec(spec_b, X.reshape(-1).view(np.float64), n * B)
    ref_b = O.dd_c2r(X, n, nthreads=8)
    e_gpu = O.rel_l2(y.reshape(B, n), ref_b)
    e_gen = O.rel_l2(O.generic_c2r(X, n, nthreads=8), ref_b)
    assert e_gpu <= 1.5 * e_gen + 1e-16, (n, e_gpu, e_gen)


def test_rdft2_rank3_roundtrip():
    shape = (6, 8, 10)
    B = 2
    x = np.random.default_rng(4).random((B,) + shape) - 0.5
    h = shape[-1] // 2 + 1
    # row-major real (B, 6, 8, 10) -> complex (B, 6, 8, 6)
    spec = [1, -1, 3, 1, 0, 0, 0, 1,
            6, 80, 2 * 8 * h, 8, 10, 2 * h, 10, 1, 2, B, 480, 2 * 6 * 8 * h]
    _, o = _exec_spec(spec, x.reshape(-1), 2 * B * 6 * 8 * h)
    X = o.view(np.complex128).reshape((B, 6, 8, h))
    ref = np.fft.rfftn(x, axes=(1, 2, 3))
    assert np.linalg.norm(X - ref) / np.linalg.norm(ref) < 1e-15
    spec_b = [1, 1, 3, 1, 0, 1, 0, 0,
              6, 2 * 8 * h, 80, 8, 2 * h, 10, 10, 2, 1, B, 2 * 6 * 8 * h, 480]
    _, y = _exec_spec(spec_b, X.reshape(-1).view(np.float64), B * 480)
    assert np.max(np.abs(y.reshape(x.shape) / 480 - x)) < 1e-14


def test_rdft2_split_complex_side():
    n, B = 64, 3
    h = n // 2 + 1
    x = np.random.default_rng(9).random((B, n)) - 0.5
    spec = [1, -1, 1, 1, 0, 0, 0, h * B, n, 1, 1, B, n, h]
    _, o = _exec_spec(spec, x.reshape(-1), 2 * h * B)
    X = (o[: h * B] + 1j * o[h * B:]).reshape(B, h)
    ref = np.fft.rfft(x, axis=-1)
    assert np.linalg.norm(X - ref) / np.linalg.norm(ref) < 1e-15
