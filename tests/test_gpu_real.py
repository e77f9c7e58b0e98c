"""GPU r2c / c2r (rank 1 and 2) against the double-double oracle.

lean-fftw computes these in its generic engine (Core/Problem.lean:142-150, 222-236); the
parity bar is the relative L2 error against the extended-precision DFT: within 1.5x of the
generic engine's own error (restated in the oracle) on the same inputs.  c2r must ignore the
imaginary parts of bins 0 and n/2 (docs/CONTRACT.md:20-23).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

SIZES = [2, 4, 6, 8, 10, 12, 16, 30, 60, 64, 210, 512, 1000, 1024, 2048, 4096, 8192, 10368]


def _r2c(x, n):
    B = x.shape[0]
    plan = lfg.plan_r2c(n, B)
    out = torch.empty((B, n // 2 + 1), dtype=torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(x).cuda(), out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _c2r(h, n):
    B = h.shape[0]
    plan = lfg.plan_c2r(n, B)
    out = torch.empty((B, n), dtype=torch.float64, device="cuda")
    plan.execute(torch.from_numpy(np.ascontiguousarray(h)).cuda(), out)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("n", SIZES)
def test_r2c_error_vs_reference(n):
    B = 4
    x = np.random.default_rng(n).random((B, n)) - 0.5
    ref = O.dd_r2c(x, nthreads=8)
    e_gpu = O.rel_l2(_r2c(x, n), ref)
    e_ref = O.rel_l2(O.generic_r2c(x, nthreads=8), ref)
    assert e_gpu <= 1.5 * e_ref + 1e-17, (n, e_gpu, e_ref)


@pytest.mark.parametrize("n", SIZES)
def test_c2r_error_vs_reference(n):
    B = 4
    rng = np.random.default_rng(n + 1)
    h = (rng.random((B, n // 2 + 1, 2)) - 0.5).view(np.complex128)[..., 0]
    ref = O.dd_c2r(h, n, nthreads=8)
    e_gpu = O.rel_l2(_c2r(h, n), ref)
    e_ref = O.rel_l2(O.generic_c2r(h, n, nthreads=8), ref)
    assert e_gpu <= 1.5 * e_ref + 1e-17, (n, e_gpu, e_ref)
    # imaginary parts of the self-conjugate bins are ignored
    h2 = h.copy()
    h2[:, 0] += 3j
    h2[:, n // 2] -= 5j
    assert np.array_equal(_c2r(h2, n), _c2r(h, n))


def test_r2c_c2r_pair_batch256_8192():
    n, B = 8192, 256
    x = np.random.default_rng(20261016).random((B, n)) - 0.5
    X = _r2c(x, n)
    e = O.rel_l2(X, O.dd_r2c(x, nthreads=16))
    assert e < 4e-16, e
    y = _c2r(X, n)
    assert np.max(np.abs(y / n - x)) < 1e-14


@pytest.mark.parametrize("n0,n1,B", [(512, 512, 3), (12, 60, 5), (64, 8, 2)])
def test_rank2_r2c_c2r(n0, n1, B):
    x = np.random.default_rng(7).random((B, n0, n1)) - 0.5
    plan = lfg.plan_r2c_2d(n0, n1, B)
    out = torch.empty((B, n0, n1 // 2 + 1), dtype=torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(x).cuda(), out)
    torch.cuda.synchronize()
    X = out.cpu().numpy()
    ref = O.dd_rank2_r2c(x, nthreads=16)
    e_gpu = O.rel_l2(X, ref)
    e_gen = O.rel_l2(O.generic_rank2_r2c(x, nthreads=16), ref)
    assert e_gpu <= 1.5 * e_gen + 1e-17, (e_gpu, e_gen)
    back = lfg.plan_c2r_2d(n0, n1, B)
    y = torch.empty((B, n0, n1), dtype=torch.float64, device="cuda")
    xin = out.clone()
    back.execute(out, y)
    torch.cuda.synchronize()
    assert torch.equal(xin, out)           # the input is not destroyed
    assert np.max(np.abs(y.cpu().numpy() / (n0 * n1) - x)) < 1e-14


def test_rdft2_spec_vector():
    """FFI encoding of a batched r2c (kind 1, sign -1): real lines with a pitch, complex
    output with a pitch (strides and offsets in doubles)."""
    n, B = 360, 3
    rpitch, cpitch = n + 6, n // 2 + 5          # doubles / complex elements
    xbuf = np.random.default_rng(3).random(2 + rpitch * B) - 0.5
    spec = [1, -1, 1, 1, 2, 2, 2, 3, n, 1, 2, B, rpitch, 2 * cpitch]
    plan = lfg.plan_spec(spec)
    out = torch.zeros(1 + cpitch * B, dtype=torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(xbuf).cuda(), out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    for b in range(B):
        x = xbuf[2 + b * rpitch: 2 + b * rpitch + n]
        got = o[1 + b * cpitch: 1 + b * cpitch + n // 2 + 1]
        e = O.rel_l2(got, O.dd_r2c(x[None, :]))
        assert e < 3e-16, e


# ---- binary32 variant -------------------------------------------------------------------
U32 = 2.0 ** -24


@pytest.mark.parametrize("n", [2, 6, 16, 60, 512, 1024, 8192, 10368])
def test_fp32_r2c_c2r_error(n):
    """Binary32 r2c and c2r (twiddles rounded once from the binary64 tables): relative L2
    error against the double-double DFT of the same binary32 data at the binary32 level."""
    B = 4
    rng = np.random.default_rng(n + 100)
    x = (rng.random((B, n)) - 0.5).astype(np.float32)
    plan = lfg.plan_r2c(n, B, precision="f32")
    out = torch.empty((B, n // 2 + 1), dtype=torch.complex64, device="cuda")
    plan.execute(torch.from_numpy(x).cuda(), out)
    torch.cuda.synchronize()
    X = out.cpu().numpy().astype(np.complex128)
    bound = 4 * U32 * max(1.0, np.sqrt(np.log2(n)))
    e = O.rel_l2(X, O.dd_r2c(x.astype(np.float64), nthreads=8))
    assert e < bound, (n, e)
    h = X.astype(np.complex64)
    back = lfg.plan_c2r(n, B, precision="f32")
    y = torch.empty((B, n), dtype=torch.float32, device="cuda")
    back.execute(torch.from_numpy(h).cuda(), y)
    torch.cuda.synchronize()
    e2 = O.rel_l2(y.cpu().numpy().astype(np.float64),
                  O.dd_c2r(h.astype(np.complex128), n, nthreads=8))
    assert e2 < bound, (n, e2)


def test_fp32_rank2_64x512x512():
    """The large-image configuration: 64 images of 512 x 512, binary32 r2c and c2r."""
    n0 = n1 = 512
    B = 64
    x = (np.random.default_rng(5).random((B, n0, n1)) - 0.5).astype(np.float32)
    plan = lfg.plan_r2c_2d(n0, n1, B, precision="f32")
    out = torch.empty((B, n0, n1 // 2 + 1), dtype=torch.complex64, device="cuda")
    plan.execute(torch.from_numpy(x).cuda(), out)
    torch.cuda.synchronize()
    X = out.cpu().numpy()
    ref = np.fft.rfft2(x[:2].astype(np.float64))           # two images checked in full
    e = np.linalg.norm(X[:2] - ref) / np.linalg.norm(ref)
    assert e < 8 * U32, e
    back = lfg.plan_c2r_2d(n0, n1, B, precision="f32")
    y = torch.empty((B, n0, n1), dtype=torch.float32, device="cuda")
    back.execute(out, y)
    torch.cuda.synchronize()
    r = y.cpu().numpy() / (n0 * n1)
    assert np.max(np.abs(r - x)) < 64 * U32, np.max(np.abs(r - x))


def test_fp32_rank2_in_fresh_process():
    """A binary32 rank-2 real plan must set up its own kernels: run it in a process that has
    made no other plan (kernel attributes are per process)."""
    import subprocess
    import sys
    from conftest import ROOT
    code = ("import sys; sys.path.insert(0, 'lean-fftw_gb300'); import numpy as np, torch, lfg\n"
            "x = torch.rand(8, 512, 512, device='cuda') - 0.5\n"
            "out = torch.empty((8, 512, 257), dtype=torch.complex64, device='cuda')\n"
            "lfg.plan_r2c_2d(512, 512, 8, precision='f32').execute(x, out)\n"
            "ref = np.fft.rfft2(x.cpu().numpy().astype(np.float64))\n"
            "e = np.linalg.norm(out.cpu().numpy() - ref) / np.linalg.norm(ref)\n"
            "assert e < 8 * 2.0 ** -24, e\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_rank2_r2c_pinned_host_matches_device(prec):
    """With pinned host buffers the rows go to device scratch and the column pass writes the
    host output; the result equals the device-resident execution bit for bit."""
    n0, n1, B = 96, 128, 5
    rdt = np.float32 if prec == "f32" else np.float64
    cdt = torch.complex64 if prec == "f32" else torch.complex128
    x = (np.random.default_rng(8).random((B, n0, n1)) - 0.5).astype(rdt)
    plan = lfg.plan_r2c_2d(n0, n1, B, precision=prec)
    dev = torch.empty((B, n0, n1 // 2 + 1), dtype=cdt, device="cuda")
    plan.execute(torch.from_numpy(x).cuda(), dev)
    torch.cuda.synchronize()
    hin = torch.from_numpy(x).pin_memory()
    hout = torch.zeros((B, n0, n1 // 2 + 1), dtype=cdt).pin_memory()
    for _ in range(2):
        plan.execute_host(hin.numpy(), hout.numpy())
    assert torch.equal(hout.view(torch.float32 if prec == "f32" else torch.float64),
                       dev.cpu().view(torch.float32 if prec == "f32" else torch.float64))
