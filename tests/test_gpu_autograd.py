"""Gradients through the adjoint kernels (lfg/torch_ops.py).

Differentiation workload: batch 256 x N = 4096 complex FP64, loss = sum |W * FFT(x)|^2 with
W iid complex normal; gradient checked against central finite differences (h = 1e-6,
relative error <= 1e-7) on random directions, and against the analytic adjoint computed by
the oracle's reference transforms (relative error <= 1e-13).  Same for the r2c / c2r pair
at batch 256 x N = 8192 real.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
from lfg import torch_ops as T  # noqa: E402
import oracle as O  # noqa: E402


def _cn(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex128)


def _fd_check(loss, x, grad, rng, ndir=3, h=1e-6):
    for _ in range(ndir):
        v = _cn(rng, x.shape) if x.is_complex() else rng.standard_normal(x.shape)
        vt = torch.from_numpy(v).cuda()
        with torch.no_grad():
            fd = (loss(x + h * vt) - loss(x - h * vt)).item() / (2 * h)
        an = torch.real(torch.sum(torch.conj(grad) * vt)).item() if x.is_complex() else \
            torch.sum(grad * vt).item()
        assert abs(fd - an) <= 1e-7 * abs(an), (fd, an)


def test_c2c_gradient_fd_and_adjoint():
    rng = np.random.default_rng(20261016)
    B, n = 256, 4096
    x0 = O.uniform_complex((B, n), seed=1)
    W = torch.from_numpy(_cn(rng, (B, n))).cuda()
    x = torch.from_numpy(x0).cuda().requires_grad_(True)
    loss = lambda z: torch.sum(torch.abs(W * T.fft(z)) ** 2)
    L = loss(x)
    L.backward()
    g = x.grad.detach()
    _fd_check(loss, x.detach(), g, rng)
    # analytic adjoint on the oracle: grad = F_+ (2 |W|^2 F_- x), reference transforms
    rs = lfg.plan_1d(n, -1, 1).radices
    y = O.ref_transform(True, n, rs, x0, nthreads=16)
    up = 2.0 * np.abs(W.cpu().numpy()) ** 2 * y
    ref = O.ref_transform(False, n, rs, up, nthreads=16)
    err = np.linalg.norm(g.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= 1e-13, err


@pytest.mark.parametrize("norm", ["backward", "ortho", "forward"])
def test_c2c_scaled_norms(norm):
    n = 360
    x = torch.from_numpy(O.uniform_complex((3, n), seed=2)).cuda().requires_grad_(True)
    y = T.fft(x, norm=norm)
    ref = torch.fft.fft(x.detach(), norm=norm)
    assert torch.allclose(y, ref, rtol=0, atol=1e-12)
    g = torch.from_numpy(O.uniform_complex((3, n), seed=3)).cuda()
    (gx,) = torch.autograd.grad(y, x, g)
    # adjoint of s F_- is s F_+
    s = {"backward": 1.0, "ortho": n ** -0.5, "forward": 1.0 / n}[norm]
    ref_g = s * torch.fft.ifft(g, norm="forward")
    assert torch.allclose(gx, ref_g, rtol=0, atol=1e-12)


def test_r2c_c2r_gradients():
    rng = np.random.default_rng(5)
    B, n = 256, 8192
    x0 = rng.random((B, n)) - 0.5
    W = torch.from_numpy(_cn(rng, (B, n // 2 + 1))).cuda()
    x = torch.from_numpy(x0).cuda().requires_grad_(True)
    loss = lambda z: torch.sum(torch.abs(W * T.rfft(z)) ** 2)
    loss(x).backward()
    g = x.grad.detach()
    _fd_check(loss, x.detach(), g, rng)
    # analytic: grad_j = Re sum_{k<=n/2} c_k e^{+2 pi i jk/n}, c = 2 |W|^2 rfft(x)
    X = np.fft.rfft(x0)
    c = 2.0 * np.abs(W.cpu().numpy()) ** 2 * X
    pad = np.zeros((B, n), np.complex128)
    pad[:, : n // 2 + 1] = c
    ref = O.ref_transform(False, n, lfg.plan_1d(n, 1, 1).radices, pad, nthreads=16).real
    err = np.linalg.norm(g.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err <= 1e-13, err

    # c2r: loss = sum (w * irfft(h))^2, with h scaled so that irfft(h) = O(1): the loss must
    # not dwarf its own h-perturbation, or binary64 cannot resolve the difference quotient
    w = torch.from_numpy(rng.standard_normal((B, n))).cuda()
    h0 = np.fft.rfft(rng.random((B, n)) - 0.5) / n
    h = torch.from_numpy(h0).cuda().requires_grad_(True)
    loss2 = lambda z: torch.sum((w * T.irfft(z, n)) ** 2)
    loss2(h).backward()
    gh = h.grad.detach()
    _fd_check(loss2, h.detach(), gh, rng)
    y = T.irfft(h.detach(), n)
    u = (2.0 * w * w * y).cpu().numpy()
    F = O.ref_transform(True, n, lfg.plan_1d(n, -1, 1).radices, u.astype(np.complex128), nthreads=16)
    ref2 = F[:, : n // 2 + 1].copy()
    ref2[:, 1: n // 2] *= 2.0
    err2 = np.linalg.norm(gh.cpu().numpy() - ref2) / np.linalg.norm(ref2)
    assert err2 <= 1e-13, err2
