"""PyTorch integration: differentiable transforms over the native kernels.

The transforms are lean-fftw's (unnormalised, forward sign -1; LeanFFTW/Spec/DFT.lean:24-29).
Every gradient runs on a hand-written adjoint kernel, never on torch.fft:

* c2c: y = s F_sign x, so grad_x = s F_{-sign} grad_y -- the conjugate-sign unnormalised
  transform with the same scale s applied in the kernel's store (`Plan.set_scale`);
* r2c: grad_x = c2r of the cotangent with its bins 1..n/2-1 halved (exact, in the c2r
  kernel's prologue: `plan_c2r(adjoint=True)`);
* c2r: grad_h = r2c of the cotangent with its bins 1..n/2-1 doubled (exact, in the r2c
  kernel's epilogue: `plan_r2c(adjoint=True)`).

Tensors are complex128 / float64 CUDA tensors; the transform runs along the last dimension,
on torch's current stream.  Plans are cached per (size, batch, direction, scale, device).
"""
from __future__ import annotations

import math
from functools import lru_cache

import torch

from .plan import plan_1d, plan_c2r, plan_r2c


@lru_cache(maxsize=64)
def _c2c_plan(n: int, sign: int, batch: int, scale: float, device: int):
    with torch.cuda.device(device):
        p = plan_1d(n, sign, batch)
        if scale != 1.0:
            p.set_scale(scale)
        return p


@lru_cache(maxsize=64)
def _real_plan(kind: str, n: int, batch: int, adjoint: bool, device: int):
    with torch.cuda.device(device):
        return (plan_r2c if kind == "r2c" else plan_c2r)(n, batch, adjoint=adjoint)


def _check(x: torch.Tensor, dtype) -> None:
    if not x.is_cuda:
        raise ValueError("lfg transforms run on CUDA tensors")
    if x.dtype != dtype:
        raise TypeError(f"expected {dtype}, got {x.dtype}")


def _scale(norm: str, n: int, inverse: bool) -> float:
    if norm == "backward":
        return 1.0 / n if inverse else 1.0
    if norm == "forward":
        return 1.0 if inverse else 1.0 / n
    if norm == "ortho":
        return 1.0 / math.sqrt(n)
    if norm == "none":
        return 1.0
    raise ValueError(f"unknown norm {norm!r}")


class _C2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, sign: int, scale: float):
        _check(x, torch.complex128)
        n = x.shape[-1]
        batch = x.numel() // n
        xc = x.contiguous()
        y = _c2c_plan(n, sign, batch, scale, x.device.index).execute(xc)
        ctx.meta = (n, sign, batch, scale, x.device.index)
        return y.view(x.shape)

    @staticmethod
    def backward(ctx, g):
        n, sign, batch, scale, dev = ctx.meta
        gc = g.contiguous()
        gx = _c2c_plan(n, -sign, batch, scale, dev).execute(gc)
        return gx.view(g.shape), None, None


class _R2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        _check(x, torch.float64)
        n = x.shape[-1]
        batch = x.numel() // n
        out = torch.empty(x.shape[:-1] + (n // 2 + 1,), dtype=torch.complex128, device=x.device)
        _real_plan("r2c", n, batch, False, x.device.index).execute(x.contiguous(), out)
        ctx.meta = (n, batch, x.device.index)
        return out

    @staticmethod
    def backward(ctx, g):
        n, batch, dev = ctx.meta
        gx = torch.empty(g.shape[:-1] + (n,), dtype=torch.float64, device=g.device)
        _real_plan("c2r", n, batch, True, dev).execute(g.contiguous(), gx)
        return gx


class _C2R(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h, n: int):
        _check(h, torch.complex128)
        batch = h.numel() // h.shape[-1]
        out = torch.empty(h.shape[:-1] + (n,), dtype=torch.float64, device=h.device)
        _real_plan("c2r", n, batch, False, h.device.index).execute(h.contiguous(), out)
        ctx.meta = (n, batch, h.device.index)
        return out

    @staticmethod
    def backward(ctx, g):
        n, batch, dev = ctx.meta
        gh = torch.empty(g.shape[:-1] + (n // 2 + 1,), dtype=torch.complex128, device=g.device)
        _real_plan("r2c", n, batch, True, dev).execute(g.contiguous(), gh)
        return gh, None


def fft(x: torch.Tensor, norm: str = "none") -> torch.Tensor:
    """Forward complex DFT along the last axis (sign -1); norm "none" (lean-fftw's
    unnormalised transform, the default), "backward", "ortho" or "forward"."""
    return _C2C.apply(x, -1, _scale(norm, x.shape[-1], False))


def ifft(x: torch.Tensor, norm: str = "none") -> torch.Tensor:
    """Backward complex DFT along the last axis (sign +1); unnormalised by default."""
    return _C2C.apply(x, 1, _scale(norm, x.shape[-1], True))


def rfft(x: torch.Tensor) -> torch.Tensor:
    """r2c along the last axis (even size): n reals -> n/2+1 complex, unnormalised."""
    return _R2C.apply(x)


def irfft(h: torch.Tensor, n: int) -> torch.Tensor:
    """c2r along the last axis: n/2+1 complex -> n reals (even n), unnormalised; the
    imaginary parts of bins 0 and n/2 are ignored."""
    return _C2R.apply(h, n)
