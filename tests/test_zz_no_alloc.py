"""lfg_execute_inplace_static: in-place execution that allocates nothing.

For callers that may not allocate device memory themselves (runtimes that own all device
memory through their own pool, or loops that cannot take cudaMalloc's implicit device
synchronisation), the library offers this one entry point: a two-group plan's intermediate
goes to a fixed 16 MiB static device array instead of a cudaMalloc'd plan buffer.  Called
through the C ABI with ctypes, its output must equal the regular entry point's (lfg_execute,
in place), bit for bit -- the tolerance every parity test here uses -- on two calls in a row,
in binary64 and binary32, one pass group and two; a plan whose intermediate would not fit the
array, or that runs another algorithm (a prime factor above 13), is refused with a clear error.

This file sorts last on purpose, so a run that stops at the first failure has run every other
test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
from lfg._lib import LFG_ERR_UNSUPPORTED, LFG_OK  # noqa: E402


def _entry():
    f = lfg.lib().lfg_execute_inplace_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def _random(shape, dtype, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    real = torch.rand(shape + (2,), generator=g, dtype=torch.float64) - 0.5
    return torch.view_as_complex(real).to(dtype).cuda()


@pytest.mark.parametrize("n,howmany,precision,groups", [
    (16384, 32, "f64", 2), (65536, 8, "f64", 2), (1024, 16, "f64", 1),
    (4096, 64, "f32", 1), (8192, 64, "f32", 2), (16384, 32, "f32", 2), (65536, 16, "f32", 2)])
def test_static_scratch_matches_regular_entry(n, howmany, precision, groups):
    dtype = torch.complex128 if precision == "f64" else torch.complex64
    plan = lfg.plan_1d(n, -1, howmany, precision=precision)
    assert plan.info().ngroups == groups           # two-group plans use the static array
    stream = torch.cuda.current_stream().cuda_stream
    f = _entry()
    for call in range(2):                           # two calls in a row share the array
        x = _random((howmany, n), dtype, seed=10 * n + call)
        ref = x.clone()
        plan.execute(ref, ref)                      # regular entry point, in place
        got = x.clone()
        rc = f(ctypes.c_void_p(plan.handle), ctypes.c_void_p(got.data_ptr()),
               ctypes.c_void_p(stream))
        assert rc == LFG_OK, lfg.lib().lfg_last_error()
        torch.cuda.synchronize()
        assert torch.equal(torch.view_as_real(got), torch.view_as_real(ref)), (n, call)


def test_oversized_intermediate_is_refused():
    n, howmany = 1 << 18, 16                        # 64 MiB intermediate > 16 MiB array
    plan = lfg.plan_1d(n, -1, howmany)
    assert plan.info().ngroups == 2
    buf = torch.zeros((howmany, n), dtype=torch.complex128, device="cuda")
    before = buf.clone()
    rc = _entry()(ctypes.c_void_p(plan.handle), ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == LFG_ERR_UNSUPPORTED
    assert b"static scratch" in lfg.lib().lfg_last_error()
    torch.cuda.synchronize()
    assert torch.equal(buf, before)                 # nothing ran


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_other_algorithms_are_refused(precision):
    """n = 17 runs the generic engine's sums (binary64) or Bluestein's convolution (binary32),
    which keep buffers of their own: refused on the host before anything is launched."""
    plan = lfg.plan_1d(17, -1, 4, precision=precision)
    dtype = torch.complex128 if precision == "f64" else torch.complex64
    buf = _random((4, 17), dtype, seed=17)
    before = buf.clone()
    rc = _entry()(ctypes.c_void_p(plan.handle), ctypes.c_void_p(buf.data_ptr()), None)
    assert rc == LFG_ERR_UNSUPPORTED
    assert b"13-smooth" in lfg.lib().lfg_last_error()
    torch.cuda.synchronize()
    assert torch.equal(buf, before)
