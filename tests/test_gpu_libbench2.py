"""The libbench2 backend (lean-fftw_gb300/csrc/tools/bench_lfg.c) driven through libbench2's
backend interface -- can_do, setup, doit, done -- by the harness of tests/libbench2_stub, on
problems as libbench2 describes them (tensors of (n, is, os), sign, split format, in place).

* 1-D complex unit-stride 13-smooth problems take the fast-engine entry points
  (lfg_lfa_plan_measure / lfg_lfa_call, the reference's lfa_plan_measure / lfa_call): the
  output equals the oracle's refTransform with the measured plan's radices, bit for bit, out
  of place, in place, and after several timed iterations;
* everything else goes through lean-fftw's FFI encoding (lfg_plan_spec on the spanned host
  ranges): multi-dimensional strided batches, split arrays, rdft2 and r2r, and a prime size,
  checked against numpy's transforms;
* problems outside the library's domain (rank 0) are refused by can_do.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
_dp = ctypes.POINTER(ctypes.c_double)


def _harness():
    sys.path.insert(0, os.path.join(HERE, "libbench2_stub"))
    import build_harness
    lfg.lib()                                   # the backend links the same liblfg.so
    L = ctypes.CDLL(build_harness.build())
    L.lfgb_run.restype = ctypes.c_int
    L.lfgb_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                           ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                           _dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return L


def _run(kind, sign, dims, vdims, inp, out, split=0, r2r=None, ini=None, outi=None, iphys=0,
         ophys=0, iters=1):
    L = _harness()
    d = np.ascontiguousarray(np.array(list(dims) + list(vdims), dtype=np.int32).reshape(-1))
    k = None if r2r is None else (ctypes.c_int * len(r2r))(*r2r)
    p = lambda a: None if a is None else a.ctypes.data_as(_dp)
    return L.lfgb_run(kind, sign, len(dims), len(vdims), d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                      k, split, p(inp), p(out), p(ini), p(outi), iphys, ophys, iters)


@pytest.mark.parametrize("n,sign,inplace,iters", [(1024, -1, False, 3), (360, 1, True, 1),
                                                  (2, -1, False, 1), (10368, -1, False, 2)])
def test_fast_engine_path_bitexact(n, sign, inplace, iters):
    x = O.uniform_complex((n,), seed=n)
    inp = x.view(np.float64).copy()
    out = inp if inplace else np.zeros_like(inp)
    assert _run(0, sign, [(n, 1, 1)], [], inp, out, iters=iters) == 0
    radices = lfg.plan_measure(n, sign < 0).radices      # the measured choice, remembered
    ref = O.ref_transform(sign < 0, n, radices, x)
    assert np.array_equal(out.view(np.uint64), ref.view(np.float64).view(np.uint64))


def test_spec_path_strided_batch():
    """A 12 x 10 complex transform over a vector of 3, interleaved, padded rows."""
    n0, n1, v = 12, 10, 3
    rows = 11                                     # complex elements per padded row
    x = O.uniform_complex((v, n0, rows), seed=5)
    out = np.zeros((v, n0, rows), dtype=np.complex128)
    dims = [(n0, rows, rows), (n1, 1, 1)]
    vd = [(v, n0 * rows, n0 * rows)]
    assert _run(0, -1, dims, vd, x.view(np.float64).reshape(-1),
                out.view(np.float64).reshape(-1)) == 0
    ref = np.fft.fft2(x[:, :, :n1])
    assert np.linalg.norm(out[:, :, :n1] - ref) <= 1e-14 * np.linalg.norm(ref)
    assert np.all(out[:, :, n1:] == 0)            # the padding is not written


def test_spec_path_split_arrays_and_prime_size():
    for n in (64, 17):
        x = O.uniform_complex((n,), seed=n)
        re, im = np.ascontiguousarray(x.real), np.ascontiguousarray(x.imag)
        ore, oim = np.zeros(n), np.zeros(n)
        assert _run(0, -1, [(n, 1, 1)], [], re, ore, split=1, ini=im, outi=oim) == 0
        ref = np.fft.fft(x)
        got = ore + 1j * oim
        assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref), n


def test_spec_path_rdft2_and_r2r():
    n, v = 256, 4
    x = np.random.default_rng(1).random((v, n)) - 0.5
    out = np.zeros((v, n // 2 + 1), dtype=np.complex128)
    assert _run(1, -1, [(n, 1, 1)], [(v, n, n // 2 + 1)], np.ascontiguousarray(x).reshape(-1),
                out.view(np.float64).reshape(-1)) == 0
    ref = np.fft.rfft(x)
    assert np.linalg.norm(out - ref) <= 1e-14 * np.linalg.norm(ref)
    # REDFT10 (DCT-II, libbench2 kind 5) of 30 points: 2 * sum x_j cos(pi k (2j + 1) / 2n)
    m = 30
    y = np.random.default_rng(2).random(m) - 0.5
    o = np.zeros(m)
    assert _run(2, -1, [(m, 1, 1)], [], y.copy(), o, r2r=[5]) == 0
    j = np.arange(m)
    ref = np.array([2 * np.sum(y * np.cos(np.pi * k * (2 * j + 1) / (2 * m))) for k in range(m)])
    assert np.linalg.norm(o - ref) <= 1e-14 * np.linalg.norm(ref)


def test_can_do_refuses_rank_zero():
    """A rank-0 problem (a plain copy) is outside the library's domain: can_do says no."""
    x = np.arange(8.0)
    assert _run(0, -1, [], [(4, 1, 1)], x, np.zeros(8)) == -1
