"""Multi-axis complex transforms (rank 2 and 3, vector rank 2) through the FFI encoding.

lean-fftw computes these in its generic engine, one axis at a time (`alongAxis`,
Core/Problem.lean:170-212).  The GPU plan runs one stage per axis (last axis first), each a
1-D transform of the fast engine over all other indices, so:

  * bit parity: the result equals the oracle's refTransform applied along each axis in the
    same order with the same radix sequences, bit for bit;
  * accuracy parity: its relative L2 error against an extended-precision multi-axis DFT is
    within 1.5x of the generic engine's (restated in the oracle) on the same input.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


def _spec(shape, sign, vec=(), layout="contiguous"):
    """Row-major complex tensor (vector dims outermost), strides in doubles."""
    dims, acc = [], 1
    for n in reversed(shape):
        dims.append((n, 2 * acc, 2 * acc))
        acc *= n
    dims.reverse()
    vdims, vacc = [], acc
    for n in reversed(vec):
        vdims.append((n, 2 * vacc, 2 * vacc))
        vacc *= n
    vdims.reverse()
    spec = [0, sign, len(shape), len(vec), 0, 1, 0, 1]
    for d in dims + vdims:
        spec += list(d)
    return spec


def _axis_apply(fn, x, axis):
    xm = np.ascontiguousarray(np.moveaxis(x, axis, -1))
    return np.ascontiguousarray(np.moveaxis(fn(xm), -1, axis))


def _split_radices(rs, sizes):
    out, i = [], 0
    for n in sizes:
        p, seq = 1, []
        while p < n:
            seq.append(rs[i])
            p *= rs[i]
            i += 1
        assert p == n
        out.append(seq)
    return out


def _run(spec, x, inplace=False):
    plan = lfg.plan_spec(spec)
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if inplace:
        plan.execute(xd, xd)
        out = xd
    else:
        out = torch.zeros_like(xd)
        plan.execute(xd, out)
    torch.cuda.synchronize()
    return plan, out.cpu().numpy()


def _dd_multi(fwd, x, axes):
    """Extended-precision DFT along `axes` (in order), carrying (hi, lo) between axes."""
    hi, lo = O.dd_dft(fwd, x, nthreads=8) if axes[0] == x.ndim - 1 else \
        tuple(_axis_apply(lambda a: O.dd_dft(fwd, a, nthreads=8)[k], x, axes[0]) for k in (0, 1))
    for ax in axes[1:]:
        parts = []
        for part in (hi, lo):
            h = _axis_apply(lambda a: O.dd_dft(fwd, a, nthreads=8)[0], part, ax)
            l = _axis_apply(lambda a: O.dd_dft(fwd, a, nthreads=8)[1], part, ax)
            parts.append((h, l))
        (ah, al), (bh, bl) = parts
        s = ah + bh
        hi, lo = s, ((ah - s) + bh) + al + bl
    return hi, lo


@pytest.mark.parametrize("shape,vec", [((64, 48), (3,)), ((12, 60), ()), ((512, 512), (2,)),
                                       ((8, 12, 10), (2,)), ((30, 16, 9), ()),
                                       ((1, 36), (4,)), ((16384, 8), ())])
@pytest.mark.parametrize("sign", [-1, 1])
def test_rank_k_bitexact_and_error(shape, vec, sign):
    x = O.uniform_complex(tuple(vec) + tuple(shape), seed=sum(shape) + len(vec))
    plan, y = _run(_spec(shape, sign, vec), x)
    axes_sizes = [n for n in reversed(shape) if n > 1]
    rs = _split_radices(plan.radices, axes_sizes)
    # bit parity: refTransform along each axis, last axis first
    ref = x.copy()
    k = 0
    for ax in reversed(range(len(shape))):
        n = shape[ax]
        if n == 1:
            continue
        axis = len(vec) + ax
        ref = _axis_apply(lambda a: O.ref_transform(sign < 0, n, rs[k], a, nthreads=8), ref, axis)
        k += 1
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64)), (shape, vec)
    if np.prod(shape) > 1 << 16:
        return
    # accuracy parity against the generic engine
    axes = [len(vec) + ax for ax in reversed(range(len(shape))) if shape[ax] > 1]
    dd = _dd_multi(sign < 0, x, axes)
    gen = x.copy()
    for ax in axes:
        gen = _axis_apply(lambda a: O.generic_dft(sign < 0, a, nthreads=8), gen, ax)
    e_gpu, e_gen = O.rel_l2(y, dd), O.rel_l2(gen, dd)
    assert e_gpu <= 1.5 * e_gen + 1e-18, (shape, e_gpu, e_gen)


def test_vector_rank2_rank1_bitexact():
    """Rank 1 with two vector dimensions, non-nesting strides (one launch over both)."""
    n, v0, v1 = 360, 5, 7
    # input: lines at distance n (inner vector) and 8*n+3 (outer); output transposed batch
    total_in = (v0 - 1) * (8 * n + 3) + (v1 - 1) * n + n
    xbuf = O.uniform_complex((total_in,), seed=9)
    spec = [0, -1, 1, 2, 0, 1, 0, 1, n, 2, 2, v1, 2 * n, 2 * n * v0, v0, 2 * (8 * n + 3), 2 * n]
    plan = lfg.plan_spec(spec)
    out = torch.zeros(v0 * v1 * n, dtype=torch.complex128, device="cuda")
    plan.execute(torch.from_numpy(xbuf).cuda(), out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    for a in range(v0):
        for b in range(v1):
            line = xbuf[a * (8 * n + 3) + b * n: a * (8 * n + 3) + b * n + n]
            got = o[b * n * v0 + a * n: b * n * v0 + a * n + n]
            assert np.array_equal(got.view(np.uint64),
                                  O.ref_transform(True, n, plan.radices, line[None])[0].view(np.uint64))


def test_rank2_inplace_matches_out_of_place():
    shape = (96, 128)
    x = O.uniform_complex((2,) + shape, seed=4)
    spec = _spec(shape, -1, (2,))
    _, y = _run(spec, x)
    _, yi = _run(spec, x, inplace=True)
    assert np.array_equal(y.view(np.uint64), yi.view(np.uint64))


def test_rank2_fp32_error():
    shape = (256, 384)
    x = O.uniform_complex(shape, seed=12).astype(np.complex64)
    plan = lfg.plan_spec(_spec(shape, -1), precision="f32")
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    plan.execute(xd, y)
    torch.cuda.synchronize()
    ref = np.fft.fft2(x.astype(np.complex128))
    e = np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert e < 8 * 2.0 ** -24, e


def test_rank2_set_scale_roundtrip():
    shape = (60, 80)
    x = O.uniform_complex(shape, seed=2)
    f = lfg.plan_spec(_spec(shape, -1))
    b = lfg.plan_spec(_spec(shape, 1)).set_scale(1.0 / (60 * 80))
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    z = torch.empty_like(xd)
    f.execute(xd, y)
    b.execute(y, z)
    torch.cuda.synchronize()
    assert np.max(np.abs(z.cpu().numpy() - x)) < 1e-14
