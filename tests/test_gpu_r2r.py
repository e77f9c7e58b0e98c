"""GPU real-to-real transforms, all eleven kinds (lean-fftw Core/Problem.lean:64-112,
151-163, and the FFI kind numbering LeanFFTW/FFI.lean:29-31).

The GPU embeds each line exactly, runs its complex transform of the embedding size and
extracts exactly, so:
  * bit parity: equal to the oracle's `fast_r2r` (the same embedding around refTransform with
    the plan's radices), bit for bit;
  * accuracy parity: relative L2 error against the extended-precision r2r within 1.5x of the
    generic engine's (the reference's own path for r2r).
Multi-dimensional r2r (one kind per axis) runs one stage per axis, last axis first.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402


def _smooth(m):
    for p in (2, 3, 5, 7, 11, 13):
        while m % p == 0:
            m //= p
    return m == 1


def _run(plan, x, out_shape=None):
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    y = torch.zeros(out_shape or x.shape, dtype=xd.dtype, device="cuda")
    plan.execute(xd, y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


SIZES = [1, 2, 3, 5, 8, 12, 16, 45, 64, 100, 360, 1000, 4096]


@pytest.mark.parametrize("kind", O.R2R_KINDS)
def test_r2r_bitexact_and_error(kind):
    checked = 0
    for n in SIZES:
        M = O.r2r_embed_size(kind, n)
        if M < 1 or (kind == "redft00" and n < 2) or not _smooth(M):
            continue
        B = 3
        x = np.random.default_rng(n + 7).random((B, n)) - 0.5
        plan = lfg.plan_r2r(n, kind, B)
        y = _run(plan, x)
        if M > 1:
            ref = O.fast_r2r(kind, x, plan.radices, nthreads=8)
            assert np.array_equal(y.view(np.uint64), ref.view(np.uint64)), (kind, n)
        dd = O.dd_r2r(kind, x, nthreads=8)
        e_gpu = O.rel_l2(y, dd)
        e_gen = O.rel_l2(O.generic_r2r(kind, x, nthreads=8), dd)
        # (at a few points the statistic is a handful of roundings: allow half an ulp)
        assert e_gpu <= 1.5 * e_gen + 1.1e-16, (kind, n, e_gpu, e_gen)
        checked += 1
    assert checked >= 8


@pytest.mark.parametrize("kind,n", [("redft00", 18), ("rodft00", 16), ("redft10", 17),
                                    ("dht", 34), ("r2hc", 19), ("hc2r", 23)])
def test_r2r_non_smooth_embedding_matches_generic_engine(kind, n):
    """Embedding sizes with a prime factor above 13 run the generic engine's own transform:
    the result is the reference's r2r bit for bit."""
    x = np.random.default_rng(n).random((2, n)) - 0.5
    y = _run(lfg.plan_r2r(n, kind, 2), x)
    ref = O.generic_r2r(kind, x)
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64)), (kind, n)


def _spec_r2r(shape, kinds, vec=()):
    dims, acc = [], 1
    for n in reversed(shape):
        dims.append((n, acc, acc))
        acc *= n
    dims.reverse()
    vdims = []
    for n in reversed(vec):
        vdims.append((n, acc, acc))
        acc *= n
    vdims.reverse()
    spec = [2, -1, len(shape), len(vec), 0, 0, 0, 0]
    for d in dims + vdims:
        spec += list(d)
    return spec + [O.R2R_KINDS.index(k) for k in kinds]


@pytest.mark.parametrize("shape,kinds,vec", [((12, 16), ("redft10", "rodft01"), (2,)),
                                            ((8, 10, 6), ("dht", "redft11", "r2hc"), ()),
                                            ((64, 64), ("redft00", "redft10"), (3,))])
def test_r2r_multidim_bitexact(shape, kinds, vec):
    x = np.random.default_rng(len(shape)).random(tuple(vec) + shape) - 0.5
    plan = lfg.plan_spec(_spec_r2r(shape, kinds, vec))
    y = _run(plan, x)
    # per axis, last first, with the radices the plan reports (one sequence per axis)
    rs_all = plan.radices
    ref, pos = x.copy(), 0
    for ax in reversed(range(len(shape))):
        kind, n = kinds[ax], shape[ax]
        M = O.r2r_embed_size(kind, n)
        rs, p = [], 1
        while p < M:
            rs.append(rs_all[pos])
            p *= rs_all[pos]
            pos += 1
        axis = len(vec) + ax
        xm = np.ascontiguousarray(np.moveaxis(ref, axis, -1))
        ref = np.ascontiguousarray(np.moveaxis(O.fast_r2r(kind, xm, rs, nthreads=8), -1, axis))
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64))


def test_r2r_fp32_error():
    for kind in ("redft10", "rodft11", "r2hc", "dht"):
        n = 360 if kind != "rodft11" else 64
        x = (np.random.default_rng(1).random((4, n)) - 0.5).astype(np.float32)
        plan = lfg.plan_r2r(n, kind, 4, precision="f32")
        y = _run(plan, x).astype(np.float64)
        e = O.rel_l2(y, O.dd_r2r(kind, x.astype(np.float64), nthreads=8))
        assert e < 4 * 2.0 ** -24 * np.sqrt(np.log2(O.r2r_embed_size(kind, n))), (kind, e)
