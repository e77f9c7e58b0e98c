"""GPU parity of the FP64 complex transforms against the oracle (refTransform restated).

For a radix sequence rs, lean-fftw's fast engine returns refTransform fwd N rs bit for bit
(LeanFFTW/Gen/Stockham.lean:296-301; checked in scripts/AsmTest.lean:41-53).  The GPU runs
the same passes with the same codelets and twiddle tables, so it must match the oracle bit
for bit for every plan it can pick, forward and backward, in and out of place, batched,
one- and two-group; and its relative L2 error against the double-double DFT must stay
within 1.5x of the reference's (the same number, since the bits agree).
Guard words after each output must stay untouched (scripts/AsmTest.lean:334-338).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no GPU", allow_module_level=True)

import lfg  # noqa: E402
import oracle as O  # noqa: E402

GUARD = 64
SENTINEL = np.float64(-1.2345678e300)


def _run(plan, x: np.ndarray, inplace: bool = False):
    """Execute on the GPU with guard words after the output; return output, guard intact."""
    n = x.size
    buf = torch.full((n + GUARD,), complex(SENTINEL, SENTINEL), dtype=torch.complex128,
                     device="cuda")
    xin = torch.from_numpy(np.ascontiguousarray(x).reshape(-1)).to("cuda")
    if inplace:
        buf[:n] = xin
        plan.execute(buf, buf)
    else:
        plan.execute(xin, buf)
    torch.cuda.synchronize()
    out = buf.cpu().numpy()
    guard_ok = bool(np.all(out[n:].real == SENTINEL) and np.all(out[n:].imag == SENTINEL))
    return out[:n].reshape(x.shape), guard_ok


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint64),
                          np.ascontiguousarray(b).view(np.uint64))


def test_golden_vectors(golden_dir):
    """Committed oracle vectors (LCG inputs of the reference tests) reproduce bit for bit."""
    z = np.load(os.path.join(golden_dir, "oracle_vectors.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    assert keys
    for key in keys:
        N = int(key.split("_")[0][1:])
        rs = [int(r) for r in key.split("_")[1].split("x")]
        x = z[key + "_in"]
        for fwd in (True, False):
            plan = lfg.plan_1d(N, -1 if fwd else 1, 1, radices=rs)
            y, ok = _run(plan, x)
            assert ok, key
            assert _bits_equal(y, z[key + ("_fwd" if fwd else "_bwd")]), (key, fwd)


POW2 = [2 ** k for k in range(1, 19)]
SMOOTH = [3, 5, 6, 7, 9, 10, 11, 12, 13, 14, 15, 18, 20, 24, 25, 27, 36, 60, 80, 108, 210, 360,
          504, 1000, 1001, 1960, 2310, 4725, 7200, 7776, 10000, 10368, 15015, 16384 * 3, 27000,
          75600, 165375]


@pytest.mark.parametrize("N", POW2 + SMOOTH)
def test_default_plan_bitexact(N):
    """The planner's own choice at each size, both directions, batched, out of place."""
    B = max(1, min(8, (1 << 16) // N))
    x = O.uniform_complex((B, N), seed=N)
    for sign in (-1, 1):
        plan = lfg.plan_1d(N, sign, B)
        y, ok = _run(plan, x)
        assert ok
        ref = O.ref_transform(sign < 0, N, plan.radices, x, nthreads=8)
        assert _bits_equal(y, ref), (N, sign, plan.radices)


@pytest.mark.parametrize("N,rs", [(16, [2, 2, 2, 2]), (64, [4, 4, 4]), (1024, [8, 8, 8, 2]),
                                  (1024, [2, 8, 8, 8]), (4096, [16, 8, 8, 4]),
                                  (8192, [8, 16, 8, 8]), (262144, [8, 16, 8, 8, 8, 4]),
                                  (10368, [8, 9, 12, 12]), (75600, [16, 3, 5, 5, 7, 9]),
                                  (165375, [15, 15, 15, 7, 7]), (1080, [12, 9, 10]),
                                  (2048, [8, 4, 4, 4, 2, 2])])
def test_explicit_plans_inplace(N, rs):
    """Published reference plans (results/repro-2026-11-04/xcheck-bits.jsonl) and others,
    in place (two-group plans then run through the plan's scratch buffer)."""
    B = 2
    x = O.lcg_rand(2 * N * B, N + 1).view(np.complex128).reshape(B, N)
    plan = lfg.plan_1d(N, -1, B, radices=rs)
    y, ok = _run(plan, x, inplace=True)
    assert ok
    assert _bits_equal(y, O.ref_transform(True, N, rs, x, nthreads=8)), (N, rs)


def test_error_vs_reference_published(golden_dir):
    """Relative L2 error against the double-double DFT: within 1.5x of the reference's
    own engine at the same size (its plan, restated), and near its published value."""
    xs = json.load(open(os.path.join(golden_dir, "xcheck.json")))
    for d in xs:
        N, rs = d["N"], d["plan"]
        if N < 4 or max(rs) > 16:
            continue
        x = O.uniform_complex((N,), seed=20261016 + N)
        ref = O.dd_dft(True, x, nthreads=8)
        e_ref = O.rel_l2(O.ref_transform(True, N, rs, x), ref)
        plan = lfg.plan_1d(N, -1, 1)
        y, _ = _run(plan, x[None, :])
        e_gpu = O.rel_l2(y[0], ref)
        assert e_gpu <= 1.5 * e_ref + 1e-18, (N, e_gpu, e_ref)
        assert e_ref <= 2.0 * d["lean_l2"] + 1e-17, (N, e_ref, d["lean_l2"])


def test_spec_strided_batch():
    """lean-fftw FFI encoding with a vector dimension and non-unit strides/offsets."""
    N, B = 360, 5
    # input: complex stride 3, line distance 3N+7 complex, offset 2 complex
    istride, idist, ioff = 3, 3 * N + 7, 2
    ostride, odist, ooff = 1, N + 4, 1
    total_in = ioff + (N - 1) * istride + (B - 1) * idist + 1
    total_out = ooff + (N - 1) * ostride + (B - 1) * odist + 1
    buf = O.uniform_complex((total_in,), seed=5)
    spec = [0, -1, 1, 1, 2 * ioff, 2 * ioff + 1, 2 * ooff, 2 * ooff + 1,
            N, 2 * istride, 2 * ostride, B, 2 * idist, 2 * odist]
    plan = lfg.plan_spec(spec)
    xin = torch.from_numpy(buf).to("cuda")
    out = torch.zeros(total_out, dtype=torch.complex128, device="cuda")
    plan.execute(xin, out)
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    lines = np.stack([buf[ioff + b * idist + istride * np.arange(N)] for b in range(B)])
    ref = O.ref_transform(True, N, plan.radices, lines)
    got = np.stack([o[ooff + b * odist + ostride * np.arange(N)] for b in range(B)])
    assert _bits_equal(got, ref)
    # untouched gaps between output lines stay zero
    mask = np.ones(total_out, bool)
    for b in range(B):
        mask[ooff + b * odist + ostride * np.arange(N)] = False
    assert np.all(o[mask] == 0)


def test_execute_host_roundtrip():
    N, B = 4096, 3
    x = O.uniform_complex((B, N), seed=11)
    plan = lfg.plan_1d(N, -1, B)
    y = plan.execute_host(x)
    assert _bits_equal(y, O.ref_transform(True, N, plan.radices, x))
    inv = lfg.plan_1d(N, 1, B).execute_host(y)
    assert np.max(np.abs(inv / N - x)) < 1e-14


@pytest.mark.parametrize("N", [64, 1000, 4096, 10368])
def test_measured_plans_bitexact(N, tmp_path, monkeypatch):
    """LFG_MEASURE times candidate (radices, grouping, tile) plans; whatever it keeps must
    still be the reference transform of its radix sequence, bit for bit, and every measured
    candidate is logged (LF_PLAN_LOG analogue)."""
    log = tmp_path / "plan.log"
    monkeypatch.setenv("LFG_PLAN_LOG", str(log))
    B = max(1, (1 << 16) // N)
    plan = lfg.plan_1d(N, -1, B, measure=True)
    x = O.uniform_complex((B, N), seed=N + 3)
    y, ok = _run(plan, x)
    assert ok
    assert _bits_equal(y, O.ref_transform(True, N, plan.radices, x, nthreads=8))
    lines = [json.loads(l) for l in open(log)]
    assert lines and all(d["n"] == N for d in lines)
    assert min(d["ms"] for d in lines) > 0
