"""The CPU oracle itself, checked before it is trusted.

* its C twiddle tables equal the Python restatement of Trig.lean (both pinned to the
  reference's published constants through test_codegen_pins);
* the double-double DFT agrees with a 200-bit mpmath DFT at small sizes;
* refTransform restated reproduces the committed golden vectors and, with the reference's
  published plans, lands on the reference's published L2 errors
  (results/repro-2026-11-04/xcheck-bits.jsonl) to within input-to-input variation;
* the generic engine restated is a DFT to binary64 accuracy.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
import trig_ref


@pytest.mark.parametrize("n", [1, 2, 5, 8, 24, 1000, 4096, 10368, 75600, 131072])
def test_c_tables_match_python_restatement(n):
    a = O.table(n)
    b = np.array(trig_ref.table(n), dtype=np.float64)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_dd_dft_against_mpmath():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    for n in (6, 16, 45, 64):
        x = O.uniform_complex((n,), seed=n)
        hi, lo = O.dd_dft(True, x)
        for k in range(n):
            s = mpmath.mpc(0)
            for j in range(n):
                s += mpmath.mpc(float(x[j].real), float(x[j].imag)) * mpmath.expjpi(-2 * mpmath.mpf(j * k) / n)
            err = abs(s - (mpmath.mpf(float(hi[k].real)) + mpmath.mpf(float(lo[k].real))
                           + 1j * (mpmath.mpf(float(hi[k].imag)) + mpmath.mpf(float(lo[k].imag)))))
            assert err < 1e-28 * max(1.0, float(abs(s))), (n, k, err)


def test_golden_vectors_reproduce(golden_dir):
    z = np.load(os.path.join(golden_dir, "oracle_vectors.npz"))
    for key in sorted({k.rsplit("_", 1)[0] for k in z.files}):
        N = int(key.split("_")[0][1:])
        rs = [int(r) for r in key.split("_")[1].split("x")]
        x = z[key + "_in"]
        assert np.array_equal(x.view(np.uint64),
                              O.lcg_rand(2 * N, N + 7).view(np.uint64)), key
        for fwd, tag in ((True, "_fwd"), (False, "_bwd")):
            y = O.ref_transform(fwd, N, rs, x)
            assert np.array_equal(y.view(np.uint64), z[key + tag].view(np.uint64)), key


def test_published_plan_errors(golden_dir):
    """Same plans as the reference's xcheck run; inputs differ (its own RNG), so the errors
    agree statistically: within 30% for N >= 64, and the same order below."""
    for d in json.load(open(os.path.join(golden_dir, "xcheck.json"))):
        N, rs = d["N"], d["plan"]
        if N < 8 or N > 70000 or max(rs) > 64:
            continue
        errs = []
        for seed in range(3):
            x = O.lcg_rand(2 * N, 1000 * seed + N).view(np.complex128)
            errs.append(O.rel_l2(O.ref_transform(True, N, rs, x), O.dd_dft(True, x)))
        e = float(np.mean(errs))
        tol = 0.3 if N >= 64 else 1.0
        assert abs(e - d["lean_l2"]) <= tol * d["lean_l2"], (N, rs, e, d["lean_l2"])


def test_published_accuracy_per_size(golden_dir):
    """The published engine's forward and backward relative L2 errors per power-of-two size
    (libbench2 --accuracy, results/emr-i12/accuracy.txt): the oracle's refTransform with the
    op-count plan, on this suite's inputs, lands within 1.5x of them at every size from 8 to
    2^14 -- the error bar the GPU path is held to, met here by the oracle it equals bit for
    bit, against the reference's own numbers (its plans were measured, so they may differ)."""
    from lfg.codegen.plans import choose_radices
    acc = json.load(open(os.path.join(golden_dir, "accuracy_emr.json")))["errors"]
    for k in range(3, 15):
        n = 1 << k
        x = O.uniform_complex((max(1, min(16, (1 << 16) // n)), n), seed=n)
        for fwd in (True, False):
            e = O.rel_l2(O.ref_transform(fwd, n, choose_radices(n), x, nthreads=4),
                         O.dd_dft(fwd, x, nthreads=4))
            pub = acc[str(n)]["fwd_l2" if fwd else "bwd_l2"]
            assert pub / 1.5 <= e <= 1.5 * pub, (n, fwd, e, pub)


@pytest.mark.parametrize("n", [8, 12, 360, 1024, 4725])
def test_generic_engine_is_a_dft(n):
    x = O.uniform_complex((3, n), seed=n)
    for fwd in (True, False):
        e = O.rel_l2(O.generic_dft(fwd, x), O.dd_dft(fwd, x))
        assert e < 5e-16 * max(1.0, np.log2(n) / 4), (n, fwd, e)


def test_ragged_oracle_matches_single_transforms():
    sizes = np.array([6, 1000, 12, 6, 243, 2048], dtype=np.int64)
    plans = {6: [6], 1000: [10, 10, 10], 12: [12], 243: [3, 9, 9], 2048: [16, 16, 8]}
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    x = O.uniform_complex((int(sizes.sum()),), seed=4)
    y = O.RaggedRef(True, sizes, plans, off, off).run(x, np.empty_like(x), nthreads=4)
    for o, n in zip(off, sizes):
        ref = O.ref_transform(True, int(n), plans[int(n)], x[o: o + n])
        assert np.array_equal(y[o: o + n].view(np.uint64), ref.view(np.uint64))
