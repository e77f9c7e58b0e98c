"""The restated codelet generator against lean-fftw's published known answers.

* every codelet constant of every butterfly of radix <= 64 (237 binary64 bit patterns,
  in order of first use): results/repro-2026-11-04/kernel-constants.txt;
* kernel operation counts: docs/ITERATIONS.md:61-62, 227-230, 285-287;
* rounding depth a, constant depth b and magnitude bound magMax of the 36 published plans,
  computed by running the Stockham schedule over depth and magnitude arithmetic
  (scripts/ErrorBound.lean:23-59): results/repro-2026-11-04/bounds.jsonl.  These are pure
  functions of every kernel's operation DAG, so they pin the generated DAGs themselves.
"""
import json
import os

import numpy as np
import pytest

from lfg.codegen import trig
from lfg.codegen.kernel import butterfly_k
from lfg.codegen.sexpr import cst_value


def _smooth(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0 and n > 1:
            n //= p
    return n == 1


def test_kernel_constants_kat(golden_dir):
    """scripts/ErrorBound.lean:64-83 enumerates constants by radix, direction, twiddling."""
    seen, lines = set(), []
    for R in range(2, 65):
        if not _smooth(R):
            continue
        for fwd in (True, False):
            for tw in (True, False):
                for c in butterfly_k(fwd, R, tw).constants():
                    if c in seen:
                        continue
                    seen.add(c)
                    nm, k, n = ("cos", 1, 8) if c[0] == "sqrthalf" else c
                    lines.append(f"{nm} {k} {n} {trig.float_to_bits(cst_value(c))}")
    ref = [l for l in open(os.path.join(golden_dir, "kernel_constants.txt")).read().split("\n") if l]
    assert len(ref) == 237
    assert lines == ref


def test_opcounts(golden_dir):
    oc = json.load(open(os.path.join(golden_dir, "opcounts.json")))
    for name, want in oc["split"].items():
        R = int(name[1:])
        assert list(butterfly_k(True, R, name[0] == "t").counts()) == want, name
        assert list(butterfly_k(False, R, name[0] == "t").counts()) == want, name
    for R, tot in oc["untwiddled_totals"].items():
        assert sum(butterfly_k(True, int(R), False).counts()) == tot, R
    assert sum(butterfly_k(True, 8, True).counts()) == oc["twiddled8_total"]


# ---- depth / magnitude arithmetic over the Stockham schedule (ErrorBound.lean:23-59)

def _eval_kernel(k, A, inputs):
    """Evaluate kernel k over arithmetic A on arrays (vectorised over butterflies)."""
    env = list(inputs)
    for op in k.ops:
        o = op[0]
        if o == "cst":
            env.append(A["cst"](op[1], inputs[0]))
        elif o == "zero":
            env.append(A["zero"](inputs[0]))
        elif o == "neg":
            env.append(env[op[1]])
        elif o in ("add", "sub", "mul"):
            env.append(A[o](env[op[1]], env[op[2]]))
        else:
            env.append(A["fma"](env[op[1]], env[op[2]], env[op[3]]))
    return [env[s] for s in k.outs]


def _stockham(A, N, rs, z, tw_of):
    """stockhamWith (Stockham.lean:287-294) with passWith/bflyInputs (Stockham.lean:263-284)
    over an arithmetic whose values are numpy arrays (one entry per scalar)."""
    ns = 1
    for t, R in enumerate(rs):
        k = butterfly_k(True, R, t >= 1)
        NR = N // R
        j = np.arange(NR)
        kk = j % ns
        b = j // ns
        ins = []
        for r in range(R):
            ins += [z[2 * (j + r * NR)], z[2 * (j + r * NR) + 1]]
        if t >= 1:
            tw = tw_of(t)
            for r in range(R - 1):
                ins += [tw[2 * r * ns + kk], tw[(2 * r + 1) * ns + kk]]
        outs = _eval_kernel(k, A, ins)
        o = np.empty_like(z)
        for r in range(R):
            c = b * ns * R + kk + r * ns
            o[2 * c] = outs[2 * r]
            o[2 * c + 1] = outs[2 * r + 1]
        z = o
        ns *= R
    return z


def _depth_mag(N, rs):
    # depthArith as a pair of int arrays packed into one complex-free structure: run twice
    def run_depth(which):
        # a: rounding depth; b: constant depth (ErrorBound.lean:24-33)
        # represent (a, b) as a*4096 + b (both stay far below 4096)
        S = 4096
        A = {
            "cst": lambda c, like: np.full_like(like, 1),
            "zero": lambda like: np.zeros_like(like),
            "add": lambda x, y: (np.maximum(x // S, y // S) + 1) * S + np.maximum(x % S, y % S),
            "sub": lambda x, y: (np.maximum(x // S, y // S) + 1) * S + np.maximum(x % S, y % S),
            "mul": lambda x, y: (x // S + y // S + 1) * S + (x % S + y % S),
            "fma": lambda x, y, z: (np.maximum(x // S + y // S, z // S) + 1) * S
                                   + np.maximum(x % S + y % S, z % S),
        }
        z = np.full(2 * N, 1, dtype=np.int64)   # inputs (0, 1)
        tws = lambda t: np.full(2 * (rs[t] - 1) * int(np.prod(rs[:t])), 1, dtype=np.int64)
        return _stockham(A, N, rs, z, tws)

    d = run_depth(0)
    a = int((d // 4096).max())
    b = int((d % 4096).max())
    ell = 2.0 ** -1022
    A = {
        "cst": lambda c, like: np.full_like(like, abs(cst_value(c)) * (1 + 2.0 ** -50) + ell),
        "zero": lambda like: np.zeros_like(like),
        "add": lambda x, y: x + y + ell,
        "sub": lambda x, y: x + y + ell,
        "mul": lambda x, y: x * y + ell,
        "fma": lambda x, y, z: x * y + z + ell,
    }
    m = _stockham(A, N, rs, np.ones(2 * N), lambda t: np.ones(2 * (rs[t] - 1) * int(np.prod(rs[:t]))))
    return a, b, float(m.max())


def _bounds(golden_dir):
    return [json.loads(l) for l in open(os.path.join(golden_dir, "bounds.jsonl"))]


@pytest.mark.parametrize("case", range(36))
def test_bounds_pin(golden_dir, case):
    d = _bounds(golden_dir)[case]
    a, b, mm = _depth_mag(d["N"], d["R"])
    assert (a, b) == (d["a"], d["b"]), d
    assert f"{mm:.6f}" == f"{d['magMax']:.6f}", (mm, d)
