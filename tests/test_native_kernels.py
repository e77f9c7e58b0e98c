"""The codelets against lean-fftw's own generated kernels (CPU).

lean-fftw ships its radix-2/4/8/16 butterflies as generated Lean source
(LeanFFTW/Native/Kernels.lean:9-1897, proved equal to refTransform by Proof/Native.lean:21-38);
tests/golden/native_kernels.json holds them as operation lists (parsed by
oracle/native_dag.py, which imports nothing from the product).  Here:

* the fixture is complete and agrees with the reference's other published pins (operation
  counts of docs/ITERATIONS.md, constant bits of kernel-constants.txt);
* the product's restated generator (lfg.codegen) emits exactly these sixteen DAGs: the same
  operations on the same operands in the same order, constants bit for bit -- so every
  binary64 result of a GPU codelet of these radices is the reference kernel's result;
* the oracle's C butterflies (now written from the fixture) give, bit for bit, the values of
  an exact evaluation of the fixture (rational arithmetic, one rounding per operation), on
  random inputs and on special values (signed zeros, subnormals, infinities, NaN, overflow).
"""
import json
import math
import os
import struct

import numpy as np
import pytest

import native_dag
import oracle as O
from lfg.codegen.kernel import butterfly_k
from lfg.codegen.sexpr import cst_value

KERNELS = native_dag.load()
CASES = [(R, tw, fwd) for R in native_dag.RADICES for tw in (False, True) for fwd in (True, False)]


def _bits(v: float) -> str:
    return f"{struct.unpack('<Q', struct.pack('<d', v))[0]:016x}"


def test_fixture_is_complete(golden_dir):
    assert len(KERNELS) == 16
    for R, tw, fwd in CASES:
        k = KERNELS[native_dag.kernel_name(fwd, R, tw)]
        assert (k["R"], k["tw"], k["fwd"]) == (R, tw, fwd)
        assert k["n_in"] == (4 * R - 2 if tw else 2 * R)
        assert len(k["outs"]) == 2 * R
        n = k["n_in"]
        for i, op in enumerate(k["ops"]):            # operands defined before use
            assert all(a < n + i for a in op[1:] if isinstance(a, int)), (R, tw, fwd, i)


def test_fixture_matches_published_counts_and_constants(golden_dir):
    oc = json.load(open(os.path.join(golden_dir, "opcounts.json")))["split"]
    assert list(native_dag.counts(KERNELS["bfly16nf"])) == oc["n16"]
    assert list(native_dag.counts(KERNELS["bfly16tf"])) == oc["t16"]
    assert sum(native_dag.counts(KERNELS["bfly8tf"])) == json.load(
        open(os.path.join(golden_dir, "opcounts.json")))["twiddled8_total"]
    published = {int(l.split()[3]) for l in open(os.path.join(golden_dir, "kernel_constants.txt"))
                 if l.strip()}
    for k in KERNELS.values():
        for op in k["ops"]:
            if op[0] == "cst":
                assert int(op[1], 16) in published


def _canon(op):
    if op[0] in ("add", "mul"):
        return (op[0],) + tuple(sorted(op[1:3]))
    if op[0] in ("fma", "fms", "fnma"):
        return (op[0],) + tuple(sorted(op[1:3])) + (op[3],)
    return tuple(op)


@pytest.mark.parametrize("R,tw,fwd", CASES)
def test_generator_emits_the_reference_dag(R, tw, fwd):
    """Slot for slot: lfg.codegen's CSE'd kernel is the reference's generated kernel.
    Operand order is compared up to the commutativity of add, mul and the product of fma,
    which IEEE binary64 arithmetic does not see."""
    ref = KERNELS[native_dag.kernel_name(fwd, R, tw)]
    k = butterfly_k(fwd, R, tw)
    assert k.n_in == ref["n_in"]
    mine = []
    for op in k.ops:
        if op[0] == "cst":
            mine.append(("cst", _bits(cst_value(op[1]))))
        else:
            mine.append(_canon(op))
    assert mine == [_canon(o) for o in ref["ops"]]
    assert list(k.outs) == ref["outs"]


SPECIALS = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, -1e-310, 1.7976931348623157e308,
            -1.7976931348623157e308, math.inf, -math.inf, math.nan, 1.0, -1.0, 0.5, 1e300, -1e300]


def _inputs(k, rng, count):
    n = k["n_in"]
    rows = [rng.uniform(-0.5, 0.5, n) for _ in range(count)]
    rows += [rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n) for _ in range(count)]
    for _ in range(count):                  # random data mixed with special values
        x = rng.uniform(-1, 1, n)
        idx = rng.choice(2 * k["R"], size=rng.integers(1, 4), replace=False)
        x[idx] = rng.choice(SPECIALS, size=idx.size)
        rows.append(x)
    if k["tw"]:                             # twiddles on the unit circle
        for x in rows[:count]:
            a = rng.uniform(0, 2 * np.pi, k["R"] - 1)
            x[2 * k["R"]::2], x[2 * k["R"] + 1::2] = np.cos(a), np.sin(a)
    return rows


def _same(a, b) -> bool:
    """Bit equality, NaN positions compared instead of payloads."""
    a, b = np.asarray(a), np.asarray(b)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint64), b[~nb].view(np.uint64)))


@pytest.mark.parametrize("R,tw,fwd", CASES)
def test_oracle_butterfly_is_the_exact_evaluation(R, tw, fwd):
    k = KERNELS[native_dag.kernel_name(fwd, R, tw)]
    rng = np.random.default_rng(1000 * R + 10 * tw + fwd)
    for x in _inputs(k, rng, 6 if R == 16 else 12):
        got = O.bfly(fwd, R, tw, x)
        want = native_dag.evaluate(k, list(map(float, x)))
        assert _same(got, want), (R, tw, fwd, x)


def test_exact_fma_against_libm():
    """native_dag.fma_exact is the correctly rounded fused multiply-add (the C library's fma
    on this host is the second opinion), on operands chosen to make the rounding matter."""
    import ctypes
    libm = ctypes.CDLL("libm.so.6")
    libm.fma.restype = ctypes.c_double
    libm.fma.argtypes = [ctypes.c_double] * 3
    rng = np.random.default_rng(7)
    vals = list(rng.standard_normal(300) * 10.0 ** rng.integers(-320, 308, 300)) + SPECIALS
    for _ in range(3000):
        a, b, c = (float(vals[i]) for i in rng.integers(0, len(vals), 3))
        if rng.random() < 0.3:
            c = -a * b                       # near-cancellation
        assert _same([native_dag.fma_exact(a, b, c)], [libm.fma(a, b, c)]), (a, b, c)
