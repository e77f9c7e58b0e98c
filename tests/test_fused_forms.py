"""The binary64 codelets' fused forms (no GPU needed).

The generated CUDA codelets write every addition, subtraction and multiplication of the
reference's DAG as a fused multiply-add with run-time operands one = 1.0 and nz = -0.0
(a*1 + b, (-b)*1 + a, a*b + (-0)), which GB300 issues faster than DADD/DMUL.  This file pins
that the emitted code has no other binary64 arithmetic and one fma per operation, and checks
the identities the bit-exactness rests on with the C library's correctly rounded fma() over
random and special operands (signed zeros, subnormals, overflow, infinities, NaNs).
"""
import ctypes
import ctypes.util
import math
import re
import struct

import numpy as np
import pytest

from lfg.codegen.emit import cuda_codelets
from lfg.codegen.kernel import butterfly_k

RADICES = list(range(2, 17))


def test_f64_codelets_use_only_fused_forms():
    text = cuda_codelets(RADICES, fp32=False)
    for intrinsic in ("__dadd_rn", "__dsub_rn", "__dmul_rn"):
        assert intrinsic not in text
    bodies = re.split(r"template <> struct BflyD<", text)[1:]
    assert len(bodies) == len(RADICES) * 4
    i = 0
    for R in RADICES:
        for fwd in (True, False):
            for tw in (False, True):
                k = butterfly_k(fwd, R, tw)
                a, m, f = k.counts()
                negs = sum(1 for op in k.ops if op[0] == "neg")
                assert bodies[i].count("__fma_rn(") == a - negs + m + f, (R, fwd, tw)
                i += 1


def test_f32_codelets_unchanged():
    text = cuda_codelets(RADICES, fp32=True)
    assert "__fadd_rn" in text and "one, " not in text.replace("float one, float nz", "")


def _libm_fma():
    name = ctypes.util.find_library("m")
    lib = ctypes.CDLL(name) if name else ctypes.CDLL(None)
    f = lib.fma
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double] * 3
    return f


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _same(a, b):
    return (math.isnan(a) and math.isnan(b)) or _bits(a) == _bits(b)


def _operands():
    rng = np.random.default_rng(7)
    vals = list(rng.standard_normal(400) * 10.0 ** rng.integers(-30, 30, size=400))
    vals += list(rng.random(100) * 1e-310)                        # subnormals
    vals += [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
             -1.7976931348623157e308, 1.5e308, math.inf, -math.inf, math.nan, 1.0, -1.0, 0.5]
    return [float(v) for v in vals]


def test_fused_identities_round_like_the_separate_operations():
    fma = _libm_fma()
    ops = _operands()
    rng = np.random.default_rng(8)
    pairs = [(ops[i], ops[j]) for i, j in rng.integers(0, len(ops), size=(20000, 2))]
    pairs += [(a, b) for a in ops[-14:] for b in ops[-14:]]     # every special pair
    for a, b in pairs:
        assert _same(fma(a, 1.0, b), a + b), (a, b)
        assert _same(fma(-b, 1.0, a), a - b), (a, b)
        assert _same(fma(a, b, -0.0), a * b), (a, b)


if __name__ == "__main__":
    pytest.main([__file__, "-q"])
