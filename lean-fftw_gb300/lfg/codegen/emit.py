"""Emit butterfly kernels as straight-line CUDA device functions or C functions.

Each kernel (a CSE'd `Kernel`, see kernel.py) becomes one function that reads its inputs
from an array, performs the operations in slot order with explicitly rounded IEEE
binary64 (or binary32) operations, and writes its outputs back.  Explicit rounding
intrinsics (`__dadd_rn`, `__dmul_rn`, `__fma_rn`, ...) keep nvcc from contracting or
reassociating anything, so the device code performs exactly the operations of the kernel,
operand for operand: the same contract the reference's C/assembly back ends keep with
`Kernel.eval` (lean-fftw `LeanFFTW/Gen/Emit.lean:91-111`).

Binary64 meaning of the fused forms (lean-fftw `LeanFFTW/Gen/Emit.lean:46-55`):
    fms(a, b, c)  = fma(a, b, -c)
    fnma(a, b, c) = fma(-a, b, c)
"""
from __future__ import annotations

from typing import List

from .kernel import Kernel, butterfly_k
from .sexpr import cst_value


def _lit(v: float, fp32: bool) -> str:
    if v == 0.0:
        return "0.0f" if fp32 else "0.0"
    # binary32 kernels use the binary64 constant rounded once to binary32
    if fp32:
        import struct
        f = struct.unpack("<f", struct.pack("<f", v))[0]
        return f.hex() + "f"
    return v.hex()


def kernel_body(k: Kernel, dialect: str, fp32: bool = False) -> List[str]:
    """Statements computing the kernel: inputs x[i] -> outputs y[i].

    dialect "cuda" uses the round-to-nearest intrinsics; dialect "c" uses plain operators
    and fma() and must be compiled with -ffp-contract=off."""
    T = "float" if fp32 else "double"
    if dialect == "cuda" and not fp32:
        # binary64 additions, subtractions and multiplications as fused multiply-adds with the
        # runtime operands one = 1.0 and nz = -0.0: a*1 + b, (-b)*1 + a and a*b + (-0) round
        # once, to the same binary64 value as a + b, a - b and a*b (signed zeros, infinities,
        # NaNs and subnormals included), and on GB300 DFMA issues ~19 % faster than DADD or
        # DMUL.  The operands must stay opaque to the compiler (loaded at run time), or it
        # folds the fma back into an add or a multiply.
        add = lambda a, b: f"__fma_rn({a}, one, {b})"
        sub = lambda a, b: f"__fma_rn(-{b}, one, {a})"
        mul = lambda a, b: f"__fma_rn({a}, {b}, nz)"
        fma_ = lambda a, b, c: f"__fma_rn({a}, {b}, {c})"
    elif dialect == "cuda":
        add = lambda a, b: f"__fadd_rn({a}, {b})"
        sub = lambda a, b: f"__fsub_rn({a}, {b})"
        mul = lambda a, b: f"__fmul_rn({a}, {b})"
        fma_ = lambda a, b, c: f"__fmaf_rn({a}, {b}, {c})"
    else:
        add = lambda a, b: f"{a} + {b}"
        sub = lambda a, b: f"{a} - {b}"
        mul = lambda a, b: f"{a} * {b}"
        fma_ = lambda a, b, c: (f"fmaf({a}, {b}, {c})" if fp32 else f"fma({a}, {b}, {c})")

    def s(i: int) -> str:
        return f"x{i}" if i < k.n_in else f"t{i}"

    lines = [f"const {T} x{i} = x[{i}];" for i in range(k.n_in)]
    for idx, op in enumerate(k.ops):
        slot = k.n_in + idx
        o = op[0]
        if o == "cst":
            e = _lit(cst_value(op[1]), fp32)
        elif o == "zero":
            e = "0.0f" if fp32 else "0.0"
        elif o == "add":
            e = add(s(op[1]), s(op[2]))
        elif o == "sub":
            e = sub(s(op[1]), s(op[2]))
        elif o == "mul":
            e = mul(s(op[1]), s(op[2]))
        elif o == "neg":
            e = f"-{s(op[1])}"
        elif o == "fma":
            e = fma_(s(op[1]), s(op[2]), s(op[3]))
        elif o == "fms":
            e = fma_(s(op[1]), s(op[2]), f"-{s(op[3])}")
        elif o == "fnma":
            e = fma_(f"-{s(op[1])}", s(op[2]), s(op[3]))
        else:
            raise ValueError(op)
        lines.append(f"const {T} t{slot} = {e};")
    for i, o in enumerate(k.outs):
        lines.append(f"y[{i}] = {s(o)};")
    return lines


def codelet_name(fwd: bool, R: int, twiddled: bool) -> str:
    return f"bf_{'f' if fwd else 'b'}{R}{'t' if twiddled else 'n'}"


def cuda_codelets(radices: List[int], fp32: bool = False) -> str:
    """A header of `__device__ __forceinline__` codelets, specialised through the
    template `Bfly<FWD, R, TW>` so that kernels pick them at compile time.

    Inputs: x[0..2R) interleaved data, then (twiddled) x[2R..4R-2) interleaved twiddles
    w_1..w_{R-1}; outputs y[0..2R) interleaved.  `one` and `nz` must be 1.0 and -0.0 read at
    run time: the binary64 codelets express additions and multiplications as fused
    multiply-adds with them (kernel_body); the binary32 codelets ignore them."""
    T = "float" if fp32 else "double"
    out = ["// Generated by lfg/codegen/emit.py from the restated lean-fftw codelet generator.",
           "// Do not edit: rebuilt by the package build step.",
           "#pragma once",
           "",
           f"template <bool FWD, int R, bool TW> struct Bfly{'F' if fp32 else 'D'};",
           ""]
    for R in radices:
        for fwd in (True, False):
            for tw in (False, True):
                k = butterfly_k(fwd, R, tw)
                a, m, f = k.counts()
                out.append(f"// radix {R} {'forward' if fwd else 'backward'} "
                           f"{'twiddled' if tw else 'untwiddled'}: {a} add/sub/neg, {m} mul, {f} fused")
                out.append(f"template <> struct Bfly{'F' if fp32 else 'D'}<{'true' if fwd else 'false'}, {R}, "
                           f"{'true' if tw else 'false'}> {{")
                out.append(f"  static constexpr int kOps = {a + m + f};")
                out.append(f"  static __device__ __forceinline__ void run(const {T}* __restrict__ x, "
                           f"{T}* __restrict__ y, {T} one, {T} nz) {{")
                out.append("    (void)one;")
                out.append("    (void)nz;")
                out += ["    " + ln for ln in kernel_body(k, "cuda", fp32)]
                out.append("  }")
                out.append("};")
                out.append("")
    return "\n".join(out) + "\n"


def c_codelets(radices: List[int]) -> str:
    """C codelets for the CPU restatement of the reference transform: per (direction, radix,
    twiddling) a codelet `lfo_bf_*` and a whole Stockham pass `lfo_pass_*` with the codelet
    inlined (the pass of lean-fftw `LeanFFTW/Gen/Stockham.lean:263-284`), plus lookups
    `lfo_codelet(fwd, R, tw)` and `lfo_pass(fwd, R, tw)` (NULL if absent).
    Compile with -ffp-contract=off."""
    out = ["/* Generated by lfg/codegen/emit.py. Compile with -ffp-contract=off. */",
           "#include <math.h>", "#include <stddef.h>", "",
           "typedef void (*lfo_codelet_fn)(const double *x, double *y);",
           "typedef void (*lfo_pass_fn)(long N, long ns, const double *tw, const double *z,",
           "                            double *o);", ""]
    table = []
    for R in radices:
        for fwd in (True, False):
            for tw in (False, True):
                k = butterfly_k(fwd, R, tw)
                name = "lfo_" + codelet_name(fwd, R, tw)
                pname = name.replace("lfo_bf_", "lfo_pass_")
                out.append(f"static inline __attribute__((always_inline)) void {name}("
                           f"const double *restrict x, double *restrict y) {{")
                out += ["  " + ln for ln in kernel_body(k, "c")]
                out.append("}")
                out.append("")
                nx = 4 * R - 2 if tw else 2 * R
                out += [
                    f"static void {pname}(long N, long ns, const double *restrict tw, "
                    f"const double *restrict z, double *restrict o) {{",
                    f"  const long NR = N / {R};",
                    "  for (long j = 0; j < NR; ++j) {",
                    "    const long k = j % ns, b = j / ns;",
                    f"    double x[{nx}], y[{2 * R}];",
                    f"    for (int r = 0; r < {R}; ++r) {{",
                    "      x[2 * r] = z[2 * (j + r * NR)];",
                    "      x[2 * r + 1] = z[2 * (j + r * NR) + 1];",
                    "    }",
                ]
                if tw:
                    out += [f"    for (int r = 0; r < {R - 1}; ++r) {{",
                            f"      x[{2 * R} + 2 * r] = tw[2 * r * ns + k];",
                            f"      x[{2 * R} + 2 * r + 1] = tw[(2 * r + 1) * ns + k];",
                            "    }"]
                out += [f"    {name}(x, y);",
                        f"    for (int r = 0; r < {R}; ++r) {{",
                        f"      const long c = b * ns * {R} + k + r * ns;",
                        "      o[2 * c] = y[2 * r];",
                        "      o[2 * c + 1] = y[2 * r + 1];",
                        "    }",
                        "  }",
                        "}", ""]
                table.append((fwd, R, tw, name, pname))
    out.append("lfo_codelet_fn lfo_codelet(int fwd, int R, int tw) {")
    for fwd, R, tw, name, _ in table:
        out.append(f"  if (fwd == {int(fwd)} && R == {R} && tw == {int(tw)}) return {name};")
    out.append("  return NULL;")
    out.append("}")
    out.append("lfo_pass_fn lfo_pass(int fwd, int R, int tw) {")
    for fwd, R, tw, _, pname in table:
        out.append(f"  if (fwd == {int(fwd)} && R == {R} && tw == {int(tw)}) return {pname};")
    out.append("  return NULL;")
    out.append("}")
    return "\n".join(out) + "\n"
