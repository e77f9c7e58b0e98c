"""ORACLE (test infrastructure only; never imported by the product): the butterfly DAGs of
lean-fftw's own generated kernels, read independently of this repository's generator.

lean-fftw ships the radix-2/4/8/16 butterflies of its Lean backend as generated Lean source,
`LeanFFTW/Native/Kernels.lean:9-1897` ("Generated by scripts/GenLeanKernels.lean from the
kernels of LeanFFTW.Gen.Stockham"): sixteen straight-line let-chains `bfly{2,4,8,16}{n,t}{f,b}`
(untwiddled / twiddled, forward / backward) over `rd`, `+`, `-`, `*`, `Float.fma` and
constants `cst <bits>`.  `Proof/Native.lean:21-38` proves the schedule that runs them equal
to the binary64 reference transform `refTransform`, so these are the reference's codelets,
operation for operation.

This module
  * parses that Lean text (`parse_lean`; used by tests/golden/make_golden.py, which commits
    the result as tests/golden/native_kernels.json, because the reference checkout is not
    available where the GPU tests run);
  * loads the committed fixture (`load`);
  * emits C functions for the oracle's restatement of refTransform (`c_source`), so that the
    oracle's radix-2/4/8/16 butterflies are the reference's own DAGs and not the output of the
    product's restated generator;
  * evaluates a kernel exactly in Python (`evaluate`, binary64 with a correctly rounded fused
    multiply-add from rational arithmetic), a cross-check of the C evaluation.

Kernel encoding (one dict per kernel): R, fwd, tw, n_in (2R, or 4R-2 twiddled), ops, outs.
Slots 0..n_in-1 are the inputs: data value r at 2r (re), 2r+1 (im); twiddle table row k of
the butterfly (`rd tw (k * ns + q)`) at 2R + k, i.e. (re, im) of w_r at 2R + 2(r-1), +1.
Slot n_in + i holds op i:
    ["cst", "<16 hex digits>"]  the binary64 constant with those bits
    ["add", a, b] / ["sub", a, b] / ["mul", a, b]
    ["fma", a, b, c]   fma(a, b, c)
    ["fms", a, b, c]   fma(a, b, -c)        (`Float.fma a b (-c)`)
    ["fnma", a, b, c]  fma(-a, b, c)        (`Float.fma (-a) b c`)
outs[2r], outs[2r+1] are the slots stored to output r (re, im).
"""
from __future__ import annotations

import json
import math
import os
import re
import struct
from fractions import Fraction
from typing import Dict, List

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(os.path.dirname(HERE), "tests", "golden", "native_kernels.json")
SOURCE = "LeanFFTW/Native/Kernels.lean"
RADICES = (2, 4, 8, 16)

_HDR = re.compile(r"^@\[inline\] unsafe def (bfly(\d+)([nt])([fb]))\b.*:=\s*$", re.M)
_WR = re.compile(r"let y := wr y \(2 \* \((?:dst|c) \+ (\d+) \* (?:dstr|ns)\)( \+ 1)?\) (\w+)$")
_RD = re.compile(r"let (\w+) := rd [xy] \(2 \* \((?:src|c) \+ (\d+) \* (?:sstr|ns)\)( \+ 1)?\)$")
_RDTW = re.compile(r"let (\w+) := rd tw \((\d+) \* ns \+ q\)$")
_CST = re.compile(r"let (\w+) := cst (\d+)$")
_BIN = re.compile(r"let (\w+) := (\w+) ([-+*]) (\w+)$")
_FMA = re.compile(r"let (\w+) := Float\.fma (\(-)?(\w+)\)? (\w+) (\(-)?(\w+)\)?$")


def parse_lean(text: str) -> Dict[str, dict]:
    """The sixteen kernels of Native/Kernels.lean, keyed by their Lean names."""
    heads = list(_HDR.finditer(text))
    out: Dict[str, dict] = {}
    for i, m in enumerate(heads):
        name, R, tw, fwd = m.group(1), int(m.group(2)), m.group(3) == "t", m.group(4) == "f"
        end = heads[i + 1].start() if i + 1 < len(heads) else len(text)
        n_in = 4 * R - 2 if tw else 2 * R
        slot: Dict[str, int] = {}
        ops: List[list] = []
        outs: List[int] = [-1] * (2 * R)

        def define(var: str, op: list) -> None:
            if var in slot:
                raise ValueError(f"{name}: {var} defined twice")
            slot[var] = n_in + len(ops)
            ops.append(op)

        for line in text[m.end():end].splitlines():
            line = line.strip()
            if not line.startswith("let "):
                if line.startswith("def ") or line.startswith("unsafe def "):
                    break            # the loop functions after the last kernel
                continue
            if (g := _WR.match(line)):
                outs[2 * int(g.group(1)) + (1 if g.group(2) else 0)] = slot[g.group(3)]
            elif (g := _RD.match(line)):
                slot[g.group(1)] = 2 * int(g.group(2)) + (1 if g.group(3) else 0)
            elif (g := _RDTW.match(line)):
                slot[g.group(1)] = 2 * R + int(g.group(2))
            elif (g := _CST.match(line)):
                define(g.group(1), ["cst", f"{int(g.group(2)):016x}"])
            elif (g := _BIN.match(line)):
                op = {"+": "add", "-": "sub", "*": "mul"}[g.group(3)]
                define(g.group(1), [op, slot[g.group(2)], slot[g.group(4)]])
            elif (g := _FMA.match(line)):
                na, nc = bool(g.group(2)), bool(g.group(5))
                if na and nc:
                    raise ValueError(f"{name}: unexpected form {line!r}")
                op = "fnma" if na else "fms" if nc else "fma"
                define(g.group(1), [op, slot[g.group(3)], slot[g.group(4)], slot[g.group(6)]])
            else:
                raise ValueError(f"{name}: unparsed line {line!r}")
        if min(outs) < 0:
            raise ValueError(f"{name}: output not written")
        out[name] = {"R": R, "fwd": fwd, "tw": tw, "n_in": n_in, "ops": ops, "outs": outs}
    return out


def load(path: str = FIXTURE) -> Dict[str, dict]:
    with open(path) as f:
        return json.load(f)["kernels"]


def kernel_name(fwd: bool, R: int, tw: bool) -> str:
    return f"bfly{R}{'t' if tw else 'n'}{'f' if fwd else 'b'}"


def counts(k: dict):
    """(adds/subs, muls, fused) of a kernel, as lean-fftw's Kernel.counts (Gen/Emit.lean:178-184)."""
    a = sum(1 for o in k["ops"] if o[0] in ("add", "sub"))
    m = sum(1 for o in k["ops"] if o[0] == "mul")
    f = sum(1 for o in k["ops"] if o[0] in ("fma", "fms", "fnma"))
    return a, m, f


# ------------------------------------------------------------------ C emission

def _c_body(k: dict, x, y) -> List[str]:
    """Statements of kernel k reading input slot i as the C expression x(i) and storing output
    i with the C statement y(i, value)."""
    n_in = k["n_in"]
    s = lambda i: f"in{i}" if i < n_in else f"t{i}"
    lines = [f"const double in{i} = {x(i)};" for i in range(n_in)]
    for idx, op in enumerate(k["ops"]):
        o, slot = op[0], n_in + idx
        if o == "cst":
            v = struct.unpack("<d", bytes.fromhex(op[1])[::-1])[0]
            e = v.hex() if v != 0.0 else ("-0.0" if op[1][0] == "8" else "0.0")
        elif o == "add":
            e = f"{s(op[1])} + {s(op[2])}"
        elif o == "sub":
            e = f"{s(op[1])} - {s(op[2])}"
        elif o == "mul":
            e = f"{s(op[1])} * {s(op[2])}"
        elif o == "neg":
            e = f"-{s(op[1])}"
        elif o == "fma":
            e = f"fma({s(op[1])}, {s(op[2])}, {s(op[3])})"
        elif o == "fms":
            e = f"fma({s(op[1])}, {s(op[2])}, -{s(op[3])})"
        elif o == "fnma":
            e = f"fma(-{s(op[1])}, {s(op[2])}, {s(op[3])})"
        else:
            raise ValueError(op)
        lines.append(f"const double t{slot} = {e};")
    lines += [y(i, s(o)) for i, o in enumerate(k["outs"])]
    return lines


def c_source(kernels: Dict[str, dict], prefix: str = "lfo_native", parts: int = 1):
    """C butterflies `<prefix>_bfly*` (x: inputs in slot order, y: outputs) and one Stockham
    pass per kernel with the butterfly inlined -- the pass of Gen/Stockham.lean:263-284:
    butterfly j = b*ns + k reads z[j + r*N/R] and, twiddled, tw[m*ns + k] (m < 2(R-1)), and
    writes output r at b*ns*R + k + r*ns -- plus the lookups `<prefix>_codelet(fwd, R, tw)`
    and `<prefix>_pass(fwd, R, tw)`.  The passes loop over k innermost (unit-stride complex
    accesses, so the compiler can vectorise across butterflies), or over b when ns = 1.
    Compile with -ffp-contract=off: every operation is rounded as the kernel prescribes.
    With parts > 1 the kernels are spread over `parts` sources (returned as a list, the
    lookups in the last), so that they compile in parallel."""
    head = ["/* ORACLE (test infrastructure only).  Generated by oracle/native_dag.py.",
            " * Compile with -ffp-contract=off. */",
            "#include <math.h>", "#include <stddef.h>", "",
            "typedef void (*lfo_codelet_fn)(const double *x, double *y);",
            "typedef void (*lfo_pass_fn)(long N, long ns, const double *tw, const double *z,",
            "                            double *o);", ""]
    files = [list(head) for _ in range(max(1, parts))]
    load = [0] * len(files)
    table = []
    for name in sorted(kernels, key=lambda n: -len(kernels[n]["ops"])):
        k = kernels[name]
        part = load.index(min(load))
        load[part] += len(k["ops"])
        out = files[part]
        R, tw = k["R"], k["tw"]
        fn, pn = f"{prefix}_{name}", f"{prefix}_pass_{name}"
        out.append(f"void {fn}(const double *restrict x, double *restrict y) {{")
        out += ["  " + l for l in _c_body(k, lambda i: f"x[{i}]", lambda i, v: f"y[{i}] = {v};")]
        out += ["}", ""]

        def xin(i, zi, ti):
            if i < 2 * R:
                r, c = divmod(i, 2)
                return f"{zi(r)}[{c}]"
            return ti(i - 2 * R)

        out += [f"void {pn}(long N, long ns, const double *restrict tw, "
                "const double *restrict z, double *restrict o) {",
                f"  const long NR = N / {R}, NB = NR / ns;",
                "  if (ns == 1) {",
                "    for (long b = 0; b < NB; ++b) {"]
        body1 = _c_body(k, lambda i: xin(i, lambda r: f"(z + 2 * (b + {r} * NR))",
                                          lambda m: f"tw[{m}]"),
                        lambda i, v: f"o[2 * (b * {R} + {i // 2}) + {i % 2}] = {v};")
        out += ["      " + l for l in body1]
        out += ["    }", "    return;", "  }",
                "  for (long b = 0; b < NB; ++b) {",
                "    const double *restrict zb = z + 2 * b * ns;",
                f"    double *restrict ob = o + 2 * b * ns * {R};",
                "    for (long kk = 0; kk < ns; ++kk) {"]
        body = _c_body(k, lambda i: xin(i, lambda r: f"(zb + 2 * (kk + {r} * NR))",
                                         lambda m: f"tw[{m} * ns + kk]"),
                       lambda i, v: f"ob[2 * (kk + {i // 2} * ns) + {i % 2}] = {v};")
        out += ["      " + l for l in body]
        out += ["    }", "  }", "}", ""]
        table.append((int(k["fwd"]), R, int(tw), fn, pn))
    out = files[-1]
    for row in table:
        out.append(f"void {row[3]}(const double *restrict x, double *restrict y);")
        out.append(f"void {row[4]}(long N, long ns, const double *restrict tw, "
                   "const double *restrict z, double *restrict o);")
    table.sort(key=lambda r: (r[1], r[2], -r[0]))
    for what, col in (("codelet", 3), ("pass", 4)):
        out.append(f"lfo_{what}_fn {prefix}_{what}(int fwd, int R, int tw) {{")
        for row in table:
            out.append(f"  if (fwd == {row[0]} && R == {row[1]} && tw == {row[2]}) return {row[col]};")
        out += ["  return NULL;", "}", ""]
    texts = ["\n".join(f) for f in files]
    return texts if parts > 1 else texts[0]


def from_ops(R: int, fwd: bool, tw: bool, n_in: int, ops, outs, cst_bits) -> dict:
    """A kernel in this module's encoding from an operation list in the same slot convention
    (operations ("add"|"sub"|"mul", a, b), ("neg", a), ("fma"|"fms"|"fnma", a, b, c),
    ("zero",), ("cst", c) with cst_bits(c) giving its 16-hex-digit binary64 bits)."""
    conv = []
    for op in ops:
        if op[0] == "cst":
            conv.append(["cst", cst_bits(op[1])])
        elif op[0] == "zero":
            conv.append(["cst", "0000000000000000"])
        else:
            conv.append([op[0], *op[1:]])
    return {"R": R, "fwd": fwd, "tw": tw, "n_in": n_in, "ops": conv, "outs": list(outs)}


# ------------------------------------------------------------------ exact evaluation

def bits_hex(v: float) -> str:
    """The 16 hex digits of a binary64 value's bits."""
    return f"{struct.unpack('<Q', struct.pack('<d', v))[0]:016x}"


def fma_exact(a: float, b: float, c: float) -> float:
    """fma(a, b, c) in binary64, round to nearest even, from exact rational arithmetic."""
    if math.isnan(a) or math.isnan(b) or math.isnan(c):
        return math.nan
    if math.isinf(a) or math.isinf(b):
        if a == 0.0 or b == 0.0:
            return math.nan                       # inf * 0
        p = math.copysign(math.inf, a) * math.copysign(1.0, b)
        if math.isinf(c) and c != p:
            return math.nan                       # inf - inf
        return p
    if math.isinf(c):
        return c
    exact = Fraction(a) * Fraction(b) + Fraction(c)
    if exact == 0:
        pz = math.copysign(1.0, a) * math.copysign(1.0, b) < 0    # sign of the zero product
        if (a == 0.0 or b == 0.0) and c == 0.0:
            neg = pz and math.copysign(1.0, c) < 0                # (-0) + (-0) = -0
            return -0.0 if neg else 0.0
        return 0.0                                # exact cancellation: +0 in round to nearest
    # beyond the largest finite binary64 by half an ulp or more: infinity
    if abs(exact) >= Fraction(2**1024 - 2**970):
        return math.inf if exact > 0 else -math.inf
    r = exact.numerator / exact.denominator       # correctly rounded (CPython int division)
    if r == 0.0:
        return 0.0 if exact > 0 else -0.0
    return r


def evaluate(k: dict, x: List[float]) -> List[float]:
    """The kernel's outputs for inputs x (len n_in), every operation rounded once."""
    v = list(x)
    for op in k["ops"]:
        o = op[0]
        if o == "cst":
            v.append(struct.unpack("<d", bytes.fromhex(op[1])[::-1])[0])
        elif o == "add":
            v.append(fma_exact(v[op[1]], 1.0, v[op[2]]))
        elif o == "sub":
            v.append(fma_exact(-v[op[2]], 1.0, v[op[1]]))
        elif o == "mul":
            v.append(fma_exact(v[op[1]], v[op[2]], -0.0))
        elif o == "neg":
            v.append(-v[op[1]])
        elif o == "fma":
            v.append(fma_exact(v[op[1]], v[op[2]], v[op[3]]))
        elif o == "fms":
            v.append(fma_exact(v[op[1]], v[op[2]], -v[op[3]]))
        else:
            v.append(fma_exact(-v[op[1]], v[op[2]], v[op[3]]))
    return [v[i] for i in k["outs"]]
