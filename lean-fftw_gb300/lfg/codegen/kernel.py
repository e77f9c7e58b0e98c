"""Butterfly kernels: common-subexpression elimination and the Stockham butterflies.

Restates lean-fftw's `LeanFFTW/Gen/Emit.lean` (straight-line `Kernel` over slots, `cse`,
`Kernel.counts`, Emit.lean:70-184) and the butterfly half of `LeanFFTW/Gen/Stockham.lean`
(`bflyIn`, `bflySym`, `butterfly`, `butterflyK`, Stockham.lean:224-252).

A kernel has `n_in` input slots; slot n_in + i holds the result of operation i.  An
operation is a tuple ("cst", c) | ("zero",) | ("add", a, b) | ("sub", a, b) | ("mul", a, b) |
("neg", a) | ("fma", a, b, c) | ("fms", a, b, c) | ("fnma", a, b, c) with slot operands.
Commutative operations take their first two operands in slot order (Emit.lean:126), which
lets CSE merge commuted duplicates; IEEE add, mul and fma are commutative in those operands,
so binary64 values are unchanged.
"""
from __future__ import annotations

import functools
from dataclasses import dataclass
from typing import Dict, List, Tuple

from . import sexpr
from .sexpr import E, inp
from .sym import SC, exec_plan, get, mk_plan, mul_gen, parts, prime_factors, val
from .symdft import pfa_dft, pfa_ok, pp_blocks, sym_dft

KOp = Tuple


@dataclass(frozen=True)
class Kernel:
    n_in: int
    ops: Tuple[KOp, ...]
    outs: Tuple[int, ...]

    def counts(self) -> Tuple[int, int, int]:
        """(adds/subs/negs, muls, fused) (Emit.lean:178-184)."""
        a = m = f = 0
        for op in self.ops:
            if op[0] in ("add", "sub", "neg"):
                a += 1
            elif op[0] == "mul":
                m += 1
            elif op[0] in ("fma", "fms", "fnma"):
                f += 1
        return a, m, f

    def flops(self) -> int:
        """Number of binary64 instructions one evaluation issues (negations included)."""
        return sum(self.counts())

    def constants(self) -> List[tuple]:
        return [op[1] for op in self.ops if op[0] == "cst"]


def cse(n_in: int, outs: List[E]) -> Kernel:
    """Emit.lean:115-175.  The slot of an expression is found depth-first, left to right;
    an operation already present (same operator, same operand slots) reuses its slot."""
    table: Dict[KOp, int] = {}
    ops: List[KOp] = []
    memo: Dict[int, int] = {}

    def node(op: KOp) -> int:
        s = table.get(op)
        if s is None:
            s = n_in + len(ops)
            table[op] = s
            ops.append(op)
        return s

    def ord2(x: int, y: int) -> Tuple[int, int]:
        return (x, y) if x <= y else (y, x)

    def go(e: E) -> int:
        r = memo.get(e.id)
        if r is not None:
            return r
        op = e.op
        if op == "input":
            r = e.args[0]
        elif op == "zero":
            r = node(("zero",))
        elif op == "cst":
            r = node(("cst", e.args[0]))
        elif op in ("add", "mul"):
            a = go(e.args[0])
            b = go(e.args[1])
            r = node((op,) + ord2(a, b))
        elif op == "sub":
            a = go(e.args[0])
            b = go(e.args[1])
            r = node(("sub", a, b))
        elif op == "neg":
            r = node(("neg", go(e.args[0])))
        else:  # fma, fms, fnma
            a = go(e.args[0])
            b = go(e.args[1])
            c = go(e.args[2])
            r = node((op,) + ord2(a, b) + (c,))
        memo[e.id] = r
        return r

    slots = [go(e) for e in outs]
    return Kernel(n_in, tuple(ops), tuple(slots))


# ---------------------------------------------------------------- butterflies (Stockham.lean)

def bfly_in(R: int, twiddled: bool, r: int) -> SC:
    """Input r: variables 2r, 2r+1, times the twiddle (variables 2R+2(r-1), +1) when
    twiddled and r >= 1 (Stockham.lean:224-228)."""
    xr = val(inp(2 * r), inp(2 * r + 1))
    if twiddled and r >= 1:
        w = val(inp(2 * R + 2 * (r - 1)), inp(2 * R + 2 * (r - 1) + 1))
        return mul_gen(w, xr)
    return xr


def bfly_sym(fwd: bool, R: int, twiddled: bool) -> List[SC]:
    """Stockham.lean:234-237."""
    x = lambda r: bfly_in(R, twiddled, r)
    if R & (R - 1) == 0:
        return exec_plan(mk_plan(fwd, prime_factors(R)), x)
    bs = pp_blocks(R)
    if pfa_ok(bs, R):
        return pfa_dft(fwd, bs, x)
    return sym_dft(fwd, prime_factors(R), x)


def butterfly(fwd: bool, R: int, twiddled: bool) -> List[E]:
    """The 2R contracted output expressions re y0, im y0, ... (Stockham.lean:242-245)."""
    y = bfly_sym(fwd, R, twiddled)
    out = []
    for i in range(2 * R):
        re, im = parts(get(y, i // 2))
        out.append(sexpr.contract(re if i % 2 == 0 else im))
    return out


def butterfly_inputs(R: int, twiddled: bool) -> int:
    """Stockham.lean:248."""
    return 4 * R - 2 if twiddled else 2 * R


@functools.lru_cache(maxsize=None)
def butterfly_k(fwd: bool, R: int, twiddled: bool) -> Kernel:
    """The CSE'd kernel of a radix-R butterfly (Stockham.lean:251-252)."""
    return cse(butterfly_inputs(R, twiddled), butterfly(fwd, R, twiddled))
