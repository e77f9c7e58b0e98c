"""Symbolic real expressions for codelet generation.

Restates lean-fftw's `LeanFFTW/Gen/SExpr.lean`: straight-line real expressions over numbered
inputs and exact trigonometric constants, with the operations the kernels execute
(`+ - * neg` and the three fused forms), the local simplifying constructors (`mk*`,
SExpr.lean:93-152) and FMA contraction (`contract`, SExpr.lean:154-176).

Expressions are hash-consed: every structurally distinct node exists once and carries a
small integer id, so structural equality is identity and the recursive passes (contract,
CSE) memoise on the id.  Structural identity is exactly what the reference's CSE merges
(its HashMap is keyed on the operation with operand slots), so hash-consing changes no
generated kernel.

Binary64 meaning of each node (SExpr.lean:77-87):
    add a+b, sub a-b, mul a*b, neg -a,
    fma  = fma(a, b, c)   (a*b + c, one rounding)
    fms  = fma(a, b, -c)  (a*b - c)
    fnma = fma(-a, b, c)  (c - a*b)
"""
from __future__ import annotations

from typing import Dict, Tuple

from . import trig

# ---------------------------------------------------------------- constants (SExpr.lean:27-45)
# A constant is a tuple: ("cos", k, n) | ("sin", k, n) | ("sqrthalf",) | ("tan", k, n).
# (k, n) is kept as given, unreduced: cos(1, 8) and cos(2, 16) are distinct constants, as in
# the reference's derived equality on `Cst`.

Cst = Tuple


def cst_value(c: Cst) -> float:
    """Binary64 value of a constant (SExpr.lean:41-45)."""
    if c[0] == "cos":
        return trig.cos_sin_2pi(c[1], c[2])[0]
    if c[0] == "sin":
        return trig.cos_sin_2pi(c[1], c[2])[1]
    if c[0] == "sqrthalf":
        return trig.cos_sin_2pi(1, 8)[0]
    if c[0] == "tan":
        return trig.tan2pi(c[1], c[2])
    raise ValueError(c)


def cst_c_literal(c: Cst) -> str:
    """Hexadecimal C literal denoting exactly the binary64 value (SExpr.lean:48-53)."""
    v = cst_value(c)
    return "0.0" if v == 0.0 else v.hex()


# ---------------------------------------------------------------- hash-consed nodes

class E:
    """One expression node. `op` is one of input, zero, cst, add, sub, mul, neg, fma, fms,
    fnma; `args` holds child nodes (or the input index / constant)."""
    __slots__ = ("op", "args", "id")

    def __init__(self, op: str, args: tuple, nid: int):
        self.op = op
        self.args = args
        self.id = nid

    def __repr__(self) -> str:  # compact, for debugging only
        if self.op == "input":
            return f"x{self.args[0]}"
        if self.op == "zero":
            return "0"
        if self.op == "cst":
            return "C" + str(self.args[0])
        return f"{self.op}({', '.join(map(repr, self.args))})"


_table: Dict[tuple, E] = {}


def _node(op: str, *args) -> E:
    key = (op,) + tuple(a.id if isinstance(a, E) else a for a in args)
    e = _table.get(key)
    if e is None:
        e = E(op, args, len(_table))
        _table[key] = e
    return e


def inp(i: int) -> E:
    return _node("input", i)


ZERO = _node("zero")


def cst(c: Cst) -> E:
    return _node("cst", c)


def add(a: E, b: E) -> E:
    return _node("add", a, b)


def sub(a: E, b: E) -> E:
    return _node("sub", a, b)


def mul(a: E, b: E) -> E:
    return _node("mul", a, b)


def neg(a: E) -> E:
    return _node("neg", a)


def fma(a: E, b: E, c: E) -> E:
    return _node("fma", a, b, c)


def fms(a: E, b: E, c: E) -> E:
    return _node("fms", a, b, c)


def fnma(a: E, b: E, c: E) -> E:
    return _node("fnma", a, b, c)


# ---------------------------------------------------------------- smart constructors

def is_zero(a: E) -> bool:
    return a.op == "zero"


def mk_neg(a: E) -> E:
    """SExpr.lean:97-100."""
    if a.op == "zero":
        return ZERO
    if a.op == "neg":
        return a.args[0]
    return neg(a)


def mk_add(a: E, b: E) -> E:
    """SExpr.lean:102-107 (first matching case wins)."""
    if a.op == "zero":
        return b
    if b.op == "zero":
        return a
    if b.op == "neg":
        return sub(a, b.args[0])
    if a.op == "neg":
        return sub(b, a.args[0])
    return add(a, b)


def mk_sub(a: E, b: E) -> E:
    """SExpr.lean:109-114."""
    if b.op == "zero":
        return a
    if a.op == "zero":
        return mk_neg(b)
    if b.op == "neg":
        return add(a, b.args[0])
    if a.op == "neg":
        return mk_neg(add(a.args[0], b))
    return sub(a, b)


def mk_mul_c(c: Cst, a: E) -> E:
    """c * a for a constant c (SExpr.lean:117-120)."""
    if a.op == "zero":
        return ZERO
    if a.op == "neg":
        return mk_neg(mul(cst(c), a.args[0]))
    return mul(cst(c), a)


def mk_fnma_c(t: Cst, b: E, a: E) -> E:
    """a - t*b (SExpr.lean:137-140)."""
    if b.op == "zero":
        return a
    return fnma(cst(t), b, a)


def mk_fma_c(t: Cst, a: E, b: E) -> E:
    """t*a + b (SExpr.lean:143-146)."""
    if a.op == "zero":
        return b
    return fma(cst(t), a, b)


def mk_fms_c(t: Cst, a: E, b: E) -> E:
    """t*a - b (SExpr.lean:149-152)."""
    if a.op == "zero":
        return mk_neg(b)
    return fms(cst(t), a, b)


# ---------------------------------------------------------------- FMA contraction

def _contract_add(a: E, b: E) -> E:
    """SExpr.lean:155-158."""
    if a.op == "mul":
        return fma(a.args[0], a.args[1], b)
    if b.op == "mul":
        return fma(b.args[0], b.args[1], a)
    return add(a, b)


def _contract_sub(a: E, b: E) -> E:
    """SExpr.lean:161-164."""
    if a.op == "mul":
        return fms(a.args[0], a.args[1], b)
    if b.op == "mul":
        return fnma(b.args[0], b.args[1], a)
    return sub(a, b)


_contract_memo: Dict[int, E] = {}


def contract(e: E) -> E:
    """Bottom-up FMA contraction (SExpr.lean:168-176)."""
    r = _contract_memo.get(e.id)
    if r is not None:
        return r
    op = e.op
    if op == "add":
        r = _contract_add(contract(e.args[0]), contract(e.args[1]))
    elif op == "sub":
        r = _contract_sub(contract(e.args[0]), contract(e.args[1]))
    elif op == "mul":
        r = mul(contract(e.args[0]), contract(e.args[1]))
    elif op == "neg":
        r = neg(contract(e.args[0]))
    elif op in ("fma", "fms", "fnma"):
        r = _node(op, contract(e.args[0]), contract(e.args[1]), contract(e.args[2]))
    else:
        r = e
    _contract_memo[e.id] = r
    return r
