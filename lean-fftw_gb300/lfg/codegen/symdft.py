"""Symbolic DFTs for butterflies whose radix is not a power of two.

Restates lean-fftw's `LeanFFTW/Gen/SymDFT.lean`:

* odd lengths by pairing terms j and p-j (`oddLeaf`, SymDFT.lean:67-115): with
  a_j = x_j + x_{p-j} and b_j = x_j - x_{p-j}, A_k = x_0 + sum cos(2*pi*j*k/p) a_j and
  S_k = sum sin(2*pi*j*k/p) b_j, so X_k = A_k -+ i S_k and X_{p-k} = A_k +- i S_k;
* factored mixed radix (`symDFT`, SymDFT.lean:126-135);
* Good-Thomas over coprime prime-power blocks (`pfaDFT`, SymDFT.lean:141-165).

Every constant is the cosine or sine of a first-quadrant angle (nonnegative); the sign of a
term is carried by the fused operation (fma or fnma).
"""
from __future__ import annotations

from typing import Callable, List, Tuple

from .sexpr import E, mk_add, mk_fma_c, mk_fnma_c, mk_mul_c, mk_neg, mk_sub, ZERO
from .sym import (SC, exec_plan, get, parts, prime_factors, sc_mul, tw, val)


def cos_h(m: int, n: int) -> Tuple[bool, tuple]:
    """cos(2*pi*m/n), 2m <= n, as (negative?, first-quadrant constant) (SymDFT.lean:33-34)."""
    if 4 * m <= n:
        return False, ("cos", m, n)
    return True, ("cos", n - 2 * m, 2 * n)


def cos_q(m: int, n: int) -> Tuple[bool, tuple]:
    """SymDFT.lean:37."""
    return cos_h(m if 2 * m <= n else n - m, n)


def sin_h(m: int, n: int) -> tuple:
    """SymDFT.lean:40-41."""
    if 4 * m <= n:
        return ("sin", m, n)
    return ("sin", n - 2 * m, 2 * n)


def sin_q(m: int, n: int) -> Tuple[bool, tuple]:
    """SymDFT.lean:45-46."""
    if 2 * m <= n:
        return False, sin_h(m, n)
    return True, sin_h(n - m, n)


def sfma(ng: bool, c: tuple, a: E, acc: E) -> E:
    """acc +- c*a (SymDFT.lean:49-50)."""
    return mk_fnma_c(c, a, acc) if ng else mk_fma_c(c, a, acc)


def smul(ng: bool, c: tuple, a: E) -> E:
    """+- c*a (SymDFT.lean:53-54)."""
    return mk_neg(mk_mul_c(c, a)) if ng else mk_mul_c(c, a)


def lacc(init: E, ts) -> E:
    """init + sum +-c_i a_i, left to right (SymDFT.lean:57-58)."""
    acc = init
    for ng, c, a in ts:
        acc = sfma(ng, c, a, acc)
    return acc


def lsum(ts) -> E:
    """SymDFT.lean:61-63."""
    if not ts:
        return ZERO
    ng, c, a = ts[0]
    return lacc(smul(ng, c, a), ts[1:])


def pair_a(p: int, x: Callable[[int], SC], i: int) -> Tuple[E, E]:
    """x_j + x_{p-j}, j = i+1 (SymDFT.lean:68-70)."""
    u, v = parts(x(i + 1)), parts(x(p - (i + 1)))
    return mk_add(u[0], v[0]), mk_add(u[1], v[1])


def pair_b(p: int, x: Callable[[int], SC], i: int) -> Tuple[E, E]:
    """x_j - x_{p-j}, j = i+1 (SymDFT.lean:73-75)."""
    u, v = parts(x(i + 1)), parts(x(p - (i + 1)))
    return mk_sub(u[0], v[0]), mk_sub(u[1], v[1])


def c_terms(p: int, k: int, x, part: int):
    """SymDFT.lean:78-80."""
    out = []
    for i in range(p // 2):
        ng, c = cos_q((i + 1) * k % p, p)
        out.append((ng, c, pair_a(p, x, i)[part]))
    return out


def s_terms(p: int, k: int, x, part: int):
    """SymDFT.lean:83-85."""
    out = []
    for i in range(p // 2):
        ng, c = sin_q((i + 1) * k % p, p)
        out.append((ng, c, pair_b(p, x, i)[part]))
    return out


def odd_a(p: int, k: int, x) -> Tuple[E, E]:
    """SymDFT.lean:88-89."""
    x0 = parts(x(0))
    return lacc(x0[0], c_terms(p, k, x, 0)), lacc(x0[1], c_terms(p, k, x, 1))


def odd_s(p: int, k: int, x) -> Tuple[E, E]:
    """SymDFT.lean:92-93."""
    return lsum(s_terms(p, k, x, 0)), lsum(s_terms(p, k, x, 1))


def odd_plus(p: int, k: int, x) -> SC:
    """A_k + i S_k (SymDFT.lean:96-97)."""
    a, s = odd_a(p, k, x), odd_s(p, k, x)
    return val(mk_sub(a[0], s[1]), mk_add(a[1], s[0]))


def odd_minus(p: int, k: int, x) -> SC:
    """A_k - i S_k (SymDFT.lean:100-101)."""
    a, s = odd_a(p, k, x), odd_s(p, k, x)
    return val(mk_add(a[0], s[1]), mk_sub(a[1], s[0]))


def odd_x0(p: int, x) -> SC:
    """SymDFT.lean:104-106."""
    x0 = parts(x(0))
    re, im = x0
    for i in range(p // 2):
        re = mk_add(re, pair_a(p, x, i)[0])
    for i in range(p // 2):
        im = mk_add(im, pair_a(p, x, i)[1])
    return val(re, im)


def odd_leaf(fwd: bool, p: int, x) -> List[SC]:
    """SymDFT.lean:111-115."""
    out = []
    for k in range(p):
        if k == 0:
            out.append(odd_x0(p, x))
        elif k <= p // 2:
            out.append(odd_minus(p, k, x) if fwd else odd_plus(p, k, x))
        else:
            out.append(odd_plus(p, p - k, x) if fwd else odd_minus(p, p - k, x))
    return out


def leaf_sym(fwd: bool, p: int, x) -> List[SC]:
    """Prime-length leaf (SymDFT.lean:119-121)."""
    if p % 2 == 1 and p >= 3:
        return odd_leaf(fwd, p, x)
    return exec_plan(("direct", p, fwd), x)


def sym_dft(fwd: bool, fs: List[int], x) -> List[SC]:
    """Factored mixed radix (SymDFT.lean:126-135)."""
    if not fs:
        return leaf_sym(fwd, 1, x)
    if len(fs) == 1:
        return leaf_sym(fwd, fs[0], x)
    r = fs[0]
    m = 1
    for f in fs[1:]:
        m *= f
    ys = [sym_dft(fwd, fs[1:], lambda j2, j1=j1: x(j1 + r * j2)) for j1 in range(r)]
    cols = [leaf_sym(fwd, r, lambda j1, k1=k1: sc_mul(tw(fwd, r * m, j1 * k1), get(ys[j1], k1)))
            for k1 in range(m)]
    return [get(cols[k % m], k // m) for k in range(r * m)]


def pp_blocks(n: int) -> List[int]:
    """Prime-power blocks, one per distinct prime, ascending (SymDFT.lean:141-143)."""
    fs = prime_factors(n)
    out = []
    for p in fs:
        if p not in [q for q, _ in out]:
            out.append((p, fs.count(p)))
    return [p ** e for p, e in out]


def pfa_ok(bs: List[int], n: int) -> bool:
    """SymDFT.lean:146-147."""
    from math import gcd, prod
    if prod(bs) != n or any(b <= 0 for b in bs):
        return False
    return all(gcd(bs[i], bs[j]) == 1 for i in range(len(bs)) for j in range(i + 1, len(bs)))


def pfa_dft(fwd: bool, bs: List[int], x) -> List[SC]:
    """Good-Thomas prime factor algorithm over coprime blocks (SymDFT.lean:156-165)."""
    if not bs:
        return sym_dft(fwd, [], x)
    if len(bs) == 1:
        return sym_dft(fwd, prime_factors(bs[0]), x)
    b = bs[0]
    m = 1
    for c in bs[1:]:
        m *= c
    ys = [pfa_dft(fwd, bs[1:], lambda j2, j1=j1: x((m * j1 + b * j2) % (b * m)))
          for j1 in range(b)]
    cols = [sym_dft(fwd, prime_factors(b), lambda j1, k2=k2: get(ys[j1], k2)) for k2 in range(m)]
    return [get(cols[k % m], k % b) for k in range(b * m)]
