"""The planner's radix rule in Python (mirror of csrc/planner.cpp `choose_radices`).

Fewest codelet operations per point: the first pass is untwiddled, every later pass
twiddled; ties go to fewer passes; radices are tried from 16 down to 2.  Used where no GPU
plan exists (the CPU baseline) and by tests that cross-check the C++ planner.
"""
from __future__ import annotations

from functools import lru_cache
from typing import List, Tuple

from .kernel import butterfly_k

RADICES = list(range(2, 17))


@lru_cache(maxsize=None)
def ops(R: int, twiddled: bool) -> int:
    return sum(butterfly_k(True, R, twiddled).counts())


@lru_cache(maxsize=None)
def _tail(m: int) -> Tuple[float, Tuple[int, ...]]:
    if m == 1:
        return 0.0, ()
    best = (float("inf"), ())
    for R in reversed(RADICES):
        if m % R:
            continue
        c, s = _tail(m // R)
        c += ops(R, True) / R
        if c < best[0] - 1e-12 or (abs(c - best[0]) <= 1e-12 and len(s) + 1 < len(best[1])):
            best = (c, (R,) + s)
    return best


def choose_radices(n: int) -> List[int]:
    best = (float("inf"), ())
    for R0 in reversed(RADICES):
        if n % R0 or n < 2:
            continue
        c, s = _tail(n // R0)
        c += ops(R0, False) / R0
        if c < best[0] - 1e-12 or (abs(c - best[0]) <= 1e-12 and len(s) + 1 < len(best[1])):
            best = (c, (R0,) + s)
    return list(best[1])
