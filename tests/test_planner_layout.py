"""The planner's choices, computed on the host (lfg_plan_layout; no GPU needed): radix
sequences with the fewest codelet operations, and the pass-group split of sizes above one
CTA's tile, including the fallbacks for the largest sizes (2^20..2^24, lfg_plan_1d's limit)
and the balanced binary32 split."""
import math

import numpy as np
import pytest

import lfg

SMEM_MAX = 7264    # largest binary64 pass group that fits two padded tile buffers


def _groups(n, rs, first):
    P = int(np.prod(rs[:first])) if first else 1
    return P, n // P


def _smooth13(n):
    for p in (2, 3, 5, 7, 11, 13):
        while n % p == 0:
            n //= p
    return n == 1


def test_known_layouts():
    assert lfg.plan_layout(1024) == ([16, 16, 4], 3)          # one group (<= 2048 points)
    rs, first = lfg.plan_layout(4096)
    assert first < len(rs) and max(_groups(4096, rs, first)) <= 2048
    rs, first = lfg.plan_layout(1 << 24)
    assert _groups(1 << 24, rs, first) == (4096, 4096)
    rs, first = lfg.plan_layout(16384, "f32")                  # balanced binary32 split
    assert _groups(16384, rs, first) == (128, 128)
    rs, first = lfg.plan_layout(4096, "f32")                   # binary32: one group to 4096
    assert first == len(rs)
    rs, first = lfg.plan_layout(8192, "f32")                   # then two register-staged groups
    assert _groups(8192, rs, first) == (128, 64)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_every_power_of_two_and_smooth_samples_plan(prec):
    rng = np.random.default_rng(1)
    sizes = [1 << k for k in range(1, 25)]
    smooth = [n for n in rng.integers(2, 1 << 22, size=4000) if _smooth13(int(n))]
    sizes += [int(n) for n in smooth[:60]] + [75600, 10368, 15015, 2310]
    for n in sizes:
        rs, first = lfg.plan_layout(n, prec)
        assert math.prod(rs) == n and all(2 <= r <= 16 for r in rs), (n, rs)
        assert 1 <= first <= len(rs)
        P, Q = _groups(n, rs, first)
        if first == len(rs):
            assert n <= SMEM_MAX * (2 if prec == "f32" else 1)
        else:
            assert P <= SMEM_MAX and Q <= SMEM_MAX, (n, rs, first)


def test_default_binary64_groups_prefer_2048():
    # up to 2048^2 points the two groups stay within the 2048-point default when the
    # fewest-operation order allows it
    for k in (12, 14, 16, 18, 19):
        rs, first = lfg.plan_layout(1 << k)
        assert max(_groups(1 << k, rs, first)) <= 2048, (k, rs, first)


def test_unsupported_sizes():
    for n in (1, 17, 2 * 17, (1 << 24) + 2, 1 << 25):
        with pytest.raises(lfg.LfgError):
            lfg.plan_layout(n)
