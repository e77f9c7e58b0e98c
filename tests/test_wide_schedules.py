"""Lane-parallel schedules of the binary64 butterflies (CPU).

The lone-transform cluster kernel (csrc/cluster_f64.cu) evaluates each butterfly level by
level of its operation DAG, one fused multiply-add per lane per level, from tables built by
lfg/codegen/wide.py.  Here the tables are replayed on the host with a correctly rounded
fused multiply-add and must give, bit for bit:

* for radices 2, 4, 8 and 16, the exact evaluation of lean-fftw's own generated kernels
  (tests/golden/native_kernels.json, LeanFFTW/Native/Kernels.lean), independently of the
  product's generator;
* for every radix 2..16, the oracle's C butterflies (lean-fftw's kernels for 2, 4, 8 and 16,
  the restated generator's for the others; compiled with -ffp-contract=off), on random
  inputs and on inputs mixed with special values.

Structure: a level reads only slots written by earlier levels, every operation appears once,
no level is wider than its lane group, and idle lanes write only a scratch slot.
"""
import numpy as np
import pytest

import native_dag
import oracle as O
from lfg.codegen.wide import replay, unpack_desc, wide_schedule

REF = native_dag.load()
SPECIALS = [0.0, -0.0, 5e-324, -1e-310, 1.7976931348623157e308, float("inf"), -float("inf"),
            float("nan"), 1.0, -1.0, 1e300]


def _same(a, b) -> bool:
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and
                np.array_equal(a[~na].view(np.uint64), b[~nb].view(np.uint64)))


def _inputs(n, R, tw, rng, count):
    rows = [rng.uniform(-1, 1, n) for _ in range(count)]
    rows += [rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n) for _ in range(count)]
    for _ in range(count):
        x = rng.uniform(-1, 1, n)
        idx = rng.choice(2 * R, size=min(3, 2 * R), replace=False)
        x[idx] = rng.choice(SPECIALS, size=idx.size)
        rows.append(x)
    if tw:
        for x in rows[:count]:
            a = rng.uniform(0, 2 * np.pi, R - 1)
            x[2 * R::2], x[2 * R + 1::2] = np.cos(a), np.sin(a)
    return rows


@pytest.mark.parametrize("R,tw,fwd", [(R, tw, fwd) for R in native_dag.RADICES
                                      for tw in (False, True) for fwd in (True, False)])
def test_schedule_is_the_reference_kernel(R, tw, fwd):
    ws = wide_schedule(fwd, R, tw)
    k = REF[native_dag.kernel_name(fwd, R, tw)]
    rng = np.random.default_rng(100 * R + 10 * tw + fwd)
    for x in _inputs(k["n_in"], R, tw, rng, 3 if R == 16 else 6):
        xs = list(map(float, x))
        assert _same(replay(ws, native_dag.fma_exact, xs), native_dag.evaluate(k, xs)), (R, tw, fwd)


@pytest.mark.parametrize("R", range(2, 17))
@pytest.mark.parametrize("tw", [False, True])
def test_schedule_matches_oracle_codelets(R, tw):
    for fwd in (True, False):
        ws = wide_schedule(fwd, R, tw)
        rng = np.random.default_rng(7 * R + tw + 3 * fwd)
        n = 4 * R - 2 if tw else 2 * R
        for x in _inputs(n, R, tw, rng, 2):
            got = replay(ws, native_dag.fma_exact, list(map(float, x)))
            want = O.bfly(fwd, R, tw, x, native=R in native_dag.RADICES)
            assert _same(got, want), (R, tw, fwd)


@pytest.mark.parametrize("R", range(2, 17))
def test_schedule_structure(R):
    for tw in (False, True):
        ws = wide_schedule(True, R, tw)
        assert ws.W in (1, 2, 4, 8, 16, 32)
        written = set(range(ws.in_base + ws.n_in))      # constants and inputs
        scratch = ws.n_slots - 1                         # where idle lanes write
        for lvl in ws.levels:
            assert len(lvl) == ws.W
            outs = []
            for d in lvl:
                u = unpack_desc(d)
                assert u is not None                     # every lane issues (no divergence)
                a, b, c, _, _, o = u
                assert {a, b, c} <= written              # reads only earlier levels
                if o != scratch:
                    outs.append(o)
            assert outs and len(set(outs)) == len(outs) and not (set(outs) & written)
            written |= set(outs)
        assert all((o & 0x7fff) in written for o in ws.outs)
        assert ws.n_slots == len(written) + 1
