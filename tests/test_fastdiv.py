"""The kernels' division by plan-time divisors (FastDiv in csrc/stockham.h): q = (umulhi(m, n)
+ n) >> l with l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, for 0 <= n < 2^31.
Checked here on the same formula, exhaustively over the dividends that matter for small
divisors (sub-problem lengths, tile widths, pass strides) and at the edges for large ones;
the GPU tests check it through the bit-exact transforms."""
import numpy as np


def make(d):
    l = 0
    while l < 31 and (1 << l) < d:
        l += 1
    m = ((1 << 32) * ((1 << l) - d)) // d + 1
    assert 0 <= m < (1 << 32)
    return m, l


def fdiv(n, m, l):
    t = (m * n) >> 32
    return (t + n) >> l


def test_small_divisors_exhaustive():
    n = np.arange(0, 1 << 17, dtype=np.uint64)
    for d in range(1, 2049):
        m, l = make(d)
        q = ((np.uint64(m) * n) >> np.uint64(32)) + n >> np.uint64(l)
        assert np.array_equal(q, n // np.uint64(d)), d


def test_edges_large():
    rng = np.random.default_rng(7)
    ds = [1, 2, 3, 7, 1000, 65535, 65536, 65537, 262144, 1 << 20, 3 ** 13, (1 << 30) + 1,
          (1 << 31) - 1] + [int(x) for x in rng.integers(1, 1 << 31, 200)]
    top = (1 << 31) - 1
    for d in ds:
        m, l = make(d)
        ns = {0, 1, d - 1, d, d + 1, top, top - 1, top - d % top} | {
            int(x) for x in rng.integers(0, top + 1, 2000)}
        for k in (1, 2, 3, 1000):
            for e in (-1, 0, 1):
                v = k * d + e
                if 0 <= v <= top:
                    ns.add(v)
        for n in ns:
            if 0 <= n <= top:
                assert fdiv(n, m, l) == n // d, (n, d)
