"""Pins the oracle's restatement of lean-fftw's r2r kinds (embedding, DFT, extraction,
Core/Problem.lean:64-112, 151-163) against independent definitions: scipy's DCT/DST types
I-IV (FFTW's REDFTxx/RODFTxx, unnormalised) and numpy's FFT for R2HC, HC2R and DHT."""
import numpy as np
import pytest

import oracle as O

sfft = pytest.importorskip("scipy.fft")

TYPES = {"redft00": ("dct", 1), "redft10": ("dct", 2), "redft01": ("dct", 3),
         "redft11": ("dct", 4), "rodft00": ("dst", 1), "rodft10": ("dst", 2),
         "rodft01": ("dst", 3), "rodft11": ("dst", 4)}


def _definition(kind, x):
    n = x.shape[-1]
    if kind in TYPES:
        f, t = TYPES[kind]
        return getattr(sfft, f)(x, type=t, axis=-1)
    F = np.fft.fft(x, axis=-1)
    if kind == "dht":
        return F.real - F.imag
    if kind == "r2hc":
        j = np.arange(n)
        return np.where(j <= n // 2, F.real[..., np.minimum(j, n - 1)], F.imag[..., (n - j) % n])
    # hc2r: halfcomplex -> Hermitian spectrum -> unnormalised inverse DFT
    h = np.zeros(x.shape[:-1] + (n // 2 + 1,), dtype=np.complex128)
    for k in range(n // 2 + 1):
        h[..., k] = x[..., k] + 1j * (x[..., n - k] if 0 < k < n - k else 0.0)
    return np.fft.irfft(h, n=n, axis=-1) * n


@pytest.mark.parametrize("kind", O.R2R_KINDS)
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 12, 15, 16, 30, 64, 100])
def test_r2r_restatement_matches_definition(kind, n):
    if kind == "redft00" and n < 2:
        return                                       # undefined (Problem.lean:241-242)
    x = np.random.default_rng(n).random((3, n)) - 0.5
    hi, lo = O.dd_r2r(kind, x)
    ref = _definition(kind, x)
    assert np.max(np.abs(hi + lo - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref))), (kind, n)


@pytest.mark.parametrize("kind", O.R2R_KINDS)
def test_generic_and_fast_r2r_accuracy(kind):
    """The generic engine's r2r and the same embedding around refTransform both land at
    binary64 accuracy against the extended-precision version."""
    from lfg.codegen.plans import choose_radices
    n = 64                    # embedding sizes 64, 126, 130, 256, 512: all 13-smooth
    x = np.random.default_rng(3).random((4, n)) - 0.5
    ref = O.dd_r2r(kind, x)
    M = O.r2r_embed_size(kind, n)
    assert O.rel_l2(O.generic_r2r(kind, x), ref) < 2e-15
    assert O.rel_l2(O.fast_r2r(kind, x, choose_radices(M)), ref) < 2e-15
