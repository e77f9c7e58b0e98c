"""The C-ABI library loads, exports every entry point include/lfg.h declares, and its
host-side twiddle tables match lean-fftw's integer trigonometry (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

import lfg
import trig_ref
from conftest import ROOT, has_gpu


def _declared():
    text = open(os.path.join(ROOT, "include", "lfg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lfg_[a-z0-9_]+)\s*\(", text)))


def test_libbench2_backend_builds_and_links():
    """The libbench2 backend compiles against the stand-in libbench2 header, links against
    liblfg.so and exports libbench2's backend interface (its GPU test drives it)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "libbench2_stub"))
    import build_harness
    lfg.lib()
    L = ctypes.CDLL(build_harness.build())
    for name in ("can_do", "setup", "doit", "done", "main_init", "initial_cleanup",
                 "final_cleanup", "bench_doc", "lfgb_run"):
        assert hasattr(L, name), name


def test_exports_every_declared_symbol():
    L = lfg.lib()
    names = _declared()
    assert "lfg_plan_spec" in names and "lfg_execute" in names
    for n in names:
        assert hasattr(L, n), n


@pytest.mark.parametrize("n", [1, 2, 3, 8, 12, 100, 1000, 1024, 10368, 65536, 75600])
def test_cos_sin_table_matches_reference_trig(n):
    got = lfg.cos_sin_table(n)
    ref = np.array(trig_ref.table(n), dtype=np.float64)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_table_values_close_to_true_trig():
    # tau (twiddle accuracy): results/repro-2026-11-04/twiddles.jsonl reports <= 0.502 ulp of 1
    n = 4096
    got = lfg.cos_sin_table(n)
    dd = np.array(trig_ref.dd_table(n))
    err = max(np.max(np.abs((got[:, 0] - dd[:, 0]) - dd[:, 1])),
              np.max(np.abs((got[:, 1] - dd[:, 2]) - dd[:, 3])))
    assert err <= 0.502 * 2.0 ** -52


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_plan_without_gpu_fails_loudly():
    with pytest.raises(lfg.LfgError):
        lfg.plan_1d(1024)


def test_unsupported_sizes_rejected_before_device_use():
    # sizes above 2^24, an explicit radix sequence for a size with a prime factor above 13
    # (the fast engine's codelets stop at 13), REDFT00 of one point (undefined, as in the
    # reference) and odd-length real transforms are refused before any device use
    with pytest.raises(lfg.Unsupported):
        lfg.plan_1d(1 << 25)
    with pytest.raises(lfg.Unsupported):
        lfg.plan_1d(17, radices=[17])
    with pytest.raises(lfg.Unsupported):
        lfg.plan_r2r(1, "redft00")
    with pytest.raises(lfg.Unsupported):
        lfg.plan_r2c(15)


def test_invalid_arguments():
    L = lfg.lib()
    h = ctypes.c_void_p()
    assert L.lfg_plan_1d(16, 0, 1, 0, 0, ctypes.byref(h)) == lfg._lib.LFG_ERR_INVALID
    assert L.lfg_plan_spec(None, 0, 0, 0, ctypes.byref(h)) == lfg._lib.LFG_ERR_INVALID
    assert L.lfg_execute(None, None, None, None) == lfg._lib.LFG_ERR_INVALID
    assert lfg.lib().lfg_strerror(1) == b"problem not supported"
