"""lfg-bench, the libbench2-style command line (lean-fftw tools/bench.py drives such
binaries with `-s <problem>` and `-v1 --verify <problem>`, tools/bench.py:44-48, 71-84).

CPU: the problem grammar (tools/classify_problems.py:7-40) maps to the FFI spec
(LeanFFTW/FFI.lean:13-21) with libbench2's row-major default strides, in doubles.
GPU: --can-do, --verify (linearity, impulse and shift errors at the binary64 level) and
the speed line in the format tools/bench.py parses."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "lean-fftw_gb300", "lfg", "lfg-bench")


def _run(*args, timeout=300):
    if not os.path.exists(EXE):
        pytest.skip("lfg-bench not built")
    r = subprocess.run([EXE, *args], capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout.strip(), r.stderr.strip()


PARSE = {
    "ocf1024": "0 -1 1 0 0 1 0 1 1024 2 2",
    "icb64x48": "0 1 2 0 0 1 0 1 64 96 96 48 2 2",
    # real sides carry im = re, as lean-fftw's libbench2 adapter encodes them
    # (bench/backends/bench-leanfftw.c:98-101)
    "orf8192*256": "1 -1 1 1 0 0 0 1 8192 1 2 256 8192 8194",
    "irb512x512*4": "1 1 2 1 0 1 0 0 512 514 514 512 2 1 4 263168 263168",
    "ocf1024:2:2*8:4096:4096": "0 -1 1 1 0 1 0 1 1024 4 4 8 8192 8192",
    "ocf16v8": "0 -1 1 1 0 1 0 1 16 16 16 8 2 2",
    "orb12x60": "1 1 2 0 0 1 0 0 12 62 60 60 2 1",
    "ir8": "1 -1 1 0 0 0 0 1 8 1 2",
    # split arrays: the imaginary array follows the real one, strides in doubles of each
    "o/cf16": "0 -1 1 0 0 16 0 16 16 1 1",
    "o/cb16*3": "0 1 1 1 0 48 0 48 16 1 1 3 16 16",
    "o/rf8": "1 -1 1 0 0 0 0 5 8 1 1",
    # r2r: kind suffixes f b h e00..e11 o00..o11 (none: R2HC forward, HC2R backward)
    "ok16": "2 -1 1 0 0 0 0 0 16 1 1 0",
    "okb64": "2 1 1 0 0 0 0 0 64 1 1 1",
    "ok30h": "2 -1 1 0 0 0 0 0 30 1 1 2",
    "ok10e10x12e01": "2 -1 2 0 0 0 0 0 10 12 12 12 1 1 5 4",
    "ik16o00*4": "2 -1 1 1 0 0 0 0 16 1 1 4 16 16 7",
    "ok12e00x16o10v3": "2 -1 2 1 0 0 0 0 12 48 48 16 3 3 3 1 1 3 9",
}


@pytest.mark.parametrize("prob", sorted(PARSE))
def test_parse_to_spec(prob):
    rc, out, _ = _run("--parse", prob)
    assert rc == 0 and out == PARSE[prob], (prob, out)


@pytest.mark.parametrize("prob", ["o/kf16", "ocf16o00", "ocfx", "ok16e02", "ok16q"])
def test_unsupported_problems_are_not_doable(prob):
    rc, out, _ = _run("--can-do", prob)
    assert rc == 0 and out == "#f"


def test_print_precision():
    assert _run("--print-precision")[1] == "double"


torch = pytest.importorskip("torch")
GPU = torch.cuda.is_available()


@pytest.mark.gpu
@pytest.mark.skipif(not GPU, reason="no GPU")
@pytest.mark.parametrize("prob,ok", [("ocf1024", True), ("ibf360*5", True), ("orf12x60", True),
                                     ("ocf64x64", True), ("ocf17", True), ("ocf19x4", True),
                                     ("orf15", True), ("ok1e00", False), ("ocf1", False)])
def test_can_do(prob, ok):
    assert _run("--can-do", prob)[1] == ("#t" if ok else "#f")


@pytest.mark.gpu
@pytest.mark.skipif(not GPU, reason="no GPU")
@pytest.mark.parametrize("prob", ["ocf1024", "ibf360*5", "icf4096", "ocb10368*3", "ocf16v8",
                                  "ocf262144", "orf8192*4", "irf1000*3", "orb8192*4",
                                  "irb360*2", "orf12x60", "orb64x48*2", "irb512x512*2",
                                  "ocf60:3:1*4:200:64", "ocf64x48", "icb12x10x8*2",
                                  "ocf16x16v3", "ok16", "okb64", "ok30h", "ok10e10x12e01",
                                  "ik16o00*4", "ok12e00x16o10v3", "ok8e11*3", "ok9o01x5e00",
                                  "o/cf1024*3", "i/cb64x48", "o/rf100*2", "o/rb30x12",
                                  "orf15*4", "orb45", "ocf101*3", "orf6x8x10"])
def test_verify(prob):
    rc, out, err = _run("--verify", prob)
    assert rc == 0, err
    m = re.match(r"^(\S+)\s+([0-9.e+-]+)\s+([0-9.e+-]+)\s+([0-9.e+-]+)$", out)
    assert m and m.group(1) == prob, out
    el, ei, es = (float(m.group(i)) for i in (2, 3, 4))
    assert max(el, ei, es) < 1e-14, out


@pytest.mark.gpu
@pytest.mark.skipif(not GPU, reason="no GPU")
@pytest.mark.parametrize("mode", [[], ["-o", "device"]])
def test_speed_line(mode):
    rc, out, err = _run("-s", "ocf1024*64", "-t", "0.002", *mode)
    assert rc == 0, err
    m = re.search(r"setup:\s*([0-9.e+-]+)\s*(ns|us|ms|s),\s*time:\s*([0-9.e+-]+)\s*(ns|us|ms|s)", out)
    assert m and out.startswith("Problem: ocf1024*64,"), out
    assert float(m.group(3)) > 0
