"""Build the libbench2 backend (lean-fftw_gb300/csrc/tools/bench_lfg.c) against the stand-in
header of this folder, with the test harness, into _build/libbench_lfg.so (test
infrastructure; linked against lean-fftw_gb300/lfg/liblfg.so, which must be built first).

    python tests/libbench2_stub/build_harness.py
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "lean-fftw_gb300", "lfg")
SO = os.path.join(HERE, "_build", "libbench_lfg.so")


def build() -> str:
    srcs = [os.path.join(ROOT, "lean-fftw_gb300", "csrc", "tools", "bench_lfg.c"),
            os.path.join(HERE, "harness.c")]
    deps = srcs + [os.path.join(HERE, "libbench2", "bench-user.h"),
                   os.path.join(ROOT, "include", "lfg.h"), os.path.join(PKG, "liblfg.so")]
    if os.path.exists(SO) and os.path.getmtime(SO) >= max(os.path.getmtime(p) for p in deps):
        return SO
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c99", "-Wall", "-fPIC", "-shared", "-I", HERE,
           "-I", os.path.join(ROOT, "include"), *srcs, "-o", SO + ".tmp", "-L", PKG, "-llfg",
           "-Wl,-rpath," + PKG]
    subprocess.run(cmd, check=True)
    os.replace(SO + ".tmp", SO)
    return SO


if __name__ == "__main__":
    print(build(), file=sys.stdout)
