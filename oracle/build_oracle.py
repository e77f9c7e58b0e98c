"""ORACLE build recipe (test infrastructure only).

Generates the C butterfly codelets of the restated lean-fftw generator and compiles them
together with refstock.c into oracle/_build/liboracle.so (git-ignored):

    python oracle/build_oracle.py

-ffp-contract=off keeps gcc from fusing a*b+c, so each generated operation is rounded
exactly as the reference kernel prescribes; fma() is called explicitly where the kernel
has a fused operation.  OpenMP gives the CPU baseline one transform per core.

The reference engine itself (Lean 4 + generated AVX-512 assembly) cannot be built here or
on an aarch64 host, so there is no oracle/_ref build; see the module docstring of
oracle.py.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")

# Radices for which C codelets are generated (every GPU radix and a few larger ones
# used by the reference's own published plans).
ORACLE_RADICES = [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 18, 20, 24, 25, 27, 32, 36, 64]


def build(force: bool = False) -> str:
    sys.path.insert(0, os.path.join(ROOT, "lean-fftw_gb300"))
    from lfg.codegen.emit import c_codelets  # noqa: E402

    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "liboracle.so")
    src = os.path.join(HERE, "refstock.c")
    trig = os.path.join(HERE, "trig_ref.c")
    cod = os.path.join(BUILD, "codelets_ref.c")
    text = c_codelets(ORACLE_RADICES)
    if not os.path.exists(cod) or open(cod).read() != text:
        with open(cod, "w") as f:
            f.write(text)
    if (not force and os.path.exists(so)
            and os.path.getmtime(so) >= max(os.path.getmtime(src), os.path.getmtime(cod),
                                        os.path.getmtime(trig))):
        return so
    # hardware fma for the explicit fma() calls (x86 needs -mfma; aarch64 always has it);
    # -ffp-contract=off still forbids fusing anything else
    arch = ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=gnu11", *arch, "-o", so + ".tmp", src, trig, cod, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(so + ".tmp", so)
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
