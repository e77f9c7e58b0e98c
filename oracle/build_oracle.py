"""ORACLE build recipe (test infrastructure only).

Writes the oracle's C butterfly codelets and compiles them together with refstock.c into
oracle/_build/liboracle.so (git-ignored):

    python oracle/build_oracle.py

Radices 2, 4, 8 and 16 (both directions, untwiddled and twiddled) are lean-fftw's own
generated kernels, read from tests/golden/native_kernels.json (LeanFFTW/Native/Kernels.lean,
see native_dag.py) -- independent of the product's code generator.  lean-fftw publishes no
generated text for its other radices; their codelets come from the restated generator
(lean-fftw_gb300/lfg/codegen), whose DAGs are pinned by the reference's published constants,
operation counts and per-plan error bounds (tests/test_codegen_pins.py).

-ffp-contract=off keeps gcc from fusing a*b+c, so each generated operation is rounded
exactly as the reference kernel prescribes; fma() is called explicitly where the kernel
has a fused operation.  -march=native / -mcpu=native lets gcc vectorise for the host (the
timed CPU baseline); OpenMP gives the CPU baseline one transform per core.

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


# lean-fftw's own generated kernels cover these radices (LeanFFTW/Native/Kernels.lean)
NATIVE_RADICES = (2, 4, 8, 16)


def _write_if_changed(path: str, text: str) -> None:
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def build(force: bool = False) -> str:
    sys.path.insert(0, HERE)
    import native_dag  # noqa: E402
    sys.path.insert(0, os.path.join(ROOT, "lean-fftw_gb300"))
    from lfg.codegen.emit import c_codelets  # noqa: E402  (radices without published kernels)

    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "liboracle.so")
    src = os.path.join(HERE, "refstock.c")
    trig = os.path.join(HERE, "trig_ref.c")
    nat = os.path.join(BUILD, "codelets_native.c")
    cod = os.path.join(BUILD, "codelets_gen.c")
    _write_if_changed(nat, native_dag.c_source(native_dag.load()))
    # the generator's lookups are renamed: refstock.c asks the native kernels first
    gen = c_codelets([R for R in ORACLE_RADICES if R not in NATIVE_RADICES])
    gen = gen.replace("lfo_codelet_fn lfo_codelet(", "lfo_codelet_fn lfo_codelet_gen(")
    gen = gen.replace("lfo_pass_fn lfo_pass(", "lfo_pass_fn lfo_pass_gen(")
    _write_if_changed(cod, gen)
    if (not force and os.path.exists(so)
            and os.path.getmtime(so) >= max(os.path.getmtime(p) for p in (src, cod, nat, trig))):
        return so
    # -march/-mcpu=native: the host's vector units (x86 also gets hardware fma this way);
    # -ffp-contract=off still forbids fusing anything the kernels do not fuse
    if platform.machine() in ("x86_64", "AMD64"):
        arch = ["-march=native", "-mfma"]
    else:
        arch = ["-mcpu=native"]
    cmd = ["gcc", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=gnu11", *arch, "-o", so + ".tmp", src, trig, nat, cod, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(so + ".tmp", so)
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
