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

import concurrent.futures as cf
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
GEN_PARTS = 6     # the generator's codelets are compiled as this many parallel sources


def _write_if_changed(path: str, text: str) -> None:
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def build(force: bool = False) -> str:
    sys.path.insert(0, HERE)
    import native_dag  # noqa: E402
    sys.path.insert(0, os.path.join(ROOT, "lean-fftw_gb300"))
    # radices without published kernels: the restated generator's DAGs
    from lfg.codegen.kernel import butterfly_k  # noqa: E402
    from lfg.codegen.sexpr import cst_value  # noqa: E402

    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "liboracle.so")
    src = os.path.join(HERE, "refstock.c")
    trig = os.path.join(HERE, "trig_ref.c")
    nat = os.path.join(BUILD, "codelets_native.c")
    cods = [os.path.join(BUILD, f"codelets_gen{i}.c") for i in range(GEN_PARTS)]
    _write_if_changed(nat, native_dag.c_source(native_dag.load(), "lfo_native"))
    bits = lambda c: native_dag.bits_hex(cst_value(c))
    gen = {}
    for R in ORACLE_RADICES:
        if R in NATIVE_RADICES:
            continue
        for fwd in (True, False):
            for tw in (False, True):
                k = butterfly_k(fwd, R, tw)
                gen[native_dag.kernel_name(fwd, R, tw)] = native_dag.from_ops(
                    R, fwd, tw, k.n_in, k.ops, k.outs, bits)
    for path, text in zip(cods, native_dag.c_source(gen, "lfo_gen", parts=GEN_PARTS)):
        _write_if_changed(path, text)
    if (not force and os.path.exists(so)
            and os.path.getmtime(so) >= max(os.path.getmtime(p) for p in (src, nat, trig, *cods))):
        return so
    # -march/-mcpu=native: the host's vector units (x86 also gets hardware fma this way);
    # -ffp-contract=off still forbids fusing anything the kernels do not fuse
    if platform.machine() in ("x86_64", "AMD64"):
        arch = ["-march=native", "-mfma"]
    else:
        arch = ["-mcpu=native"]
    flags = ["gcc", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
             "-std=gnu11", *arch]
    srcs = (src, trig, nat, *cods)
    objs = [os.path.join(BUILD, os.path.basename(c) + ".o") for c in srcs]
    # the generated files are large: compile the sources in parallel
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        for r in ex.map(lambda co: subprocess.run([*flags, "-c", co[0], "-o", co[1]]),
                        zip(srcs, objs)):
            if r.returncode != 0:
                raise RuntimeError("oracle compile failed")
    subprocess.run([*flags, "-shared", "-o", so + ".tmp", *objs, "-lm"], check=True)
    os.replace(so + ".tmp", so)
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
