"""Build step of the package: generate the codelets and compile the native library.

    python -m lfg.build            (from lean-fftw_gb300/)

1. Runs the restated lean-fftw codelet generator (lfg.codegen) and writes
   csrc/generated/codelets_f64.cuh (device butterflies, one template specialisation per
   radix, direction and twiddling), csrc/generated/opcounts.h (operation counts used by
   the planner) and csrc/generated/wide_f64.h (lane-parallel schedules of the
   binary64 butterflies for the lone-transform cluster kernel).
2. Compiles csrc/*.cu for sm_103a (nvcc -gencode arch=compute_103a,code=sm_103a) and the
   host sources with g++, in parallel, and links lfg/liblfg.so.
3. Builds the libbench2-style command line lfg/lfg-bench (csrc/tools/lfg_bench.cpp) against
   liblfg.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # lean-fftw_gb300/
CSRC = os.path.join(ROOT, "csrc")
GEN = os.path.join(CSRC, "generated")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "liblfg.so")
REPO = os.path.dirname(ROOT)

GPU_RADICES = list(range(2, 17))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# sources compiled several times, once per -DLFG_PART value (large template instantiations
# split over translation units so they compile in parallel)
PARTS = {"ragged_f64.cu": 10}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _write_if_changed(path: str, text: str) -> None:
    if os.path.exists(path) and open(path).read() == text:
        return
    with open(path, "w") as f:
        f.write(text)


def generate() -> None:
    sys.path.insert(0, ROOT)
    from lfg.codegen.emit import cuda_codelets
    from lfg.codegen.kernel import butterfly_k

    os.makedirs(GEN, exist_ok=True)
    _write_if_changed(os.path.join(GEN, "codelets_f64.cuh"), cuda_codelets(GPU_RADICES, fp32=False))
    _write_if_changed(os.path.join(GEN, "codelets_f32.cuh"), cuda_codelets(GPU_RADICES, fp32=True))
    un = [0] * 17
    tw = [0] * 17
    for R in GPU_RADICES:
        un[R] = sum(butterfly_k(True, R, False).counts())
        tw[R] = sum(butterfly_k(True, R, True).counts())
    text = ("// Generated by lfg/build.py: operations of the radix-R codelets\n"
            "// (adds/subs/negs + muls + fused), from the restated lean-fftw generator.\n"
            "#pragma once\nnamespace lfg {\n"
            f"constexpr int kOpsUntw[17] = {{{', '.join(map(str, un))}}};\n"
            f"constexpr int kOpsTw[17] = {{{', '.join(map(str, tw))}}};\n"
            "}  // namespace lfg\n")
    _write_if_changed(os.path.join(GEN, "opcounts.h"), text)
    from lfg.codegen.wide import c_tables
    _write_if_changed(os.path.join(GEN, "wide_f64.h"), c_tables(GPU_RADICES))


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(p.encode())
        h.update(open(p, "rb").read())
    return h.hexdigest()[:16]


def compile_all(verbose: bool = False, jobs: int = 0) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(GEN, f) for f in sorted(os.listdir(GEN))]
    headers.append(os.path.join(REPO, "include", "lfg.h"))
    common = _digest(headers + [os.path.abspath(__file__)])
    inc = ["-I", CSRC, "-I", os.path.join(REPO, "include")]
    jobs_list = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        for part in range(PARTS.get(f, 0)) if f in PARTS else [None]:
            tag = "" if part is None else f".p{part}"
            obj = os.path.join(BUILD, f"{f}{tag}.{_digest([src])}.{common}.o")
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xptxas", "-v" if verbose else "-O3", *inc]
            if part is not None:
                cmd.append(f"-DLFG_PART={part}")
            cmd += ["-c", src, "-o", obj]
            jobs_list.append((obj, cmd))
            objs.append(obj)
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f"{f}.{_digest([src])}.{common}.o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", *inc, "-I",
               os.path.join(cuda_home(), "include"), "-c", src, "-o", obj]
        jobs_list.append((obj, cmd))
        objs.append(obj)

    def run(job):
        obj, cmd = job
        if os.path.exists(obj):
            return obj, ""
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    # longest compiles first, so the pool's tail is short
    jobs_list.sort(key=lambda j: 0 if any(k in j[0] for k in ("ragged_f64", "stockham")) else 1)
    with cf.ThreadPoolExecutor(max_workers=jobs or max(4, os.cpu_count() or 4)) as ex:
        for obj, log in ex.map(run, jobs_list):
            if verbose and log:
                print(log)
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


CLI = os.path.join(PKG, "lfg-bench")


def build_cli() -> str:
    src = os.path.join(CSRC, "tools", "lfg_bench.cpp")
    stamp = CLI + ".digest"
    d = _digest([src, LIB, os.path.join(REPO, "include", "lfg.h")])
    if os.path.exists(CLI) and os.path.exists(stamp) and open(stamp).read() == d:
        return CLI
    cuda = cuda_home()
    tmp = CLI + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(cuda, "include"), src, "-o", tmp, "-L", PKG, "-llfg",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath,$ORIGIN",
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    with open(stamp, "w") as f:
        f.write(d)
    return CLI


def build(verbose: bool = False) -> str:
    generate()
    lib = compile_all(verbose=verbose)
    build_cli()
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
