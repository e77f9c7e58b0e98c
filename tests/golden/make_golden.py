"""Regenerate the committed golden fixtures under tests/golden/.

    python tests/golden/make_golden.py --reference DIR     (or LEAN_FFTW_REFERENCE=DIR)

Two kinds of fixture:

1. Known answers published by lean-fftw (read from a checkout of the reference given by
   --reference or the LEAN_FFTW_REFERENCE variable; without one only the oracle vectors are
   rewritten).  They are copied verbatim or re-encoded as JSON, never re-derived:
     kernel_constants.txt  results/repro-2026-11-04/kernel-constants.txt (237 binary64
                           bit patterns of every codelet constant, radix <= 64)
     bounds.jsonl          results/repro-2026-11-04/bounds.jsonl (rounding depth a,
                           constant depth b and magnitude bound of 36 published plans)
     xcheck.json           results/repro-2026-11-04/xcheck-bits.jsonl (chosen plan and
                           relative L2 error against long-double FFTW, 36 sizes)
     opcounts.json         docs/ITERATIONS.md:227-230 and :285-287 (kernel op counts)
     accuracy_emr.json     results/emr-i12/accuracy.txt:1-36 (libbench2 --accuracy of the
                           published engine, power-of-two sizes: forward and backward
                           relative L1/L2/Linf errors against a multiple-precision FFT)
     published_times.json  docs/RESULTS.md:72-89 (median single-core time of the published
                           engine, i12, and of FFTW per power-of-two size, Emerald Rapids)
     native_kernels.json   LeanFFTW/Native/Kernels.lean:9-1897 (the sixteen generated
                           radix-2/4/8/16 butterflies, parsed by oracle/native_dag.py into
                           operation lists with their constant bits)
2. Input/output vectors of the CPU oracle (oracle/oracle.py, refTransform restated) on the
   reference tests' own LCG inputs (scripts/AsmTest.lean:7-13): oracle_vectors.npz.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (N, plan) pairs of the oracle vectors: pow-2 and 13-smooth sizes, every radix 2..16
VECTOR_CASES = [
    (2, [2]), (3, [3]), (5, [5]), (7, [7]), (11, [11]), (13, [13]), (14, [14]),
    (16, [4, 4]), (60, [4, 15]), (64, [8, 8]), (120, [10, 12]), (210, [15, 7, 2]),
    (1024, [16, 8, 8]), (1080, [6, 9, 4, 5]), (2048, [16, 16, 8]), (1001, [7, 11, 13]),
]


def copy_reference_pins(ref: str) -> None:
    rr = os.path.join(ref, "results", "repro-2026-11-04")
    shutil.copyfile(os.path.join(rr, "kernel-constants.txt"),
                    os.path.join(HERE, "kernel_constants.txt"))
    shutil.copyfile(os.path.join(rr, "bounds.jsonl"), os.path.join(HERE, "bounds.jsonl"))
    xs = []
    with open(os.path.join(rr, "xcheck-bits.jsonl")) as f:
        for line in f:
            d = json.loads(line)
            xs.append({"N": d["N"], "plan": [int(r) for r in d["lean_R"].split("x")],
                       "lean_l2": d["lean_l2"], "fftw_l2": d["fftw_l2"],
                       "bitexact_oop": d["lean_bitexact_oop"]})
    with open(os.path.join(HERE, "xcheck.json"), "w") as f:
        json.dump(xs, f, indent=0)
    # op counts quoted in docs/ITERATIONS.md
    it = open(os.path.join(ref, "docs", "ITERATIONS.md")).read()
    counts = {}
    for name, a, m, fu in re.findall(r"([nt]\d+)\s+\(\d+, \d+, \d+\)\s*→\s*\((\d+), (\d+), (\d+)\)", it):
        counts[name] = [int(a), int(m), int(fu)]
    m = re.search(r"Operations per untwiddled kernel.*?radix 3: \d+ → (\d+),\s*5: \d+ → (\d+), "
                  r"7: \d+ → (\d+), 11: \d+ → (\d+), 13: \d+ → (\d+), 6: \d+ → (\d+), "
                  r"10: \d+ → (\d+),\s*12: \d+ → (\d+), 15: \d+ → (\d+)", it, re.S)
    totals = dict(zip(["3", "5", "7", "11", "13", "6", "10", "12", "15"],
                      [int(v) for v in m.groups()]))
    m8 = re.search(r"R=8 (\d+) \(= \d+\)", it)
    with open(os.path.join(HERE, "opcounts.json"), "w") as f:
        json.dump({"split": counts, "untwiddled_totals": totals,
                   "twiddled8_total": int(m8.group(1)),
                   "source": "lean-fftw docs/ITERATIONS.md:61-62, 227-230, 285-287"}, f, indent=1)
    native_kernels(ref)
    published_times(ref)
    acc = {}
    for line in open(os.path.join(ref, "results", "emr-i12", "accuracy.txt")):
        d = json.loads(line)
        if d["impl"] == "lean-i12" and d["rc"] == 0:
            acc[str(d["n"])] = dict(zip(["fwd_l1", "fwd_l2", "fwd_linf", "bwd_l1", "bwd_l2",
                                         "bwd_linf"], d["err"]))
    with open(os.path.join(HERE, "accuracy_emr.json"), "w") as f:
        json.dump({"source": "lean-fftw results/emr-i12/accuracy.txt (impl lean-i12, "
                             "libbench2 --accuracy, problem ocfN)", "errors": acc}, f, indent=0)


def published_times(ref: str) -> None:
    unit = {"ns": 1e-9, "µs": 1e-6, "ms": 1e-3}
    rows = {}
    lines = open(os.path.join(ref, "docs", "RESULTS.md")).read().splitlines()
    start = next(i for i, l in enumerate(lines) if l.startswith("| N | FFTW best | mode | i11 | i12"))
    for i, line in enumerate(lines[start + 2:], start + 3):
        m = re.match(r"\| (\d+) \| ([\d.]+) (ns|µs|ms) \| \w+ \| ([\d.]+) (ns|µs|ms) \| "
                     r"([\d.]+) (ns|µs|ms) \|", line)
        if not m:
            break
        rows[m.group(1)] = {"fftw_s": float(m.group(2)) * unit[m.group(3)],
                            "i12_s": float(m.group(6)) * unit[m.group(7)], "line": i}
    with open(os.path.join(HERE, "published_times.json"), "w") as f:
        json.dump({"source": "lean-fftw docs/RESULTS.md (median of 10 runs, one core, "
                             "libbench2 protocol)", "times": rows}, f, indent=0)


def native_kernels(ref: str) -> None:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import native_dag
    text = open(os.path.join(ref, native_dag.SOURCE)).read()
    ks = native_dag.parse_lean(text)
    with open(native_dag.FIXTURE, "w") as f:
        f.write('{"source": "lean-fftw ' + native_dag.SOURCE + '",\n "kernels": {\n')
        rows = []
        for name in sorted(ks, key=lambda n: (ks[n]["R"], ks[n]["tw"], not ks[n]["fwd"])):
            rows.append(f'  "{name}": ' + json.dumps(ks[name], separators=(",", ":")))
        f.write(",\n".join(rows) + "\n}}\n")


def oracle_vectors() -> None:
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    arrays = {}
    for N, rs in VECTOR_CASES:
        x = O.lcg_rand(2 * N, N + 7).view(np.complex128)
        key = f"N{N}_" + "x".join(map(str, rs))
        arrays[key + "_in"] = x
        for fwd in (True, False):
            arrays[key + ("_fwd" if fwd else "_bwd")] = O.ref_transform(fwd, N, rs, x)
    np.savez_compressed(os.path.join(HERE, "oracle_vectors.npz"), **arrays)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("LEAN_FFTW_REFERENCE"),
                    help="checkout of lean-fftw (default: $LEAN_FFTW_REFERENCE)")
    a = ap.parse_args()
    if a.reference:
        if not os.path.isdir(a.reference):
            sys.exit(f"make_golden: {a.reference} is not a directory")
        copy_reference_pins(a.reference)
    else:
        print("make_golden: no reference checkout given; published pins left as they are")
    oracle_vectors()
    print("golden fixtures written to", HERE)
