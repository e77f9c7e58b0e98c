"""Benchmark of the GB300 execute path (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

Workloads (synthetic inputs, re/im iid uniform[-0.5, 0.5) from numpy default_rng(20261016)):

  ragged     (default, the headline) 8192 1-D complex FP64 forward transforms, sizes drawn
             log-uniformly from [2, 16384] and snapped to the nearest 13-smooth integer in
             log distance (859 distinct sizes, sum 14,922,904 points), packed back to back
             in size order; one persistent launch replayed from a CUDA graph.  The same batch
             with one launch per distinct size is timed beside it, the launches in one chain
             (`per_size`) and spread over 64 independent graph branches so that different
             sizes run at the same time (`per_size_concurrent`).
  c2c_<N>    1-D complex FP64 forward, N = 2^k (k = 1..18), batch 2^26 / N (1 GiB in and
             out): the power-of-two sweep; also the small sizes N = 3, 5, 6, 7, 9 .. 15, 21,
             25, 27 (batch floor(2^26 / N)).
  small_1024 one transform of N = 1024 (the plain small case: latency-bound).
  large_262144[_f32]  32 transforms of N = 2^18, binary64 (or binary32: the FP32 variant with
             compensated last-pass twiddles).
  c2c_1024_f32  the binary32 variant at N = 1024, batch 2^17 (1 GiB in and out).
  r2c_512x512[_f32]  64 real 512 x 512 images to 64 x 512 x 257 half spectra (fused r2c
             rows, then the column transforms in place); GFLOP/s counts 2.5 N log2 N per image.
  grad_4096  differentiation: batch 256 x N = 4096, loss = sum |W * FFT(x)|^2 (W iid complex
             normal), one forward transform and one adjoint transform (the backward pass) per
             step through torch.autograd; GFLOP/s counts both transforms.

A step is one execution over the whole batch.  `value` is GFLOP/s with the conventional
5 N log2 N flops per transform, inputs resident in HBM; `e2e` is the same metric through
the C ABI's host-pointer entry points (lfg_execute_host / lfg_execute_ragged_host),
host-to-device and device-to-host copies inside the timed region.  The ragged batch moves
239 MB in and out per step and the sweep 2 GiB, both above the 129 MB L2, so no L2 flush
is needed between steps.

`--impl reference` times lean-fftw's reference algorithm on the host cores instead: the
oracle's C restatement of refTransform with the reference's codelets (the reference engine
itself, Lean 4 + AVX-512 assembly, cannot be built or run on this aarch64 host), all host
threads, one transform per thread, on a bounded sample of the same workload.

Multi-GPU: transforms are independent, so N ranks each run the full per-GPU batch with no
collective (weak scaling); the barrier and max-over-ranks timing follow torchrun's env.  With
--shard the ranks split one ragged batch instead (lfg.shard_ragged: cost-balanced, the same
split computed on every rank; strong scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lean-fftw_gb300"))

SEED = 20261016
WORKLOADS = {"ragged": dict(kind="ragged", count=8192, sign=-1)}
for _k in range(1, 19):
    WORKLOADS[f"c2c_{1 << _k}"] = dict(kind="c2c", n=1 << _k, batch=(1 << 26) >> _k, sign=-1)
# small sizes that are not powers of two (one butterfly, or two passes): 1 GiB in and out
for _n in (3, 5, 6, 7, 9, 10, 11, 12, 13, 14, 15, 21, 25, 27):
    WORKLOADS[f"c2c_{_n}"] = dict(kind="c2c", n=_n, batch=(1 << 26) // _n, sign=-1)
# the other configurations of the reference's measurement plan, each as its own line
WORKLOADS.update({
    "small_1024": dict(kind="c2c", n=1024, batch=1, sign=-1),           # latency-bound
    "large_262144": dict(kind="c2c", n=1 << 18, batch=32, sign=-1),
    "large_262144_f32": dict(kind="c2c", n=1 << 18, batch=32, sign=-1, precision="f32"),
    "c2c_1024_f32": dict(kind="c2c", n=1024, batch=1 << 17, sign=-1, precision="f32"),
    # differentiation: loss = sum |W * FFT(x)|^2, forward transform + adjoint per step
    "grad_4096": dict(kind="grad", n=4096, batch=256, sign=-1),
    # large images: 64 real 512 x 512 images to 64 x 512 x 257 half spectra
    "r2c_512x512": dict(kind="r2c2d", n0=512, n1=512, batch=64, sign=-1),
    "r2c_512x512_f32": dict(kind="r2c2d", n0=512, n1=512, batch=64, sign=-1, precision="f32"),
})


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def figures():
    """Figures measured outside the timed run (profiles/figures.json): the DFMA issue rate
    (`--workload fp64_peak`) and the ncu DRAM traffic of each workload's dominant kernel."""
    p = os.path.join(ROOT, "profiles", "figures.json")
    return json.load(open(p)) if os.path.exists(p) else {}


def fp64_peak():
    """DFMA issue rate of a GB300 in T instructions/s (the binding roofline of binary64)."""
    return figures().get("fp64_issue", {}).get("dfma_tinstr_per_s")


def traffic_key(args):
    """Key of a run in the traffic figures: the workload, with "_f32" for a binary32 run of a
    binary64 workload; None when --batch changes the size the figure was scaled to."""
    if args.batch > 0:
        return None
    key = args.workload
    if args.precision == "f32" and not key.endswith("_f32"):
        key += "_f32"
    return key


def ncu_traffic(workload):
    """DRAM bytes per launch of the dominant kernel, from its committed ncu capture."""
    t = figures().get("traffic", {}).get(workload)
    return float(t["bytes_per_launch"]) if t else None


# Issue-rate probe of the FP64 pipe: every warp runs 8 independent chains of one binary64
# instruction form over operands read from device memory (so the compiler cannot fold the
# fused forms back into an add or a multiply); 8 CTAs of 256 threads per SM.
FP64_PROBE_SRC = r"""
#include <cuda_runtime.h>
template <int OP>
__global__ void __launch_bounds__(256) chains(double* out, const double* p, int iters) {
  const double one = p[0], c = p[1], m = p[2], nz = p[3];
  double v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = (double)(threadIdx.x + i) * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (OP == 0) v[i] = __dadd_rn(v[i], c);
      if (OP == 1) v[i] = __fma_rn(v[i], one, c);
      if (OP == 2) v[i] = __fma_rn(v[i], m, c);
      if (OP == 3) v[i] = __dmul_rn(v[i], m);
      if (OP == 4) v[i] = __fma_rn(v[i], m, nz);
    }
  }
  double s = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += v[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
template <int OP>
static float time_op(double* out, const double* p, int grid, int iters) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  chains<OP><<<grid, 256>>>(out, p, iters);
  cudaEventRecord(a);
  for (int r = 0; r < 5; ++r) chains<OP><<<grid, 256>>>(out, p, iters);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / 5;
}
// rates[0..4]: T instr/s of DADD, DFMA(x,1,c), DFMA(x,m,c), DMUL, DFMA(x,m,-0)
extern "C" int lfg_fp64_probe(double* rates) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return -1;
  const int grid = sms * 8, iters = 4096;
  double *out = nullptr, *p = nullptr;
  if (cudaMalloc(&out, (size_t)grid * 256 * sizeof(double)) != cudaSuccess) return -1;
  if (cudaMalloc(&p, 4 * sizeof(double)) != cudaSuccess) return -1;
  const double h[4] = {1.0, 1e-9, 1.0000001, -0.0};
  cudaMemcpy(p, h, sizeof h, cudaMemcpyHostToDevice);
  const double ops = (double)grid * 256 * 8 * iters;
  const float t[5] = {time_op<0>(out, p, grid, iters), time_op<1>(out, p, grid, iters),
                      time_op<2>(out, p, grid, iters), time_op<3>(out, p, grid, iters),
                      time_op<4>(out, p, grid, iters)};
  for (int i = 0; i < 5; ++i) rates[i] = ops / (t[i] * 1e-3) / 1e12;
  cudaFree(out);
  cudaFree(p);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
"""


def run_fp64_peak(args):
    """`--workload fp64_peak`: the FP64 pipe's issue rates on this GPU (one JSON line)."""
    import ctypes
    import tempfile
    from lfg.build import ARCH, nvcc
    with tempfile.TemporaryDirectory() as d:
        src, so = os.path.join(d, "probe.cu"), os.path.join(d, "probe.so")
        open(src, "w").write(FP64_PROBE_SRC)
        subprocess.run([nvcc(), *ARCH, "-O3", "-shared", "-Xcompiler", "-fPIC", src, "-o", so],
                       check=True)
        lib = ctypes.CDLL(so)
        rates = (ctypes.c_double * 5)()
        with Clocks(0) as clk:
            rc = lib.lfg_fp64_probe(rates)
    if rc != 0:
        raise SystemExit("fp64_peak: the probe failed")
    names = ["dadd", "dfma_one", "dfma", "dmul", "dfma_nz"]
    line = {"metric": "FP64 issue rate (T instr/s)", "value": round(rates[2], 4),
            "unit": "T instr/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f64",
            "config": {"workload": "fp64_peak", "grid": "8 CTAs x 256 threads per SM",
                       "chains_per_thread": 8, "iterations": 4096},
            "rates": {k: round(v, 4) for k, v in zip(names, rates)}, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, dev: int):
        self.dev = dev
        self.p = None
        self.path = os.path.join("/tmp", f"lfg_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=clocks.sm,clocks.max.sm,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if not self.p or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def flops_per_transform(n):
    return 5.0 * n * math.log2(n)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value, device=None):
    """Max of a per-rank scalar over the process group (identity when not distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(rank):
    """Weak scaling: every rank transforms its own full per-GPU batch, seeded by rank; the
    transforms are independent, so no data moves between ranks."""
    return SEED + rank


def cpu_reference(wl, runs=10, budget_s=None):
    """Time the oracle's restatement of refTransform on all host threads (one transform per
    thread) on a bounded sample of the workload, by libbench2's protocol; returns a dict with
    GFLOP/s, threads, a description of the sample and the published engine's figures."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    threads = os.cpu_count() or 1
    if wl["kind"] == "ragged":
        sizes = ragged_workload_sizes(wl)
        plans = {int(n): reference_plan(int(n)) for n in set(sizes.tolist())}
        off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        runner = O.RaggedRef(wl["sign"] < 0, sizes, plans, off, off)
        x = O.uniform_complex((int(sizes.sum()),), seed=SEED)
        y = np.empty_like(x)
        call = lambda: runner.run(x, y, nthreads=threads)
        flops = float(sum(flops_per_transform(int(n)) for n in sizes))
        sample = f"the whole batch ({len(sizes)} transforms, {len(plans)} sizes) per timed call"
    elif wl["kind"] == "r2c2d":
        sizes = None
        # lean-fftw runs rdft2 in its generic engine (Core/Problem.lean:222-236): restated
        n0, n1 = wl["n0"], wl["n1"]
        count = min(wl["batch"], max(1, threads // 2))
        x = np.random.default_rng(SEED).random((count, n0, n1)) - 0.5
        call = lambda: O.generic_rank2_r2c(x, nthreads=threads)
        flops = 2.5 * n0 * n1 * math.log2(n0 * n1) * count
        sample = (f"{count} of the {wl['batch']} images ({n0}x{n1}, binary64) per timed call "
                  "through the generic engine's rdft2")
    else:
        sizes = None
        n = wl["n"]
        rs = reference_plan(n)
        count = max(threads, min(wl["batch"], threads * max(1, (1 << 15) // n)))
        x = O.uniform_complex((count, n), seed=SEED)
        call = lambda: O.ref_transform(wl["sign"] < 0, n, rs, x, nthreads=threads)
        flops = flops_per_transform(n) * count
        sample = f"{count} of the {wl['batch']} transforms of N={n} (plan {'x'.join(map(str, rs))}) per timed call"
    t, runs = libbench2_time(call, runs=runs, budget_s=budget_s)
    out = {"gflops": flops / t / 1e9, "threads": threads,
           "sample": sample + f"; libbench2 protocol: iterations doubled to >= 10 ms, best of 8, "
                              f"median of {runs} runs"}
    pub = published_engine(wl, sizes if wl["kind"] == "ragged" else None)
    if pub:
        out["published"] = pub
    return out


def libbench2_time(call, runs=10, budget_s=None):
    """Seconds per call by libbench2's protocol (lean-fftw docs/BENCHMARK_PROTOCOL.md:15-19,
    33-37): the iteration count doubles until one measurement takes at least 10 ms; a run is
    the best of 8 measurements; the result is the median of `runs` runs (fewer if `budget_s`
    of measuring is spent).  Returns (seconds per call, runs done)."""
    call()
    iters = 1
    while True:
        t0 = time.perf_counter()
        for _ in range(iters):
            call()
        if time.perf_counter() - t0 >= 0.01:
            break
        iters *= 2
    per_run, start = [], time.perf_counter()
    for _ in range(runs):
        best = math.inf
        for _ in range(8):
            t0 = time.perf_counter()
            for _ in range(iters):
                call()
            best = min(best, (time.perf_counter() - t0) / iters)
        per_run.append(best)
        if budget_s and time.perf_counter() - start > budget_s:
            break
    return statistics.median(per_run), len(per_run)


def published_engine(wl, sizes=None):
    """lean-fftw's published engine on one core (docs/RESULTS.md:72-89, i12 on Emerald Rapids,
    AVX-512; it cannot run on this host): GFLOP/s per core at N = 1024 and, for the workload,
    the single-core rate its per-size medians imply (log-linear interpolation in log2 N
    between the published power-of-two sizes; non-power-of-two sizes are an estimate)."""
    p = os.path.join(ROOT, "tests", "golden", "published_times.json")
    if not os.path.exists(p):
        return None
    tab = {int(k): v["i12_s"] for k, v in json.load(open(p))["times"].items()}
    ks = sorted(tab)
    rate = {n: flops_per_transform(n) / tab[n] / 1e9 for n in ks}

    def core_rate(n):
        if n <= ks[0]:
            return rate[ks[0]]
        if n >= ks[-1]:
            return rate[ks[-1]]
        hi = next(k for k in ks if k >= n)
        lo = ks[ks.index(hi) - 1]
        f = (math.log2(n) - math.log2(lo)) / (math.log2(hi) - math.log2(lo))
        return rate[lo] + f * (rate[hi] - rate[lo])

    out = {"engine": "lean-fftw i12, one Emerald Rapids core (AVX-512), published medians",
           "source": "docs/RESULTS.md:72-89", "core_gflops_n1024": round(rate[1024], 2)}
    if sizes is not None:
        t = sum(flops_per_transform(int(n)) / core_rate(int(n)) for n in sizes)
        out["core_gflops_workload_estimate"] = round(
            sum(flops_per_transform(int(n)) for n in sizes) / t, 2)
    elif wl.get("n"):
        out["core_gflops_workload_estimate"] = round(core_rate(wl["n"]), 2)
    return out


def ragged_workload_sizes(wl):
    """The benchmark's ragged sizes, in increasing order (so that the per-size strategy can
    run one batched launch per distinct size)."""
    import numpy as np
    from lfg.ragged import ragged_sizes
    return np.sort(ragged_sizes(wl["count"], SEED), kind="stable")


def reference_plan(n):
    """The reference's own plan where published (results/repro-2026-11-04/xcheck-bits.jsonl,
    committed as tests/golden/xcheck.json), else the planner's op-count rule."""
    p = os.path.join(ROOT, "tests", "golden", "xcheck.json")
    for d in json.load(open(p)):
        if d["N"] == n and max(d["plan"]) <= 64:
            return d["plan"]
    from lfg.codegen.plans import choose_radices
    return choose_radices(n)


METRIC = "FP64 c2c FFT GFLOP/s (5 N log2 N)"


def metric_name(wl):
    m = METRIC
    if wl["kind"] == "r2c2d":
        m = "FP64 r2c FFT GFLOP/s (2.5 N log2 N)"
    return m if wl.get("precision", "f64") == "f64" else m.replace("FP64", "FP32")


def workload_config(name, wl):
    if wl["kind"] == "ragged":
        return {"workload": name, "transforms": wl["count"], "sizes": "13-smooth in [2, 16384], "
                "log-uniform, seed 20261016", "sign": wl["sign"], "layout": "packed, size order"}
    if wl["kind"] == "r2c2d":
        return {"workload": name, "n0": wl["n0"], "n1": wl["n1"], "batch": wl["batch"],
                "sign": wl["sign"]}
    return {"workload": name, "n": wl["n"], "batch": wl["batch"], "sign": wl["sign"]}


def ragged_accuracy(sizes, host, out, count=64):
    """"At ref error" for the ragged batch: a sample of `count` transforms spread over the
    sizes (evenly in size order) against the double-double DFT, beside lean-fftw's reference
    transform of the same inputs (the oracle's refTransform, reference plans): aggregate
    relative L2 over the sample for both, their ratio, and the worst per-transform ratio."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    pick = np.unique(np.linspace(0, len(sizes) - 1, count).round().astype(np.int64))
    e_gpu = e_ref = den = 0.0
    worst = 0.0
    for i in pick:
        n, a = int(sizes[i]), int(off[i])
        x = np.ascontiguousarray(host[a:a + n])[None]
        hi, lo = O.dd_dft(True, x)
        norm2 = float(np.sum(np.abs(hi) ** 2))
        eg = O.rel_l2(np.ascontiguousarray(out[a:a + n]), (hi[0], lo[0]))
        er = O.rel_l2(O.ref_transform(True, n, reference_plan(n), x)[0], (hi[0], lo[0]))
        e_gpu += eg * eg * norm2
        e_ref += er * er * norm2
        den += norm2
        if er > 0:
            worst = max(worst, eg / er)
    l2, rl2 = math.sqrt(e_gpu / den), math.sqrt(e_ref / den)
    return {"sample": f"{len(pick)} transforms, evenly spaced in size order "
                      f"(N = {int(sizes[pick[0]])} .. {int(sizes[pick[-1]])})",
            "oracle": "double-double DFT", "l2_err": float(f"{l2:.4g}"),
            "ref_l2_err": float(f"{rl2:.4g}"), "ratio": round(l2 / rl2, 4),
            "worst_transform_ratio": round(worst, 4), "bar": 1.5}


def published_accuracy():
    """lean-fftw's published forward/backward relative L2 errors per power-of-two size
    (results/emr-i12/accuracy.txt, committed as tests/golden/accuracy_emr.json)."""
    p = os.path.join(ROOT, "tests", "golden", "accuracy_emr.json")
    return {int(k): v for k, v in json.load(open(p))["errors"].items()} if os.path.exists(p) else {}


def run_precision(args):
    """`--workload precision`: relative L2 error per size against the double-double DFT, for
    the binary64 path, the binary32 path (compensated last-pass twiddles from 2^16, and plain
    products), lean-fftw's reference transform (the oracle's refTransform with the reference's
    plans) and the reference's published errors: c2c N = 2^k (k = 1..18; 32 transforms of
    2^18, as in the large-N configuration) and 64 real 512 x 512 images (rdft2)."""
    import numpy as np
    import torch

    import lfg
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    torch.cuda.set_device(0)
    threads = os.cpu_count() or 1
    pub = published_accuracy()
    rows = []
    t0 = time.perf_counter()
    for k in range(1, 19):
        n = 1 << k
        B = 32 if k == 18 else max(1, min(64, (1 << 20) // n))
        x = O.uniform_complex((B, n), seed=SEED + k)
        x32 = x.astype(np.complex64)
        row = {"n": n, "batch": B}
        for fwd in (True, False):
            d = "fwd" if fwd else "bwd"
            ref = O.dd_dft(fwd, x, nthreads=threads)
            ref32 = O.dd_dft(fwd, x32.astype(np.complex128), nthreads=threads)
            plan = lfg.plan_1d(n, -1 if fwd else 1, B)
            y = plan.execute(torch.from_numpy(x).cuda()).cpu().numpy()
            row[f"f64_{d}"] = O.rel_l2(y, ref)
            r = O.ref_transform(fwd, n, reference_plan(n), x, nthreads=threads)
            row[f"ref_{d}"] = O.rel_l2(r, ref)
            for comp in ((True, False) if k >= 16 else (True,)):
                p32 = lfg.plan_1d(n, -1 if fwd else 1, B, precision="f32", compensated=comp)
                y32 = p32.execute(torch.from_numpy(x32).cuda()).cpu().numpy()
                row[f"f32_{d}" if comp else f"f32_plain_{d}"] = O.rel_l2(y32.astype(np.complex128), ref32)
            if n in pub:
                row[f"published_{d}"] = pub[n][f"{d}_l2"]
        row["ratio_f64_to_ref"] = max(row["f64_fwd"] / row["ref_fwd"] if row["ref_fwd"] else 1.0,
                                      row["f64_bwd"] / row["ref_bwd"] if row["ref_bwd"] else 1.0)
        rows.append({k2: (float(f"{v:.4g}") if isinstance(v, float) else v) for k2, v in row.items()})
    # rank-2 real: 64 images of 512 x 512 (the generic engine is the reference's rdft2 path)
    xi = np.random.default_rng(SEED).random((64, 512, 512)) - 0.5
    ref = O.dd_rank2_r2c(xi, nthreads=threads)
    img = {"shape": [512, 512], "batch": 64}
    for prec in ("f64", "f32"):
        xin = xi.astype(np.float32) if prec == "f32" else xi
        refp = ref if prec == "f64" else O.dd_rank2_r2c(xin.astype(np.float64), nthreads=threads)
        plan = lfg.plan_r2c_2d(512, 512, 64, precision=prec)
        yd = torch.empty((64, 512, 257), device="cuda",
                         dtype=torch.complex64 if prec == "f32" else torch.complex128)
        y = plan.execute(torch.from_numpy(np.ascontiguousarray(xin)).cuda(), yd).cpu().numpy()
        img[f"{prec}"] = float(f"{O.rel_l2(y.astype(np.complex128), refp):.4g}")
    img["ref_generic"] = float(f"{O.rel_l2(O.generic_rank2_r2c(xi, nthreads=threads), ref):.4g}")
    worst = max(r["ratio_f64_to_ref"] for r in rows)
    line = {"metric": "relative L2 error vs double-double DFT, binary64 / reference (worst size)",
            "value": round(worst, 4), "unit": "ratio", "n_gpus": 1, "higher_is_better": False,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "precision", "inputs": "re/im iid uniform[-0.5, 0.5), seed "
                       "20261016 + log2 N", "oracle": "double-double DFT",
                       "reference": "refTransform restated, reference plans"},
            "c2c": rows, "r2c_512x512": img,
            "wall_s": round(time.perf_counter() - t0, 1)}
    print(json.dumps(line), flush=True)


def run_reference(args, wl):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    cb = cpu_reference(wl, runs=max(1, min(args.steps, 10)), budget_s=60)
    gf, threads, sample = cb["gflops"], cb["threads"], cb["sample"]
    line = {"metric": metric_name(wl), "value": round(gf, 3),
            "unit": "GFLOP/s", "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.workload, wl),
            "cpu_baseline": {"value": round(gf, 3), "unit": "GFLOP/s", "cores": threads,
                             "kind": "port", "sample": sample,
                             "published": cb.get("published")},
            "e2e": {"value": round(gf, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


L2_BYTES = 129e6            # GB300 L2


def timed(step, steps, stream, local, barrier, flush=None):
    """K steps bracketed by a barrier and a synchronize, CUDA events on `stream`.

    With `flush` (workloads whose input fits in 1.5x L2), every step is preceded by a write
    of a buffer twice the L2 size and timed by its own pair of events, so each step starts
    from a cold L2 and the flush itself is not timed."""
    import torch
    barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        if flush is None:
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(steps):
                step()
            ev1.record(stream)
            torch.cuda.synchronize()
            total = ev0.elapsed_time(ev1)
        else:
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                   for _ in range(steps)]
            # a head start for the host: the device sleeps (untimed) while the host queues
            # the first steps, so no event pair ever waits for the host's next launch
            if hasattr(torch.cuda, "_sleep"):
                torch.cuda._sleep(int(min(steps, 4000) * 60000))
            for a, b in evs:
                flush()
                a.record(stream)
                step()
                b.record(stream)
            torch.cuda.synchronize()
            total = sum(a.elapsed_time(b) for a, b in evs)
    barrier()
    return total / steps, clk.summary()


def make_flush(dev):
    import torch
    buf = torch.empty(int(2 * L2_BYTES) // 4, dtype=torch.float32, device=dev)
    return lambda: buf.fill_(1.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)   # ~1 s timed: several clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="ragged",
                    choices=sorted(WORKLOADS) + ["fp64_peak", "precision"])
    ap.add_argument("--impl", default="lfg", choices=["lfg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shard", action="store_true",
                    help="ragged, N > 1: split the one batch over the ranks (lfg.shard_ragged, "
                         "cost-balanced) instead of a full batch per rank (strong scaling)")
    ap.add_argument("--untuned", action="store_true",
                    help="ragged: plan with the default schedule instead of autotuning it "
                         "(profiling runs, where the tuner's candidate launches would be captured)")
    ap.add_argument("--precision", choices=["f64", "f32"], default=None,
                    help="c2c workloads: compute in this precision (the sweep's binary32 leg); "
                         "binary32 batches double so each size still moves 1 GiB")
    ap.add_argument("--batch", type=int, default=0,
                    help="override the batch of a c2c workload (smaller cases for profiling)")
    args = ap.parse_args()
    if args.workload == "fp64_peak":
        return run_fp64_peak(args)
    if args.workload == "precision":
        return run_precision(args)
    wl = dict(WORKLOADS[args.workload])
    if args.precision and wl["kind"] == "c2c" and wl.get("precision", "f64") != args.precision:
        wl["precision"] = args.precision
        if args.precision == "f32" and args.workload.startswith("c2c_") and wl["batch"] > 1:
            wl["batch"] *= 2
    if args.batch > 0 and "batch" in wl:
        wl["batch"] = args.batch
    if args.impl == "reference":
        return run_reference(args, wl)

    import numpy as np
    import torch

    import lfg
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    stream = torch.cuda.current_stream()
    rng = np.random.default_rng(rank_seed(rank))
    extra = {}
    out_shape, out_dtype, alg_bytes_override = None, None, None
    job_flops = None      # whole-job flops per step when the ranks split one batch
    if wl["kind"] == "ragged":
        sizes = ragged_workload_sizes(wl)
        if args.shard and ws > 1:
            shard, _ = lfg.shard_ragged(sizes, ws)
            job_flops = float(sum(flops_per_transform(int(n)) for n in sizes))
            sizes = sizes[shard == rank]
            extra["shard"] = {"ranks": ws, "transforms_this_rank": int(sizes.size)}
        total = int(sizes.sum())
        t_plan = time.perf_counter()
        plan = lfg.plan_ragged(sizes, wl["sign"], measure=not args.untuned)   # autotuned
        t_plan = time.perf_counter() - t_plan
        per_size = lfg.plan_ragged(sizes, wl["sign"], per_size=True)
        per_size_conc = lfg.plan_ragged(sizes, wl["sign"], per_size=True, concurrent=True)
        rinfo = plan.info()
        host = (rng.random((total, 2)) - 0.5).view(np.complex128).reshape(total)
        flops_step = float(sum(flops_per_transform(int(n)) for n in sizes))
        points = total
        launches_per_step = int(rinfo.launches)
        codelet_ops = rinfo.flops
        step_fn = lambda: plan.execute(x, y)
        host_fn = lambda a, b: plan.execute_host(a, b)
        extra["config_extra"] = {"distinct_sizes": int(rinfo.classes), "points": total,
                                 "work_items": int(rinfo.items), "grid": int(rinfo.grid),
                                 "smem_bytes": int(rinfo.smem_bytes),
                                 "autotuned": {"block_shape": int(rinfo.block_shape),
                                               "tile": int(rinfo.tile_target),
                                               "single_group_max": int(rinfo.single_max),
                                               "planning_s": round(t_plan, 2)}}
    elif wl["kind"] == "r2c2d":
        n0, n1, B = wl["n0"], wl["n1"], wl["batch"]
        prec = wl.get("precision", "f64")
        rdt = np.float32 if prec == "f32" else np.float64
        plan = lfg.plan_r2c_2d(n0, n1, B, precision=prec)
        info = plan.info()
        host = (rng.random((B, n0, n1)) - 0.5).astype(rdt)
        out_shape = (B, n0, n1 // 2 + 1)
        out_dtype = torch.complex64 if prec == "f32" else torch.complex128
        flops_step = 2.5 * n0 * n1 * math.log2(n0 * n1) * B      # half a complex transform
        launches_per_step = 2                                      # rows (fused r2c), columns
        codelet_ops = info.flops
        step_fn = lambda: plan.execute(x, y)
        host_fn = lambda a, b: plan.execute_host(a, b)
        esz_r = 4 if prec == "f32" else 8
        alg_bytes_override = B * (n0 * n1 * esz_r + n0 * (n1 // 2 + 1) * 2 * esz_r)
        points = n0 * n1 * B
        extra["config_extra"] = {"images": B, "shape": [n0, n1], "radices": plan.radices}
    elif wl["kind"] == "grad":
        from lfg import torch_ops
        n, B = wl["n"], wl["batch"]
        host = (rng.random((B, n, 2)) - 0.5).view(np.complex128).reshape(B, n)
        W = torch.from_numpy((rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n)))).to(dev)
        flops_step = 2 * flops_per_transform(n) * B      # forward + adjoint
        points = 2 * n * B
        launches_per_step = 2
        fplan = lfg.plan_1d(n, -1, B)
        codelet_ops = 2 * fplan.info().flops

        def grad_step():
            xg = x.detach().requires_grad_(True)
            loss = torch.sum(torch.abs(W * torch_ops.fft(xg)) ** 2)
            loss.backward()
            return xg.grad

        step_fn = grad_step

        def host_fn(a, b):
            xg = torch.from_numpy(a).to(dev, non_blocking=True).requires_grad_(True)
            loss = torch.sum(torch.abs(W * torch_ops.fft(xg)) ** 2)
            loss.backward()
            torch.from_numpy(b).copy_(xg.grad)        # device -> pinned host, then synchronise

        extra["config_extra"] = {"loss": "sum |W * FFT(x)|^2", "radices": fplan.radices}
    else:
        n, B = wl["n"], wl["batch"]
        prec = wl.get("precision", "f64")
        plan = lfg.plan_1d(n, wl["sign"], B, precision=prec)
        info = plan.info()
        host = (rng.random((B, n, 2)) - 0.5).view(np.complex128).reshape(B, n)
        if prec == "f32":
            host = host.astype(np.complex64)
        flops_step = flops_per_transform(n) * B
        points = n * B
        launches_per_step = int(info.ngroups)
        codelet_ops = info.flops
        step_fn = lambda: plan.execute(x, y)
        host_fn = lambda a, b: plan.execute_host(a, b)
        extra["config_extra"] = {"radices": [info.radices[i] for i in range(info.npass)]}
    x = torch.from_numpy(host).to(dev)
    y = torch.empty(out_shape, dtype=out_dtype, device=dev) if out_shape else torch.empty_like(x)
    for _ in range(max(3, args.warmup)):
        step_fn()
    torch.cuda.synchronize()
    in_bytes = x.numel() * x.element_size()
    flush = make_flush(dev) if in_bytes < 1.5 * L2_BYTES else None

    # headline: device-resident inputs
    ms, clocks = timed(step_fn, args.steps, stream, local, barrier, flush)
    ms = max_over_ranks(ms, dev)
    scaling = "weak" if job_flops is None else "strong"
    if job_flops is None:
        job_flops = flops_step * ws
    value = job_flops / (ms * 1e-3) / 1e9

    if wl["kind"] == "ragged":
        # the comparison point: one launch per distinct size, in one chain (each size after
        # the previous one) and spread over 64 independent graph branches (sizes overlap; of 16, 32, 64 and
        # 128 branches, 64 measured fastest)
        for key, ps_plan in (("per_size", per_size), ("per_size_concurrent", per_size_conc)):
            y2 = torch.empty_like(x)
            ps_step = lambda: ps_plan.execute(x, y2)
            for _ in range(3):
                ps_step()
            ps_ms, _ = timed(ps_step, min(20, max(5, args.steps // 4)), stream, local, barrier)
            ps_ms = max_over_ranks(ps_ms, dev)
            torch.cuda.synchronize()
            extra[key] = {"value": round(job_flops / (ps_ms * 1e-3) / 1e9, 3),
                          "unit": "GFLOP/s", "ms_per_step": round(ps_ms, 4),
                          "launches_per_step": int(ps_plan.info().launches),
                          "speedup_of_persistent": round(ps_ms / ms, 3),
                          "same_bits": bool(torch.equal(y.view(torch.float64),
                                                        y2.view(torch.float64)))}
            del y2

    if wl["kind"] == "ragged" and rank == 0:
        extra["accuracy"] = ragged_accuracy(sizes, host, y.cpu().numpy())

    # roofline of the dominant kernel (one launch per step for ragged and single-group sizes)
    esz = 8.0 if wl.get("precision") == "f32" else 16.0
    alg_bytes = 2 * esz * points         # read + write of the data once
    if alg_bytes_override is not None:   # real input, half-spectrum output
        alg_bytes = float(alg_bytes_override)
    hbm_peak, peak_kind = peaks()
    kernel_ms = ms / launches_per_step
    achieved = alg_bytes / launches_per_step / (kernel_ms * 1e-3) / 1e9
    fp64p = fp64_peak()
    fp64_ach = codelet_ops / (ms * 1e-3) / 1e12

    # end to end through the C ABI's host-pointer entry point (pinned host buffers)
    hin = torch.from_numpy(host).pin_memory()
    hout = torch.empty(tuple(y.shape), dtype=y.dtype).pin_memory()
    hin_np, hout_np = hin.numpy(), hout.numpy()
    host_fn(hin_np, hout_np)
    e2e_steps = max(2, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_fn(hin_np, hout_np)
    t_e2e = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dev)
    e2e = job_flops / t_e2e / 1e9

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cb = cpu_reference(wl, runs=10, budget_s=20)
        cpu = {"value": round(cb["gflops"], 3), "unit": "GFLOP/s", "cores": cb["threads"],
               "kind": "port", "sample": cb["sample"], "published": cb.get("published")}

    if rank == 0:
        config = workload_config(args.workload, wl)
        config.update(extra.pop("config_extra"))
        config["l2_flush"] = ("inputs larger than L2 (129 MB)" if flush is None else
                              "L2 flushed before every timed step (258 MB write, not timed)")
        config["parallelism"] = f"replicas{ws}" if scaling == "weak" else f"shards{ws}"
        metric = metric_name(wl)
        line = {
            "metric": metric, "value": round(value, 3), "unit": "GFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": scaling, "vs_baseline": None,
            "dtype": wl.get("precision", "f64"),
            "data": "synthetic", "config": config,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                         "peak_kind": peak_kind, "traffic": ncu_traffic(traffic_key(args)),
                         "algorithmic_bytes_per_launch": alg_bytes / launches_per_step},
            "fp64_issue": None if wl.get("precision") == "f32" else
                          {"achieved": round(fp64_ach, 4), "unit": "T FP64 instr/s",
                           "peak": fp64p, "frac": round(fp64_ach / fp64p, 4) if fp64p else None,
                           "note": "codelet binary64 instructions per step / step time; peak = "
                                   "measured DFMA issue rate (every codelet operation is a DFMA)"},
            "e2e": {"value": round(e2e, 3), "unit": "GFLOP/s",
                    "h2d_bytes_per_step": int(hin.numel() * hin.element_size()),
                    "d2h_bytes_per_step": int(hout.numel() * hout.element_size())},
            "gpu_launches": int(launches_per_step * args.steps),
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
