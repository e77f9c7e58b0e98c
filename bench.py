"""Benchmark of the GB300 execute path (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

Workloads (synthetic inputs, re/im iid uniform[-0.5, 0.5) from numpy default_rng(20261016)):

  c2c_1024   1-D complex FP64 forward, N = 1024, batch 65536 (1 GiB in, 1 GiB out); the
             power-of-two sweep's shape at N = 1024 (batch = 2^26 / N).

A step is one execution of the plan over the whole batch.  `value` is GFLOP/s with the
conventional 5 N log2 N flops per transform, inputs resident in HBM; `e2e` is the same
metric through the C ABI's host-pointer entry point (lfg_execute_host), host-to-device and
device-to-host copies inside the timed region.  Inputs are larger than L2 (129 MB), so no
L2 flush is needed between steps.

`--impl reference` times lean-fftw's reference algorithm on the host cores instead: the
oracle's C restatement of refTransform with the reference's codelets (the reference engine
itself, Lean 4 + AVX-512 assembly, cannot be built or run on this aarch64 host), all host
threads, one transform per thread, on a bounded sample of the same workload.

Multi-GPU: transforms are independent, so N ranks each run the full per-GPU batch with no
collective (weak scaling); the barrier and max-over-ranks timing follow torchrun's env.
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
WORKLOADS = {
    "c2c_1024": dict(kind="c2c", n=1024, batch=65536, sign=-1),
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_peak():
    """DFMA issue rate measured on this machine's GB300 (profiles/fp64_issue_rate.md)."""
    p = os.path.join(ROOT, "profiles", "fp64_issue_rate.md")
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("dfma_tinstr_per_s:"):
                return float(line.split(":")[1])
    return None


def ncu_traffic(workload):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", f"stockham_f64_{workload}.md")
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    return None


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


def cpu_reference(wl, steps, warmup, sample_transforms=None, budget_s=None):
    """Time the oracle's restatement of refTransform on all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    threads = os.cpu_count() or 1
    n = wl["n"]
    rs = reference_plan(n)
    if sample_transforms is None:
        sample_transforms = max(threads, min(wl["batch"], threads * max(1, (1 << 14) // n)))
    x = O.uniform_complex((sample_transforms, n), seed=SEED)
    O.ref_transform(wl["sign"] < 0, n, rs, x[:threads], nthreads=threads)  # warm caches/tables
    times = []
    for _ in range(warmup):
        O.ref_transform(wl["sign"] < 0, n, rs, x, nthreads=threads)
    for _ in range(steps):
        t0 = time.perf_counter()
        O.ref_transform(wl["sign"] < 0, n, rs, x, nthreads=threads)
        times.append(time.perf_counter() - t0)
        if budget_s and sum(times) > budget_s:
            break
    t = statistics.median(times)
    gflops = flops_per_transform(n) * sample_transforms / t / 1e9
    return gflops, threads, f"{sample_transforms} transforms of N={n} (plan {'x'.join(map(str, rs))}) " \
                            f"per timed call, median of {len(times)}"


def reference_plan(n):
    """The reference's own plan where published (results/repro-2026-11-04/xcheck-bits.jsonl,
    committed as tests/golden/xcheck.json), else the planner's op-count rule."""
    p = os.path.join(ROOT, "tests", "golden", "xcheck.json")
    for d in json.load(open(p)):
        if d["N"] == n and max(d["plan"]) <= 64:
            return d["plan"]
    from lfg.codegen.plans import choose_radices
    return choose_radices(n)


def run_reference(args, wl):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    gf, threads, sample = cpu_reference(wl, max(1, args.steps), max(0, min(args.warmup, 2)),
                                        budget_s=60)
    line = {"metric": "FP64 c2c FFT GFLOP/s (5 N log2 N)", "value": round(gf, 3),
            "unit": "GFLOP/s", "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n": wl["n"], "batch": wl["batch"],
                       "sign": wl["sign"]},
            "cpu_baseline": {"value": round(gf, 3), "unit": "GFLOP/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(gf, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="c2c_1024", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="lfg", choices=["lfg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)

    import numpy as np
    import torch

    import lfg
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    n, B, sign = wl["n"], wl["batch"], wl["sign"]
    plan = lfg.plan_1d(n, sign, B)
    info = plan.info()
    rng = np.random.default_rng(SEED + rank)
    host = (rng.random((B, n, 2)) - 0.5).view(np.complex128).reshape(B, n)
    x = torch.from_numpy(host).to(dev)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()

    for _ in range(max(3, args.warmup)):
        plan.execute(x, y)
    torch.cuda.synchronize()

    # headline: K steps, device-resident inputs, CUDA events on the launching stream
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            plan.execute(x, y)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    total_flops = flops_per_transform(n) * B * ws
    value = total_flops / (ms * 1e-3) / 1e9

    # dominant kernel: per-launch duration of each group, events around each launch
    group_ms = []
    if info.ngroups == 1:
        group_ms = [ms]
    kernel_ms = ms / info.ngroups if info.ngroups > 1 else ms
    alg_bytes = 32.0 * n * B            # read + write of the data, one pass over HBM
    hbm_peak, peak_kind = peaks()
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9 if info.ngroups == 1 else \
        alg_bytes * info.ngroups / (ms * 1e-3) / 1e9
    traffic = ncu_traffic(args.workload)
    fp64p = fp64_peak()
    fp64_ach = info.flops / (ms * 1e-3) / 1e12

    # end to end through the C ABI's host-pointer entry point (pinned host buffers)
    hin = torch.from_numpy(host).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    hin_np, hout_np = hin.numpy(), hout.numpy()
    plan.execute_host(hin_np, hout_np)
    e2e_steps = max(2, min(args.steps, 5))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.execute_host(hin_np, hout_np)
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    if ws > 1:
        t = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    e2e = total_flops / t_e2e / 1e9

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        gf, threads, sample = cpu_reference(wl, 3, 1, budget_s=20)
        cpu = {"value": round(gf, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
               "sample": sample}

    if rank == 0:
        line = {
            "metric": "FP64 c2c FFT GFLOP/s (5 N log2 N)", "value": round(value, 3),
            "unit": "GFLOP/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "n": n, "batch": B, "sign": sign,
                       "radices": [info.radices[i] for i in range(info.npass)],
                       "l2_flush": "inputs (1 GiB) larger than L2", "parallelism": f"replicas{ws}"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                         "peak_kind": peak_kind,
                         "traffic": traffic},
            "fp64_issue": {"achieved": round(fp64_ach, 4), "unit": "T FP64 instr/s",
                           "peak": fp64p, "frac": round(fp64_ach / fp64p, 4) if fp64p else None,
                           "note": "codelet binary64 instructions per step / step time; peak = "
                                   "measured DFMA issue rate"},
            "e2e": {"value": round(e2e, 3), "unit": "GFLOP/s",
                    "h2d_bytes_per_step": int(hin.numel() * 16),
                    "d2h_bytes_per_step": int(hout.numel() * 16)},
            "gpu_launches": int(info.ngroups * args.steps),
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
