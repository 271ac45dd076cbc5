#!/usr/bin/env python
"""Throughput of the PIV window path on one GB300 (or N replicas).

Workload: one 4096 x 4096 uint16 image pair (12-bit particle images, seeded
synthetic data), 32 x 32 interrogation windows at step 8 (75 % overlap):
509 x 509 = 259,081 windows.  One step = one pass over the pair: every
window extracted, FFT cross-correlated (reference default "complex" mode,
FFT::cross_correlate), peak-searched, Gaussian-fitted, vector written.

  value  vectors/s with the frames already in HBM (device-buffer C ABI call,
         CUDA events on the launching stream); four resident copies of the
         pair (268 MB > 129 MB L2) are rotated so that no step reads frames
         another step left in L2;
  e2e    the same through the host-buffer C ABI call opiv_process_pair:
         pinned host frames in, vectors (and peak codes) back in host
         memory, host-to-device and device-to-host copies inside the timed
         region;
  roofline  the fused FP32 kernel: algorithmic FLOPs (2 complex 2-D FFTs of
         5 N log2 N each + 8 N, N = 32*32, per window) per launch over its
         CUDA-event duration, against the FP32 CUDA-core peak;
  cpu_baseline  the reference's CPU path (the compiled reference where this
         host has it, else the oracle's restatement) on the host cores.

`--impl reference` times the reference's own CPU implementation of the path
(thread pool over all host cores) on the same workload instead.
Multi-GPU: the path does not exchange data between windows; N ranks run N
independent replicas (one pair each), value is the sum.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "openpiv-cxx_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

IMG = 4096
IA = 32
STEP = 8
N_WIN = (1 + (IMG - IA) // STEP) ** 2
FLOP_PER_WINDOW = 2 * 5 * IA * IA * math.log2(IA * IA) + 8 * IA * IA   # 110,592
METRIC = "vectors/s"
WORKLOAD = f"piv_pair_{IMG}x{IMG}_u16_ia{IA}_step{STEP}"
L2_ROTATION = 4


def peaks_file():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the GPU is under load."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) == 9:
                    rows.append(parts)
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


def dist_setup(args=None):
    """Rank, world size and local rank from the torchrun environment; for
    N > 1 joins the process group (NCCL with GPUs, gloo without)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", init_method="env://")
        else:
            dist.init_process_group("gloo", init_method="env://")
    return rank, world, local


def dist_max(x: float, world: int) -> float:
    """Maximum of x over the ranks (the slowest replica's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def cpu_path(kind_pref: str = "ref"):
    """The fastest available CPU implementation of the path: the compiled
    reference if this host has it, else the oracle's restatement."""
    from oracle import oracle

    if kind_pref == "ref" and oracle.available("ref", fast=True):
        return oracle.get("ref", fast=True), "reference"
    if not oracle.available("port", fast=True):
        oracle.build(ref=False)
    return oracle.get("port", fast=True), "port"


def cpu_baseline(a, b, grid, budget_s: float = 15.0):
    impl, kind = cpu_path()
    threads = os.cpu_count() or 1
    fa, fb = a.astype(np.float64), b.astype(np.float64)
    # bounded sample: contiguous blocks of window rows, about budget_s of work
    _, _, t = impl.process_windows(fa, fb, grid[:2000], IA, 1, False, threads)
    rate = 2000 / max(t, 1e-6)
    n = int(min(len(grid), max(2000, rate * budget_s / 2)))
    done, secs = 0, 0.0
    while secs < budget_s * 0.5 and done < 4 * len(grid):
        _, _, t = impl.process_windows(fa, fb, grid[:n], IA, 1, False, threads)
        done += n
        secs += t
    return {"value": done / secs, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{done} windows ({n} per run, first rows of the {len(grid)}-window grid), "
                      f"complex mode, {threads} threads, {secs:.1f} s"}


def run_ours(args):
    import torch

    import opiv_gb300 as og
    from opiv_gb300 import synth

    rank, world, local = dist_setup(args)
    dev = local
    torch.cuda.set_device(dev)
    a, b = synth.config2(pair=rank)
    plan = og.Plan(IMG, IMG, np.uint16, IA, STEP, mode=og.CORR_COMPLEX, device=dev)
    assert plan.n == N_WIN
    plan.set_timing(True)
    stream = torch.cuda.Stream(device=dev)
    # resident copies of the pair at distinct addresses (defeats L2 reuse)
    frames = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)) for _ in range(L2_ROTATION)]
    dvec = torch.empty((plan.n, 5), dtype=torch.float32, device=dev)
    dpk = torch.empty(plan.n, dtype=torch.int32, device=dev)
    pitch = IMG * 2
    launches0 = og.kernel_launch_count()

    def step(k):
        fa, fb = frames[k % L2_ROTATION]
        plan.process_device(fa.data_ptr(), fb.data_ptr(), pitch, dvec.data_ptr(), dpk.data_ptr(),
                            stream.cuda_stream)

    sampler = ClockSampler(dev)
    sampler.start()
    for k in range(args.warmup):
        step(k)
    stream.synchronize()
    torch.cuda.synchronize()
    dist_barrier(world)
    torch.cuda.synchronize()
    launches_before = og.kernel_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    fp32_ms, exact_ms, exact_windows = [], [], 0
    ev0.record(stream)
    for k in range(args.steps):
        step(k)
        f, e = plan.last_timing()
        fp32_ms.append(f)
        exact_ms.append(e)
    ev1.record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    dist_barrier(world)
    elapsed = ev0.elapsed_time(ev1) / 1e3
    elapsed = dist_max(elapsed, world)
    gpu_launches = og.kernel_launch_count() - launches_before
    exact_windows = plan.exact_count()

    # ---- end to end through the host-buffer call (pinned host memory)
    ha = torch.from_numpy(a).pin_memory()
    hb = torch.from_numpy(b).pin_memory()
    hvec = torch.empty((plan.n, 5), dtype=torch.float32).pin_memory()
    hpk = torch.empty(plan.n, dtype=torch.int32).pin_memory()
    for _ in range(max(1, args.warmup)):
        plan.process_into(ha.data_ptr(), hb.data_ptr(), pitch, hvec.data_ptr(), hpk.data_ptr())
    dist_barrier(world)
    e2e_steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.process_into(ha.data_ptr(), hb.data_ptr(), pitch, hvec.data_ptr(), hpk.data_ptr())
    t_e2e = dist_max(time.perf_counter() - t0, world)
    dist_barrier(world)
    clocks = sampler.stop()

    # parity spot check of the timed output against the host call's output
    assert torch.equal(dvec.cpu(), hvec), "device and host calls disagree"

    if rank != 0:
        return
    peaks = peaks_file()
    fp32_s = statistics.mean(fp32_ms) / 1e3
    achieved = FLOP_PER_WINDOW * plan.n / fp32_s / 1e12
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    value = args.steps * plan.n * world / elapsed
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded particle images, 0.03 ppp, 12-bit)",
        "config": {"workload": WORKLOAD, "windows_per_step": plan.n, "ia": IA, "step": STEP,
                   "mode": "complex (FFT::cross_correlate)", "parallelism": f"replicas x{world}",
                   "l2": f"{L2_ROTATION} resident copies of the pair rotated per step "
                         f"({L2_ROTATION * 2 * IMG * IMG * 2 / 1e6:.0f} MB > 129 MB L2)",
                   "exact_pass_windows_last_step": exact_windows},
        "e2e": {"value": e2e_steps * plan.n * world / t_e2e, "unit": METRIC,
                "h2d_bytes_per_step": 2 * IMG * IMG * 2,
                "d2h_bytes_per_step": plan.n * (20 + 4)},
        "gpu_launches": gpu_launches,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": None,
                     "kernel": "piv_fp32_kernel<32,COMPLEX,u16>",
                     "kernel_ms": statistics.mean(fp32_ms),
                     "exact_pass_ms": statistics.mean(exact_ms),
                     "peak_source": f"152 SMs x 128 FP32 lanes x 2 x {sm_max:.0f} MHz "
                                    f"(sm_max_mhz of MEASURED_PEAKS.json)",
                     "hbm_gbs_achieved": (2 * IMG * IMG * 2 + plan.n * 24) / fp32_s / 1e9,
                     "hbm_gbs_peak": peaks.get("hbm_gbs")},
        "clocks": clocks,
    }
    if world == 1:
        grid = plan.grid()
        line["cpu_baseline"] = cpu_baseline(a, b, grid)
    print(json.dumps(line), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from opiv_gb300 import synth

    impl, kind = cpu_path()
    threads = os.cpu_count() or 1
    a, b = synth.config2()
    fa, fb = a.astype(np.float64), b.astype(np.float64)
    from oracle import oracle

    grid = oracle.get("port").grid_offsets(IMG, IMG, IA, IA, STEP, STEP)
    # size each step so that warmup + steps take about two minutes
    _, _, t = impl.process_windows(fa, fb, grid[:2000], IA, 1, False, threads)
    rate = 2000 / max(t, 1e-6)
    per_step = int(min(len(grid), max(1000, rate * 120.0 / max(1, args.steps + args.warmup))))
    for _ in range(args.warmup):
        impl.process_windows(fa, fb, grid[:per_step], IA, 1, False, threads)
    secs = 0.0
    for _ in range(args.steps):
        _, _, t = impl.process_windows(fa, fb, grid[:per_step], IA, 1, False, threads)
        secs += t
    value = args.steps * per_step / secs
    sample = (f"{per_step} of the {len(grid)} windows per step (first window rows), complex mode, "
              f"{threads} threads, thread pool of one task per window")
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded particle images, 0.03 ppp, 12-bit)", "impl": "reference",
        "config": {"workload": WORKLOAD, "windows_per_step": per_step, "ia": IA, "step": STEP,
                   "mode": "complex (FFT::cross_correlate)"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
