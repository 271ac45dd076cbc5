#!/usr/bin/env python
"""Throughput of the PIV window path on one GB300 (or N replicas).

Workload: one 4096 x 4096 uint16 image pair (12-bit particle images, seeded
synthetic data), 32 x 32 interrogation windows at step 8 (75 % overlap):
509 x 509 = 259,081 windows.  One step = one pass over the pair: every
window extracted, cross-correlated (reference default "complex" mode,
FFT::cross_correlate), peak-searched, Gaussian-fitted, vector written.

  value  vectors/s of the tensor-core split-BF16 path (DFT matrix products
         on tcgen05, hi*hi + hi*lo + lo*hi, FP32 accumulation) with the
         frames already in HBM (device-buffer C ABI call, CUDA events on the
         launching stream); four resident copies of the pair (268 MB >
         129 MB L2) are rotated so that no step reads frames another step
         left in L2;
  e2e    the same through the host-buffer C ABI call opiv_process_pair:
         pinned host frames in, vectors (and peak codes) back in host
         memory, host-to-device and device-to-host copies inside the timed
         region;
  roofline  the tensor-core kernel: executed MMA FLOPs per launch over its
         CUDA-event duration, against the measured BF16 tensor peak;
  plain_fp32  the plain FP32 FFT path (reference-exact integer peaks):
         vectors/s, e2e, and its kernel's algorithmic FLOPs (2 complex 2-D
         FFTs of 5 N log2 N each + 8 N, N = 32*32, per window) against the
         FP32 CUDA-core peak;
  accuracy_vs_fp64  RMS / max displacement error and peak-mismatch rate of
         each precision against the FP64 pass (every window through the
         exact kernel: the reference's arithmetic);
  cpu_baseline  the reference's CPU path (the compiled reference where this
         host has it, else the oracle's restatement) on the host cores.

`--impl reference` times the reference's own CPU implementation of the path
(thread pool over all host cores) on the same workload instead.
`--workload batch` times 48 pairs of mixed sizes through the 64/32/16 px
multi-pass schedule (CUDA-graph replay).
Multi-GPU: the path does not exchange data between windows; N ranks run N
independent replicas (one pair each), value is the sum.
"""
from __future__ import annotations

import argparse
import hashlib
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
# DRAM bytes (read + write) of one launch of the timed kernels on this
# workload, from an ncu capture (the bench cannot profile itself), with the
# SHA-256 prefixes of the kernel sources that capture ran: when a source no
# longer matches, the line reports no traffic instead of a stale figure
KERNEL_TRAFFIC = {
    "tc": {"bytes": 67_346_944 + 819_456,
           "sources": {"piv_tc_kernel.cuh": "52baeb2ef1e34e1b", "tc_ptx.cuh": "74cf252d23d6309a"}},
    "fp32": {"bytes": 67_165_440 + 4_344_832,
             "sources": {"piv_fp32.cuh": "916731b6afc83819", "fft_reg.cuh": "b328bf1c452ce151"}},
}


def kernel_traffic(kind):
    """(bytes, source note) of one launch of the tc or fp32 kernel, or
    (None, why) when its sources changed since the capture."""
    rec = KERNEL_TRAFFIC[kind]
    for name, digest in rec["sources"].items():
        with open(os.path.join(PKG, "csrc", name), "rb") as f:
            if hashlib.sha256(f.read()).hexdigest()[:16] != digest:
                return None, f"{name} changed since the ncu capture of its traffic"
    return rec["bytes"], "dram__bytes_read.sum + dram__bytes_write.sum of one launch, ncu capture of this workload"


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
    # the other legs, a shorter sample each: one thread, and the real mode
    # (FFT::cross_correlate_real) on all threads and on one
    legs = {"complex_all_threads": done / secs}
    for name, mode, nt in (("complex_1_thread", 1, 1), ("real_all_threads", 0, threads),
                           ("real_1_thread", 0, 1)):
        m = max(200, int(n * nt / threads) // 2)
        _, _, t = impl.process_windows(fa, fb, grid[:m], IA, mode, False, nt)
        legs[name] = m / max(t, 1e-9)
    return {"value": done / secs, "unit": METRIC, "cores": threads, "kind": kind,
            "sample": f"{done} windows ({n} per run, first rows of the {len(grid)}-window grid), "
                      f"complex mode, {threads} threads, {secs:.1f} s",
            "legs": legs}


# executed tensor-core FLOPs per 32 x 32 window of the DFT-GEMM kernel
# (vertical tiles of 4 windows): per tile and operand pass, 2 M N K FLOPs
# with K = 16 for stage 1 (two products of M x N = 128 x 32), stage 2 (four
# of 128 x 64), stage 3 (four of 64 x 64) and stage 4 (two of 128 x 32);
# split BF16 runs 3 passes (hi*hi, hi*lo, lo*hi)
TC_FLOP_PER_WINDOW_PASS = 2 * 16 * (2 * 128 * 32 + 4 * 128 * 64 + 4 * 64 * 64 + 2 * 128 * 32) / 4


def accuracy(vec, pk, ref_vec, ref_pk):
    """Displacement error against the FP64 pass: RMS and max of (u, v) over
    windows with the same integer peak, and the peak-mismatch rate."""
    mask = 0xFFFF
    a = np.where(pk >= 0, pk & mask, pk)
    r = np.where(ref_pk >= 0, ref_pk & mask, ref_pk)
    same = a == r
    d = (vec[:, 2:4] - ref_vec[:, 2:4])[same]
    ok = np.isfinite(d).all(1)
    d = d[ok]
    return {"rms_px": float(np.sqrt(np.mean(d ** 2))) if d.size else None,
            "max_px": float(np.abs(d).max()) if d.size else None,
            "peak_mismatch_rate": float(1.0 - same.mean()),
            "nan_mismatch": int((~ok).sum())}


def run_ours(args):
    import torch

    import opiv_gb300 as og
    from opiv_gb300 import synth

    rank, world, local = dist_setup(args)
    dev = local
    torch.cuda.set_device(dev)
    a, b = synth.config2(pair=rank)
    stream = torch.cuda.Stream(device=dev)
    # resident copies of the pair at distinct addresses (defeats L2 reuse)
    frames = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)) for _ in range(L2_ROTATION)]
    pitch = IMG * 2

    tiles = {}

    def make_plan(precision):
        plan = og.Plan(IMG, IMG, np.uint16, IA, STEP, mode=og.CORR_COMPLEX, device=dev)
        assert plan.n == N_WIN
        plan.set_precision(precision)
        # tensor-core plans: the autotuner times both tile shapes on the pair
        fa, fb = frames[0]
        tiles[precision] = plan.autotune(fa.data_ptr(), fb.data_ptr(), pitch, stream.cuda_stream)
        plan.set_timing(True)
        return plan

    def timed(precision, steps, warmup, n_plans=2):
        """Device-resident passes over the pair, `steps` of them, alternating
        two plans on two streams (a pass's exact re-decision, a few SMs,
        overlaps the next pass's main kernel), or one plan on one stream with
        n_plans = 1: (seconds over all ranks, main-kernel ms per step,
        exact-pass ms per step, launches, device outputs of the last step)."""
        plans = [make_plan(precision) for _ in range(n_plans)]
        streams = [stream, torch.cuda.Stream(device=dev)][:n_plans]
        outs = [(torch.empty((N_WIN, 5), dtype=torch.float32, device=dev),
                 torch.empty(N_WIN, dtype=torch.int32, device=dev)) for _ in plans]

        def step(k, i=None):
            i = k % n_plans if i is None else i
            fa, fb = frames[k % L2_ROTATION]
            plans[i].process_device(fa.data_ptr(), fb.data_ptr(), pitch, outs[i][0].data_ptr(),
                                    outs[i][1].data_ptr(), streams[i].cuda_stream)

        for k in range(warmup):
            step(k)
        torch.cuda.synchronize()
        dist_barrier(world)
        torch.cuda.synchronize()
        launches_before = og.kernel_launch_count()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev_side = torch.cuda.Event()
        ev0.record(streams[0])
        streams[-1].wait_event(ev0)
        for k in range(steps):      # back to back: no host synchronisation inside
            step(k)
        ev_side.record(streams[-1])
        streams[0].wait_event(ev_side)
        ev1.record(streams[0])
        torch.cuda.synchronize()
        dist_barrier(world)
        elapsed = dist_max(ev0.elapsed_time(ev1) / 1e3, world)
        launches = og.kernel_launch_count() - launches_before
        for p in plans:
            p.status()
        last = (steps - 1) % n_plans
        # kernel durations (the plan's events around its kernels) from a
        # separate loop on one plan that waits for each step
        main_ms, exact_ms = [], []
        for k in range(min(steps, 50)):
            step(k, last)
            f, e = plans[last].last_timing()
            main_ms.append(f)
            exact_ms.append(e)
        return elapsed, main_ms, exact_ms, launches, outs[last][0], outs[last][1], plans[last]

    sampler = ClockSampler(dev)
    sampler.start()
    # ---- the tensor-core split-BF16 path (headline) and the plain FP32 path
    tc_el, tc_ms, _, tc_launches, tc_vec, tc_pk, tc_plan = timed(og.PREC_TC_SPLIT_BF16, args.steps,
                                                                  args.warmup)
    fp_el, fp_ms, ex_ms, fp_launches, fp_vec, fp_pk, fp_plan = timed(og.PREC_FP32, args.steps,
                                                                     args.warmup)
    exact_windows = fp_plan.exact_count()
    # the same two paths with one plan on one stream (no overlap of
    # neighbouring passes): a shorter run
    n_single = max(3, args.steps // 2)
    tc1_el = timed(og.PREC_TC_SPLIT_BF16, n_single, args.warmup, n_plans=1)[0]
    fp1_el = timed(og.PREC_FP32, n_single, args.warmup, n_plans=1)[0]

    # ---- end to end through the host-buffer call (pinned host memory)
    ha = torch.from_numpy(a).pin_memory()
    hb = torch.from_numpy(b).pin_memory()

    outs = [(torch.empty((N_WIN, 5), dtype=torch.float32).pin_memory(),
             torch.empty(N_WIN, dtype=torch.int32).pin_memory()) for _ in range(2)]

    def e2e(plan):
        """Every step: the pair's frames up from pinned host memory, one pass,
        vectors and peak codes back, through the pipelined host call
        opiv_process_pairs (step i's copies overlap the passes of steps
        i - 1 and i + 1)."""
        def call(n):
            plan.process_pairs_into([ha.data_ptr()] * n, [hb.data_ptr()] * n, pitch,
                                    [outs[i % 2][0].data_ptr() for i in range(n)],
                                    [outs[i % 2][1].data_ptr() for i in range(n)])
        call(max(2, args.warmup))
        dist_barrier(world)
        n = max(1, args.steps)
        t0 = time.perf_counter()
        call(n)
        t = dist_max(time.perf_counter() - t0, world)
        dist_barrier(world)
        return n * N_WIN * world / t

    fp_e2e = e2e(fp_plan)
    assert torch.equal(fp_vec.cpu(), outs[0][0]), "device and host calls disagree (FP32 path)"
    tc_e2e = e2e(tc_plan)
    assert torch.equal(tc_vec.cpu(), outs[0][0]), "device and host calls disagree (tensor-core path)"
    clocks = sampler.stop()

    # ---- accuracy against the FP64 pass (the reference's arithmetic on every window)
    f64_plan = make_plan(og.PREC_FP64)
    f64_vec, f64_pk = f64_plan.process(a, b)
    acc = {"tc_split_bf16": accuracy(tc_vec.cpu().numpy(), tc_pk.cpu().numpy(), f64_vec, f64_pk),
           "fp32": accuracy(fp_vec.cpu().numpy(), fp_pk.cpu().numpy(), f64_vec, f64_pk)}
    # the other tensor-core precisions: throughput (a shorter run) and accuracy
    others = {}
    for name, prec in (("tc_bf16", og.PREC_TC_BF16), ("tc_split_fp16", og.PREC_TC_SPLIT_FP16),
                       ("tc_fp16", og.PREC_TC_FP16), ("tc_split2_fp16", og.PREC_TC_SPLIT2_FP16)):
        n_o = max(3, args.steps // 10)
        el, ms, _, _, v, k, _ = timed(prec, n_o, 3)
        others[name] = {"value": n_o * N_WIN * world / el, "kernel_ms": statistics.mean(ms)}
        acc[name] = accuracy(v.cpu().numpy(), k.cpu().numpy(), f64_vec, f64_pk)

    if rank != 0:
        return
    peaks = peaks_file()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    tc_s = statistics.mean(tc_ms) / 1e3
    fp_s = statistics.mean(fp_ms) / 1e3
    tc_flops = 3 * TC_FLOP_PER_WINDOW_PASS * N_WIN
    achieved = tc_flops / tc_s / 1e12
    value = args.steps * N_WIN * world / tc_el
    plain_value = args.steps * N_WIN * world / fp_el
    tc_traffic, fp_traffic = kernel_traffic("tc"), kernel_traffic("fp32")
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": tc_el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3",
        "data": "synthetic (seeded particle images, 0.03 ppp, 12-bit)",
        "config": {"workload": WORKLOAD, "windows_per_step": N_WIN, "ia": IA, "step": STEP,
                   "mode": "complex (FFT::cross_correlate)", "parallelism": f"replicas x{world}",
                   "path": "tensor-core DFT-GEMM, split BF16 (hi*hi + hi*lo + lo*hi), FP32 accumulate",
                   "tile": {og.TILE_VERTICAL: "4 windows stacked in a grid column",
                            og.TILE_HORIZONTAL: "4 windows side by side in a grid row"}.get(
                                tiles.get(og.PREC_TC_SPLIT_BF16), "n/a") + " (autotuned)",
                   "streams": "steps alternate between two plans on two streams "
                              "(one plan on one stream: single_stream_value)",
                   "l2": f"{L2_ROTATION} resident copies of the pair rotated per step "
                         f"({L2_ROTATION * 2 * IMG * IMG * 2 / 1e6:.0f} MB > 129 MB L2)"},
        "single_stream_value": n_single * N_WIN * world / tc1_el,
        "e2e": {"value": tc_e2e, "unit": METRIC, "h2d_bytes_per_step": 2 * IMG * IMG * 2,
                "d2h_bytes_per_step": N_WIN * (20 + 4),
                "call": "opiv_process_pairs (pinned host frames, copies overlapped with the passes)"},
        "gpu_launches": tc_launches,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": achieved / bf16_peak, "traffic": tc_traffic[0],
                     "traffic_source": f"{tc_traffic[1]}; algorithmic bytes {2 * IMG * IMG * 2 + N_WIN * 24}",
                     "kernel": "piv_tc_kernel<split,COMPLEX,u16>", "kernel_ms": statistics.mean(tc_ms),
                     "flop": "executed MMA FLOPs: 3 passes x (2 128x32 + 4 128x64 + 4 64x64 + 2 128x32 products, K=16) per 4 windows",
                     "peak_source": "bf16_tflops of MEASURED_PEAKS.json (cuBLAS burst, of measured)",
                     "hbm_gbs_achieved": (2 * IMG * IMG * 2 + N_WIN * 24) / tc_s / 1e9,
                     "hbm_gbs_peak": peaks.get("hbm_gbs")},
        "accuracy_vs_fp64": acc,
        "plain_fp32": {
            "value": plain_value, "e2e": fp_e2e, "gpu_launches": fp_launches,
            "ms_per_step": fp_el * 1e3 / args.steps,
            "tc_speedup": value / plain_value,
            "exact_pass_windows_last_step": exact_windows,
            "roofline": {"bound": "fp32", "achieved": FLOP_PER_WINDOW * N_WIN / fp_s / 1e12,
                         "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": FLOP_PER_WINDOW * N_WIN / fp_s / 1e12 / fp32_peak,
                         "traffic": fp_traffic[0], "traffic_source": fp_traffic[1],
                         "kernel": "piv_fp32_kernel<32,COMPLEX,u16>", "kernel_ms": statistics.mean(fp_ms),
                         "exact_pass_ms": statistics.mean(ex_ms),
                         "flop": "algorithmic: 2 x 5 N log2 N + 8 N, N = 1024, per window",
                         "peak_source": f"{n_sm} SMs x 128 FP32 lanes x 2 x {sm_max:.0f} MHz"},
            "single_stream_value": n_single * N_WIN * world / fp1_el},
        "other_precisions": others,
        "clocks": clocks,
    }
    if world == 1:
        grid = fp_plan.grid()
        line["cpu_baseline"] = cpu_baseline(a, b, grid)
        if not args.no_other_workloads:
            line["other_workloads"] = other_workloads(args)
    print(json.dumps(line), flush=True)


def other_workloads(args) -> dict:
    """Compact records of the other workloads, measured in the same run as
    the headline (one GPU): the 48-pair multi-pass batch (20 steps), the
    precision sweep on a 1024^2 crop of the config-2 field (base
    statistics, every window size and precision), and the adjoint with
    Monte Carlo over 200 noise seeds (the full workloads: --workload
    batch / sweep / adjoint)."""
    import argparse as ap

    t0 = time.perf_counter()
    b = batch_line(ap.Namespace(steps=20, warmup=3))
    t1 = time.perf_counter()
    sw = sweep_line(1024, variants=("base",))
    t2 = time.perf_counter()
    adj = adjoint_line(200)
    t3 = time.perf_counter()
    keep = ("variant", "ia", "precision", "windows", "kernel_ms", "rms_px", "max_px", "peak_mismatch_rate")
    return {
        "batch_48_pairs_64_32_16": {
            "metric": b["metric"], "value": b["value"], "ms_per_step": b["ms_per_step"],
            "e2e": b["e2e"]["value"], "e2e_call_ms_streams": b["e2e"]["call_ms_streams"],
            "schedules": {k: v for k, v in b["schedules"].items() if k != "autotune"},
            "gpu_launches_per_step": b["gpu_launches"] / b["steps"],
            "roofline_frac_fp32": b["roofline"]["frac"],
            "cpu_baseline": b.get("cpu_baseline", {}).get("value"), "seconds": t1 - t0},
        "precision_sweep_1024": {"rows": [{k: r[k] for k in keep} for r in sw["rows"]],
                                 "seconds": t2 - t1},
        "adjoint_2048_f32": {k: adj[k] for k in ("windows", "vjp_ms", "sigma_ms", "fd_check", "monte_carlo")}
        | {"seconds": t3 - t2},
    }


# ---- batched multi-pass workload ---------------------------------------------------
BATCH_PAIRS = 48
BATCH_PASSES = [(64, 32), (32, 16), (16, 8)]
BATCH_WORKLOAD = "piv_batch_48_pairs_u16_multipass_64_32_16_step_half"


def flop_per_window(ia: int) -> float:
    n = ia * ia
    return 2 * 5 * n * math.log2(n) + 8 * n


def _config3_pair(args):
    from opiv_gb300 import synth

    return synth.config3(*args)


def batch_frames(seed_offset: int = 0):
    """The 48 pairs of the batched workload, rendered in a spawned process
    pool (before any CUDA call of this process)."""
    import concurrent.futures as cf
    import multiprocessing as mp

    from opiv_gb300 import synth

    layout = synth.config3_layout(BATCH_PAIRS)
    jobs = [(seed_offset + i, size, off) for i, (size, off) in enumerate(layout)]
    workers = max(1, min(len(jobs), (os.cpu_count() or 2)))
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        frames = list(ex.map(_config3_pair, jobs))
    return [size for size, _ in layout], frames


def batch_cpu_rate(sizes, frames, budget_s: float = 15.0):
    """The CPU path's multi-pass chain (reference calls per window) over as
    many of the batch's pairs, smallest first, as fit in about budget_s."""
    from oracle import oracle

    impl, kind = cpu_path()
    threads = os.cpu_count() or 1
    order = sorted(range(len(sizes)), key=lambda i: sizes[i][0] * sizes[i][1])
    vectors, windows, secs, used = 0, 0, 0.0, 0
    for i in order:
        a, b = frames[i]
        t0 = time.perf_counter()
        out = oracle.multipass(impl, a, b, BATCH_PASSES, 1, False, threads)
        secs += time.perf_counter() - t0
        vectors += len(out[-1]["grid"])
        windows += sum(len(o["grid"]) for o in out)
        used += 1
        if secs > budget_s:
            break
    return {"value": vectors / secs, "unit": "vectors/s (final pass)", "cores": threads,
            "kind": kind, "windows_per_s": windows / secs,
            "sample": f"{used} pairs (smallest first), 3-pass chain, complex mode, "
                      f"{threads} threads, {secs:.1f} s"}


def run_batch(args):
    line = batch_line(args)
    if line is not None:
        print(json.dumps(line), flush=True)


def batch_line(args):
    """The batched multi-pass workload's JSON line (None on ranks > 0)."""
    rank, world, local = dist_setup(args)
    sizes, frames = batch_frames(seed_offset=BATCH_PAIRS * rank)
    import torch

    import opiv_gb300 as og

    dev = local
    torch.cuda.set_device(dev)
    batch = og.Batch(sizes, np.uint16, BATCH_PASSES, mode=og.CORR_COMPLEX, device=dev)
    for i, (a, b) in enumerate(frames):
        batch.upload(i, a, b)
    n_pass = len(BATCH_PASSES)
    win = [[batch.window_count(i, k) for k in range(n_pass)] for i in range(len(sizes))]
    final = sum(w[-1] for w in win)
    total = sum(sum(w) for w in win)
    flops = sum(flop_per_window(BATCH_PASSES[k][0]) * w[k] for w in win for k in range(n_pass))
    stream = torch.cuda.Stream(device=dev)
    h = stream.cuda_stream

    def timed(use_graph: bool, steps: int) -> float:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        dist_barrier(world)
        ev0.record(stream)
        for _ in range(steps):
            batch.run(use_graph=use_graph, stream=h)
        ev1.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        dist_barrier(world)
        return dist_max(ev0.elapsed_time(ev1) / 1e3, world)

    sampler = ClockSampler(dev)
    sampler.start()
    # streams schedule: every pair's pass chain on 8 fork streams
    for _ in range(args.warmup):
        batch.run(use_graph=False, stream=h)
    eager = timed(False, args.steps)
    for _ in range(args.warmup):
        batch.run(use_graph=True, stream=h)
    launches_before = og.kernel_launch_count()
    graph_streams = timed(True, args.steps)
    launches_streams = og.kernel_launch_count() - launches_before
    # queue schedule: per pass one persistent kernel over a device work queue
    # of all pairs' windows; untuned (resident grid, chunk 1), then autotuned
    batch.set_schedule(og.BATCH_QUEUE)
    for _ in range(args.warmup):
        batch.run(use_graph=True, stream=h)
    graph_queue0 = timed(True, args.steps)
    t_tune = time.perf_counter()
    batch.autotune(stream=h)
    t_tune = time.perf_counter() - t_tune
    tuning = [batch.tuning(k) for k in range(n_pass)]
    lanes = batch.lanes()
    for _ in range(args.warmup):
        batch.run(use_graph=True, stream=h)
    launches_before = og.kernel_launch_count()
    graph_queue = timed(True, args.steps)
    launches_queue = og.kernel_launch_count() - launches_before
    # windows the exact FP64 pass re-decided, per pass (peak codes' flag bit)
    exact_per_pass = [int(sum(np.count_nonzero(batch.results(i, k)[1] & og.PEAK_EXACT)
                              for i in range(len(sizes)))) for k in range(n_pass)]
    use_queue = graph_queue <= graph_streams
    graph = graph_queue if use_queue else graph_streams
    gpu_launches = launches_queue if use_queue else launches_streams

    # end to end: pinned host frames in, every pair's final-pass vectors out
    pinned = [(torch.from_numpy(a).pin_memory(), torch.from_numpy(b).pin_memory())
              for a, b in frames]
    h2d = sum(2 * a.numel() * 2 for a, _ in pinned)
    last = n_pass - 1
    outs = [(torch.empty((win[i][last], 5), dtype=torch.float32).pin_memory(),
             torch.empty(win[i][last], dtype=torch.int32).pin_memory()) for i in range(len(sizes))]
    d2h = sum(w[last] * 24 for w in win)

    ptrs = ([a.data_ptr() for a, _ in pinned], [b.data_ptr() for _, b in pinned],
            [a.shape[1] * 2 for a, _ in pinned], [v.data_ptr() for v, _ in outs],
            [p.data_ptr() for _, p in outs])

    def e2e_step():
        # opiv_batch_process: pair i's passes start once its frames are up,
        # its vectors come back once its last pass ends
        batch.process_into(*ptrs)

    e2e_steps = max(5, args.steps // 4)
    call_ms = {}

    def e2e_time(schedule):
        batch.set_schedule(schedule)
        if schedule == og.BATCH_QUEUE:
            batch.run(use_graph=True, stream=h)   # records the queue graph the call replays
            stream.synchronize()
        e2e_step()
        dist_barrier(world)
        t0 = time.perf_counter()
        per = []
        for _ in range(e2e_steps):
            t1 = time.perf_counter()
            e2e_step()
            per.append((time.perf_counter() - t1) * 1e3)
        call_ms[schedule] = per
        return dist_max(time.perf_counter() - t0, world)

    # the host-to-device bandwidth of these pinned frames, one stream, timed
    # on the device (the upload is most of an end-to-end call's copies)
    dev_frames = [(torch.empty_like(a, device=dev), torch.empty_like(b, device=dev)) for a, b in pinned]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for rep in range(2):
            ev0.record(stream)
            for (da, db), (a, b) in zip(dev_frames, pinned):
                da.copy_(a, non_blocking=True)
                db.copy_(b, non_blocking=True)
            ev1.record(stream)
    stream.synchronize()
    h2d_gbs = h2d / (ev0.elapsed_time(ev1) / 1e3) / 1e9
    del dev_frames

    t_e2e_streams = e2e_time(og.BATCH_STREAMS)
    t_e2e_queue = e2e_time(og.BATCH_QUEUE)
    t_e2e = min(t_e2e_streams, t_e2e_queue)
    clocks = sampler.stop()
    batch.close()
    if rank != 0:
        return None
    peaks = peaks_file()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12
    achieved = flops * args.steps / graph / 1e12
    line = {
        "metric": "vectors/s (final pass)", "value": args.steps * final * world / graph,
        "unit": "vectors/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": graph * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded particle images, 0.03 ppp, 12-bit, Lamb-Oseen vortex)",
        "config": {"workload": BATCH_WORKLOAD, "pairs": len(sizes),
                   "sizes": {f"{w}x{h}": sizes.count((w, h)) for w, h in sorted(set(sizes))},
                   "passes": BATCH_PASSES, "final_vectors_per_step": final,
                   "windows_per_step_all_passes": total, "mode": "complex",
                   "submission": ("CUDA graph of the queue schedule: per pass one persistent FP32 "
                                  "kernel over a device work queue of all pairs' windows + one exact "
                                  "launch, autotuned grid and chunk" if use_queue else
                                  "CUDA graph of all pairs' passes on 8 forked streams"),
                   "l2": f"{sum(2 * w * h * 2 for w, h in sizes) / 1e9:.2f} GB of frames per "
                         f"step (> 129 MB L2)",
                   "parallelism": f"replicas x{world}"},
        "windows_per_s_all_passes": args.steps * total * world / graph,
        "eager_value": args.steps * final * world / eager,
        "schedules": {
            "streams_graph": args.steps * final * world / graph_streams,
            "streams_eager": args.steps * final * world / eager,
            "queue_graph_untuned": args.steps * final * world / graph_queue0,
            "queue_graph_autotuned": args.steps * final * world / graph_queue,
            "launches_per_step": {"streams": launches_streams / args.steps,
                                  "queue": launches_queue / args.steps},
            "exact_windows_per_pass": exact_per_pass,
            "autotune": {"seconds": t_tune, "lanes": lanes,
                         "per_pass": [{"ia": BATCH_PASSES[k][0], "ctas_per_sm": c, "chunk": ch,
                                       "resident_limit": mx, "pass_ms": ms}
                                      for k, (c, ch, mx, ms) in enumerate(tuning)]},
        },
        "e2e": {"value": e2e_steps * final * world / t_e2e, "unit": "vectors/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "call": ("opiv_batch_process, streams schedule (pinned host frames; per-pair "
                         "uploads, pass chains and downloads overlapped)"
                         if t_e2e_streams <= t_e2e_queue else
                         "opiv_batch_process, queue schedule (all uploads, the queue graph, "
                         "all downloads)"),
                "streams": e2e_steps * final * world / t_e2e_streams,
                "queue": e2e_steps * final * world / t_e2e_queue,
                "call_ms_streams": [round(x, 2) for x in call_ms[og.BATCH_STREAMS]],
                "call_ms_queue": [round(x, 2) for x in call_ms[og.BATCH_QUEUE]],
                "pinned_h2d_gbs": h2d_gbs},
        "gpu_launches": gpu_launches,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": None,
                     "kernel": "whole step (all FP32 and exact launches of the graph)"},
        "clocks": clocks,
    }
    if world == 1:
        line["cpu_baseline"] = batch_cpu_rate(sizes, frames)
    return line


# ---- precision sweep -----------------------------------------------------------
def fp64_numpy_pass(a, b, grid, ia, img_h, chunk=2048):
    """Vectors and peak codes of the reference's chain on numpy FP64
    correlation planes, for window sizes the FP64 GPU pass does not take
    (48 px: not a power of two).  Complex mode: IFFT(FFT(b) conj FFT(a)),
    unnormalised, quadrant-swapped (fft.h:188-206); find_peaks(plane, 2, 1):
    strict 4-neighbour maxima over rows [1, W-2), columns [1, W-1), the two
    largest (ties: lower row-major index) (image_utils.impl.h:42-74); the
    3-point Gaussian fit (impl:77-101); the vector of main.cpp:220-236."""
    n = len(grid)
    vec = np.zeros((n, 5), np.float64)
    pk = np.full(n, -1, np.int64)
    for s0 in range(0, n, chunk):
        g = grid[s0:s0 + chunk]
        wa = np.stack([a[y:y + ia, x:x + ia] for x, y in g]).astype(np.float64)
        wb = np.stack([b[y:y + ia, x:x + ia] for x, y in g]).astype(np.float64)
        r = np.fft.ifft2(np.fft.fft2(wb) * np.conj(np.fft.fft2(wa))).real * (ia * ia)
        pl = np.fft.fftshift(r, axes=(1, 2))
        c = pl[:, 1:ia - 2, 1:ia - 1]
        strict = ((c > pl[:, 0:ia - 3, 1:ia - 1]) & (c > pl[:, 2:ia - 1, 1:ia - 1]) &
                  (c > pl[:, 1:ia - 2, 0:ia - 2]) & (c > pl[:, 1:ia - 2, 2:ia]))
        cand = np.where(strict, c, -np.inf).reshape(len(g), -1)
        order = np.argsort(-cand, axis=1, kind="stable")[:, :2]
        v0 = np.take_along_axis(cand, order[:, :1], 1)[:, 0]
        v1 = np.take_along_axis(cand, order[:, 1:2], 1)[:, 0]
        ok = np.isfinite(v1)
        cw = ia - 2
        py, px = order[:, 0] // cw + 1, order[:, 0] % cw + 1
        idx = np.arange(len(g))
        C, L, R = pl[idx, py, px], pl[idx, py, px - 1], pl[idx, py, px + 1]
        U, D = pl[idx, py - 1, px], pl[idx, py + 1, px]
        with np.errstate(all="ignore"):
            fx = np.where((L > 0) & (C > 0) & (R > 0),
                          (np.log(L) - np.log(R)) / (2 * (np.log(L) + np.log(R) - 2 * np.log(C))), np.nan)
            fy = np.where((U > 0) & (C > 0) & (D > 0),
                          (np.log(U) - np.log(D)) / (2 * (np.log(U) + np.log(D) - 2 * np.log(C))), np.nan)
            sn = np.where(v1 > 0, v0 / v1, 0.0)
        out = np.stack([g[:, 0] + ia // 2, img_h - (g[:, 1] + ia // 2), ia // 2 - px - fx,
                        ia // 2 - py - fy, sn], axis=1)
        vec[s0:s0 + chunk] = np.where(ok[:, None], out, 0.0)
        pk[s0:s0 + chunk] = np.where(ok, py * ia + px, -1)
    return vec, pk


def run_sweep(args):
    sizes = tuple(int(w) for w in args.sweep_windows.split(","))
    variants = tuple(args.sweep_variants.split(","))
    print(json.dumps(sweep_line(args.sweep_size, variants=variants, sizes=sizes)), flush=True)


def sweep_line(size, variants=("base", "sparse", "noisy"), sizes=(16, 32, 48, 64)):
    """Displacement error of every precision against the FP64 reference on
    the config-2 field: windows 16 / 32 / 48 / 64 px at 75 % overlap, at
    config-2 statistics, low seeding (0.005 ppp) and high noise (sigma 80).
    The FP64 reference is the FP64 GPU pass for powers of two and numpy
    FP64 planes through the reference's peak search and fit for 48 px, which
    the reference's FFT rejects (fft.h:76-84): no FP32-FFT row there."""
    import torch

    import opiv_gb300 as og
    from opiv_gb300 import synth

    torch.cuda.set_device(0)
    precisions = [("fp32", og.PREC_FP32), ("tc_split_bf16", og.PREC_TC_SPLIT_BF16),
                  ("tc_bf16", og.PREC_TC_BF16), ("tc_split_fp16", og.PREC_TC_SPLIT_FP16),
                  ("tc_fp16", og.PREC_TC_FP16), ("tc_split2_fp16", og.PREC_TC_SPLIT2_FP16)]
    rows = []
    for variant in variants:
        a, b = synth.config4(variant, size)
        for ia in sizes:
            step = ia // 4

            def plan(prec):
                if ia == 48:
                    return og.Plan(size, size, np.uint16, ia, step, mode=og.CORR_COMPLEX, tensor_core=prec)
                p = og.Plan(size, size, np.uint16, ia, step, mode=og.CORR_COMPLEX)
                p.set_precision(prec)
                return p

            if ia == 48:
                ref_vec, ref_pk = fp64_numpy_pass(a, b, og.grid_offsets(size, size, ia, ia, step, step),
                                                  ia, size)
            else:
                ref_vec, ref_pk = plan(og.PREC_FP64).process(a, b)
            for name, prec in precisions:
                if prec == og.PREC_FP32 and ia == 48:
                    continue   # the FFT path takes powers of 2
                p = plan(prec)
                vec, pk = p.process(a, b)
                p.set_timing(True)
                for _ in range(3):
                    vec, pk = p.process(a, b)
                ms, _ = p.last_timing()
                rows.append({"variant": variant, "ia": ia, "step": step, "precision": name,
                             "windows": p.n, "kernel_ms": ms,
                             **accuracy(vec, pk, ref_vec, ref_pk)})
    return {"metric": "precision sweep vs FP64 reference", "size": size,
            "data": "synthetic config-2 field (seeded particle images, 12-bit)", "rows": rows}


# ---- adjoint and uncertainty ------------------------------------------------------
def run_adjoint(args):
    print(json.dumps(adjoint_line(args.mc_seeds)), flush=True)


def adjoint_line(mc_seeds):
    """The config-5 workload: a 2048^2 float32 pair (0.02 ppp, shift (0.40,
    0.25), noise sigma 0.02), 32 px windows at step 16 (16,129 windows).
    The adjoint of every vector against FP64 central differences through
    the oracle (h = 1e-3, 256 sampled windows, the 4 pixels with the
    largest adjoint entries of frame A each), and the propagated sigma_u,
    sigma_v against Monte Carlo over 1000 noise seeds."""
    import torch

    import opiv_gb300 as og
    from opiv_gb300 import synth
    from oracle import oracle

    torch.cuda.set_device(0)
    size, ia, step, sig = 2048, 32, 16, 0.02
    a, b = synth.config5(size=size)
    plan = og.Plan(size, size, np.float32, ia, step)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    pitch = size * 4
    vec = torch.empty((plan.n, 5), dtype=torch.float32, device="cuda")
    pk = torch.empty(plan.n, dtype=torch.int32, device="cuda")
    plan.process_device(da.data_ptr(), db.data_ptr(), pitch, vec.data_ptr(), pk.data_ptr(), 0)
    torch.cuda.synchronize()
    grid = plan.grid()
    pkn = pk.cpu().numpy()
    rng = np.random.default_rng(5)
    nx = len(np.unique(grid[:, 0]))
    # 256 windows on a lattice of every 4th window: no two share a pixel
    lattice = np.arange(plan.n).reshape(-1, nx)[::4, ::4].ravel()
    lattice = lattice[pkn[lattice] >= 0]
    sample = np.sort(rng.choice(lattice, size=min(256, len(lattice)), replace=False))
    cot = torch.zeros((plan.n, 2), dtype=torch.float32, device="cuda")
    cot[torch.from_numpy(sample).cuda(), 0] = 1.0
    ga = torch.zeros_like(da)
    gb = torch.zeros_like(db)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    plan.adjoint_device(da.data_ptr(), db.data_ptr(), pitch, pk.data_ptr(), cot.data_ptr(),
                        ga.data_ptr(), gb.data_ptr(), pitch)
    ev1.record()
    torch.cuda.synchronize()
    vjp_ms = ev0.elapsed_time(ev1)
    gan = ga.cpu().numpy()
    orc = oracle.get("port")
    h, errs = 1e-3, []
    for w in sample:
        x, y = grid[w]
        wa = a[y:y + ia, x:x + ia].astype(np.float64)
        wb = b[y:y + ia, x:x + ia].astype(np.float64)
        g = gan[y:y + ia, x:x + ia]
        for flat in np.argsort(-np.abs(g).ravel())[:4]:
            py, px = divmod(int(flat), ia)
            us = []
            for sgn in (1, -1):
                wp = wa.copy()
                wp[py, px] += sgn * h
                us.append(orc.process_windows(wp, wb, np.array([[0, 0]], np.int32), ia,
                                              og.CORR_COMPLEX)[0][0, 2])
            fd = (us[0] - us[1]) / (2 * h)
            if np.isfinite(fd):
                errs.append(abs(fd - g[py, px]) / max(abs(fd), 1e-3))
    errs = np.array(errs)

    # propagated sigma at the clean pair against Monte Carlo over noise seeds
    a0, b0 = synth.config5(size=size, noise=0.0)
    c0a, c0b = torch.from_numpy(a0).cuda(), torch.from_numpy(b0).cuda()
    plan.process_device(c0a.data_ptr(), c0b.data_ptr(), pitch, vec.data_ptr(), pk.data_ptr(), 0)
    dsig = torch.zeros((plan.n, 2), dtype=torch.float32, device="cuda")
    ev0.record()
    plan.adjoint_device(c0a.data_ptr(), c0b.data_ptr(), pitch, pk.data_ptr(), var_a=sig * sig,
                        var_b=sig * sig, d_sigma=dsig.data_ptr())
    ev1.record()
    torch.cuda.synchronize()
    sigma_ms = ev0.elapsed_time(ev1)
    pred = dsig.cpu().numpy()
    pk0 = pk.cpu().numpy()
    gen = torch.Generator(device="cuda").manual_seed(20261203 + 5000)
    s1 = torch.zeros((plan.n, 2), dtype=torch.float64, device="cuda")
    s2 = torch.zeros_like(s1)
    same = torch.ones(plan.n, dtype=torch.bool, device="cuda")
    dpk = torch.empty_like(pk)
    pk0d = pk.clone()
    seeds = mc_seeds
    for _ in range(seeds):
        na = c0a + sig * torch.randn(c0a.shape, generator=gen, device="cuda")
        nb = c0b + sig * torch.randn(c0b.shape, generator=gen, device="cuda")
        plan.process_device(na.data_ptr(), nb.data_ptr(), pitch, vec.data_ptr(), dpk.data_ptr(), 0)
        uv = vec[:, 2:4].double()
        s1 += uv
        s2 += uv * uv
        same &= dpk == pk0d
    mean = s1 / seeds
    mc = torch.sqrt(torch.clamp(s2 / seeds - mean * mean, min=0) * seeds / (seeds - 1)).cpu().numpy()
    ok = same.cpu().numpy() & (pk0 >= 0) & np.isfinite(pred).all(1) & (pred > 0).all(1) & np.isfinite(mc).all(1)
    ratio = mc[ok] / pred[ok]
    q = np.percentile(ratio, [25, 50, 75], axis=0)
    return {
        "metric": "adjoint and propagated uncertainty", "workload": "config5_2048sq_f32_ia32_step16",
        "windows": plan.n, "vjp_ms": vjp_ms, "sigma_ms": sigma_ms,
        "fd_check": {"windows": int(len(sample)), "pixels": int(len(errs)), "h": h,
                     "rel_err_median": float(np.median(errs)), "rel_err_p99": float(np.percentile(errs, 99)),
                     "rel_err_max": float(errs.max())},
        "monte_carlo": {"seeds": seeds, "sigma": sig, "windows_compared": int(ok.sum()),
                        "ratio_mc_over_propagated_u": {"p25": q[0, 0], "median": q[1, 0], "p75": q[2, 0]},
                        "ratio_mc_over_propagated_v": {"p25": q[0, 1], "median": q[1, 1], "p75": q[2, 1]},
                        "median_sigma_u_px": float(np.median(pred[ok, 0])),
                        "median_sigma_v_px": float(np.median(pred[ok, 1]))},
        "data": "synthetic (seeded float32 particle images, config 5)"}


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
    per_step = int(min(len(grid), max(1000, rate * args.reference_seconds / max(1, args.steps + args.warmup))))
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
                   "mode": "complex (FFT::cross_correlate)",
                   "ranks": int(os.environ.get("WORLD_SIZE", "1")),
                   "note": "the reference is a CPU library: rank 0 runs it, the other ranks exit"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def launch_replicas(n: int, argv: list[str]) -> int:
    """`--gpus N` outside a torchrun launch: N ranks on this node, one per
    GPU, by re-running this script under torch.distributed.run (rendezvous
    on 127.0.0.1, a free port); returns the launcher's exit status."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + argv
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 1000 for pair, 20 for batch)")
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="pair", choices=["pair", "batch", "sweep", "adjoint"],
                    help="pair: one 4096^2 pair, 32 px windows at step 8 (default); "
                         "batch: 48 pairs of mixed sizes through the 64/32/16 px schedule; "
                         "sweep: accuracy of every precision against the FP64 pass; "
                         "adjoint: d(u, v)/d(pixels) and propagated uncertainty (config 5)")
    ap.add_argument("--mc-seeds", type=int, default=1000, help="Monte Carlo seeds of the adjoint workload")
    ap.add_argument("--sweep-size", type=int, default=2048,
                    help="image size of the precision sweep")
    ap.add_argument("--sweep-windows", default="16,32,48,64",
                    help="window sizes of the precision sweep (comma-separated)")
    ap.add_argument("--sweep-variants", default="base,sparse,noisy",
                    help="field variants of the precision sweep (comma-separated)")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="pair workload: skip the compact batch / sweep / adjoint records")
    ap.add_argument("--reference-seconds", type=float, default=120.0,
                    help="CPU seconds of the reference arm's warm-up plus timed steps")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_replicas(args.gpus, sys.argv[1:]))
    if args.steps is None:
        args.steps = 20 if args.workload == "batch" and args.impl == "ours" else 1000
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "sweep":
        run_sweep(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
