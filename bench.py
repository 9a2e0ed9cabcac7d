"""Benchmark: out-of-core left-looking FP64 Cholesky on GB300.

One JSON line on rank 0 (see the keys below).  A step is one factorization of one
synthetic SPD matrix A = (R + R^T)/2 + n I (R uniform in [-0.5, 0.5), SplitMix64,
seed 100 + rank):

* ``value`` -- TFLOP/s (n^3/3 flops) of the factorization with A already resident in
  HBM (device pointer, factored in place).  Every step first restores A from a
  pristine device copy (a device-to-device copy inside the timed region; A is larger
  than L2, so no L2 flush is needed).
* ``e2e``  -- the same metric through the C-ABI with A in page-locked HOST memory,
  streamed through a device budget that forces the left-looking out-of-core schedule:
  every host-to-device panel/column copy and device-to-host copy-back is inside the
  timed region (byte counts are the library's own).
* ``roofline`` -- the dominant kernel (the panel update: syrk + gemm on FP64 DMMA),
  achieved = its algorithmic flops / its CUDA-event time on the launching stream over
  the timed steps; peak = FP64 DMMA issue rate measured live by the library's probe.
* ``cpu_baseline`` -- the oracle (a C++ restatement of the reference's QUARK task graph
  on host BLAS) timed on this host's cores on a bounded sample.

``--impl reference`` times the reference algorithm's CPU path (the oracle: QUARK-style
task graph + host BLAS; the reference itself cannot be built here) on the same
workload with all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Cholesky TFLOP/s (n^3/3 flops), mixed vs FP64 at backward err<=1e-14; p99 ms"

# DRAM bytes per algorithmic flop of k_panel_update, from one ncu capture of two launches
# at n=8192, nb=1024 (dram__bytes_read.sum + dram__bytes_write.sum = 348.1 MB for
# 44.02 GFLOP; profiles/k_panel_update_fp64_n8192.md).  The kernel's traffic is the
# operand and C tiles, which scale with the flops of a launch at fixed nb.
UPDATE_DRAM_BYTES_PER_FLOP = 348.1e6 / 44.02e9


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=24576)
    p.add_argument("--nb", type=int, default=1024)
    p.add_argument("--budget-mb", type=int, default=1024, help="device panel budget for the e2e (host) leg")
    p.add_argument("--seed", type=int, default=100)
    p.add_argument("--cpu-sample-n", type=int, default=12288)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--skip-e2e", action="store_true")
    return p.parse_args()


# ----------------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
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
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(pw) if pw else None}


# ----------------------------------------------------------------------------------
# distributed helpers (N > 1: independent replicas, one per GPU)
# ----------------------------------------------------------------------------------
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ----------------------------------------------------------------------------------
# CPU legs (oracle): the reported baseline and the reference arm
# ----------------------------------------------------------------------------------
def cpu_factor_tflops(n: int, nb: int, budget_bytes: int, seed: int, reps: int = 1) -> tuple[float, int, list]:
    import oracle

    ncores = os.cpu_count() or 1
    oracle.set_blas_threads(1)  # one BLAS thread per task, as the reference links sequential MKL
    times = []
    for r in range(reps):
        A = oracle.gen_uniform(n, seed, float(n))
        t, info, npan = oracle.cholesky(A, nb, budget_bytes, ncores, 2)
        if info != 0:
            raise RuntimeError(f"oracle info={info}")
        times.append(t)
    return (n ** 3 / 3.0) / (sum(times) / len(times)) / 1e12, ncores, times


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    n, nb = args.n, args.nb
    budget = args.budget_mb << 20
    import oracle

    ncores = os.cpu_count() or 1
    oracle.set_blas_threads(1)
    for _ in range(args.warmup):
        A = oracle.gen_uniform(n, args.seed, float(n))
        oracle.cholesky(A, nb, budget, ncores, 2)
    total = 0.0
    for _ in range(args.steps):
        A = oracle.gen_uniform(n, args.seed, float(n))
        t, info, npan = oracle.cholesky(A, nb, budget, ncores, 2)
        if info != 0:
            raise RuntimeError(f"oracle info={info}")
        total += t
    ms = total / args.steps * 1e3
    val = (n ** 3 / 3.0) / (ms / 1e3) / 1e12
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: A=(R+R^T)/2+n*I, R~U[-0.5,0.5) SplitMix64 seed {args.seed}",
        "config": {"workload": f"plain FP64 out-of-core lower Cholesky n={n} nb={nb} budget={args.budget_mb}MiB",
                   "n": n, "nb": nb, "device_budget_bytes": budget},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": ncores, "kind": "port",
                         "sample": f"full workload (n={n}), QUARK-style task graph of the reference restated "
                                   f"in C++ on {ncores} worker threads, host OpenBLAS one thread per task; "
                                   "timer = factorization only (oocdag.cpp:51,90)"},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------------
def run_ours(args):
    rank, world, local = dist_env()
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import oocdag_gb300 as ooc

    ooc.load()
    n, nb = args.n, args.nb
    seed = args.seed + rank
    flops = n ** 3 / 3.0
    h = ooc.Handle(local)
    comp = torch.cuda.ExternalStream(h.stream(0))

    # FP64 roofline denominator: live DMMA issue-rate probe (no FP64 entry exists in the
    # measured peaks file).
    peak_tf = h.fp64_peak(300.0)

    # ---- value: device-resident A -------------------------------------------------
    A0 = torch.empty((n, n), dtype=torch.float64, device="cuda")  # column-major view (ld = n)
    h.matgen_uniform(A0, n, n, seed, float(n))
    A = torch.empty_like(A0)
    torch.cuda.synchronize()

    def dev_step():
        with torch.cuda.stream(comp):
            A.copy_(A0)
        r = h.dpotrf_L(A, n, n, nb, 0)
        if r.info != 0:
            raise RuntimeError(f"info={r.info}")
        return r

    for _ in range(args.warmup):
        dev_step()
    h.set_option(ooc.OPT_PROFILE, 1)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    upd_ms = upd_flops = 0.0
    upd_launch = 0
    launches = 0
    for _ in range(args.steps):
        r = dev_step()
        s = r.stats
        upd_ms += s["update_ms"]
        upd_flops += s["update_flops"]
        upd_launch += s["update_launches"]
        launches += s["kernel_launches"] + 1  # + the restore copy kernel
    e1.record(comp)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    h.set_option(ooc.OPT_PROFILE, 0)
    ms_local = e0.elapsed_time(e1) / args.steps
    ms = allreduce_max(ms_local, world)
    value = flops * world / (ms / 1e3) / 1e12

    # check the last factor (not timed): scaled residual on the device
    resid = h.residual(A, n, n, "uniform", seed, float(n))

    # ---- e2e: host A through the C-ABI, out of core ------------------------------
    e2e = None
    npanels = None
    if not args.skip_e2e:
        budget = args.budget_mb << 20
        Hpr = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        Hw = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
        h.matgen_uniform(Hpr, n, n, seed, float(n))
        for _ in range(args.warmup):
            Hw.copy_(Hpr)
            h.dpotrf_L(Hw, n, n, nb, budget)
        tot_ms = 0.0
        h2d = d2h = 0.0
        barrier(world)
        for _ in range(args.steps):
            Hw.copy_(Hpr)  # restore the input (host memcpy, outside the per-step events)
            torch.cuda.synchronize()
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(comp)
            r = h.dpotrf_L(Hw, n, n, nb, budget)
            s1.record(comp)
            torch.cuda.synchronize()
            if r.info != 0:
                raise RuntimeError(f"e2e info={r.info}")
            tot_ms += s0.elapsed_time(s1)
            h2d += r.stats["h2d_bytes"]
            d2h += r.stats["d2h_bytes"]
            npanels = r.stats["npanels"]
            launches += r.stats["kernel_launches"]
        e2e_ms = allreduce_max(tot_ms / args.steps, world)
        e2e = {"value": flops * world / (e2e_ms / 1e3) / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
               "ms_per_step": e2e_ms, "device_budget_bytes": budget, "panels": npanels,
               "host_link_gbs": (h2d + d2h) / args.steps / (e2e_ms / 1e3) / 1e9}
        del Hpr, Hw

    # ---- roofline of the dominant kernel -----------------------------------------
    achieved = upd_flops / (upd_ms / 1e3) / 1e12 if upd_ms > 0 else None
    roofline = {"bound": "fp64-dmma", "kernel": "k_panel_update (syrk+gemm, FP64 mma.sync m8n8k4)",
                "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                "frac": (achieved / peak_tf) if achieved else None,
                "peak_source": "measured live: FP64 DMMA issue loop on all SMs (ooc_fp64_peak_probe); "
                               "MEASURED_PEAKS.json has no FP64 entry",
                "launches": upd_launch, "avg_launch_ms": upd_ms / max(1, upd_launch),
                "share_of_step": upd_ms / (ms_local * args.steps) if ms_local > 0 else None,
                "traffic": (UPDATE_DRAM_BYTES_PER_FLOP * upd_flops / upd_launch) if upd_launch else None,
                "traffic_unit": "bytes per launch (ncu capture at n=8192 scaled by flops per launch)",
                "algorithmic_bytes_note": "operand tiles read once + C tiles read and written"}

    # ---- CPU baseline (rank 0, N=1 only) -----------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        ns = min(args.cpu_sample_n, n)
        bud = max(args.budget_mb << 20 >> 4, 1)  # keep the sample out of core as well
        bb = (ns + nb - 1) // nb
        bud = max(bud, (3 * bb + 2) * nb * nb * 8)
        tf, cores, times = cpu_factor_tflops(ns, nb, bud, seed)
        cpu = {"value": tf, "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": f"n={ns} nb={nb} budget={bud >> 20}MiB, {times[0]:.1f}s: the reference's QUARK task "
                         f"graph restated in C++ on {cores} host threads, OpenBLAS one thread per task"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic: A=(R+R^T)/2+n*I, R~U[-0.5,0.5) SplitMix64 seed {args.seed}+rank",
            "config": {"workload": f"plain FP64 out-of-core lower Cholesky n={n} nb={nb} "
                                   f"(e2e: host A, device budget {args.budget_mb} MiB)",
                       "form": "fp64-plain", "n": n, "nb": nb, "parallelism": f"replicas x{world}",
                       "l2": f"inputs larger than L2 ({n * n * 8 / 1e9:.1f} GB per matrix)"},
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": launches, "scaled_residual": resid,
        }
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
