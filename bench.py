#!/usr/bin/env python3
"""Benchmark: phase-space cell-updates/s of the Vlasov–Maxwell RK step on GB300.

Workload: the single-level FP64 laser / plasma-slab case (Nx=2048, Np=256, x in [0,100]
lambda, p in [-2,2] m_e c, 0.01 n_c slab on [20,80] with 5-lambda ramps, T=1 keV,
a0=1 Gaussian pulse of FWHM 10 periods, CFL 0.5) on synthetic seeded inputs.
One step = CalculateDt + one full six-stage RK step (moments, Poisson, Vlasov FCT stage,
Maxwell stage, six times).  The metric counts every phase-space cell of every patch
once per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 (torchrun) runs N independent replicas, one per GPU ("replicas only": a single solve
has no sharded data path here); value sums the replicas' cells over the max-over-ranks
time.  --impl reference times the reference algorithm on the host cores instead: the
oracle port (C++ restatement pinned to the reference build), with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "phase-space cell-updates/s"
UNIT = "cell-updates/s"
WORKLOAD = "laser_slab_Nx2048_Np256_1level_fp64"
MEASURED = ROOT / "MEASURED_PEAKS.json"

# Compulsory DRAM bytes per padded cell of each profiled kernel (each plane read or
# written once; stage-0 variants, which is what the profile launches).
KERNEL_BYTES = {"gamma": 8, "faces": 48, "flux": 72, "ds_f2": 64, "limR": 48, "limC": 48, "update": 48,
                "moments": 24, "assemble": 0}
# Algorithmic FP64 operations per padded cell (a division counts as one operation).
KERNEL_FLOPS = {"gamma": 6, "faces": 125, "flux": 20, "ds_f2": 8, "limR": 34, "limC": 4, "update": 8,
                "moments": 30, "assemble": 0}


def problem_config1():
    from veritas_gb300 import Problem

    return Problem(L=100.0, nx=2048, np=256, Lfinest=1, pmax=2.0, dens=0.01, x1=15, x2=20, x3=80, x4=85, Te=1.0,
                   a0=1.0, fwhm=10.0, delay=10.0, cfl=0.5, quadDepth=2, precision=64)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        self.tmp.flush()
        rows = []
        for line in Path(self.tmp.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, fl in rows for i, v in enumerate(fl) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_reference(args, cells_per_step_full: int, sample_steps: int, threads: int, nx: int, np_: int) -> dict:
    """Time the oracle port (reference algorithm, C++ OpenMP) on the host cores."""
    exe = ROOT / "oracle" / "_port" / "veritas_port"
    if not exe.exists():
        return {"unavailable": "oracle port not built (run __graft_entry__.build())"}
    p = problem_config1()
    p.nx, p.np = nx, np_
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    cmd = [str(exe), *p.harness_args(), f"time_steps={sample_steps}"]
    out = subprocess.run(cmd, capture_output=True, text=True, env=env, check=True).stdout
    rec = json.loads(out.strip().splitlines()[-1])
    return {"value": rec["cells"] / rec["median_s"], "best": rec["cells"] / rec["best_s"], "cells": rec["cells"],
            "median_s": rec["median_s"], "threads": rec["threads"]}


def run_reference(args) -> None:
    world, rank, _ = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    rec = cpu_reference(args, 0, steps, threads, 2048, 256)
    if "unavailable" in rec:
        print(json.dumps({"impl": "reference", "unavailable": rec["unavailable"]}))
        return
    v = rec["value"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": 1, "ms_per_step": rec["median_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells_per_step": rec["cells"]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": rec["threads"], "kind": "port",
                             "sample": f"{steps} timed RK steps (median) of the full 2048x256 case after 1 warm-up"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lite", action="store_true",
                    help="only the warm-up and timed steps (used under ncu); no e2e, kernel timing or CPU baseline")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    world, rank, local = dist_info()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist
    warmup = max(3, args.warmup)

    from veritas_gb300 import Context, PinnedArray, SolverManager

    ctx = Context(local)
    s = SolverManager(ctx, problem_config1())
    cells = s.cell_count()
    for _ in range(warmup):
        s.Advance(s.CalculateDt())
    ctx.sync()

    # ---- timed region: K steps, L2 flushed before each, CUDA events on the ctx stream
    if dist:
        dist.barrier()
    ctx.sync()
    l0 = ctx.kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            ctx.timer_begin()
            s.Advance(s.CalculateDt())
            times.append(ctx.timer_end())
    ctx.sync()
    launches = ctx.kernel_launches() - l0 - args.steps  # minus the flush memsets (not kernels of ours)
    total_ms = sum(times)
    if dist:
        import torch

        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    ms_step = total_ms / args.steps
    value = cells * world * args.steps / (total_ms * 1e-3)
    if args.lite:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_step, "lite": True}))
        s.close()
        ctx.close()
        return

    # ---- end to end through the C ABI with pinned host buffers
    n = s.state_size()
    hin, hout = PinnedArray(n), PinnedArray(n)
    s.state_to_host(hin.array)
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dt = s.CalculateDt()
        s.step_host(hin.array, hout.array, dt)
        hin, hout = hout, hin
    e2e_s = time.perf_counter() - t0
    e2e = {"value": cells * world * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n,
           "d2h_bytes_per_step": 8 * n + 8}

    # ---- dominant kernel, live CUDA-event timing
    prof = s.profile_kernels(reps=5)
    padded = (2048 + 4) * (256 + 4)
    launches_per_step = {"gamma": 6, "faces": 6, "flux": 6, "ds_f2": 6, "limR": 6, "limC": 6, "update": 6,
                         "moments": 6, "assemble": 6}
    share = {k: prof[k] * launches_per_step[k] for k in prof}
    dom = max(share, key=share.get)
    peaks = json.loads(MEASURED.read_text()) if MEASURED.exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    ach = KERNEL_BYTES[dom] * padded / (prof[dom] * 1e-3) / 1e9
    fp64_peak = ctx.measure_fp64_peak()
    fp64_ach = KERNEL_FLOPS[dom] * padded / (prof[dom] * 1e-3) / 1e9
    traffic = _read_traffic(dom)
    roofline = {"kernel": f"k64_{dom}", "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": ach / hbm_peak, "traffic": traffic, "peak_source": "measured" if peaks else "fallback",
                "algorithmic_bytes_per_launch": KERNEL_BYTES[dom] * padded,
                "fp64": {"achieved_gflops": fp64_ach, "peak_gflops": fp64_peak, "frac": fp64_ach / fp64_peak,
                         "note": "FP64 issue rate is the binding roofline of the plain path; peak measured live "
                                 "with a DFMA chain kernel"},
                "kernel_ms": prof}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rec = cpu_reference(args, cells, 3, os.cpu_count() or 1, 2048, 256)
        if "unavailable" not in rec:
            cpu = {"value": rec["value"], "unit": UNIT, "cores": rec["threads"], "kind": "port",
                   "sample": "3 timed RK steps (median) of the full 2048x256 case after 1 warm-up"}
        else:
            cpu = {"value": None, "unavailable": rec["unavailable"]}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "cells_per_step": cells, "l2": "flushed before every timed step",
                           "parallelism": f"replicas{world}"},
                "clocks": clk.summary(), "gpu_launches": launches, "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu}
        print(json.dumps(line))
    hin.close()
    hout.close()
    s.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


def _read_traffic(kernel: str):
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get(kernel)
    return None


if __name__ == "__main__":
    main()
