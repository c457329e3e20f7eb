#!/usr/bin/env python3
"""Benchmark: phase-space cell-updates/s of the Vlasov–Maxwell RK step on GB300.

Workload: the block-structured AMR FP64 laser / plasma-slab case — base grid Nx=4096,
Np=512, two levels with refinement ratio 2, refinement criterion 1e-6 with size weight 1
(x in [0,100] lambda, p in [-2,2] m_e c, 0.01 n_c slab on [20,80] with 5-lambda ramps,
T=1 keV, a0=1 Gaussian pulse of FWHM 10 periods, CFL 0.5), the hierarchy built by the
initial flagging / clustering.  Inputs are synthetic (the analytic initial plasma).
One step = CalculateDt + one full six-stage RK step (moments, Poisson, Vlasov FCT stage
of every patch of every level with the ghost fills, interface fluxes and limiter
exchange, Maxwell stage, six times); regridding is outside the timed region, as in the
reference's own timing of SolverManager::Advance.  The metric counts every phase-space
cell of every patch of every level (covered coarse cells included) once per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 (torchrun) runs N independent replicas, one per GPU ("replicas only": a single solve
has no sharded data path here); value sums the replicas' cells over the max-over-ranks
time.  --impl reference times the reference algorithm on the host cores instead: the
oracle port (C++ restatement pinned bit-exact to the reference build), with all host
threads, from the same initial hierarchy.
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
WORKLOAD = "laser_slab_amr_Nx4096_Np512_2level_r2_fp64"
MEASURED = ROOT / "MEASURED_PEAKS.json"

# Compulsory DRAM bytes per padded cell of each profiled kernel (each plane read or
# written once; stage-0 variants, which is what the profile launches).
KERNEL_BYTES = {"gamma": 8, "faces": 48, "flux": 72, "ds_f2": 64, "limR": 48, "limC": 48, "update": 48,
                "moments": 24, "assemble": 0}
# Algorithmic FP64 operations per padded cell (a division counts as one operation).
KERNEL_FLOPS = {"gamma": 6, "faces": 125, "flux": 20, "ds_f2": 8, "limR": 34, "limC": 4, "update": 8,
                "moments": 30, "assemble": 0}
KERNEL_NAMES = {"gamma": "k64_gamma", "faces": "k64_faces", "flux": "k64_flux", "ds_f2": "k64_ds_f2",
                "limR": "k64_limR", "limC": "k64_limC", "update": "k64_update", "moments": "k64_moments",
                "assemble": "k_assemble", "poisson": "k_poisson", "maxwell": "k_maxwell*", "ghost": "k_ghost",
                "iface": "k_iface", "csync": "k_csync", "moments_poisson": "k64_moments_poisson"}
# The pipelined launch does the work of these three kernels (FP64 runs with the exact solve).
PIPELINED = ("moments", "assemble", "poisson")


def problem_config1():
    from veritas_gb300.workloads import laser_slab_2048x256

    return laser_slab_2048x256()


def problem_config3():
    """Larger wakefield case: base 16384 x 1024, three levels, 0.005 n_c, a0 = 2, 0.5 keV."""
    from veritas_gb300.workloads import laser_wakefield_amr_16384x1024

    return laser_wakefield_amr_16384x1024()


def run_config3(args) -> None:
    """--form config3: the larger three-level case alone, as one JSON line."""
    from veritas_gb300 import Context

    ctx = Context(0)
    print(json.dumps(measure_config3(ctx, args.steps)))
    ctx.close()


def measure_config3(ctx, steps: int) -> dict:
    """The precision form on the larger case: FP32 throughput, and the error of f, E_x,
    E_y and the field energy against the FP64 path over the same steps from the same
    initial hierarchy."""
    import dataclasses

    import numpy as np

    from veritas_gb300 import SolverManager

    sys.path.insert(0, str(ROOT / "tests"))
    import vxstate

    t0 = time.perf_counter()
    s32 = SolverManager(ctx, dataclasses.replace(problem_config3(), precision=32))
    init32 = time.perf_counter() - t0
    cells = s32.cell_count()
    layout = s32.layout()
    with tempfile.TemporaryDirectory() as td:
        t0 = time.perf_counter()
        s64 = SolverManager(ctx, problem_config3())
        init64 = time.perf_counter() - t0
        s64.save_state(Path(td) / "init.bin")
        s32.load_state(Path(td) / "init.bin")  # the same initial f (FP64 values, rounded)
        p = problem_config3()
        e0 = p.a0 * 9.10938291e-31 * 299792458.0 * (2 * np.pi * 299792458.0 / p.lambda_) / 1.60217657e-19
        ew = ee = ey = 0.0
        t64 = t32 = 0.0
        for _ in range(steps):
            dt = s64.CalculateDt()
            ctx.timer_begin()
            s64.Advance(dt)
            t64 += ctx.timer_end()
            ctx.timer_begin()
            s32.Advance(dt)
            t32 += ctx.timer_end()
            wa, wb = field_energy(s64), field_energy(s32)
            ew = max(ew, abs(wb - wa) / max(abs(wa), 1e-300))
            ee = max(ee, float(np.max(np.abs(s32.field("Ex") - s64.field("Ex")))) / e0)
            ey = max(ey, float(np.max(np.abs(s32.field("Ey") - s64.field("Ey")))) / e0)
        s64.save_state(Path(td) / "a.bin")
        s32.save_state(Path(td) / "b.bin")
        sa, sb = vxstate.read_state(Path(td) / "a.bin"), vxstate.read_state(Path(td) / "b.bin")
    num = den = 0.0
    for la, lb in zip(sa["species"][0], sb["species"][0]):
        for ra, rb in zip(la, lb):
            fa, fb = ra["f"][2:-2, 2:-2, 0], rb["f"][2:-2, 2:-2, 0]
            num = max(num, float(np.max(np.abs(fb - fa))))
            den = max(den, float(np.max(np.abs(fa))))
    line = {"form": "precision", "workload": "laser_wakefield_amr_Nx16384_Np1024_3level_r2",
            "cells_per_step": cells, "patches": len(layout), "steps": steps,
            "fp32": {"value": cells * steps / (t32 * 1e-3), "unit": UNIT, "ms_per_step": t32 / steps},
            "fp64": {"value": cells * steps / (t64 * 1e-3), "unit": UNIT, "ms_per_step": t64 / steps},
            "init_s": {"fp32": init32, "fp64": init64},
            "error_vs_fp64": {"from": "the FP64 run's initial hierarchy (t = 0), same dt sequence",
                              "f_rel_linf": num / den, "field_energy_rel_max": ew,
                              "Ex_abs_max_over_laser_E0": ee, "Ey_abs_max_over_laser_E0": ey}}
    s32.close()
    s64.close()
    return line


def problem_config2():
    """Two-level AMR laser / slab case: base 4096 x 512, refinement ratio 2."""
    from veritas_gb300.workloads import laser_slab_amr_4096x512

    return laser_slab_amr_4096x512()


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


def max_over_ranks(total_ms: float, dist, device: str) -> float:
    """The job's timed-region length: the slowest rank's (all-reduce MAX), then a barrier
    so that no rank starts the next phase while another is still timing."""
    import torch

    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_value(cells_per_rank: int, world: int, steps: int, total_ms: float) -> float:
    """Whole-job cell-updates/s: every rank advances its own replica of the workload."""
    return cells_per_rank * world * steps / (total_ms * 1e-3)


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_reference(state_path: Path | None, sample_steps: int, threads: int, warmup: int = 1) -> dict:
    """Time the oracle port (reference algorithm, C++ OpenMP) on the host cores.  It
    starts from `state_path` (a state file of the workload) or, when None, builds the
    workload's initial hierarchy itself (flagging, clustering, quadrature; untimed)."""
    exe = ROOT / "oracle" / "_port" / "veritas_port"
    if not exe.exists():
        return {"unavailable": "oracle port not built (run __graft_entry__.build())"}
    p = problem_config2()
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    cmd = [str(exe), *p.harness_args(), f"time_steps={sample_steps}", f"warmup={warmup}"]
    if state_path is not None:
        cmd.append(f"load={state_path}")
    out = subprocess.run(cmd, capture_output=True, text=True, env=env, check=True).stdout
    rec = json.loads(out.strip().splitlines()[-1])
    return {"value": rec["cells"] / rec["median_s"], "best": rec["cells"] / rec["best_s"], "cells": rec["cells"],
            "patches": rec["patches"], "median_s": rec["median_s"], "threads": rec["threads"],
            "init_s": rec["init_s"]}


def workload_config(cells: int, patches: int, world: int) -> dict:
    """The `config` of both arms' lines: the workload, its size and layout, the L2 rule."""
    return {"workload": WORKLOAD, "cells_per_step": cells, "levels": 2, "patches": patches,
            "l2": "inputs larger than L2 (the step streams about 620 MB of patch planes; the GPU arm also "
                  "flushes L2 before every timed step)",
            "parallelism": f"replicas{world}"}


def run_reference(args) -> None:
    """The reference arm: the oracle port (C++/OpenMP restatement pinned bit-exact to the
    reference build) on all host cores, building the workload's initial hierarchy itself
    (the CUDA library is never loaded in this process).  Under torchrun rank 0 alone runs."""
    world, rank, local = dist_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    warm = max(3, args.warmup)
    rec = cpu_reference(None, steps, threads, warm)
    if "unavailable" in rec:
        print(json.dumps({"impl": "reference", "unavailable": rec["unavailable"]}))
        return
    v = rec["value"]
    sample = (f"{steps} timed RK steps (median) of the full workload ({rec['cells']} cells) after {warm} "
              "warm-up steps, from the initial hierarchy the port builds itself")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": warm, "ms_per_step": rec["median_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(rec["cells"], rec["patches"], world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": rec["threads"], "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


EPS0, MU0 = 8.854187817e-12, 1.0 / 795774.715482


def field_energy(s):
    import numpy as np

    nf = s.field("Ey").size // 8
    Ey, Ez, By, Bz = (s.field(k)[:nf] for k in ("Ey", "Ez", "By", "Bz"))
    Ex = s.field("Ex")
    return 0.5 * EPS0 * float(np.sum(Ey * Ey) + np.sum(Ez * Ez) + np.sum(Ex * Ex)) + \
        0.5 / MU0 * float(np.sum(By * By) + np.sum(Bz * Bz))


def measure_form(ctx, init_path: Path, steps: int, warmup: int, variant: dict, dtype: str,
                 persistent: int = 0) -> dict:
    """A variant of the plain path (`variant` overrides Problem fields: the FP32 precision
    form, or FP64 with the scan Poisson solve) on the same workload: throughput, and its
    error against the plain FP64 path over `steps` steps from the same state with the same
    dt sequence."""
    import dataclasses

    import numpy as np

    from veritas_gb300 import SolverManager

    sys.path.insert(0, str(ROOT / "tests"))
    import vxstate

    p32 = dataclasses.replace(problem_config2(), **variant)
    s = SolverManager(ctx, p32)
    cells = s.cell_count()
    from veritas_gb300 import autotune_many

    tile = autotune_many([s])
    ctx.set_persistent(bool(persistent))  # FP32: the persistent stage kernels
    for _ in range(warmup):
        s.Advance(s.CalculateDt())
    ctx.sync()
    times = []
    for _ in range(steps):
        ctx.flush_l2()
        ctx.timer_begin()
        s.Advance(s.CalculateDt())
        times.append(ctx.timer_end())
    ctx.set_persistent(False)
    prof = s.profile_kernels(reps=5)
    s.close()
    ms = sum(times) / len(times)
    # error against the FP64 path from the FP64 initial state
    a, b = SolverManager(ctx, problem_config2()), SolverManager(ctx, p32)
    a.load_state(init_path)
    b.load_state(init_path)
    # E_x is normalised by the laser's field amplitude a0 m c omega / |q| (near t = 0 the
    # plasma is neutral and E_x itself is rounding noise, so a relative error means nothing)
    e0 = p32.a0 * 9.10938291e-31 * 299792458.0 * (2 * np.pi * 299792458.0 / p32.lambda_) / 1.60217657e-19
    ew = ee = ey = exr = 0.0
    for _ in range(steps):
        dt = a.CalculateDt()
        a.Advance(dt)
        b.Advance(dt)
        wa, wb = field_energy(a), field_energy(b)
        ew = max(ew, abs(wb - wa) / max(abs(wa), 1e-300))
        xa, xb = a.field("Ex"), b.field("Ex")
        ee = max(ee, float(np.max(np.abs(xb - xa))) / e0)
        exr = max(exr, float(np.max(np.abs(xb - xa))) / max(float(np.max(np.abs(xa))), 1e-300))
        ya, yb = a.field("Ey"), b.field("Ey")
        ey = max(ey, float(np.max(np.abs(yb - ya))) / e0)
    with tempfile.TemporaryDirectory() as td:
        a.save_state(Path(td) / "a.bin")
        b.save_state(Path(td) / "b.bin")
        sa, sb = vxstate.read_state(Path(td) / "a.bin"), vxstate.read_state(Path(td) / "b.bin")
    num = den = 0.0
    for la, lb in zip(sa["species"][0], sb["species"][0]):
        for ra, rb in zip(la, lb):
            fa, fb = ra["f"][2:-2, 2:-2, 0], rb["f"][2:-2, 2:-2, 0]
            num = max(num, float(np.max(np.abs(fb - fa))))
            den = max(den, float(np.max(np.abs(fa))))
    a.close()
    b.close()
    return {"value": cells / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "dtype": dtype,
            "variant": variant, "persistent": persistent, "tile_p_x": list(tile),
            "error_vs_fp64": {"steps": steps, "from": "the FP64 run's initial hierarchy (t = 0), same dt sequence",
                              "f_rel_linf": num / den, "field_energy_rel_max": ew, "Ex_rel_linf_max": exr,
                              "Ex_abs_max_over_laser_E0": ee, "Ey_abs_max_over_laser_E0": ey},
            "kernel_ms": prof}


def measure_batched(ctx, count: int, steps: int, warmup: int, precision: int, fast: int = 0,
                    persistent: int = 0) -> dict:
    """The seeded ensemble of `count` independent runs advanced together: one launch per
    sub-step for all runs (captured in one CUDA graph per step), or with persistent = 1
    (FP32) three launches per RK stage, two of them persistent cooperative stage kernels.
    fast = 1: FP64 runs with the contracted FCT kernels."""
    import dataclasses

    from veritas_gb300 import SolverManager, advance_many, calculate_dt_many
    from veritas_gb300.ensemble import ensemble_problems

    t0 = time.perf_counter()
    runs = [SolverManager(ctx, dataclasses.replace(p, fast=fast))
            for p in ensemble_problems(count, precision=precision)]
    init_s = time.perf_counter() - t0
    cells = sum(r.cell_count() for r in runs)
    from veritas_gb300 import autotune_many

    tile = autotune_many(runs)
    ctx.set_persistent(bool(persistent))
    for _ in range(warmup):
        advance_many(runs, calculate_dt_many(runs))
    ctx.sync()
    times = []
    l0 = ctx.kernel_launches()
    for _ in range(steps):
        ctx.timer_begin()
        advance_many(runs, calculate_dt_many(runs))
        times.append(ctx.timer_end())
    ctx.sync()
    launches = (ctx.kernel_launches() - l0) / steps - 1  # minus the CFL kernel of each step
    ctx.set_persistent(False)
    for r in runs:
        r.close()
    ms = sum(times) / len(times)
    return {"value": cells / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "runs": count, "cells_per_step": cells,
            "init_s": init_s, "precision": precision, "fast": fast, "persistent": persistent,
            "launches_per_rk_stage": launches / 6, "tile_p_x": list(tile),
            "sampler": "splitmix64 seed 0x5EED0004, stream r = run r (veritas_gb300/ensemble.py)"}


def measure_serving(ctx, count: int, steps: int, precision: int, budget_gb: float = 150.0) -> dict:
    """Serving loop: Poisson arrivals at 20 solves/s (seed 0x5EED0005) of ensemble-sampled
    problems, each run for `steps` RK steps, admitted under the HBM budget and batched
    with whatever else is live.  48-step solves take a regrid each and overload the GPU at
    this arrival rate (their latency is mostly queueing); 16-step solves (no regrid) are
    a load it keeps up with."""
    import dataclasses

    import numpy as np

    from veritas_gb300 import Server
    from veritas_gb300.ensemble import arrival_times, ensemble_problems

    probs = [dataclasses.replace(p, precision=precision) for p in ensemble_problems(count)]
    arr = arrival_times(count)
    srv = Server(ctx, int(budget_gb * (1 << 30)), max_live=count)
    srv.set_regrid(True, 0.0)  # the reference driver's rule: a regrid after every 21 steps
    start = srv.clock()
    ids, nxt = [], 0
    done_cells = 0
    while True:
        now = srv.clock() - start
        while nxt < count and arr[nxt] <= now:
            ids.append(srv.submit(probs[nxt], steps, arrival=start + arr[nxt]))
            nxt += 1
        live, waiting = srv.step()
        if nxt >= count and live == 0 and waiting == 0:
            break
        if live == 0 and waiting == 0 and nxt < count:
            time.sleep(max(0.0, arr[nxt] - (srv.clock() - start)))
    end = srv.clock()
    res = [srv.result(i) for i in ids]
    srv.close()
    ok = [r for r in res if r["status"] == 3]
    lat = np.array([r["finish"] - r["arrival"] for r in ok])
    wait = np.array([r["bound"] - r["arrival"] for r in ok])
    cells = sum(r["cells"] for r in ok) * steps
    return {"solves": count, "completed": len(ok), "steps_per_solve": steps, "precision": precision,
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean())},
            "queue_and_build_s": {"p50": float(np.percentile(wait, 50)), "p99": float(np.percentile(wait, 99))},
            "regrids_per_solve": float(np.mean([r["regrids"] for r in ok])),
            "solves_per_s": count / (end - start), "cell_updates_per_s": cells / (end - start),
            "arrivals": "Poisson, 20 solves/s, splitmix64 seed 0x5EED0005", "hbm_budget_gb": budget_gb,
            "note": "each solve is scaled to a fixed step count (the full 50-period solves of this size mix "
                    "exceed one GPU's throughput at this arrival rate by two orders of magnitude); runs are built "
                    "and regridded on the server's worker threads while the batch steps; regrid after every 21 steps"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--poisson", type=int, default=0, choices=[0, 1],
                    help="Poisson solver of the headline run: 0 the LU's rounding order, 1 the O(n) scan solve")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32],
                    help="precision of the headline workload (64, the plain path, unless profiling the FP32 form)")
    ap.add_argument("--form", default="", choices=["", "config3", "batched", "served"],
                    help="config3: the precision form on the larger three-level case; batched: the 64-run "
                         "ensemble alone; served: the serving loop alone (each its own JSON line; --precision "
                         "selects the form's precision)")
    ap.add_argument("--runs", type=int, default=64, help="ensemble size of --form batched / solves of --form served")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the FP32 / batched / served forms (FP64 headline line only)")
    ap.add_argument("--persistent", action="store_true",
                    help="FP32 runs (--form batched, or --precision 32): the persistent stage kernels")
    ap.add_argument("--lite", action="store_true",
                    help="only the warm-up and timed steps (used under ncu); no e2e, kernel timing or CPU baseline")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.form == "config3":
        run_config3(args)
        return
    if args.form in ("batched", "served"):
        from veritas_gb300 import Context

        ctx = Context(0)
        if args.form == "batched":
            out = measure_batched(ctx, args.runs, args.steps, max(1, args.warmup), args.precision,
                                  persistent=int(args.persistent))
        else:
            out = measure_serving(ctx, args.runs, args.steps, args.precision)
        print(json.dumps({"form": args.form, **out}))
        ctx.close()
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
    import dataclasses

    s = SolverManager(ctx, dataclasses.replace(problem_config2(), precision=args.precision, poisson=args.poisson))
    cells = s.cell_count()
    if args.persistent:
        ctx.set_persistent(True)
    init_path = Path(tempfile.mkdtemp()) / "init.bin"
    if rank == 0 and not args.lite and not (args.no_cpu_baseline and args.no_forms):
        s.save_state(init_path)  # the CPU baseline and the FP32 error check start from it
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
        total_ms = max_over_ranks(total_ms, dist, f"cuda:{local}")
    ms_step = total_ms / args.steps
    value = job_value(cells, world, args.steps, total_ms)
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

    # ---- per-kernel live CUDA-event timing (context stream); shares per step
    prof = s.profile_kernels(reps=5)
    layout = s.layout()
    padded = sum((l[4] + 4) * (l[5] + 4) for l in layout)
    per_step = {k: 6 for k in prof}
    per_step["ghost"] = 12  # two fills (slots 2 and 1) per stage
    # the kernels a step launches: the pipelined launch in place of its three kernels
    # (which are still timed alone, for reference), or the three when it is not used
    pipelined = prof.get("moments_poisson", 0.0) > 0.0
    in_step = [k for k in prof if (k not in PIPELINED if pipelined else k != "moments_poisson")]
    share = {k: prof[k] * per_step[k] for k in in_step}
    tot = sum(share.values())
    dom = max(share, key=share.get)
    peaks = json.loads(MEASURED.read_text()) if MEASURED.exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = ctx.measure_fp64_peak()
    n_fine = s.field("phi").size

    def kernel_roofline(k):
        if k in ("poisson", "moments_poisson"):
            # the two band factors (4 coefficients per row each), the diagonal and its
            # two-word reciprocal, the permutation, the right-hand side and the result
            bpl = n_fine * (8 * 8 + 3 * 8 + 4 + 8 + 8)
            flops = n_fine * 20
            if k == "moments_poisson":  # and the moments' f reads and column sums
                bpl += KERNEL_BYTES["moments"] * padded
                flops += KERNEL_FLOPS["moments"] * padded
        else:
            bpl = KERNEL_BYTES.get(k, 0) * padded
            flops = KERNEL_FLOPS.get(k, 0) * padded
        ach = bpl / (prof[k] * 1e-3) / 1e9
        return {"kernel": k, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": ach / hbm_peak, "algorithmic_bytes_per_launch": bpl, "ms_per_launch": prof[k],
                "fp64": {"achieved_gflops": flops / (prof[k] * 1e-3) / 1e9, "peak_gflops": fp64_peak,
                         "frac": flops / (prof[k] * 1e-3) / 1e9 / fp64_peak}}

    roofline = kernel_roofline(dom)
    roofline.update({"kernel": KERNEL_NAMES.get(dom, dom), "traffic": _read_traffic(dom),
                     "peak_source": "measured" if peaks else "fallback",
                     "share_of_step": share[dom] / tot,
                     "note": ("the exact Poisson solve is two serial triangular recurrences in the reference's "
                              "rounding order: one thread's FP64 latency chain, not bandwidth, bounds it"
                              if dom == "poisson" else
                              "moments (FP64 issue bound) with the exact solve's forward sweep following them, "
                              "then the backward sweep: the moments' FP64 issue rate and the solve's FP64 latency "
                              "chain bound it, not bandwidth" if dom == "moments_poisson" else
                              "FP64 issue rate is the binding roofline of the plain path"),
                     "kernel_ms": prof, "kernel_share": {k: share[k] / tot for k in share},
                     "pipelined": pipelined})
    if dom in ("poisson", "moments_poisson"):
        # the solve's own bound: per row, forward one dependent multiply-subtract and the
        # shuffle that hands x_{i-1} to the lanes, backward the multiply-subtract, the
        # two-operation quotient and the shuffle; cycles measured live on one lane
        ms_cyc, sh_cyc = ctx.measure_fp64_latency()
        mhz = clk.summary().get("sm_mhz") or 2070.0
        fwd_cyc, bwd_cyc = ms_cyc + sh_cyc, 2 * ms_cyc + sh_cyc
        row_cyc = fwd_cyc + bwd_cyc
        min_ms = n_fine * row_cyc / (mhz * 1e3)
        roofline["latency"] = {"bound": "FP64 dependent chain", "mul_sub_cycles": ms_cyc, "shuffle_cycles": sh_cyc,
                               "cycles_per_row": row_cyc, "rows": n_fine, "sm_mhz": mhz, "min_ms": min_ms,
                               "achieved_ms": prof["poisson"], "frac": min_ms / prof["poisson"]}
        if dom == "moments_poisson":
            # pipelined: at best the forward sweep hides entirely behind the moments (timed
            # alone, FP64 issue bound), then the backward sweep's chain
            fwd_ms, bwd_ms = n_fine * fwd_cyc / (mhz * 1e3), n_fine * bwd_cyc / (mhz * 1e3)
            best = max(prof["moments"], fwd_ms) + bwd_ms
            roofline["latency"].update({"bound": "moments (FP64 issue) overlapped with the forward chain, then the "
                                                 "backward chain",
                                        "moments_ms": prof["moments"], "forward_chain_ms": fwd_ms,
                                        "backward_chain_ms": bwd_ms, "min_ms": best,
                                        "achieved_ms": prof["moments_poisson"],
                                        "frac": best / prof["moments_poisson"],
                                        "separate_kernels_ms": prof["moments"] + prof["assemble"] + prof["poisson"]})
    stencil = max((k for k in share if k in KERNEL_BYTES and KERNEL_BYTES[k] > 0), key=share.get)
    roofline["stencil"] = kernel_roofline(stencil)
    roofline["stencil"]["kernel"] = KERNEL_NAMES.get(stencil, stencil)

    forms = None
    if rank == 0 and not args.no_forms:
        forms = {"fp32": measure_form(ctx, init_path, args.steps, warmup, {"precision": 32},
                                      "f32 (moments, fields, Poisson f64)"),
                 "fp64_scan_poisson": measure_form(ctx, init_path, args.steps, warmup, {"poisson": 1},
                                                   "f64 (O(n) scan Poisson instead of the LU's rounding order)"),
                 "fp64_fast": measure_form(ctx, init_path, args.steps, warmup, {"fast": 1},
                                           "f64 (FCT kernels with fused multiply-add; the LU's rounding order)"),
                 "fp64_fast_scan_poisson": measure_form(ctx, init_path, args.steps, warmup, {"fast": 1, "poisson": 1},
                                                        "f64 (fused multiply-add FCT kernels, O(n) scan Poisson)"),
                 "fp32_persistent": measure_form(ctx, init_path, args.steps, warmup, {"precision": 32},
                                                 "f32, persistent stage kernels (3 launches per RK stage)",
                                                 persistent=1),
                 "batched_fp32": measure_batched(ctx, 64, 20, 3, 32),
                 "batched_fp32_persistent": measure_batched(ctx, 64, 20, 3, 32, persistent=1),
                 "batched_fp64": measure_batched(ctx, 64, 20, 3, 64),
                 "batched_fp64_fast": measure_batched(ctx, 64, 20, 3, 64, fast=1),
                 "served_fp32": measure_serving(ctx, 200, 48, 32),
                 "served_fp32_short": measure_serving(ctx, 200, 16, 32),
                 "served_fp64": measure_serving(ctx, 24, 24, 64),
                 "precision_wakefield_16384x1024": measure_config3(ctx, args.steps)}
        forms["fp32_speedup_vs_fp64"] = forms["fp32"]["value"] / value
        forms["fp64_scan_poisson_speedup_vs_fp64"] = forms["fp64_scan_poisson"]["value"] / value
        forms["fp64_fast_speedup_vs_fp64"] = forms["fp64_fast"]["value"] / value
        forms["fp64_fast_scan_poisson_speedup_vs_fp64"] = forms["fp64_fast_scan_poisson"]["value"] / value
        forms["batched_fp32_speedup_vs_fp64"] = forms["batched_fp32"]["value"] / value
        forms["batched_fp32_speedup_vs_batched_fp64"] = forms["batched_fp32"]["value"] / forms["batched_fp64"]["value"]
        forms["served_fp32_speedup_vs_fp64"] = forms["served_fp32"]["cell_updates_per_s"] / value

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rec = cpu_reference(init_path, 3, os.cpu_count() or 1, 3)
        if "unavailable" not in rec:
            cpu = {"value": rec["value"], "unit": UNIT, "cores": rec["threads"], "kind": "port",
                   "sample": f"3 timed RK steps (median) of the full workload ({rec['cells']} cells) after 3 "
                             "warm-up steps, from the same initial hierarchy"}
        else:
            cpu = {"value": None, "unavailable": rec["unavailable"]}
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        parity = parity_vs_port(ctx, 2)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(cells, len(layout), world),
                "clocks": clk.summary(), "gpu_launches": launches, "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu, "parity_vs_port": parity, "forms": forms}
        print(json.dumps(line))
    hin.close()
    hout.close()
    s.close()
    ctx.close()
    if init_path.exists():
        init_path.unlink()
    if dist:
        dist.destroy_process_group()


def parity_vs_port(ctx, steps: int) -> dict:
    """The headline workload's parity: the GPU path and the oracle port (pinned bit-exact
    to the reference build) each build the initial hierarchy from t = 0, then advance
    `steps` RK steps with the same dt; compared array by array (relative L-inf; the bar is
    1e-10; the patch layouts must be identical)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from helpers import gpu_vs_port

    with tempfile.TemporaryDirectory() as td:
        try:
            err = gpu_vs_port(ctx, problem_config2(), steps, Path(td))
        except AssertionError as e:  # compare_states found a different patch layout
            return {"steps": steps, "layouts_identical": False, "error": str(e)}
    after = {k: v for k, v in err.items() if not k.startswith("init_")}
    return {"steps": steps, "from": "t = 0: each side builds the initial hierarchy, then the same dt sequence",
            "tolerance": 1e-10, "layouts_identical": True, "init_rel_linf": max(v for k, v in err.items()
                                                                                if k.startswith("init_")),
            "f_rel_linf": after["f"], "fields_rel_linf": max(v for k, v in after.items() if k not in ("f", "time")),
            "per_array": err}


def _read_traffic(kernel: str):
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get(kernel)
    return None


if __name__ == "__main__":
    main()
