"""Shared helpers for the parity tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import vxstate

GOLDEN = Path(__file__).resolve().parent / "golden"


def case_args(name: str) -> dict:
    out = {}
    for kv in (GOLDEN / f"{name}.args").read_text().split():
        k, v = kv.split("=")
        out[k] = v
    return out


def problem_for(name: str):
    from veritas_gb300 import Problem

    a = case_args(name)
    p = Problem()
    for k, v in a.items():
        if k == "levels":
            p.Lfinest = int(v)
        elif k in ("nx", "np", "r", "quadDepth"):
            setattr(p, k, int(v))
        else:
            setattr(p, k, float(v))
    return p


def golden(name: str, step: int) -> dict:
    return vxstate.from_npz(GOLDEN / f"{name}_s{step}.npz")


def golden_named(name: str, tag: str) -> dict:
    return vxstate.from_npz(GOLDEN / f"{name}_{tag}.npz")


def compare_states(got: dict, ref: dict, tol: float) -> dict:
    """Relative L-inf errors of f (slots 0 and 1, whole padded block) and the fields."""
    err = {}
    fmax = 0.0
    for sg, sr in zip(got["species"], ref["species"]):
        for lg, lr in zip(sg, sr):
            assert len(lg) == len(lr)
            for rg, rr in zip(lg, lr):
                for k in ("x_pos", "p_pos", "n_x", "n_p", "depth", "up", "down", "left", "right"):
                    assert rg[k] == rr[k], k
                for slot in (0, 1):
                    e = vxstate.rel_linf(rg["f"][..., slot], rr["f"][..., slot])
                    fmax = max(fmax, e)
    err["f"] = fmax
    nf = ref["n"] + ref["pre"] + ref["post"]
    for k in ("By", "Bz", "Ey", "Ez", "Ay", "Az"):
        err[k] = vxstate.rel_linf(got[k][:nf], ref[k][:nf])
    for k in ("a_squared", "phi", "charge", "J"):
        err[k] = vxstate.rel_linf(got[k], ref[k])
    err["Ex0"] = abs(got["Ex0"] - ref["Ex0"]) / max(abs(ref["Ex0"]), 1e-300)
    err["time"] = abs(got["time"] - ref["time"]) / max(abs(ref["time"]), 1e-300)
    return err


def total_mass(st: dict) -> float:
    m = 0.0
    for levels in st["species"]:
        for rects in levels:
            for r in rects:
                m += float(np.sum(r["f"][2:-2, 2:-2, 0]))
    return m


ROOT = GOLDEN.parent.parent
PORT = ROOT / "oracle" / "_port" / "veritas_port"


def port_exe() -> Path:
    """The oracle port (built by build(); built here if missing)."""
    import subprocess

    if not PORT.exists():
        subprocess.run(["bash", str(ROOT / "oracle" / "port" / "build_port.sh")], check=True, capture_output=True)
    return PORT


def gpu_vs_port(ctx, problem, steps: int, workdir: Path, init_state: Path | None = None,
                threads: int | None = None) -> dict:
    """The GPU path and the oracle port advanced `steps` RK steps with the GPU path's dt
    sequence; returns compare_states' relative L-inf errors after the steps (f slots 0 and
    1, every field array, Ex0, time).  Both start from `init_state` when given.  When None,
    each builds the initial hierarchy itself (flagging, clustering, quadrature) and the
    errors of the two initial states are returned too, under keys prefixed "init_"."""
    import os
    import subprocess

    from veritas_gb300 import SolverManager

    workdir = Path(workdir)
    s = SolverManager(ctx, problem)
    if init_state is not None:
        s.load_state(init_state)
    else:
        s.save_state(workdir / "gpu_init.bin")
    dts = []
    for _ in range(steps):
        dt = s.CalculateDt()
        dts.append(dt)
        s.Advance(dt)
    s.save_state(workdir / "gpu.bin")
    s.close()
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    cmd = [str(port_exe()), *problem.harness_args(), "dts=" + ",".join(repr(d) for d in dts), f"steps={steps}",
           f"dump_every={steps}", f"dumpdir={workdir}"]
    if init_state is not None:
        cmd.append(f"load={init_state}")
    subprocess.run(cmd, check=True, capture_output=True, env=env)
    err = compare_states(vxstate.read_state(workdir / "gpu.bin"), vxstate.read_state(workdir / f"state_{steps:05d}.bin"),
                         0.0)
    if init_state is None:
        e0 = compare_states(vxstate.read_state(workdir / "gpu_init.bin"), vxstate.read_state(workdir / "state_00000.bin"),
                            0.0)
        err.update({"init_" + k: v for k, v in e0.items()})
    return err
