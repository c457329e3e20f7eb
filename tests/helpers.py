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
