"""Builds the C user problem of this folder into a shared library and hands its hooks
to the library the way a C caller would (function pointers in a vx_hooks struct)."""
from __future__ import annotations

import ctypes
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
_BUILT = {}


class Sin2Params(ctypes.Structure):
    """sin2_params of sin2_problem.h."""
    _fields_ = [("nx", ctypes.c_uint32), ("np", ctypes.c_uint32), ("Lfinest", ctypes.c_uint32)] + [
        (n, ctypes.c_double) for n in ("L", "pad", "x_lo", "x_hi", "dens", "mod_k", "mod_amp", "Te", "Ti", "mi",
                                       "pmax_e", "pmax_i", "drift", "a0", "ramp", "crit", "minEff", "sizeWeight",
                                       "cfl")] + [("quadDepth", ctypes.c_int32)] + [
        (n, ctypes.c_double) for n in ("ref_x0", "ref_x1", "ref_p")]


def problem_library() -> ctypes.CDLL:
    """sin2_problem.c compiled with -ffp-contract=off (as the reference build links it)."""
    if "lib" not in _BUILT:
        out = Path(tempfile.mkdtemp()) / "libsin2_problem.so"
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(out),
                        str(HERE / "sin2_problem.c"), "-lm"], check=True)
        _BUILT["lib"] = ctypes.CDLL(str(out))
    return _BUILT["lib"]


def sin2_hooks(args: dict):
    """(hooks, params): the problem's defaults overridden by the fixture's key=value args
    (nx, np, levels, L, pad, a0, ramp, crit, minEff) — the keys the reference harness reads."""
    from veritas_gb300 import VxHooks

    lib = problem_library()
    prm = Sin2Params()
    lib.sin2_defaults(ctypes.byref(prm))
    for k, v in args.items():
        if k == "levels":
            prm.Lfinest = int(v)
        elif k in ("nx", "np"):
            setattr(prm, k, int(v))
        else:
            setattr(prm, k, float(v))
    h = VxHooks()
    h.user = ctypes.cast(ctypes.pointer(prm), ctypes.c_void_p)
    for field, sym in (("initial_conditions", "sin2_initial_conditions"),
                       ("settings_override", "sin2_settings_override"),
                       ("initial_distribution", "sin2_initial_distribution"), ("get_by", "sin2_get_by"),
                       ("get_bz", "sin2_get_bz"), ("refinement_override", "sin2_refinement_override")):
        setattr(h, field, ctypes.cast(getattr(lib, sym), ctypes.c_void_p))
    return h, prm
