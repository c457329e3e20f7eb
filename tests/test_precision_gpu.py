"""FP32 precision form against the FP64 path (the form's oracle), through the C ABI.

Both forms start from the same state (a reference dump) and take the same dt sequence.
Errors after 5 steps (the bar and what was measured on GB300):
  f   : max |f32 - f64| / max |f64| over all patches (slot 0)  bar 1e-5, measured 3e-7..5e-7
  W   : relative error of the field energy, every step        bar 1e-5, measured 4e-11..4e-8
  E_x : relative L-inf on the finest grid, stated              guard 1e-4, measured 7e-7..4e-5
The FP32 form keeps moments, fields and the Poisson solve in FP64, so the field errors
come from f alone.  E_x is the largest: it follows the net charge, a small difference
between the electron charge and the neutralising background, so the FP32 rounding of
f is amplified by (electron charge / net charge).
"""
import numpy as np
import pytest

import vxstate
from helpers import golden, problem_for

TOL_F, TOL_E, TOL_W = 1e-5, 1e-4, 1e-5
EPS0, MU0 = 8.854187817e-12, 1.0 / 795774.715482


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


def field_energy(s):
    nf = s.field("Ey").size // 8
    Ey, Ez, By, Bz = (s.field(k)[:nf] for k in ("Ey", "Ez", "By", "Bz"))
    Ex = s.field("Ex")
    return 0.5 * EPS0 * (np.sum(Ey * Ey) + np.sum(Ez * Ez) + np.sum(Ex * Ex)) + 0.5 / MU0 * (np.sum(By * By) + np.sum(Bz * Bz))


def f_error(st32, st64):
    num, den = 0.0, 0.0
    for l32, l64 in zip(st32["species"][0], st64["species"][0]):
        assert len(l32) == len(l64)
        for r32, r64 in zip(l32, l64):
            a, b = r32["f"][2:-2, 2:-2, 0], r64["f"][2:-2, 2:-2, 0]
            num = max(num, float(np.max(np.abs(a - b))))
            den = max(den, float(np.max(np.abs(b))))
    return num / den


def run_pair(ctx, tmp_path, prob, start=None, steps=5):
    from veritas_gb300 import SolverManager

    p64 = prob
    s64 = SolverManager(ctx, p64)
    if start is not None:
        vxstate.write_state(start, tmp_path / "start.bin")
        s64.load_state(tmp_path / "start.bin")
    s64.save_state(tmp_path / "init.bin")
    p32 = problem_for_precision(prob, 32)
    s32 = SolverManager(ctx, p32)
    s32.load_state(tmp_path / "init.bin")
    errs = []
    for k in range(steps):
        dt = s64.CalculateDt()
        s64.Advance(dt)
        s32.Advance(dt)
        w64, w32 = field_energy(s64), field_energy(s32)
        e64, e32 = s64.field("Ex"), s32.field("Ex")
        errs.append({"W": abs(w32 - w64) / max(abs(w64), 1e-300),
                     "Ex": float(np.max(np.abs(e32 - e64)) / max(np.max(np.abs(e64)), 1e-300))})
    s64.save_state(tmp_path / "a64.bin")
    s32.save_state(tmp_path / "a32.bin")
    ef = f_error(vxstate.read_state(tmp_path / "a32.bin"), vxstate.read_state(tmp_path / "a64.bin"))
    s32.close()
    s64.close()
    return ef, errs


def problem_for_precision(prob, precision):
    import dataclasses

    return dataclasses.replace(prob, precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("slab64", 0), ("drift128", 0), ("amr2", 0), ("beam2", 0), ("beam3", 0),
                                    ("ions2", 0), ("ragged2", 0)])
def test_fp32_form_error_vs_fp64(ctx, tmp_path, name, k):
    ef, errs = run_pair(ctx, tmp_path, problem_for(name), golden(name, k), steps=5)
    ew = max(e["W"] for e in errs)
    ee = max(e["Ex"] for e in errs)
    print(f"{name}: f {ef:.2e}  Ex {ee:.2e}  W {ew:.2e}")
    assert ef <= TOL_F and ee <= TOL_E and ew <= TOL_W, (ef, ee, ew)


@pytest.mark.gpu
def test_fp32_form_from_its_own_initialisation(ctx, tmp_path):
    """The FP32 run built from t=0 (its own flagging, clustering and quadrature) has the
    FP64 run's layout and f to FP32 rounding."""
    from veritas_gb300 import SolverManager

    prob = problem_for("amr2")
    s64 = SolverManager(ctx, prob)
    s32 = SolverManager(ctx, problem_for_precision(prob, 32))
    assert s32.layout() == s64.layout()
    s64.save_state(tmp_path / "a.bin")
    s32.save_state(tmp_path / "b.bin")
    ef = f_error(vxstate.read_state(tmp_path / "b.bin"), vxstate.read_state(tmp_path / "a.bin"))
    assert ef <= 1e-7, ef
    s32.close()
    s64.close()


@pytest.mark.gpu
def test_fp32_state_roundtrip(ctx, tmp_path):
    from veritas_gb300 import SolverManager

    s = SolverManager(ctx, problem_for_precision(problem_for("beam2"), 32))
    s.Advance(s.CalculateDt())
    s.save_state(tmp_path / "a.bin")
    s.load_state(tmp_path / "a.bin")
    s.save_state(tmp_path / "b.bin")
    assert (tmp_path / "a.bin").read_bytes() == (tmp_path / "b.bin").read_bytes()
    s.close()


@pytest.mark.gpu
def test_fp32_full_size_amr_runs_and_conserves():
    """Config-2 size in the FP32 form: mass conserved to FP32 rounding, fields finite."""
    import os
    import tempfile

    from veritas_gb300 import Context, SolverManager
    import bench

    c = Context(0)
    s = SolverManager(c, problem_for_precision(bench.problem_config2(), 32))
    with tempfile.TemporaryDirectory() as td:
        s.save_state(os.path.join(td, "a.bin"))
        st0 = vxstate.read_state(os.path.join(td, "a.bin"))
        for _ in range(3):
            s.Advance(s.CalculateDt())
        s.save_state(os.path.join(td, "b.bin"))
        st1 = vxstate.read_state(os.path.join(td, "b.bin"))
    base0 = st0["species"][0][-1][0]["f"][2:-2, 2:-2, 0].sum()
    base1 = st1["species"][0][-1][0]["f"][2:-2, 2:-2, 0].sum()
    assert abs(base1 - base0) <= 1e-5 * abs(base0)
    for k in ("By", "Bz", "Ey", "Ez", "phi"):
        assert np.all(np.isfinite(st1[k]))
    s.close()
    c.close()
