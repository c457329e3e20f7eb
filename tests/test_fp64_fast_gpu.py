"""The fast FP64 form (vx_problem.fast = 1: the FCT kernels with fused multiply-add and
the WENO weights from one ratio) against the reference's states.

It gives up the reference's rounding, not its precision: after one step from every
fixture state the f slots and every field array stay within 1e-10 relative L-inf of the
reference build (the plain path's bar), and on the benchmarked sizes f and the transverse
fields stay within 1e-10 of the oracle port after two steps.  The patch layouts are
untouched (the step does not regrid)."""
import dataclasses

import numpy as np
import pytest

import vxstate
from helpers import compare_states, golden, port_exe, problem_for

TOL = 1e-10
ONE_STEP = [("slab64", 0), ("drift128", 0), ("edge64", 0), ("amr2", 0), ("beam2", 0), ("beam3", 0), ("ions2", 0),
            ("ragged2", 0)]


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", ONE_STEP)
def test_fast_form_one_step_within_bar(ctx, tmp_path, name, k):
    from veritas_gb300 import SolverManager

    s = SolverManager(ctx, dataclasses.replace(problem_for(name), fast=1))
    vxstate.write_state(golden(name, k), tmp_path / "in.bin")
    s.load_state(tmp_path / "in.bin")
    ref = golden(name, k + 1)
    s.Advance(ref["dt"])
    s.save_state(tmp_path / "out.bin")
    err = compare_states(vxstate.read_state(tmp_path / "out.bin"), ref, TOL)
    print(name, {kk: f"{v:.2e}" for kk, v in err.items()})
    for kk, v in err.items():
        assert v <= TOL, (kk, v)
    s.close()


@pytest.mark.gpu
def test_fast_form_differs_from_exact_form(ctx, tmp_path):
    """The two forms are different kernels: their states after a step are not identical."""
    from veritas_gb300 import SolverManager

    out = []
    for fast in (0, 1):
        s = SolverManager(ctx, dataclasses.replace(problem_for("beam2"), fast=fast))
        vxstate.write_state(golden("beam2", 0), tmp_path / "in.bin")
        s.load_state(tmp_path / "in.bin")
        s.Advance(golden("beam2", 1)["dt"])
        s.save_state(tmp_path / f"o{fast}.bin")
        out.append((tmp_path / f"o{fast}.bin").read_bytes())
        s.close()
    assert out[0] != out[1]


@pytest.mark.gpu
@pytest.mark.parametrize("workload", ["laser_slab_2048x256", "laser_slab_amr_4096x512"])
def test_fast_form_at_benchmark_size(ctx, tmp_path, workload):
    """Both forms from the same initial hierarchy, two steps with the exact form's dt; f and
    the transverse fields of the fast form within 1e-10 of the oracle port."""
    import subprocess

    from veritas_gb300 import SolverManager
    from veritas_gb300.workloads import WORKLOADS

    p = WORKLOADS[workload]()
    a = SolverManager(ctx, p)
    a.save_state(tmp_path / "init.bin")
    dts = [a.CalculateDt()]
    a.Advance(dts[0])
    dts.append(a.CalculateDt())
    a.close()
    b = SolverManager(ctx, dataclasses.replace(p, fast=1))
    b.load_state(tmp_path / "init.bin")
    for dt in dts:
        b.Advance(dt)
    b.save_state(tmp_path / "fast.bin")
    b.close()
    subprocess.run([str(port_exe()), *p.harness_args(), f"load={tmp_path / 'init.bin'}",
                    "dts=" + ",".join(repr(d) for d in dts), "steps=2", "dump_every=2", f"dumpdir={tmp_path}"],
                   check=True, capture_output=True)
    err = compare_states(vxstate.read_state(tmp_path / "fast.bin"), vxstate.read_state(tmp_path / "state_00002.bin"),
                         TOL)
    print(workload, {k: f"{v:.2e}" for k, v in err.items()})
    for k in ("f", "By", "Bz", "Ey", "Ez", "Ay", "Az", "a_squared", "time"):
        assert err[k] <= TOL, (k, err[k])
