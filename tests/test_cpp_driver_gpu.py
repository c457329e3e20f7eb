"""The C++ host interface (include/veritas_gb300.hpp) end to end: the stand-alone driver
veritas_gb300_run steps a solve from t = 0 with its own CFL time step — and regrids —
through SolverManager::CalculateDt / Advance / reGrid, and its final state must equal
the reference's dump of the same run (1e-10 relative, observed exact)."""
import os
import subprocess
from pathlib import Path

import pytest

import vxstate
from helpers import case_args, compare_states, golden, golden_named

DRIVER = Path(__file__).resolve().parent.parent / "veritas_gb300" / "veritas_gb300_run"
TOL = 1e-10


def _run(tmp_path, name, *extra):
    args = [f"{k}={v}" for k, v in case_args(name).items()]
    out = tmp_path / "final.bin"
    r = subprocess.run([str(DRIVER), *args, *extra, f"dump={out}"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return vxstate.read_state(out)


def _check(got, ref):
    err = compare_states(got, ref, TOL)
    for k, v in err.items():
        assert v <= TOL, (k, v)


@pytest.mark.gpu
def test_driver_steps_match_reference(tmp_path):
    assert DRIVER.exists(), "run __graft_entry__.build() first"
    _check(_run(tmp_path, "amr2", "steps=3"), golden("amr2", 3))


@pytest.mark.gpu
def test_driver_regrid_matches_reference(tmp_path):
    _check(_run(tmp_path, "beam2", "steps=5", "regrid_every=4"), golden_named("beam2", "post1"))
