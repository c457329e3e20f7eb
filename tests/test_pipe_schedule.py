"""The read schedule of the pipelined FP64 moments + Poisson launch, on CPU.

The pipelined solve (k64_moments_poisson) gathers each row's right-hand side in the
staging of the forward chunk that first reads it, while the sweep runs the chunk before.
PoissonLU::first_read_chunk computes that chunk from the sweep's read pattern; the checker
(tests/native/pipe_schedule_check.cpp) derives the first read of every row independently
from the factor's band form, for sizes from 5 to 16384 rows, and requires the two to agree
and no gathered row to be one the sweep writes beside the gather.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_pipelined_solve_read_schedule(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    csrc = ROOT / "veritas_gb300" / "csrc"
    exe = tmp_path / "pipe_schedule_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(csrc),
                    str(ROOT / "tests" / "native" / "pipe_schedule_check.cpp"), str(csrc / "poisson_lu.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "consistent" in r.stdout
