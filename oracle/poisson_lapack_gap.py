"""ORACLE / TEST INFRASTRUCTURE — how far apart LAPACK's LU variants put the reference's
Poisson solution.

The reference factorises its dense Poisson matrix (EMSolver.cpp:28-88) with dgetrf and
solves with dgetrs every stage (EMSolver.cpp:156-192); which LAPACK it links decides the
rounding.  This script takes the workload's charge after a few steps of the oracle port
(the port solves with the unblocked right-looking LU, oracle/lu_exact.hpp, bit-identical
to the reference build that links the same restatement) and solves the same system with
SciPy's OpenBLAS dgetrf/dgetrs (a blocked LU, what a non-MKL build of the reference links)
and with iterative refinement on longdouble residuals (the exact solution of the discrete
system, to far below double rounding).  It prints the relative L-inf gaps in phi and in
E_x (the reference's 4th-order difference, GetEfield EMSolver.cpp:137-154, without Ex0).

  python oracle/poisson_lapack_gap.py [workload ...]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

EPS0_INV = 1.1294e+11  # veritas.hpp:22


def reference_matrix(n: int) -> np.ndarray:
    """The matrix as LAPACK reads the reference's pM (column-major, EMSolver.cpp:41-67)."""
    w1, w2, w3 = -16.0 / 30.0 / 0.4, 1.0 / 30.0 / 0.4, 1 / 0.4
    P = np.zeros((n, n))
    for i in range(2, n - 2):
        P[i, i], P[i, i + 1], P[i, i - 1], P[i, i + 2], P[i, i - 2] = w3, w1, w1, w2, w2
    P[0, 0] = 1.0
    P[1, 1], P[1, 2], P[1, 0], P[1, 3], P[1, n - 1] = w3, w1, w1, w2, w2
    P[n - 2, n - 2], P[n - 2, n - 1], P[n - 2, n - 3], P[n - 2, 0], P[n - 2, n - 4] = w3, w1, w1, w2, w2
    P[n - 1, n - 1], P[n - 1, 0], P[n - 1, n - 2], P[n - 1, 1], P[n - 1, n - 3] = w3, w1, w1, w2, w2
    return P.T.copy()


def efield(phi: np.ndarray, dx: float) -> np.ndarray:
    n = phi.size
    i = np.arange(n)
    return -(1.0 / (12 * dx)) * (8 * (phi[(i + 1) % n] - phi[(i - 1) % n]) - phi[(i + 2) % n] + phi[(i - 2) % n])


def measure(workload: str, steps: int = 20, threads: int | None = None) -> dict:
    from scipy.linalg import lapack

    import vxstate
    from helpers import port_exe
    from veritas_gb300.workloads import WORKLOADS

    p = WORKLOADS[workload]()
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, OMP_NUM_THREADS=str(threads or os.cpu_count() or 1))
        subprocess.run([str(port_exe()), *p.harness_args(), f"steps={steps}", f"dump_every={steps}", f"dumpdir={td}"],
                       check=True, capture_output=True, env=env)
        st = vxstate.read_state(Path(td) / f"state_{steps:05d}.bin")
    n = st["phi"].size
    dx = p.L * p.lambda_ / p.nx / p.r ** (p.Lfinest - 1)
    b = EPS0_INV * (st["charge"] + st["neut"])  # UpdatePotential's right-hand side
    b = b * dx ** 2
    A = reference_matrix(n)
    lu, piv, info = lapack.dgetrf(A)
    assert info == 0
    x_blocked, info = lapack.dgetrs(lu, piv, b)
    x_unblocked = st["phi"]
    Al, bl, xl = A.astype(np.longdouble), b.astype(np.longdouble), x_blocked.astype(np.longdouble)
    for _ in range(6):
        d, _ = lapack.dgetrs(lu, piv, np.asarray(bl - Al @ xl, dtype=np.float64))
        xl = xl + d.astype(np.longdouble)
    x_exact = np.asarray(xl, dtype=np.float64)
    sp, se = np.max(np.abs(x_exact)), np.max(np.abs(efield(x_exact, dx)))

    def gaps(x, y):
        return (float(np.max(np.abs(x - y)) / sp), float(np.max(np.abs(efield(x, dx) - efield(y, dx))) / se))

    out = {"n": n, "steps": steps}
    for k, (x, y) in {"blocked_vs_unblocked": (x_blocked, x_unblocked), "blocked_vs_exact": (x_blocked, x_exact),
                      "unblocked_vs_exact": (x_unblocked, x_exact)}.items():
        out[k] = dict(zip(("phi", "Ex"), gaps(x, y)))
    return out


if __name__ == "__main__":
    for w in sys.argv[1:] or ["laser_slab_2048x256", "laser_slab_amr_4096x512"]:
        r = measure(w)
        print(w, "n =", r["n"])
        for k in ("blocked_vs_unblocked", "blocked_vs_exact", "unblocked_vs_exact"):
            print(f"  {k:22s} phi {r[k]['phi']:.2e}  E_x {r[k]['Ex']:.2e}")
