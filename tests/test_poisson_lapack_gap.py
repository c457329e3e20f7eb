"""The LU variant question on CPU: a blocked LAPACK LU (SciPy's OpenBLAS) and the
unblocked LU the reference build is pinned to put the one-level workload's potential
within 1e-10 of each other, and each within 1e-10 of the exact discrete solution (E_x
relative to its largest value).  oracle/poisson_lapack_gap.py prints the same gaps at
n = 8192."""
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))


def test_lapack_variants_agree_at_n2048():
    pytest.importorskip("scipy")
    import poisson_lapack_gap as g

    r = g.measure("laser_slab_2048x256", steps=5)
    assert r["n"] == 2048
    for k in ("blocked_vs_unblocked", "blocked_vs_exact", "unblocked_vs_exact"):
        assert r[k]["Ex"] < 1e-10, (k, r[k])
    # the two LAPACK variants are closer to each other than either is to the exact solution
    assert r["blocked_vs_unblocked"]["phi"] < r["unblocked_vs_exact"]["phi"]
