"""The CFL bound entry point that allocates no device memory, against the run's own.

vx_cfl_bound_noalloc serves callers that cannot allocate device memory — a time-step
controller running beside solves whose memory is committed up front, or one that must
not cause the synchronisation cudaMalloc / cudaFree may imply.  It takes device field
arrays the caller already owns; here they are device copies of a run's fields, and the
result must equal vx_run_calculate_dt's for the same state (the tolerance of the parity
tests, 1e-10 relative; the arithmetic is the same, so it is expected to be exact) on two
calls in a row with the state advanced in between.  It must also refuse grids beyond its
fixed scratch.  This file is collected last so that a stop at its first failure has run
everything else.
"""
import ctypes
import dataclasses

import pytest

from helpers import problem_for

TOL = 1e-10
ME, QE, CS = 9.10938291e-31, -1.60217657e-19, 299792458.0


def _fn():
    from veritas_gb300 import lib

    f = lib().vx_cfl_bound_noalloc
    d = ctypes.POINTER(ctypes.c_double)
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, d, d, d, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_void_p, d]
    f.restype = ctypes.c_int
    return f


def _species(prob):
    """(q, m, finest-level dp) per species, as EMFieldSolver::EstimateCFLBound reads them
    (Settings::GetDp(0, i) = r^-maxDepth times the base dp)."""
    mc = ME * CS
    fine = float(prob.r) ** -(prob.Lfinest - 1)
    out = [(QE, ME, 2.0 * prob.pmax * mc / prob.np * fine)]
    if prob.mi > 0:
        mi = prob.mi * ME
        out.append((-QE, mi, 2.0 * prob.ipmax * mi * CS / prob.np * fine))
    return out


def _bound(torch, s, prob, n_override=None):
    """Calls the no-alloc entry point on device copies of the run's current fields."""
    n = s.field("Ex").size
    dev = {k: torch.from_numpy(s.field(k)[:n].copy()).cuda() for k in ("Ay", "Az", "By", "Bz", "Ex")}
    torch.cuda.synchronize()
    sp = _species(prob)
    q = (ctypes.c_double * len(sp))(*(x[0] for x in sp))
    m = (ctypes.c_double * len(sp))(*(x[1] for x in sp))
    dp0 = (ctypes.c_double * len(sp))(*(x[2] for x in sp))
    dx0 = prob.L * prob.lambda_ / prob.nx / float(prob.r) ** (prob.Lfinest - 1)
    dt = ctypes.c_double()
    rc = _fn()(*(ctypes.c_void_p(dev[k].data_ptr()) for k in ("Ay", "Az", "By", "Bz", "Ex")),
               n if n_override is None else n_override, q, m, dp0, len(sp), dx0, prob.cfl, None, ctypes.byref(dt))
    return rc, dt.value


def _free_bytes(torch):
    free, _ = torch.cuda.mem_get_info()
    return free


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["slab64", "ions2_wide"])
def test_noalloc_cfl_equals_run_bound_twice(case):
    """One level and one species (a single block of 256 cells), and two levels with two
    species on a 512-cell finest grid (two blocks folded, the species loop, the
    finest-level dp)."""
    torch = pytest.importorskip("torch")
    from veritas_gb300 import Context, SolverManager

    prob = problem_for("slab64") if case == "slab64" else dataclasses.replace(problem_for("ions2"), nx=256)
    ctx = Context(0)
    s = SolverManager(ctx, prob)
    assert s.field("Ex").size > (256 if case != "slab64" else 0)
    for _ in range(2):
        s.Advance(s.CalculateDt())
    for call in range(2):
        rc, dt = _bound(torch, s, prob)
        assert rc == 0
        ref = s.CalculateDt()
        assert abs(dt - ref) <= TOL * ref, (call, dt, ref)
        s.Advance(ref)  # the second call sees a different state
    s.close()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_cfl_allocates_nothing():
    """Once the first call has looked up its scratch, a call leaves the device's free
    memory exactly as it was."""
    torch = pytest.importorskip("torch")
    from veritas_gb300 import Context, SolverManager

    prob = problem_for("slab64")
    ctx = Context(0)
    s = SolverManager(ctx, prob)
    rc, _ = _bound(torch, s, prob)  # first call on the device: symbol lookup
    assert rc == 0
    n = s.field("Ex").size
    dev = {k: torch.from_numpy(s.field(k)[:n].copy()).cuda() for k in ("Ay", "Az", "By", "Bz", "Ex")}
    sp = _species(prob)
    q, m, dp0 = ((ctypes.c_double * 1)(sp[0][i]) for i in range(3))
    dt = ctypes.c_double()
    torch.cuda.synchronize()
    before = _free_bytes(torch)
    for _ in range(3):
        rc = _fn()(*(ctypes.c_void_p(dev[k].data_ptr()) for k in ("Ay", "Az", "By", "Bz", "Ex")), n, q, m, dp0, 1,
                   prob.L * prob.lambda_ / prob.nx, prob.cfl, None, ctypes.byref(dt))
        assert rc == 0
    assert _free_bytes(torch) == before
    s.close()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_cfl_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from veritas_gb300 import Context, SolverManager, lib

    prob = problem_for("slab64")
    ctx = Context(0)
    s = SolverManager(ctx, prob)
    rc, _ = _bound(torch, s, prob, n_override=(1 << 20) + 1)
    assert rc == -1
    assert b"exceeds the limit" in lib().vx_last_error()
    s.close()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_cfl_rejects_bad_species_values():
    torch = pytest.importorskip("torch")
    from veritas_gb300 import lib

    dev = torch.zeros(64, dtype=torch.float64, device="cuda")
    dt = ctypes.c_double()
    for bad in ((QE, ME, 0.0), (QE, 0.0, 1e-24), (QE, float("nan"), 1e-24)):
        q, m, dp0 = ((ctypes.c_double * 1)(bad[i]) for i in range(3))
        rc = _fn()(*([ctypes.c_void_p(dev.data_ptr())] * 5), 64, q, m, dp0, 1, 1e-8, 0.5, None, ctypes.byref(dt))
        assert rc == -1
        assert b"finite positive" in lib().vx_last_error()
