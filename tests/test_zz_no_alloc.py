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


def _bound(torch, s, prob, n_override=None):
    """Calls the no-alloc entry point on device copies of the run's current fields."""
    n = s.field("Ex").size
    dev = {k: torch.from_numpy(s.field(k)[:n].copy()).cuda() for k in ("Ay", "Az", "By", "Bz", "Ex")}
    torch.cuda.synchronize()
    mc = ME * CS
    q = (ctypes.c_double * 1)(QE)
    m = (ctypes.c_double * 1)(ME)
    dp0 = (ctypes.c_double * 1)(2.0 * prob.pmax * mc / prob.np)  # one level: the base dp
    dx0 = prob.L * prob.lambda_ / prob.nx
    dt = ctypes.c_double()
    rc = _fn()(*(ctypes.c_void_p(dev[k].data_ptr()) for k in ("Ay", "Az", "By", "Bz", "Ex")),
               n if n_override is None else n_override, q, m, dp0, 1, dx0, prob.cfl, None, ctypes.byref(dt))
    return rc, dt.value


@pytest.mark.gpu
def test_noalloc_cfl_equals_run_bound_twice():
    torch = pytest.importorskip("torch")
    from veritas_gb300 import Context, SolverManager

    prob = problem_for("slab64")
    ctx = Context(0)
    s = SolverManager(ctx, prob)
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
