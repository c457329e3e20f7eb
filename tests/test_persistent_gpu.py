"""Persistent stage form of FP32 launch sets: the same bits as one launch per sub-step.

With the persistent form on, each RK stage of an FP32 set is three launches (a
cooperative kernel for the moments and the rho/J assembly, the Poisson solve, and a
cooperative kernel for the whole FCT stage with the Maxwell stage beside it); every phase
runs the same device body as the per-sub-step kernel that does it in the default form, so
the states must be byte-identical — alone, batched and across a regrid.  A grid barrier
whose wait runs out must come back as VX_ERR_TIMEOUT at the next synchronisation, with
the context still usable.
"""
import dataclasses

import pytest

from helpers import problem_for

NAMES = ["slab64", "amr2", "drift128", "beam2", "ragged2", "ions2", "beam3"]


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.set_persistent(False)
    c.close()


def _states(ctx, tmp_path, tag, probs, steps, persistent, batched, regrid_after=None):
    from veritas_gb300 import SolverManager, advance_many, calculate_dt_many

    ctx.set_persistent(persistent)
    sms = [SolverManager(ctx, p) for p in probs]
    for step in range(steps):
        if batched:
            advance_many(sms, calculate_dt_many(sms))
        else:
            for s in sms:
                s.Advance(s.CalculateDt())
        if step == regrid_after:
            for s in sms:
                s.reGrid()
    out = []
    for k, s in enumerate(sms):
        path = tmp_path / f"{tag}{k}.bin"
        s.save_state(path)
        out.append(path.read_bytes())
        s.close()
    ctx.set_persistent(False)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [False, True])
def test_persistent_equals_per_substep(ctx, tmp_path, batched):
    probs = [dataclasses.replace(problem_for(n), precision=32) for n in NAMES]
    ref = _states(ctx, tmp_path, "a", probs, 3, False, batched)
    got = _states(ctx, tmp_path, "b", probs, 3, True, batched)
    for n, a, b in zip(NAMES, ref, got):
        assert a == b, n


@pytest.mark.gpu
def test_persistent_across_regrid(ctx, tmp_path):
    probs = [dataclasses.replace(problem_for(n), precision=32) for n in ("amr2", "beam3", "ions2")]
    ref = _states(ctx, tmp_path, "a", probs, 3, False, True, regrid_after=1)
    got = _states(ctx, tmp_path, "b", probs, 3, True, True, regrid_after=1)
    assert ref == got


@pytest.mark.gpu
def test_persistent_three_launches_per_stage(ctx):
    from veritas_gb300 import SolverManager

    ctx.set_persistent(True)
    s = SolverManager(ctx, dataclasses.replace(problem_for("beam2"), precision=32))
    s.Advance(s.CalculateDt())
    ctx.sync()
    k0 = ctx.kernel_launches()
    s.Advance(s.CalculateDt())
    ctx.sync()
    launches = ctx.kernel_launches() - k0 - 1  # minus the CFL kernel
    s.close()
    ctx.set_persistent(False)
    assert launches == 18  # 6 stages x (stage_pre, Poisson, stage_fct)


@pytest.mark.gpu
def test_persistent_barrier_timeout_reported(ctx, tmp_path):
    from veritas_gb300 import SolverManager, VxError

    p = dataclasses.replace(problem_for("amr2"), precision=32)
    ctx.set_persistent(True)
    # every barrier waits for one arrival more than the grid makes: the first wait runs out
    # after 2 ms, the rest of the step passes its barriers without waiting
    ctx.set_persistent_limit(2_000_000, 1)
    s = SolverManager(ctx, p)
    s.Advance(s.CalculateDt())
    with pytest.raises(VxError) as e:
        ctx.sync()
    assert e.value.code == -6
    s.close()
    ctx.set_persistent_limit()
    ctx.sync()  # the record was cleared
    # the context stays usable: a fresh run gives the per-sub-step form's bits
    ref = _states(ctx, tmp_path, "a", [p], 2, False, False)
    got = _states(ctx, tmp_path, "b", [p], 2, True, False)
    assert ref == got
