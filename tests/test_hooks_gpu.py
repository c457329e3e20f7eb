"""A user problem given only through the C hooks (vx_run_create_hooks) against the
reference build running the same user code behind its own Settings hooks, and the
per-class stage calls against vx_run_advance.

The problem (tests/hooks/sin2_problem.c) has two mobile species, vacuum pads of five
cells, a circularly polarised laser ramped by sin^2 (GetBY and GetBZ), an x-dependent
electron drift and a RefinementOverride window; nothing of it is compiled into the
library.  Bar: 1e-10 relative L-inf, layouts identical (bit-exact is expected)."""
import numpy as np
import pytest

import vxstate
from helpers import case_args, compare_states, golden, golden_named, problem_for

TOL = 1e-10


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


def _hooks_run(ctx, name="sin2hooks"):
    from hooks.loader import sin2_hooks
    from veritas_gb300 import SolverManager

    h, prm = sin2_hooks(case_args(name))
    s = SolverManager(ctx, None, hooks=h)
    s._keep = prm  # the parameter block the hooks' user pointer refers to
    return s


def _check(got, ref, label):
    err = compare_states(got, ref, TOL)
    print(label, {k: f"{v:.2e}" for k, v in err.items()})
    for k, v in err.items():
        assert v <= TOL, (k, v)


def _state(s, path):
    s.save_state(path)
    return vxstate.read_state(path)


@pytest.mark.gpu
def test_hooks_initial_hierarchy(ctx, tmp_path):
    s = _hooks_run(ctx)
    _check(_state(s, tmp_path / "i.bin"), golden("sin2hooks", 0), "init")
    st = s.settings()
    assert st.nspecies == 2 and st.maxDepth == 1 and st.fMax[0] > 0
    s.close()


@pytest.mark.gpu
def test_hooks_steps(ctx, tmp_path):
    s = _hooks_run(ctx)
    vxstate.write_state(golden("sin2hooks", 0), tmp_path / "in.bin")
    s.load_state(tmp_path / "in.bin")
    ref1 = golden("sin2hooks", 1)
    s.Advance(ref1["dt"])
    _check(_state(s, tmp_path / "a.bin"), ref1, "step 1")
    for _ in range(2):
        s.Advance(s.CalculateDt())
    _check(_state(s, tmp_path / "b.bin"), golden("sin2hooks", 3), "step 3 (own dt)")
    s.close()


@pytest.mark.gpu
def test_hooks_regrid(ctx, tmp_path):
    s = _hooks_run(ctx)
    vxstate.write_state(golden_named("sin2hooks", "pre"), tmp_path / "pre.bin")
    s.load_state(tmp_path / "pre.bin")
    s.reGrid()
    _check(_state(s, tmp_path / "post.bin"), golden_named("sin2hooks", "post"), "regrid")
    ref = golden_named("sin2hooks", "post1")
    s.Advance(ref["dt"])
    _check(_state(s, tmp_path / "post1.bin"), ref, "step after regrid")
    s.close()


def _composed_step(s, dt):
    """SolverManager::Advance (SolverManager.cpp:28-39) from the per-class calls."""
    for st in range(6):
        s.moments()
        s.poisson()
        s.vlasov_stage(st, dt)
        s.update_time(st, dt)
        s.maxwell_stage(st, dt)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sin2hooks", "beam2", "ions2", "slab64"])
def test_per_class_calls_equal_advance(ctx, tmp_path, name):
    """One step composed of vx_run_moments / _poisson / _vlasov_stage / _update_time /
    _maxwell_stage equals vx_run_advance byte for byte and the reference's next state."""
    from veritas_gb300 import SolverManager

    def make():
        return _hooks_run(ctx) if name == "sin2hooks" else SolverManager(ctx, problem_for(name))

    vxstate.write_state(golden(name, 0), tmp_path / "in.bin")
    ref = golden(name, 1)
    a, b = make(), make()
    a.load_state(tmp_path / "in.bin")
    b.load_state(tmp_path / "in.bin")
    a.Advance(ref["dt"])
    _composed_step(b, ref["dt"])
    a.save_state(tmp_path / "a.bin")
    b.save_state(tmp_path / "b.bin")
    assert (tmp_path / "a.bin").read_bytes() == (tmp_path / "b.bin").read_bytes()
    _check(vxstate.read_state(tmp_path / "b.bin"), ref, name + " composed")
    a.close()
    b.close()


@pytest.mark.gpu
def test_sub_steps_in_parts_equal_whole(ctx, tmp_path):
    """vlasov_stage's sub-step bits run separately give the whole stage's result."""
    from veritas_gb300 import SUB_COPY, SUB_FLUX, SUB_LIMIT, SUB_UPDATE, SolverManager

    vxstate.write_state(golden("beam2", 0), tmp_path / "in.bin")
    dt = golden("beam2", 1)["dt"]
    a, b = SolverManager(ctx, problem_for("beam2")), SolverManager(ctx, problem_for("beam2"))
    for s in (a, b):
        s.load_state(tmp_path / "in.bin")
    _composed_step(a, dt)
    for st in range(6):
        b.moments()
        b.poisson()
        for bit in (SUB_FLUX, SUB_LIMIT, SUB_UPDATE, SUB_COPY):
            b.vlasov_stage(st, dt, bit)
        b.update_time(st, dt)
        b.maxwell_stage(st, dt)
    a.save_state(tmp_path / "a.bin")
    b.save_state(tmp_path / "b.bin")
    assert (tmp_path / "a.bin").read_bytes() == (tmp_path / "b.bin").read_bytes()
    a.close()
    b.close()


@pytest.mark.gpu
def test_flag_matches_error_estimate_and_override(ctx, tmp_path):
    """vx_run_flag on the pre-regrid state: every flagged cell has ErrorEstimate > crit
    (restated in numpy, Rectangle.hpp:128-130, weights Rectangle.cpp:68-74) or lies in the
    problem's RefinementOverride window, and every cell that satisfies either is flagged."""
    s = _hooks_run(ctx)
    pre = golden_named("sin2hooks", "pre")
    vxstate.write_state(pre, tmp_path / "pre.bin")
    s.load_state(tmp_path / "pre.bin")
    st = s.settings()
    prm = s._keep
    r = st.refinementRatio
    lam, me, c = 1e-6, 9.10938291e-31, 299792458.0
    for sp in range(2):
        for depth in range(st.maxDepth + 1):
            got = s.flag(sp, depth)
            want = []
            for R in _level(pre, sp, depth, st.maxDepth):
                f = R["f"][..., 1]
                fm = st.fMax[sp]
                w = [0.5 / fm * r ** (-0.5 * depth), 0.5 / fm * r ** (-0.5 * depth), 0.5 / fm * r ** (-2.0 * depth),
                     0.5 / fm * r ** (-2.0 * depth), st.sizeWeight / fm * r ** (-st.maxDepth + depth)]
                band = 3 * sum(r ** k for k in range(st.maxDepth - depth + 1))
                xs = st.x_size * r ** (st.maxDepth - depth)
                ps = st.p_size[sp] * r ** (st.maxDepth - depth)
                dx = r ** (depth - st.maxDepth) * st.dx
                dp = r ** (depth - st.maxDepth) * st.dp[sp]
                for i in range(max(R["x_pos"], band), min(R["x_pos"] + R["n_x"], xs - band)):
                    for j in range(max(R["p_pos"], band), min(R["p_pos"] + R["n_p"], ps - band)):
                        a, b = i - R["x_pos"] + 2, j - R["p_pos"] + 2
                        e = (w[0] * abs(f[a + 1, b] - f[a - 1, b]) + w[1] * abs(f[a, b + 1] - f[a, b - 1])
                             + w[2] * abs(f[a + 1, b] - 2 * f[a, b] + f[a - 1, b])
                             + w[3] * abs(f[a, b + 1] - 2 * f[a, b] + f[a, b - 1]) + w[4] * abs(f[a, b]))
                        x, p = (i + 0.5) * dx, st.pmin[sp] + dp * j
                        ovr = sp == 0 and prm.ref_x0 <= x / lam <= prm.ref_x1 and abs(p) < prm.ref_p * me * c
                        if e > st.refinementCriteria or ovr:
                            want.append((i, j))
            assert got == want, (sp, depth, len(got), len(want))
    s.close()


def _level(state, sp, depth, max_depth):
    """Patches of one depth from a state dict (levels listed finest first: index = depth)."""
    return state["species"][sp][depth]
