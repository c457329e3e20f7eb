"""Pipelined moments and exact Poisson solve of FP64 runs: the same bits as separate kernels.

With the pipelined form on (the default), each RK stage of an FP64 run with the exact
solve launches the moments, the rho/J assembly and the solve as one kernel whose solve
block starts its forward sweep as soon as the moment columns of its first rows are done,
and assembles rho and J row chunk by row chunk.  The arithmetic is that of the separate
k64_moments, k_assemble and k_poisson kernels, so the states must be byte-identical —
alone, in sets of up to four runs, across a regrid and on the benchmarked two-level
4096 x 512 workload.  A wait of the solve that runs out must come back as VX_ERR_TIMEOUT
at the next synchronisation, with the context still usable.
"""
import pytest

from helpers import problem_for

NAMES = ["slab64", "amr2", "drift128", "edge64", "beam2", "ragged2", "ions2", "beam3"]


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.set_pipelined(True)
    c.set_persistent_limit()
    c.close()


def _states(ctx, tmp_path, tag, probs, steps, pipelined, batched, regrid_after=None):
    from veritas_gb300 import SolverManager, advance_many, calculate_dt_many

    ctx.set_pipelined(pipelined)
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
    ctx.set_pipelined(True)
    return out


@pytest.mark.gpu
def test_pipelined_equals_separate_kernels(ctx, tmp_path):
    probs = [problem_for(n) for n in NAMES]
    ref = _states(ctx, tmp_path, "a", probs, 3, False, False)
    got = _states(ctx, tmp_path, "b", probs, 3, True, False)
    for n, a, b in zip(NAMES, ref, got):
        assert a == b, n


@pytest.mark.gpu
def test_pipelined_sets_of_runs(ctx, tmp_path):
    """Two and four runs of different sizes in one launch (their units interleaved by the
    chunk that first needs them, one solve block per run)."""
    for names in (["amr2", "ions2"], ["slab64", "beam2", "ragged2", "beam3"]):
        probs = [problem_for(n) for n in names]
        ref = _states(ctx, tmp_path, "a", probs, 2, False, True)
        got = _states(ctx, tmp_path, "b", probs, 2, True, True)
        for n, a, b in zip(names, ref, got):
            assert a == b, n


@pytest.mark.gpu
def test_pipelined_across_regrid(ctx, tmp_path):
    probs = [problem_for(n) for n in ("amr2", "beam3", "ions2")]
    ref = _states(ctx, tmp_path, "a", probs, 3, False, False, regrid_after=1)
    got = _states(ctx, tmp_path, "b", probs, 3, True, False, regrid_after=1)
    assert ref == got


@pytest.mark.gpu
def test_pipelined_at_benchmark_size(ctx, tmp_path):
    """The two-level 4096 x 512 workload (finest n = 8192: 32 row chunks, hundreds of
    moment units), two steps each way."""
    from veritas_gb300.workloads import laser_slab_amr_4096x512

    p = laser_slab_amr_4096x512()
    ref = _states(ctx, tmp_path, "a", [p], 2, False, False)
    got = _states(ctx, tmp_path, "b", [p], 2, True, False)
    assert ref == got


@pytest.mark.gpu
def test_pipelined_launch_count(ctx):
    """One launch instead of moments + assembly + solve: two launches fewer per stage."""
    from veritas_gb300 import SolverManager

    counts = []
    for on in (False, True):
        ctx.set_pipelined(on)
        s = SolverManager(ctx, problem_for("beam2"))
        s.Advance(s.CalculateDt())
        ctx.sync()
        k0 = ctx.kernel_launches()
        s.Advance(s.CalculateDt())
        ctx.sync()
        counts.append(ctx.kernel_launches() - k0)
        s.close()
    ctx.set_pipelined(True)
    assert counts[1] == counts[0] - 12, counts


@pytest.mark.gpu
def test_pipelined_wait_timeout_reported(ctx, tmp_path):
    from veritas_gb300 import SolverManager, VxError

    p = problem_for("amr2")
    ctx.set_pipelined(True)
    # every wait expects one unit more than the launch has: the first wait runs out after
    # 2 ms, the later ones pass at once; the moment units themselves always finish
    ctx.set_persistent_limit(2_000_000, 1)
    s = SolverManager(ctx, p)
    s.Advance(s.CalculateDt())
    with pytest.raises(VxError) as e:
        ctx.sync()
    assert e.value.code == -6
    s.close()
    ctx.set_persistent_limit()
    ctx.sync()  # the record was cleared
    # the context stays usable: a fresh run gives the separate kernels' bits
    ref = _states(ctx, tmp_path, "a", [p], 2, False, False)
    got = _states(ctx, tmp_path, "b", [p], 2, True, False)
    assert ref == got
