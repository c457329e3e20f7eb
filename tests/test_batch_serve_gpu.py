"""Batched and served forms: every solve's result is the same alone and in a mix.

The batched launch set runs one kernel per sub-step over all patches of all runs, and
the serving loop admits and retires solves between steps; neither lets one run's data
reach another's arithmetic, so the states must match bit for bit (both precisions).
"""
import dataclasses

import pytest

import vxstate
from helpers import golden, problem_for


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


def _bytes(s, path):
    s.save_state(path)
    return path.read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_batched_equals_separate(ctx, tmp_path, precision):
    from veritas_gb300 import SolverManager, advance_many, calculate_dt_many

    names = ["slab64", "amr2", "drift128", "beam2", "ragged2", "ions2"]
    probs = [dataclasses.replace(problem_for(n), precision=precision) for n in names]
    alone = [SolverManager(ctx, p) for p in probs]
    mixed = [SolverManager(ctx, p) for p in probs]
    for step in range(3):
        dts = calculate_dt_many(mixed)
        for s, dt in zip(alone, dts):
            assert s.CalculateDt() == dt
            s.Advance(dt)
        advance_many(mixed, dts)
    for k, (a, m) in enumerate(zip(alone, mixed)):
        assert _bytes(a, tmp_path / f"a{k}.bin") == _bytes(m, tmp_path / f"m{k}.bin"), names[k]
    for s in alone + mixed:
        s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_served_result_same_alone_and_in_mix(ctx, tmp_path, precision):
    from veritas_gb300 import Server

    X = dataclasses.replace(problem_for("amr2"), precision=precision)
    Y = dataclasses.replace(problem_for("drift128"), precision=precision)
    Z = dataclasses.replace(problem_for("beam3"), precision=precision)
    srv = Server(ctx, 8 << 30)
    rid = srv.submit(X, 3, state_path=tmp_path / "alone.bin")
    while srv.step() != (0, 0):
        pass
    assert srv.result(rid)["finished"] == 1
    srv.close()

    srv = Server(ctx, 8 << 30)
    ry = srv.submit(Y, 4)
    while srv.result(ry)["steps_done"] == 0:  # Y runs alone for a step
        srv.step()
    rx = srv.submit(X, 3, state_path=tmp_path / "mix.bin")  # joins while Y is live
    rz = srv.submit(Z, 2)
    while srv.step() != (0, 0):
        pass
    for r in (rx, ry, rz):
        assert srv.result(r)["finished"] == 1
    assert srv.result(rx)["admitted"] >= srv.result(ry)["admitted"]
    assert (tmp_path / "alone.bin").read_bytes() == (tmp_path / "mix.bin").read_bytes()
    srv.close()


@pytest.mark.gpu
def test_server_admits_by_memory_budget(ctx):
    """A budget that holds one solve at a time: the second waits for the first to retire."""
    from veritas_gb300 import Server

    P = problem_for("slab64")
    srv = Server(ctx, 1 << 30)
    a = srv.submit(P, 2)
    while srv.result(a)["device_bytes"] == 0:  # built on the server's thread, then bound
        srv.step()
    used = srv.result(a)["device_bytes"]
    srv.close()
    srv = Server(ctx, int(used * 1.5))
    a = srv.submit(P, 2)
    b = srv.submit(P, 2)
    while srv.step() != (0, 0):
        pass
    ra, rb = srv.result(a), srv.result(b)
    assert ra["finished"] and rb["finished"]
    assert rb["admitted"] >= ra["finish"]
    srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_autotuned_tiles_change_nothing(ctx, tmp_path, precision):
    """The tile shape the autotuner picks changes no arithmetic: results are identical to
    the default 32 x 8 tiles."""
    from veritas_gb300 import SolverManager, advance_many, autotune_many

    P = dataclasses.replace(problem_for("beam3"), precision=precision)
    a, b = SolverManager(ctx, P), SolverManager(ctx, P)
    for _ in range(2):
        a.Advance(a.CalculateDt())
    shape = autotune_many([b])
    assert shape[0] * shape[1] <= 1024
    for _ in range(2):
        b.Advance(b.CalculateDt())
    assert _bytes(a, tmp_path / "a.bin") == _bytes(b, tmp_path / "b.bin")
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_launch_mode_changes_nothing(ctx, tmp_path, precision):
    """Steps with and without the CUDA graph and programmatic dependent launch give the
    same bits (every kernel waits for its predecessor before touching memory)."""
    from veritas_gb300 import Problem, SolverManager

    out = []
    for graphs, pdl in ((True, True), (False, False), (True, False)):
        ctx.set_launch_mode(graphs=graphs, pdl=pdl)
        s = SolverManager(ctx, Problem(nx=512, np=64, Lfinest=2, precision=precision))
        for _ in range(3):
            s.Advance(s.CalculateDt())
        s.save_state(tmp_path / f"s{len(out)}.bin")
        out.append((tmp_path / f"s{len(out)}.bin").read_bytes())
        s.close()
    ctx.set_launch_mode(graphs=True, pdl=True)
    assert out[0] == out[1] == out[2]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
def test_served_solve_regrids_and_is_the_same_alone_and_in_mix(ctx, tmp_path, precision):
    """A served solve of 25 steps regrids after step 22 (the reference driver's rule:
    more than 20 steps since the last regrid); its final state is the same alone as in a
    mix with solves that join, regrid and retire around it, and equals a plain run that
    regrids at the same step."""
    from veritas_gb300 import Server, SolverManager

    X = dataclasses.replace(problem_for("beam2"), precision=precision)
    Y = dataclasses.replace(problem_for("amr2"), precision=precision)
    Z = dataclasses.replace(problem_for("ions2"), precision=precision)
    srv = Server(ctx, 8 << 30)
    rid = srv.submit(X, 25, state_path=tmp_path / "alone.bin")
    while srv.step() != (0, 0):
        pass
    r = srv.result(rid)
    assert r["status"] == 3 and r["regrids"] == 1 and r["steps_done"] == 25
    srv.close()

    srv = Server(ctx, 8 << 30)
    ry = srv.submit(Y, 30)
    while srv.result(ry)["steps_done"] < 5:
        srv.step()
    rx = srv.submit(X, 25, state_path=tmp_path / "mix.bin")
    rz = srv.submit(Z, 12)
    while srv.step() != (0, 0):
        pass
    assert [srv.result(k)["status"] for k in (rx, ry, rz)] == [3, 3, 3]
    assert srv.result(ry)["regrids"] == 1
    assert (tmp_path / "alone.bin").read_bytes() == (tmp_path / "mix.bin").read_bytes()
    srv.close()

    s = SolverManager(ctx, X)
    for k in range(25):
        s.Advance(s.CalculateDt())
        if k + 1 == 22:
            s.reGrid()
    assert _bytes(s, tmp_path / "plain.bin") == (tmp_path / "alone.bin").read_bytes()
    s.close()


@pytest.mark.gpu
def test_server_cancels_waiting_and_live_requests(ctx, tmp_path):
    """Cancelling a waiting request removes it from the queue; cancelling a live one
    retires it at once without writing its state; the others finish unaffected."""
    from veritas_gb300 import REQ_CANCELLED, REQ_DONE, Server

    P = problem_for("amr2")
    srv = Server(ctx, 8 << 30)
    keep = srv.submit(P, 40, state_path=tmp_path / "keep_alone.bin")
    while srv.step() != (0, 0):
        pass
    srv.close()

    srv = Server(ctx, 8 << 30, max_live=2)
    a = srv.submit(P, 40, state_path=tmp_path / "keep_mix.bin")
    b = srv.submit(problem_for("drift128"), 50, state_path=tmp_path / "never.bin")
    c = srv.submit(problem_for("slab64"), 4)  # waits while a and b hold both slots
    while srv.result(b)["steps_done"] < 2:
        srv.step()
    assert srv.result(a)["status"] == 2 and srv.result(c)["status"] == 0
    srv.cancel(c)
    srv.cancel(b)
    while srv.step() != (0, 0):
        pass
    ra, rb, rc = srv.result(a), srv.result(b), srv.result(c)
    assert ra["status"] == REQ_DONE and rb["status"] == REQ_CANCELLED and rc["status"] == REQ_CANCELLED
    assert rb["finished"] == 1 and 2 <= rb["steps_done"] < 50 and rc["steps_done"] == 0
    assert not (tmp_path / "never.bin").exists()
    assert (tmp_path / "keep_alone.bin").read_bytes() == (tmp_path / "keep_mix.bin").read_bytes()
    srv.close()


@pytest.mark.gpu
def test_server_cancels_a_solve_out_for_regrid(ctx, tmp_path):
    """A solve regrids on a worker thread, out of the batch; cancelled meanwhile, it is
    dropped when the regrid ends (the regrid not counted), and the solve beside it
    finishes with the same bits as alone."""
    from veritas_gb300 import REQ_CANCELLED, REQ_DONE, Server

    srv = Server(ctx, 8 << 30)
    srv.submit(problem_for("beam2"), 30, state_path=tmp_path / "alone.bin")
    while srv.step() != (0, 0):
        pass
    srv.close()

    srv = Server(ctx, 8 << 30)
    a = srv.submit(problem_for("amr2"), 40)
    k = srv.submit(problem_for("beam2"), 30, state_path=tmp_path / "mix.bin")
    while srv.result(a)["steps_done"] < 22:
        srv.step()
    srv.cancel(a)  # its regrid, due after step 22, was handed to a worker by that step
    while srv.step() != (0, 0):
        pass
    ra, rk = srv.result(a), srv.result(k)
    assert ra["status"] == REQ_CANCELLED and ra["finished"] == 1
    assert ra["steps_done"] == 22 and ra["regrids"] == 0
    assert rk["status"] == REQ_DONE and rk["regrids"] == 1
    assert (tmp_path / "alone.bin").read_bytes() == (tmp_path / "mix.bin").read_bytes()
    srv.close()


@pytest.mark.gpu
def test_server_retires_a_solve_gone_non_finite_alone(ctx, tmp_path):
    """A request whose laser amplitude is NaN (a bad host-side input) fails its health
    check after its first step and is retired alone; the solve stepping beside it in the
    same launches finishes with the same bits as alone."""
    from veritas_gb300 import REQ_DONE, REQ_FAILED, Server

    P = problem_for("amr2")
    bad = dataclasses.replace(problem_for("slab64"), a0=float("nan"))
    srv = Server(ctx, 8 << 30)
    srv.submit(P, 4, state_path=tmp_path / "alone.bin")
    while srv.step() != (0, 0):
        pass
    srv.close()
    srv = Server(ctx, 8 << 30)
    g = srv.submit(P, 4, state_path=tmp_path / "mix.bin")
    b = srv.submit(bad, 4)
    while srv.step() != (0, 0):
        pass
    rg, rb = srv.result(g), srv.result(b)
    assert rg["status"] == REQ_DONE
    assert rb["status"] == REQ_FAILED and "not finite" in rb["error"] and rb["steps_done"] <= 1
    assert (tmp_path / "alone.bin").read_bytes() == (tmp_path / "mix.bin").read_bytes()
    srv.close()


@pytest.mark.gpu
def test_server_refuses_a_request_larger_than_its_budget(ctx):
    from veritas_gb300 import Problem, Server, VxError

    srv = Server(ctx, 64 << 20)
    with pytest.raises(VxError) as e:
        srv.submit(Problem(nx=16384, np=1024, Lfinest=3), 10)
    assert e.value.code == -1 and "larger than the whole memory budget" in str(e.value)
    ok = srv.submit(problem_for("slab64"), 1)
    while srv.step() != (0, 0):
        pass
    assert srv.result(ok)["status"] == 3
    srv.close()
