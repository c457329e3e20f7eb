"""FP64 GPU path vs the reference build, through the C ABI.

Each case loads a state the reference dumped, advances with the dt the reference used,
and compares f (slots 0 and 1 over the padded block), the six transverse field arrays
with all 8 RK slots, a^2, phi, rho, J and Ex0.  Tolerance: 1e-10 relative L-inf
(max|gpu - ref| / max|ref|), the plain path's parity bar; the GPU kernels keep the
reference's operation order, so the observed errors are at rounding level.
"""
import numpy as np
import pytest

import vxstate
from helpers import compare_states, golden, golden_named, gpu_vs_port, problem_for, total_mass

TOL = 1e-10
ONE_STEP = [("slab64", 0), ("slab64", 1), ("drift128", 0), ("edge64", 0),
            ("amr2", 0), ("beam2", 0), ("beam3", 0), ("ions2", 0), ("ragged2", 0)]


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


def _solver(ctx, name):
    from veritas_gb300 import SolverManager

    return SolverManager(ctx, problem_for(name))


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", ONE_STEP)
def test_one_step_from_reference_state(ctx, tmp_path, name, k):
    s = _solver(ctx, name)
    vxstate.write_state(golden(name, k), tmp_path / "in.bin")
    s.load_state(tmp_path / "in.bin")
    ref = golden(name, k + 1)
    s.Advance(ref["dt"])
    s.save_state(tmp_path / "out.bin")
    got = vxstate.read_state(tmp_path / "out.bin")
    err = compare_states(got, ref, TOL)
    print(name, k, {kk: f"{v:.2e}" for kk, v in err.items()})
    for kk, v in err.items():
        assert v <= TOL, (kk, v)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name,k0,k1", [("slab64", 0, 5), ("drift128", 1, 3), ("edge64", 1, 3), ("amr2", 1, 3),
                                        ("ions2", 1, 3), ("ragged2", 0, 3),
                                        ("beam2", 1, 3), ("beam3", 0, 3)])
def test_multi_step_with_own_dt(ctx, tmp_path, name, k0, k1):
    s = _solver(ctx, name)
    vxstate.write_state(golden(name, k0), tmp_path / "in.bin")
    s.load_state(tmp_path / "in.bin")
    for _ in range(k1 - k0):
        s.Advance(s.CalculateDt())
    ref = golden(name, k1)
    assert abs(s.time - ref["time"]) <= 1e-12 * ref["time"]
    s.save_state(tmp_path / "out.bin")
    got = vxstate.read_state(tmp_path / "out.bin")
    err = compare_states(got, ref, TOL)
    print(name, k0, k1, {kk: f"{v:.2e}" for kk, v in err.items()})
    for kk, v in err.items():
        assert v <= TOL, (kk, v)
    s.close()


@pytest.mark.gpu
def test_initialisation_matches_reference(ctx, tmp_path):
    """f(t=0) from the quadrature and neutralising charge (host-side hooks)."""
    s = _solver(ctx, "slab64")
    s.save_state(tmp_path / "init.bin")
    got = vxstate.read_state(tmp_path / "init.bin")
    ref = golden("slab64", 0)
    assert np.array_equal(got["species"][0][0][0]["f"][..., :2], ref["species"][0][0][0]["f"][..., :2])
    assert vxstate.rel_linf(got["neut"], ref["neut"]) <= 1e-14
    s.close()


def _check(got, ref, label):
    err = compare_states(got, ref, TOL)
    print(label, {kk: f"{v:.2e}" for kk, v in err.items()})
    for kk, v in err.items():
        assert v <= TOL, (kk, v)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["amr2", "beam2", "beam3", "ions2", "ragged2"])
def test_initial_hierarchy_matches_reference(ctx, tmp_path, name):
    """Mesh::Mesh: base level, maxDepth rounds of flagging / clustering with every patch
    from the quadrature, then the ghost fill and the neutralising charge."""
    s = _solver(ctx, name)
    s.save_state(tmp_path / "init.bin")
    _check(vxstate.read_state(tmp_path / "init.bin"), golden(name, 0), name + " init")
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["amr2", "beam2", "beam3", "ions2", "ragged2"])
def test_regrid_matches_reference(ctx, tmp_path, name):
    """SolverManager::reGrid on the reference's state: the new layout, the transferred
    f (slots 0 and 1, ghosts included), then one step on the new layout."""
    s = _solver(ctx, name)
    vxstate.write_state(golden_named(name, "pre"), tmp_path / "pre.bin")
    s.load_state(tmp_path / "pre.bin")
    s.reGrid()
    s.save_state(tmp_path / "post.bin")
    _check(vxstate.read_state(tmp_path / "post.bin"), golden_named(name, "post"), name + " regrid")
    ref1 = golden_named(name, "post1")
    s.Advance(ref1["dt"])
    s.save_state(tmp_path / "post1.bin")
    _check(vxstate.read_state(tmp_path / "post1.bin"), ref1, name + " step after regrid")
    s.close()


@pytest.mark.gpu
def test_deterministic_repeat(ctx, tmp_path):
    outs = []
    for rep in range(2):
        s = _solver(ctx, "drift128")
        vxstate.write_state(golden("drift128", 0), tmp_path / "in.bin")
        s.load_state(tmp_path / "in.bin")
        for _ in range(2):
            s.Advance(s.CalculateDt())
        s.save_state(tmp_path / f"o{rep}.bin")
        outs.append((tmp_path / f"o{rep}.bin").read_bytes())
        s.close()
    assert outs[0] == outs[1]


@pytest.mark.gpu
def test_full_size_conservation_and_fields():
    """Config-1 size (2048 x 256): mass conserved by the flux form, fields finite."""
    from veritas_gb300 import Context, Problem, SolverManager

    c = Context(0)
    s = SolverManager(c, Problem())
    import tempfile, os

    with tempfile.TemporaryDirectory() as td:
        s.save_state(os.path.join(td, "a.bin"))
        m0 = total_mass(vxstate.read_state(os.path.join(td, "a.bin")))
        for _ in range(3):
            s.Advance(s.CalculateDt())
        s.save_state(os.path.join(td, "b.bin"))
        st = vxstate.read_state(os.path.join(td, "b.bin"))
    m1 = total_mass(st)
    assert abs(m1 - m0) <= 1e-12 * abs(m0)
    for k in ("By", "Bz", "Ey", "Ez", "Ay", "Az", "phi"):
        assert np.all(np.isfinite(st[k]))
    assert np.abs(st["Bz"]).max() > 0
    s.close()
    c.close()


@pytest.mark.gpu
def test_gpu_matches_port_at_512x128(tmp_path):
    """Larger than the fixtures: GPU and oracle port from t=0 for 3 steps, own dt."""
    import subprocess
    from pathlib import Path
    from veritas_gb300 import Context, Problem, SolverManager

    root = Path(__file__).resolve().parent.parent
    port = root / "oracle" / "_port" / "veritas_port"
    if not port.exists():
        subprocess.run(["bash", str(root / "oracle" / "port" / "build_port.sh")], check=True)
    p = Problem(L=40.0, nx=512, np=128, Te=5.0, pmax=1.0, x1=5, x2=8, x3=30, x4=34, pert_amp=0.05, pert_k=4,
                a0=1.5, fwhm=4, delay=2)
    subprocess.run([str(port), *p.harness_args(), "steps=3", "dump_every=3", f"dumpdir={tmp_path}"], check=True)
    ref = vxstate.read_state(tmp_path / "state_00003.bin")
    c = Context(0)
    s = SolverManager(c, p)
    for _ in range(3):
        s.Advance(s.CalculateDt())
    s.save_state(tmp_path / "gpu.bin")
    got = vxstate.read_state(tmp_path / "gpu.bin")
    err = compare_states(got, ref, TOL)
    print("512x128 vs port", {k: f"{v:.2e}" for k, v in err.items()})
    for k, v in err.items():
        assert v <= TOL, (k, v)
    s.close()
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("workload", ["laser_slab_2048x256", "laser_slab_amr_4096x512"])
def test_gpu_matches_port_at_benchmark_size(ctx, tmp_path, workload):
    """The benchmarked workloads at full size (one level 2048 x 256; two levels on a
    4096 x 512 base): the GPU path and the oracle port each build the initial hierarchy
    (same patch layout, every array within 1e-10), then take two RK steps with the same
    dt (every array within 1e-10)."""
    from veritas_gb300.workloads import WORKLOADS

    err = gpu_vs_port(ctx, WORKLOADS[workload](), 2, tmp_path)
    print(workload, "vs port", {k: f"{v:.2e}" for k, v in err.items()})
    for k, v in err.items():
        assert v <= TOL, (k, v)
