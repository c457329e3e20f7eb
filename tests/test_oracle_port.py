"""The oracle port (oracle/port, C++ restatement) is pinned to the reference build.

The golden fixtures were dumped by the reference itself; the port, started from the same
problem arguments (t=0: its own initial hierarchy and quadrature, multi-level cases
included) or from a dumped state with the reference's dt sequence, must reproduce them
bit for bit.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import vxstate
from helpers import GOLDEN, case_args, compare_states, golden

ROOT = Path(__file__).resolve().parent.parent
PORT = ROOT / "oracle" / "_port" / "veritas_port"
# single-level cases, and the one-species AMR cases from t = 0: the port builds the
# initial hierarchy itself (maxDepth rounds of flagging, clustering and quadrature)
CASES = {"slab64": [0, 1, 2, 5], "drift128": [0, 1, 3], "edge64": [0, 1, 3],
         "amr2": [0, 1, 3], "beam2": [0, 1, 3], "beam3": [0, 1, 3], "ragged2": [0, 1, 3]}


@pytest.fixture(scope="module")
def port():
    subprocess.run(["bash", str(ROOT / "oracle" / "port" / "build_port.sh")], check=True, capture_output=True)
    assert PORT.exists()
    return PORT


def _args(name):
    return [f"{k}={v}" for k, v in case_args(name).items()]


@pytest.mark.parametrize("name", sorted(CASES))
def test_port_from_t0_matches_reference(port, tmp_path, name):
    ks = CASES[name]
    dts = [golden(name, k)["dt"] for k in range(1, ks[-1] + 1) if (GOLDEN / f"{name}_s{k}.npz").exists()]
    # dt is recomputed by the port from its own state; it must agree with the reference
    subprocess.run([str(port), *_args(name), f"steps={ks[-1]}", "dump_every=1", f"dumpdir={tmp_path}"],
                   check=True, capture_output=True, env={"OMP_NUM_THREADS": "4"})
    for k in ks:
        got = vxstate.read_state(tmp_path / f"state_{k:05d}.bin")
        ref = golden(name, k)
        err = compare_states(got, ref, 0.0)
        assert max(err.values()) == 0.0, (k, err)
        assert got["dt"] == ref["dt"]


def test_port_from_loaded_state(port, tmp_path):
    vxstate.write_state(golden("drift128", 1), tmp_path / "in.bin")
    dts = ",".join(repr(golden("drift128", 3)["dt"]) for _ in range(1))
    subprocess.run([str(port), *_args("drift128"), f"load={tmp_path / 'in.bin'}", "steps=2", "dump_every=2",
                    f"dumpdir={tmp_path}"], check=True, capture_output=True, env={"OMP_NUM_THREADS": "2"})
    got = vxstate.read_state(tmp_path / "state_00002.bin")
    err = compare_states(got, golden("drift128", 3), 0.0)
    assert max(err.values()) == 0.0, err


def test_port_thread_count_invariant(port, tmp_path):
    outs = []
    for th in ("1", "3"):
        d = tmp_path / th
        d.mkdir()
        subprocess.run([str(port), *_args("slab64"), "steps=2", "dump_every=2", f"dumpdir={d}"], check=True,
                       capture_output=True, env={"OMP_NUM_THREADS": th})
        outs.append((d / "state_00002.bin").read_bytes())
    assert outs[0] == outs[1]


def test_port_detects_planted_error(port, tmp_path):
    """A one-ulp change planted in the oracle's input state shows up in the comparison."""
    st = golden("slab64", 1)
    f = st["species"][0][0][0]["f"]
    i, j = 30, 16
    f[i, j, 0] = np.nextafter(f[i, j, 0], np.inf)
    f[i, j, 1] = f[i, j, 0]
    vxstate.write_state(st, tmp_path / "in.bin")
    subprocess.run([str(port), *_args("slab64"), f"load={tmp_path / 'in.bin'}", "steps=1", "dump_every=1",
                    f"dumpdir={tmp_path}", f"dts={golden('slab64', 2)['dt']!r}"], check=True, capture_output=True)
    got = vxstate.read_state(tmp_path / "state_00001.bin")
    err = compare_states(got, golden("slab64", 2), 0.0)
    assert err["f"] > 0.0


@pytest.mark.parametrize("name,k0,k1", [("amr2", 0, 3), ("beam2", 1, 3), ("beam3", 0, 3), ("ragged2", 0, 3)])
def test_port_amr_steps_match_reference(port, tmp_path, name, k0, k1):
    """Multi-level step (ghost fills, interface fluxes, limiter exchange, nested moments)
    from a reference state with the port's own dt."""
    vxstate.write_state(golden(name, k0), tmp_path / "in.bin")
    subprocess.run([str(port), *_args(name), f"load={tmp_path / 'in.bin'}", f"steps={k1 - k0}", "dump_every=1",
                    f"dumpdir={tmp_path}"], check=True, capture_output=True, env={"OMP_NUM_THREADS": "4"})
    for k in range(k0 + 1, k1 + 1):
        if not (GOLDEN / f"{name}_s{k}.npz").exists():
            continue
        got = vxstate.read_state(tmp_path / f"state_{k - k0:05d}.bin")
        err = compare_states(got, golden(name, k), 0.0)
        assert max(err.values()) == 0.0, (k, err)


@pytest.mark.parametrize("name", ["amr2", "beam2", "beam3", "ragged2"])
def test_port_amr_step_after_regrid(port, tmp_path, name):
    from helpers import golden_named

    vxstate.write_state(golden_named(name, "post"), tmp_path / "in.bin")
    ref = golden_named(name, "post1")
    subprocess.run([str(port), *_args(name), f"load={tmp_path / 'in.bin'}", "steps=1", "dump_every=1",
                    f"dumpdir={tmp_path}", f"dts={ref['dt']!r}"], check=True, capture_output=True,
                   env={"OMP_NUM_THREADS": "4"})
    err = compare_states(vxstate.read_state(tmp_path / "state_00001.bin"), ref, 0.0)
    assert max(err.values()) == 0.0, err
