"""Generate the golden parity fixtures by running the reference Veritas build.

The reference (its unmodified sources) is compiled by ``oracle/ref/build_ref.sh`` into
``oracle/_ref/veritas_ref`` together with the harness problem file; this script runs it
for each case below and stores the dumped states as compressed ``.npz`` files next to
this script.  It needs the reference tree, so it only runs where that tree is mounted:

    python tests/golden/make_golden.py [--ref /path/to/veritas/sources]

Cases are small enough for the oracle to finish in seconds; every parameter is the
harness's key=value argument.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(HERE.parent))
import vxstate  # noqa: E402

# name -> (harness args, steps, states to keep)
CASES = {
    # Plasma slab with a density modulation and a strong injected pulse on 64 x 32 cells.
    "slab64": (["L=8", "nx=64", "np=32", "Te=50", "pmax=2", "x1=1.5", "x2=2", "x3=6", "x4=6.5", "pert_amp=0.2",
                "pert_k=2", "a0=2", "fwhm=2", "delay=1", "levels=1"], 5, [0, 1, 2, 5]),
    # Drifting plasma (net current) on 128 x 64 cells.
    "drift128": (["L=16", "nx=128", "np=64", "Te=20", "pmax=1.5", "p0=0.15", "x1=3", "x2=4", "x3=12", "x4=13",
                  "pert_amp=0.1", "pert_k=3", "a0=1.5", "fwhm=3", "delay=1.5", "levels=1"], 3, [0, 1, 3]),
    # Plasma touching both x edges and both p edges: exercises the skipped domain-edge faces.
    "edge64": (["L=4", "nx=64", "np=32", "Te=50", "pmax=0.5", "x1=-1", "x2=0", "x3=3", "x4=5", "pert_amp=0.3",
                "pert_k=1", "a0=1", "fwhm=2", "delay=0.5", "levels=1"], 3, [0, 1, 3]),
    # Two refinement levels, one fine patch over the slab.
    "amr2": (["L=8", "nx=64", "np=32", "Te=50", "pmax=2", "x1=1.5", "x2=2", "x3=6", "x4=6.5", "pert_amp=0.2",
              "pert_k=2", "a0=2", "fwhm=2", "delay=1", "levels=2"], 3, [0, 1, 3]),
    # Slab plus a drifting beam: four fine patches, three of them side by side in x with
    # staggered p extents (same-level ghost copies and limiter exchange between patches).
    "beam2": (["L=8", "nx=64", "np=32", "Te=0.5", "pmax=2", "x1=1", "x2=1.5", "x3=3", "x4=3.5", "pert_amp=0.2",
               "pert_k=2", "a0=2", "fwhm=2", "delay=1", "bdens=0.5", "bp0=1.2", "bTe=0.5", "crit=1e-3",
               "minEff=0.9", "levels=2"], 3, [0, 1, 3]),
    # Three levels: two finest patches inside one intermediate patch.
    "beam3": (["L=8", "nx=64", "np=32", "Te=1", "pmax=2", "x1=1.5", "x2=2", "x3=6", "x4=6.5", "pert_amp=0.2",
               "pert_k=2", "a0=2", "fwhm=2", "delay=1", "bdens=0.5", "bp0=-1.2", "bTe=1", "crit=1e-3",
               "minEff=0.9", "levels=3"], 3, [0, 1, 3]),
    # Electrons and mobile ions (mass 4 m_e, charge +e): two species, each with its own
    # two-level hierarchy; moments, Poisson and CFL sum over both.
    "ions2": (["L=8", "nx=64", "np=32", "Te=50", "pmax=2", "x1=1.5", "x2=2", "x3=6", "x4=6.5", "pert_amp=0.2",
               "pert_k=2", "a0=2", "fwhm=2", "delay=1", "mi=4", "iTe=50", "ipmax=0.6", "levels=2"], 3, [0, 1, 3]),
    # Ragged sizes: 50 x 38 base cells (n_p not a multiple of 8 or of the kernels' tiles,
    # n_x not a multiple of 8), one fine patch of 68 x 64.
    "ragged2": (["L=8", "nx=50", "np=38", "Te=50", "pmax=2", "x1=1.5", "x2=2", "x3=6", "x4=6.5", "pert_amp=0.2",
                 "pert_k=2", "a0=2", "fwhm=2", "delay=1", "levels=2"], 3, [0, 1, 3]),
}


# Cases of a user problem given through the C hooks (tests/hooks/sin2_problem.c), run by
# the reference build linked behind its Settings hooks (oracle/_ref/veritas_ref_hooks):
# two mobile species, vacuum pads of 5 cells, a circularly polarised sin^2-ramped laser
# (both GetBY and GetBZ), a refinement window from RefinementOverride; args are the
# problem's own keys (sin2_params).
HOOK_CASES = {
    "sin2hooks": (["nx=64", "np=32", "levels=2"], 3, [0, 1, 3]),
}
HOOK_REGRID = {"sin2hooks": 4}


# name -> regrid interval for the regrid fixtures of that case: the state just before
# SolverManager::reGrid ("_pre"), just after it ("_post") and one step later ("_post1").
REGRID = {
    "amr2": 4,
    "ragged2": 4,
    "ions2": 4,
    "beam2": 4,
    "beam3": 4,
}


# name -> (steps, interval) of the text-output fixtures: the files SolverManager::fileOutput
# and OutputRectangles write at t = 0 and after every interval-th step, stored byte for
# byte (one-thread run: Rectangle::CalculateEnergy's OpenMP loop adds into shared bins).
DIAG = {
    "ions2": (2, 2),
    "beam3": (2, 2),
}


def run_diag(exe: Path, name: str, args: list[str], steps: int, every: int) -> None:
    import numpy as np

    with tempfile.TemporaryDirectory() as td:
        out = Path(td) / "output"
        (out / "rectangleData").mkdir(parents=True)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        cmd = [str(exe), *args, f"steps={steps}", f"diag_every={every}"]
        subprocess.run(cmd, check=True, env=env, cwd=td, stdout=subprocess.DEVNULL)
        files = {}
        for f in sorted(out.rglob("*.txt")):
            files[str(f.relative_to(out))] = np.frombuffer(f.read_bytes(), dtype=np.uint8)
        np.savez_compressed(HERE / f"{name}_diag.npz", **files)


def run_case(exe: Path, name: str, args: list[str], steps: int, keep: list[int]) -> None:
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, OMP_NUM_THREADS="4")
        cmd = [str(exe), *args, f"steps={steps}", "dump_every=1", f"dumpdir={td}"]
        subprocess.run(cmd, check=True, env=env, stdout=subprocess.DEVNULL)
        for k in keep:
            st = vxstate.read_state(Path(td) / f"state_{k:05d}.bin")
            vxstate.to_npz(st, HERE / f"{name}_s{k}.npz")
    (HERE / f"{name}.args").write_text(" ".join(args) + "\n")


def run_regrid(exe: Path, name: str, args: list[str], every: int) -> None:
    with tempfile.TemporaryDirectory() as td:
        env = dict(os.environ, OMP_NUM_THREADS="4")
        cmd = [str(exe), *args, f"steps={every + 1}", f"regrid_every={every}", "dump_every=1", f"dumpdir={td}"]
        subprocess.run(cmd, check=True, env=env, stdout=subprocess.DEVNULL)
        vxstate.to_npz(vxstate.read_state(Path(td) / f"state_{every:05d}.bin"), HERE / f"{name}_pre.npz")
        vxstate.to_npz(vxstate.read_state(Path(td) / f"regrid_{every:05d}.bin"), HERE / f"{name}_post.npz")
        vxstate.to_npz(vxstate.read_state(Path(td) / f"state_{every + 1:05d}.bin"), HERE / f"{name}_post1.npz")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("VERITAS_REFERENCE_DIR"),
                    help="the reference's source tree (default: $VERITAS_REFERENCE_DIR)")
    ap.add_argument("--only", action="append", default=[], help="regenerate only these cases")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set VERITAS_REFERENCE_DIR to the reference's source tree")
    subprocess.run(["bash", str(REPO / "oracle" / "ref" / "build_ref.sh"), a.ref], check=True)
    exe = REPO / "oracle" / "_ref" / "veritas_ref"
    for name, (args, steps, keep) in CASES.items():
        if a.only and name not in a.only:
            continue
        run_case(exe, name, args, steps, keep)
        print("wrote", name)
    for name, every in REGRID.items():
        if a.only and name not in a.only:
            continue
        run_regrid(exe, name, CASES[name][0], every)
        print("wrote", name, "regrid")
    exe_hooks = REPO / "oracle" / "_ref" / "veritas_ref_hooks"
    for name, (args, steps, keep) in HOOK_CASES.items():
        if a.only and name not in a.only:
            continue
        run_case(exe_hooks, name, args, steps, keep)
        if name in HOOK_REGRID:
            run_regrid(exe_hooks, name, args, HOOK_REGRID[name])
        print("wrote", name, "(C hooks)")
    for name, (steps, every) in DIAG.items():
        if a.only and name not in a.only:
            continue
        run_diag(exe, name, CASES[name][0], steps, every)
        print("wrote", name, "diag")


if __name__ == "__main__":
    main()
