"""Text diagnostics (SolverManager::fileOutput, Mesh::outputRectangleData) vs the files the
reference build wrote for the same run.

The fixtures hold every file the reference wrote at t = 0 and after two steps with its
own dt (tests/golden/make_golden.py, DIAG).  The GPU run starts from its own
initialisation, takes the same two steps with its own CalculateDt and writes through the
C ABI.  Checks: the same file names (the rectangle files carry t in their names), the
same number of lines and tokens per line, every field value in the reference's format,
integers and patch headers identical, and values within 1e-10 relative to the largest
|value| of their line (the plain path's parity bar) for the 15-digit files; the
4-significant-digit rectangle values within one unit of their last digit.
"""
import re

import numpy as np
import pytest

from helpers import GOLDEN, problem_for

FIELD_TOL = 1e-10
SCI15 = re.compile(r"-?\d\.\d{15}e[+-]\d{2,3}")
SCI4 = re.compile(r"-?\d\.\d{4}e[+-]\d{2,3}")


def reference_files(name):
    z = np.load(GOLDEN / f"{name}_diag.npz")
    return {k: bytes(z[k]).decode() for k in z.files}


def written_files(root):
    return {str(p.relative_to(root)): p.read_text() for p in sorted(root.rglob("*.txt"))}


def run_and_write(ctx, name, root, precision=64, steps=2):
    from veritas_gb300 import SolverManager

    prob = problem_for(name)
    prob.precision = precision
    s = SolverManager(ctx, prob)
    (root / "rectangleData").mkdir(parents=True)
    for k in range(steps + 1):
        if k:
            s.Advance(s.CalculateDt())
        if k in (0, steps):
            s.fileOutput(s.time, root)
            s.OutputRectangles(s.time, root / "rectangleData")
    s.close()
    return written_files(root)


def compare_fields(got, ref, label, tol):
    gl, rl = got.splitlines(), ref.splitlines()
    assert len(gl) == len(rl), label
    worst = 0.0
    for n, (a, b) in enumerate(zip(gl, rl)):
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (label, n)
        assert a.endswith(" ") == b.endswith(" "), (label, n)
        for t in ta:
            assert SCI15.fullmatch(t), (label, n, t)
        va, vb = np.array(ta, dtype=np.float64), np.array(tb, dtype=np.float64)
        scale = np.max(np.abs(vb))
        if scale > 0:
            worst = max(worst, float(np.max(np.abs(va - vb)) / scale))
        else:
            assert np.all(va == 0), (label, n)
    assert worst <= tol, (label, worst)
    return worst


def compare_rectangles(got, ref, label, rtol):
    gl, rl = got.splitlines(), ref.splitlines()
    assert len(gl) == len(rl), label
    for n, (a, b) in enumerate(zip(gl, rl)):
        if b.startswith("r "):
            assert a == b, (label, n)
            continue
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb) == 3 and ta[:2] == tb[:2], (label, n)
        assert SCI4.fullmatch(ta[2]), (label, n, ta[2])
        # "x p  value": two spaces before the value, as the reference writes
        assert a.count("  ") == b.count("  "), (label, n)
        va, vb = float(ta[2]), float(tb[2])
        assert abs(va - vb) <= rtol * abs(vb) + 1e-300, (label, n, a, b)


@pytest.fixture(scope="module")
def ctx():
    from veritas_gb300 import Context

    c = Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ions2", "beam3"])
def test_file_output_matches_reference(ctx, tmp_path, name):
    ref = reference_files(name)
    got = run_and_write(ctx, name, tmp_path / "output")
    assert sorted(got) == sorted(ref)
    errs, identical = {}, 0
    for fname, text in ref.items():
        identical += got[fname] == text
        if fname.startswith("rectangleData/"):
            compare_rectangles(got[fname], text, fname, 1.01e-4)
        else:
            errs[fname] = compare_fields(got[fname], text, fname, FIELD_TOL)
    print(name, f"{identical}/{len(ref)} files byte-identical", {k: f"{v:.1e}" for k, v in errs.items()})


@pytest.mark.gpu
def test_file_output_precision_form(ctx, tmp_path):
    """The FP32 form writes the same files; values within its stated error."""
    ref = reference_files("ions2")
    got = run_and_write(ctx, "ions2", tmp_path / "output", precision=32)
    assert sorted(got) == sorted(ref)
    for fname, text in ref.items():
        if fname.startswith("rectangleData/"):
            gl, rl = got[fname].splitlines(), text.splitlines()
            assert len(gl) == len(rl)
            va = np.array([float(l.split()[2]) for l in gl if not l.startswith("r ")])
            vb = np.array([float(l.split()[2]) for l in rl if not l.startswith("r ")])
            # FP32 error (1e-5 of the level's peak) plus the 4-digit rounding of either side
            assert np.all(np.abs(va - vb) <= 1e-5 * np.max(np.abs(vb)) + 1.01e-4 * np.abs(vb)), fname
        else:
            compare_fields(got[fname], text, fname, 1e-4)


@pytest.mark.gpu
def test_file_output_selected_and_appended(ctx, tmp_path):
    """Only the selected files are created; later calls append one record each."""
    from veritas_gb300 import SolverManager

    s = SolverManager(ctx, problem_for("amr2"))
    out = tmp_path / "o"
    out.mkdir()
    for _ in range(3):
        s.fileOutput(s.time, out, outputs=["charge", "time"], precision=6)
    s.close()
    assert sorted(p.name for p in out.iterdir()) == ["charge.txt", "time.txt"]
    assert len((out / "charge.txt").read_text().splitlines()) == 3
    assert (out / "time.txt").read_text().splitlines() == ["0.000000e+00"] * 3


@pytest.mark.gpu
def test_file_output_missing_directory_is_an_io_error(ctx, tmp_path):
    from veritas_gb300 import SolverManager, VxError

    s = SolverManager(ctx, problem_for("slab64"))
    with pytest.raises(VxError) as e:
        s.fileOutput(s.time, tmp_path / "absent")
    assert e.value.code == -4  # VX_ERR_IO
    with pytest.raises(VxError):
        s.OutputRectangles(s.time, tmp_path / "absent")
    s.close()
