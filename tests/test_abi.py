"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w \*]*?[\s\*])(vx_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "vx_run_advance" in syms and "vx_ctx_create" in syms
    assert len(syms) >= 15


def test_library_exports_all_declared():
    from veritas_gb300 import LIB_PATH

    lib = ctypes.CDLL(str(LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_problem_defaults_roundtrip():
    from veritas_gb300 import Problem, _Problem, lib

    c = _Problem()
    lib().vx_problem_defaults(ctypes.byref(c))
    d = Problem()
    assert c.nx == d.nx and c.np == d.np and c.precision == 64
    assert c.L == d.L and c.a0 == d.a0


def test_errors_without_arguments():
    from veritas_gb300 import lib

    assert lib().vx_run_advance(None, 1.0) == -1
    assert lib().vx_ctx_sync(None) == -1


def test_input_defaults_are_the_references():
    """vx_input_defaults fills the reference's struct defaults (Settings.hpp:4-33)."""
    from veritas_gb300 import VxInput, VxOutput, VxParticles, lib

    g, p, o = VxInput(), VxParticles(), VxOutput()
    lib().vx_input_defaults(ctypes.byref(g), ctypes.byref(p), ctypes.byref(o))
    assert (g.minEfficiency, g.dx, g.k, g.refinementCriteria, g.cfl, g.sizeWeight) == (0.6, 0.5, 0.01, 1e-8, 0.9, 0.0)
    assert (g.preLength, g.postLength, g.nx, g.r, g.Lfinest) == (2, 2, 304, 2, 5)
    assert (g.plasma_xl_bound, g.plasma_xr_bound, g.ntempEM, g.tempEM[0]) == (3.0e-6, 7.0e-6, 1, 0.0)
    assert p.nspecies == 1 and p.mass[0] == 9.10938291e-31 and p.charge[0] == -1.60217657e-19
    assert (p.np[0], p.dp[0], p.pmin[0], p.nmisc[0], p.misc[0][0], p.misc[0][1]) == (50, 0.1, 0.1, 2, 0.0, 0.01)
    assert o.time == 1 and o.AFieldSquared == 1 and o.precision == 15


def test_hooks_struct_layouts_match_the_header():
    """The Python mirror's struct sizes equal the C header's (compiled here with gcc)."""
    import subprocess
    import tempfile

    from veritas_gb300 import VxHooks, VxInput, VxOutput, VxParticles, VxSettings, _Problem, _RequestResult

    src = ('#include <stdio.h>\n#include "vx.h"\nint main(void){printf("%zu %zu %zu %zu %zu %zu %zu",'
           'sizeof(vx_input),sizeof(vx_particles),sizeof(vx_output),sizeof(vx_settings),sizeof(vx_hooks),'
           'sizeof(vx_problem),sizeof(vx_request_result));return 0;}\n')
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "s.c").write_text(src)
        subprocess.run(["gcc", "-I", str(ROOT / "include"), "-o", str(Path(td) / "s"), str(Path(td) / "s.c")],
                       check=True)
        got = subprocess.run([str(Path(td) / "s")], capture_output=True, text=True, check=True).stdout.split()
    want = [ctypes.sizeof(t) for t in (VxInput, VxParticles, VxOutput, VxSettings, VxHooks, _Problem, _RequestResult)]
    assert [int(x) for x in got] == want
