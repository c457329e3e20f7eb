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
