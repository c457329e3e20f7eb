"""The three-level wakefield case (base 16384 x 1024, 36 M cells) builds and steps: its
finest patch is 45888 cells wide (more than any 16-bit index holds), and its 65536
finest cells take the scan Poisson solve to its largest blocks (512 threads per CTA,
16 unknowns per thread)."""
import dataclasses
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.gpu
def test_three_level_wakefield_fp32_steps():
    sys.path.insert(0, str(ROOT))
    import bench
    from veritas_gb300 import Context, SolverManager

    ctx = Context(0)
    s = SolverManager(ctx, dataclasses.replace(bench.problem_config3(), precision=32))
    layout = s.layout()
    assert max(l[4] for l in layout) > 32767
    for _ in range(2):
        s.Advance(s.CalculateDt())
    for name in ("charge", "J", "phi", "Ey", "Bz"):
        assert np.all(np.isfinite(s.field(name))), name
    assert s.field("phi").size == 65536
    s.close()
    ctx.close()
