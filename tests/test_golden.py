"""Golden fixtures produced by the reference build: well-formed and physically sane."""
import numpy as np
import pytest

import vxstate
from helpers import GOLDEN, golden, total_mass

CASES = {"slab64": [0, 1, 2, 5], "drift128": [0, 1, 3], "edge64": [0, 1, 3]}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_layout(name):
    for k in CASES[name]:
        st = golden(name, k)
        assert st["step"] == k
        nf = st["n"] + st["pre"] + st["post"]
        assert st["By"].size == 8 * nf and st["a_squared"].size == st["n"] + 1
        r = st["species"][0][-1][0]
        assert r["f"].shape == (r["n_x"] + 4, r["n_p"] + 4, 3)
        # slots 0 and 1 agree at the start of every step (Rectangle.cpp:1614-1621)
        assert np.array_equal(r["f"][..., 0], r["f"][..., 1])


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_conserves_mass(name):
    ks = CASES[name]
    m0 = total_mass(golden(name, ks[0]))
    for k in ks[1:]:
        assert abs(total_mass(golden(name, k)) - m0) <= 1e-13 * abs(m0)


def test_roundtrip_bin(tmp_path):
    st = golden("slab64", 1)
    p = tmp_path / "s.bin"
    vxstate.write_state(st, p)
    back = vxstate.read_state(p)
    assert back["time"] == st["time"]
    assert np.array_equal(back["species"][0][0][0]["f"], st["species"][0][0][0]["f"])
