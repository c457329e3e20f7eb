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


# ---------------------------------------------------------------- text-output fixtures

DIAG = {"ions2": 2, "beam3": 1}  # case -> species


def _diag(name):
    z = np.load(GOLDEN / f"{name}_diag.npz")
    return {k: bytes(z[k]).decode() for k in z.files}


def _rows(text):
    return [np.array(l.split(), dtype=np.float64) for l in text.splitlines()]


def _dndp(st, sp, L, lam, nx, r):
    """Rectangle::CalculateEnergy + Level/Mesh sums (Rectangle.cpp:284-305,
    Level.cpp:31-40, 64-78) on a dumped state: f slot 1 of the cells not covered by a finer
    patch, interpolated onto the finest p sub-cells, times the patch's dx."""
    M = np.array([[0.104166666666667, -0.708333333333334, 0.708333333333334, -0.104166666666667],
                  [0.117647058823529, 0.029411764705882, 0.029411764705882, 0.117647058823529],
                  [-0.083333333333333, 0.166666666666667, -0.166666666666667, 0.083333333333334]])
    levels = st["species"][sp]  # index = depth; depth 0 is the finest level
    top = len(levels) - 1
    base = levels[top][0]
    total = np.zeros(base["n_p"] * r ** top)
    for d, lvl in enumerate(levels):
        rtb = r ** d  # finest cells per cell of this level (Rectangle::relativeToBottom)
        tl = -0.5 + np.arange(rtb) / rtb
        tr = -0.5 + (np.arange(rtb) + 1.0) / rtb
        w = np.stack([(tl + tr) * 0.5, (tl * tl + tl * tr + tr * tr) / 3.0 - 1.0 / 12,
                      (tl ** 3 + tl * tl * tr + tl * tr * tr + tr ** 3) * 0.25], axis=1)
        finer = levels[d - 1] if d > 0 else []
        for R in lvl:
            f = R["f"][..., 1]
            n_x, n_p = R["n_x"], R["n_p"]
            nested = np.zeros((n_x, n_p), bool)
            gx = (R["x_pos"] + np.arange(n_x)) * r
            gp = (R["p_pos"] + np.arange(n_p)) * r
            for F in finer:
                nested |= (((gx >= F["x_pos"]) & (gx < F["x_pos"] + F["n_x"]))[:, None]
                           & ((gp >= F["p_pos"]) & (gp < F["p_pos"] + F["n_p"]))[None, :])
            e = np.zeros((n_p, rtb))
            for j in range(n_p):
                st5 = f[2:n_x + 2, j:j + 5] - f[2:n_x + 2, j + 2:j + 3]
                a = st5[:, [0, 1, 3, 4]] @ M.T
                vals = a @ w.T + f[2:n_x + 2, j + 2][:, None]
                e[j] = np.where(nested[:, j][:, None], 0.0, vals).sum(axis=0)
            e *= L * lam / nx * float(r) ** (d - top)  # Settings::GetDx(depth)
            total[R["p_pos"] * rtb:(R["p_pos"] + n_p) * rtb] += e.reshape(-1)
    return total


@pytest.mark.parametrize("name", sorted(DIAG))
def test_diag_fixture_against_states(name):
    """The reference's text files at t = 0 against its own t = 0 state dump: the species
    charges add up to rho, the dN/dp spectra follow from f slot 1, the rectangle files
    list the patches with f slot 0 to four digits."""
    files, st = _diag(name), golden(name, 0)
    ns = DIAG[name]
    args = dict(kv.split("=") for kv in (GOLDEN / f"{name}.args").read_text().split())
    ch = _rows(files["charge.txt"])
    assert len(ch) == 2 * ns and all(c.size == st["n"] for c in ch)
    rho = sum(ch[:ns])
    # 16 significant digits per species term (the species charges cancel to rho)
    assert np.max(np.abs(rho - st["charge"])) <= 1e-14 * max(np.max(np.abs(c)) for c in ch[:ns])
    for sp in range(ns):
        got = _dndp(st, sp, float(args["L"]), 1e-6, int(args["nx"]), 2)
        ref = _rows(files[f"dNdP_{sp}.txt"])[0]
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), sp
    assert _rows(files["time.txt"])[0][0] == 0.0
    nf = st["n"] + st["pre"] + st["post"]
    assert np.array_equal(_rows(files["EFieldTrans.txt"])[0], st["Ey"][:nf])
    assert np.array_equal(_rows(files["potential.txt"])[0], st["phi"])
    for sp in range(ns):
        for d, lvl in enumerate(st["species"][sp]):
            lines = files[f"rectangleData/rectangleData_p{sp}_l{d}_t0.000000e+00.txt"].splitlines()
            pos = 0
            for R in lvl:
                assert lines[pos] == f"r {R['x_pos']} {R['p_pos']} {R['n_x']} {R['n_p']}"
                v = np.array([float(l.split()[2]) for l in lines[pos + 1:pos + 1 + R["n_x"] * R["n_p"]]])
                f0 = R["f"][2:R["n_x"] + 2, 2:R["n_p"] + 2, 0].reshape(-1)
                assert np.all(np.abs(v - f0) <= 5.01e-4 * np.abs(f0) + 1e-300)
                pos += 1 + R["n_x"] * R["n_p"]
            assert pos == len(lines)
