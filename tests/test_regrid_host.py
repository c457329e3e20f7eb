"""Regrid clustering on the host (Mesh::updateHierarchy, Mesh.cpp:132-208) against the
reference's own regrid.

The flags are recomputed here from the reference's pre-regrid state with the error
estimate of Rectangle.hpp:128-130 (elementwise float64, the same operations and order as
the C++), on the range of Rectangle::getError (Rectangle.cpp:866-890); the clustering
itself runs in the library's host code through vx_update_hierarchy.  The result must be
the reference's post-regrid layout, boundary flags included.
"""
import numpy as np
import pytest

from helpers import golden_named, problem_for

CASES = ["amr2", "beam2", "beam3", "ragged2"]


def _flags(st, prob, maxdepth):
    from veritas_gb300 import error_weights

    r = prob.r
    patches, flags = [], []
    for depth, rects in enumerate(st["species"][0]):
        w, crit = error_weights(prob, 0, depth)
        offset = 3 * sum(r ** i for i in range(maxdepth - depth + 1))
        xsize = prob.nx * r ** (maxdepth - depth)
        psize = prob.np * r ** (maxdepth - depth)
        for R in rects:
            x0, p0, nx, np_ = R["x_pos"], R["p_pos"], R["n_x"], R["n_p"]
            patches.append((depth, x0, p0, nx, np_))
            lx, ux = max(x0, offset), min(x0 + nx, xsize - offset)
            lp, up = max(p0, offset), min(p0 + np_, psize - offset)
            cells = []
            if lx < ux and lp < up:
                f = R["f"][..., 1]
                ii = np.arange(lx - x0, ux - x0) + 2
                jj = np.arange(lp - p0, up - p0) + 2
                c = f[np.ix_(ii, jj)]
                xp, xm = f[np.ix_(ii + 1, jj)], f[np.ix_(ii - 1, jj)]
                pp, pm = f[np.ix_(ii, jj + 1)], f[np.ix_(ii, jj - 1)]
                e = (w[0] * np.abs(xp - xm) + w[1] * np.abs(pp - pm) + w[2] * np.abs(xp - 2 * c + xm)
                     + w[3] * np.abs(pp - 2 * c + pm) + w[4] * np.abs(c))
                fi, fj = np.nonzero(e > crit)
                cells = list(zip((fi + lx).tolist(), (fj + lp).tolist()))
            flags.append(cells)
    return patches, flags


def _layout(st):
    out = []
    for depth, rects in enumerate(st["species"][0]):
        for R in rects:
            out.append((depth, R["x_pos"], R["p_pos"], R["n_x"], R["n_p"], R["up"], R["down"], R["left"], R["right"]))
    return out


@pytest.mark.parametrize("name", CASES)
def test_clustering_matches_reference_regrid(name):
    from veritas_gb300 import update_hierarchy

    prob = problem_for(name)
    pre, post = golden_named(name, "pre"), golden_named(name, "post")
    patches, flags = _flags(pre, prob, prob.Lfinest - 1)
    assert sum(len(f) for f in flags) > 0
    got = update_hierarchy(prob, 0, patches, flags)
    assert got == _layout(post)


def test_partial_hierarchy_boundary_flags():
    """A hierarchy with fewer levels than maxDepth + 1 gets the reference's boundary
    flags (Mesh.cpp:803-813 compares with the size of level N - lvl): on a 3-level
    problem, one refinement round leaves the base patch open at its upper and right
    edges."""
    from veritas_gb300 import update_hierarchy

    prob = problem_for("beam3")
    pre = golden_named("beam3", "pre")
    base = pre["species"][0][2][0]
    patches = [(2, 0, 0, base["n_x"], base["n_p"])]
    _, flags = _flags({"species": [[[], [], [base]]]}, prob, 2)
    got = update_hierarchy(prob, 0, patches, flags)
    depths = [g[0] for g in got]
    assert depths[-1] == 2 and 1 in depths and 0 not in depths
    b = got[-1]
    assert b[5:] == (0, 1, 1, 0)  # up, down, left, right


def test_no_flags_keeps_base_only():
    """Nothing flagged: the hierarchy stays at the base level, which (being shorter than
    maxDepth + 1 levels) is open at its upper and right edges."""
    from veritas_gb300 import update_hierarchy

    prob = problem_for("amr2")
    got = update_hierarchy(prob, 0, [(1, 0, 0, prob.nx, prob.np)], [[]])
    assert got == [(1, 0, 0, prob.nx, prob.np, 0, 1, 1, 0)]
