"""The oracle's facet rules and boundary integrals (tensorquad.c:309-355 restated), pinned by geometry: rule
nodes on the right side with outward X x Y orientation, surface areas and the divergence theorem on the perturbed
unit cube, and exact reproduction of linear fields (uniform and per-element orders)."""
import numpy as np
import pytest

import pyoracle as po

OUTWARD = {0: (0, -1, 0), 1: (1, 0, 0), 2: (0, 1, 0), 3: (-1, 0, 0), 4: (0, 0, -1), 5: (0, 0, 1)}


@pytest.mark.parametrize("side", range(6))
def test_facet_rule_lies_on_its_side_and_is_outward(side):
    for order in (0, 2, 4, 8, 16):
        nodes, w = po.facet_rule(side, order)
        n1 = int(round(np.sqrt(len(w))))
        assert n1 * n1 == len(w) == (order // 2 + 1) ** 2
        nrm = np.array(OUTWARD[side], float)
        d = int(np.argmax(np.abs(nrm)))
        np.testing.assert_array_equal(nodes[:, d], nrm[d])  # on the side
        assert np.all(np.abs(np.delete(nodes, d, axis=1)) < 1)  # strictly inside the face
        assert abs(w.sum() - 4.0) < 1e-14
        if n1 > 1:  # X (slowest) x Y points outward
            g = nodes.reshape(n1, n1, 3)
            tx, ty = g[1, 0] - g[0, 0], g[0, 1] - g[0, 0]
            c = np.cross(tx, ty)
            assert np.dot(c, nrm) > 0 and np.linalg.norm(np.cross(c, nrm)) < 1e-14


def test_areas_and_divergence_theorem():
    o = po.FS(6, 5, 7, degree=3, perturb=0.1, seed=2, dirichlet_mask=0)
    # masks: walls, top, bottom, all; int x.n over the unit cube's walls / top / bottom / all
    for mask, area, xn in ((1, 4.0, 2.0), (2, 1.0, 1.0), (4, 1.0, 0.0), (7, 6.0, 3.0)):
        jw, x, nrm, _ = o.facet_points(mask)
        assert abs(jw.sum() - area) < 1e-13
        assert abs((np.einsum("qd,qd->q", x, nrm) * jw).sum() - xn) < 1e-13
        np.testing.assert_allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-15)
        assert np.all(np.isclose(np.abs(nrm).max(axis=1), 1.0))  # the box's faces are axis-aligned planes
    fel, side, qoff = o.facets(7)
    assert len(fel) == 2 * (5 * 4 + 5 * 6 + 4 * 6) and qoff[-1] == 16 * len(fel)
    assert np.all(np.diff(fel) >= 0)


def nodal_coordinates(o):
    """physical coordinates of every expanded node (trilinear map at the GLL nodes of each element)"""
    ce, xs, ed = o.coords_expanded(), o.xstart(), o.elem_degree()
    out = np.zeros((o.nexp, 3))
    for e in range(o.nelem):
        P = ed[e] + 1
        g = [po.lobatto(P[c])[0] for c in range(3)]
        loc = 0
        for i in range(P[0]):
            for j in range(P[1]):
                for k in range(P[2]):
                    xi = (g[0][i], g[1][j], g[2][k])
                    x = np.zeros(3)
                    for t in range(8):
                        b = ((t >> 2) & 1, (t >> 1) & 1, t & 1)
                        x += np.prod([(1 + (2 * b[c] - 1) * xi[c]) / 2 for c in range(3)]) * ce[e, t]
                    out[xs[e] + loc] = x
                    loc += 1
    return out


def interpolant(o, f):
    """global vector of the nodal interpolant of f (no Dirichlet sets; rows of E that are plain copies)"""
    xn = nodal_coordinates(o)
    em = o.emap()
    g = np.zeros(o.n)
    ok = em >= 0
    g[em[ok]] = f(xn[ok])
    return g


@pytest.mark.parametrize("hp", [False, True])
def test_linear_fields_are_reproduced(hp):
    ed = np.random.default_rng(4).integers(2, 5, size=27).astype(np.int32) if hp else None
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=5, dirichlet_mask=0, elem_degree=ed)
    a, c0 = np.array([0.3, -1.2, 0.7]), 0.4
    b, c1 = np.array([1.1, 0.5, -0.2]), -0.3
    f = lambda x: x @ a + c0
    h = lambda x: x @ b + c1
    gf, gh = interpolant(o, f), interpolant(o, h)
    jw, x, nrm, u = o.facet_points(7, gf)
    np.testing.assert_allclose(u[:, 0], f(x), rtol=0, atol=1e-13)
    for d in range(3):
        y = o.facet_commit(7, jw * f(x) * nrm[:, d])
        # sum_i y_i = int_G f n_d = int_O df/dx_d; y.h = int_G f h n_d = int_O d(f h)/dx_d (linear integrands:
        # value at the centroid of the unit cube)
        assert abs(y.sum() - a[d]) < 1e-12
        cen = np.full(3, 0.5)
        assert abs(y @ gh - (a[d] * h(cen) + b[d] * f(cen))) < 1e-12
