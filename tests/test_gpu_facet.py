"""Facet rules and the batched facet iterator on the device against the oracle (rules, facet lists, area weights,
points, normals, field values, committed boundary integrals; uniform and per-element orders, bs 1 and 3), and a
Poisson problem with a Neumann face (weak set 200) solved to its manufactured solution at the expected rate."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

BIT = {100: 1, 200: 2, 300: 4}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_facet_rules_match_oracle():
    for side in range(6):
        for order in range(0, 17, 2):
            n, w = dg.facet_rule(side, order)
            no, wo = po.facet_rule(side, order)
            np.testing.assert_allclose(n, no, rtol=0, atol=1e-15)
            np.testing.assert_allclose(w, wo, rtol=1e-15, atol=0)


CASES = [  # npoints, degree, per-element orders, bs, Dirichlet sets, weak sets
    ((5, 6, 5), 3, False, 1, (100,), (200, 300)),
    ((4, 4, 5), 4, True, 3, (300,), (100, 200)),
    ((5, 5, 5), 2, False, 3, (), (100, 200, 300)),
]


@pytest.mark.parametrize("npts,deg,hp,bs,dirichlet,weak", CASES)
def test_facet_iterator_matches_oracle(npts, deg, hp, bs, dirichlet, weak):
    ne = (npts[0] - 1) * (npts[1] - 1) * (npts[2] - 1)
    ed = np.random.default_rng(7).integers(2, 7, size=ne).astype(np.int32) if hp else None
    fs = dg.FS(npts, degree=deg, perturb=0.1, seed=2, bs=bs, dirichlet=dirichlet, weak=weak, elem_degree=ed)
    o = po.FS(*npts, degree=deg, perturb=0.1, seed=2, bs=bs, dirichlet_mask=sum(BIT[s] for s in dirichlet), elem_degree=ed)
    wm = sum(BIT[s] for s in weak)
    it = dg.FacetIterator(fs)
    fel, side, qoff = it.facets()
    oel, oside, oqoff = o.facets(wm)
    np.testing.assert_array_equal(fel, oel)
    np.testing.assert_array_equal(side, oside)
    np.testing.assert_array_equal(qoff, oqoff)
    g = np.random.default_rng(1).uniform(-1, 1, fs.n * bs)
    it.start(torch.as_tensor(g, device="cuda"))
    a = it.get()
    jw, x, nrm, u = o.facet_points(wm, g)
    np.testing.assert_allclose(host(a["jw"]), jw, rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(host(a["x"]), x, rtol=0, atol=1e-14)
    np.testing.assert_allclose(host(a["normal"]), nrm, rtol=0, atol=1e-14)
    assert np.linalg.norm(host(a["u"]) - u) <= 1e-12 * np.linalg.norm(u)
    v = np.random.default_rng(2).uniform(-1, 1, (len(jw), bs))
    a["v"].copy_(torch.as_tensor(v, device="cuda"))
    it.commit()
    y = torch.full((fs.n * bs,), 5.0, dtype=torch.float64, device="cuda")
    it.finish(y, dg.ADD_VALUES)
    yo = o.facet_commit(wm, v, np.full(fs.n * bs, 5.0), add=True)
    assert np.linalg.norm(host(y) - yo) <= 1e-12 * np.linalg.norm(yo)
    # INSERT commit replaces the earlier one; INSERT finish overwrites y
    it.start(None)
    it.get()["v"].copy_(torch.as_tensor(2 * v, device="cuda"))
    it.commit(dg.ADD_VALUES)
    it.commit(dg.INSERT_VALUES)
    it.finish(y, dg.INSERT_VALUES)
    yo = o.facet_commit(wm, 2 * v)
    assert np.linalg.norm(host(y) - yo) <= 1e-12 * np.linalg.norm(yo)


def test_no_weak_sets_is_empty():
    fs = dg.FS((4, 4, 4), degree=2, perturb=0.1, seed=1)
    it = dg.FacetIterator(fs)
    fel, _, qoff = it.facets()
    assert len(fel) == 0 and qoff[-1] == 0
    it.start(None)
    assert it.get()["jw"].numel() == 0
    it.commit()
    y = torch.ones(fs.n, dtype=torch.float64, device="cuda")
    it.finish(y, dg.INSERT_VALUES)
    assert float(torch.abs(y).max()) == 0.0


def exact(x):
    s0, s1 = torch.sin(np.pi * x[:, 0]), torch.sin(np.pi * x[:, 1])
    c0, c1 = torch.cos(np.pi * x[:, 0]), torch.cos(np.pi * x[:, 1])
    sh, ch = torch.sinh(x[:, 2]), torch.cosh(x[:, 2])
    u = s0 * s1 * sh
    du = torch.stack([np.pi * c0 * s1 * sh, np.pi * s0 * c1 * sh, s0 * s1 * ch], dim=1)
    return u, du


def neumann_poisson(M, p, neumann=True):
    """-lap u = (2 pi^2 - 1) u, u = sin(pi x) sin(pi y) sinh(z): zero on the walls (100) and the bottom (300),
    du/dn given on the top (weak set 200)"""
    fs = dg.FS((M + 1,) * 3, degree=p, perturb=0.1, seed=3, dirichlet=(100, 300), weak=(200,))
    it = dg.RulesetIterator(fs)
    it.start(None)
    a = it.get()
    u, _ = exact(a["x"])
    a["v"].copy_((a["jw"] * (2 * np.pi ** 2 - 1) * u)[:, None])
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    b = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    it.finish(b)
    if neumann:
        fi = dg.FacetIterator(fs)
        fi.start(None)
        c = fi.get()
        _, du = exact(c["x"])
        c["v"].copy_((c["jw"] * (du * c["normal"]).sum(1))[:, None])
        fi.commit()
        fi.finish(b, dg.ADD_VALUES)
    op = fs.operator()
    m = fs.matrix()
    m.assemble()
    x = torch.zeros_like(b)
    its, rn = dg.KSP(op, m, ksp_type=dg.dKSP_CG).solve(b, x, rtol=1e-12, maxit=3000)
    it.start(x)
    a = it.get()
    ue, du = exact(a["x"])
    uerr, gerr = it.error_norms(ue[:, None].contiguous(), du[:, None, :].contiguous())
    return uerr[1], gerr[1]


def test_neumann_poisson_converges():
    e4, g4 = neumann_poisson(4, 3)
    e8, g8 = neumann_poisson(8, 3)
    assert e8 < 2e-5
    assert e4 / e8 > 10 and g4 / g8 > 5  # h^4 in L2, h^3 in H1 at p = 3
    e8n, _ = neumann_poisson(8, 3, neumann=False)  # without the boundary term the top flux is wrong
    assert e8n > 100 * e8
