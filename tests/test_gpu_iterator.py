"""Batched dRulesetIterator: a q-function written in torch between GetPatchApplied and CommitPatchApplied
reproduces the fused operator applies and the oracle (src/fs/interface/fsrulesetit.c, the Start /
GetPatchApplied / CommitPatchApplied / Finish cycle used by src/fs/tests/elast.c and src/fs/tests/ellip.c)."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

E0, NU = 1.0, 0.3
LAM, MU = E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def cycle(fs, g, qfun, use_v=False, use_dv=True):
    it = dg.RulesetIterator(fs)
    it.start(torch.as_tensor(g, device="cuda"))
    a = it.get()
    qfun(a)
    it.commit(dg.INSERT_VALUES, use_v, use_dv)
    y = torch.zeros(fs.n * fs.bs, dtype=torch.float64, device="cuda")
    it.finish(y)
    torch.cuda.synchronize()
    return y.cpu().numpy(), it, a


def poisson(a):
    a["dv"].copy_(a["jw"][:, None, None] * a["du"])


@pytest.mark.parametrize("p", [1, 2, 4, 7])
def test_poisson_qfunction_matches_operator_and_oracle(p):
    npoints = (4, 5, 4)
    fs = dg.FS(npoints, degree=p, perturb=0.1, seed=p)
    o = po.FS(*npoints, degree=p, perturb=0.1, seed=p)
    g = np.random.default_rng(p).uniform(-1, 1, fs.n)
    y, _, _ = cycle(fs, g, poisson)
    yo = o.apply(g)
    assert np.linalg.norm(y - yo) / np.linalg.norm(yo) < 1e-12
    yf = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    fs.operator().mult(torch.as_tensor(g, device="cuda"), yf)
    torch.cuda.synchronize()
    assert np.linalg.norm(y - yf.cpu().numpy()) / np.linalg.norm(yo) < 1e-13


def test_elasticity_qfunction_matches_operator():
    npoints = (4, 4, 3)
    fs = dg.FS(npoints, degree=3, perturb=0.1, seed=3, bs=3)
    o = po.FS(*npoints, degree=3, perturb=0.1, seed=3, bs=3)
    g = np.random.default_rng(0).uniform(-1, 1, fs.n * 3)

    def elast(a):  # ElastPointwiseFunction (src/fs/tests/elast.c): sigma = lam tr(eps) I + 2 mu eps
        du = a["du"]
        eps = 0.5 * (du + du.transpose(1, 2))
        tr = eps.diagonal(dim1=1, dim2=2).sum(-1)
        sig = LAM * tr[:, None, None] * torch.eye(3, dtype=du.dtype, device=du.device) + 2 * MU * eps
        a["dv"].copy_(a["jw"][:, None, None] * sig)

    y, _, _ = cycle(fs, g, elast)
    yo = o.apply(g, kind=2, param=np.array([LAM, MU]))
    assert np.linalg.norm(y - yo) / np.linalg.norm(yo) < 1e-12


def test_energy_identities_mass_and_stiffness():
    """g^T M g = sum jw u^2 and g^T A g = sum jw |grad u|^2 (restriction is E^T, homogeneous Dirichlet)."""
    fs = dg.FS((5, 4, 4), degree=4, perturb=0.15, seed=9)
    g = np.random.default_rng(3).standard_normal(fs.n)
    mass = lambda a: a["v"].copy_(a["jw"][:, None] * a["u"])
    y, _, a = cycle(fs, g, mass, use_v=True, use_dv=False)
    e = float((a["jw"][:, None] * a["u"] ** 2).sum())
    assert abs(g @ y - e) < 1e-12 * abs(e)
    y, _, a = cycle(fs, g, poisson)
    e = float((a["jw"][:, None, None] * a["du"] ** 2).sum())
    assert abs(g @ y - e) < 1e-12 * abs(e)


def test_coordinates_and_jacobian():
    """x matches dFSGetQuadratureCoordinates; jw sums to the mesh volume (the box [0,1]^3)."""
    fs = dg.FS((4, 4, 5), degree=3, perturb=0.1, seed=2)
    _, _, a = cycle(fs, np.zeros(fs.n), poisson)
    xq = torch.zeros(fs.nq * 3, dtype=torch.float64, device="cuda")
    fs.qpt_coords(xq)
    torch.cuda.synchronize()
    np.testing.assert_allclose(a["x"].cpu().numpy().ravel(), xq.cpu().numpy(), rtol=0, atol=1e-14)
    assert abs(float(a["jw"].sum()) - 1.0) < 1e-13
    assert float(a["jw"].min()) > 0


def test_restart_and_add_mode():
    fs = dg.FS((4, 4, 4), degree=2, perturb=0.1, seed=4)
    g = np.random.default_rng(4).uniform(-1, 1, fs.n)
    y1, it, _ = cycle(fs, g, poisson)
    y = torch.as_tensor(y1, device="cuda").clone()
    it.start(torch.as_tensor(g, device="cuda"))
    poisson(it.get())
    it.commit()
    it.finish(y, dg.ADD_VALUES)
    torch.cuda.synchronize()
    np.testing.assert_allclose(y.cpu().numpy(), 2 * y1, rtol=1e-15, atol=1e-15)


def test_errors():
    fs = dg.FS((3, 3, 3), degree=2, seed=1)
    with pytest.raises(dg.DohpError):
        dg.RulesetIterator(fs, method=dg.SELF)
    it = dg.RulesetIterator(fs)
    with pytest.raises(dg.DohpError):
        it.get()


@pytest.mark.parametrize("bs", [1, 3])
def test_mixed_order_space_matches_oracle_and_operator(bs):
    """per-element orders 1..7: one batched apply per order bucket, each element at its own offsets"""
    npoints = (4, 5, 4)
    ne = 3 * 4 * 3
    ed = np.random.default_rng(11 + bs).integers(1, 8, size=ne).astype(np.int32)
    fs = dg.FS(npoints, degree=4, perturb=0.1, seed=5, bs=bs, elem_degree=ed)
    o = po.FS(*npoints, degree=4, perturb=0.1, seed=5, bs=bs, elem_degree=ed)
    assert fs.nq == o.num_qpts()[0]
    g = np.random.default_rng(bs).uniform(-1, 1, fs.n * bs)
    mass = lambda a: a["v"].copy_(a["jw"][:, None] * a["u"])
    y, it, a = cycle(fs, g, mass, use_v=True, use_dv=False)
    if bs == 1:  # the oracle's mass apply is scalar
        yo = o.apply(g, kind=3)
        assert np.linalg.norm(y - yo) / np.linalg.norm(yo) < 1e-12
    np.testing.assert_allclose(a["x"].cpu().numpy(), o.qpt_coords(), rtol=0, atol=1e-14)
    assert abs(float(a["jw"].sum()) - 1.0) < 1e-13
    if bs == 1:
        y, _, _ = cycle(fs, g, poisson)
        yo = o.apply(g)
        yf = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        fs.operator().mult(torch.as_tensor(g, device="cuda"), yf)
    else:
        def elast(a):
            du = a["du"]
            eps = 0.5 * (du + du.transpose(1, 2))
            tr = eps.diagonal(dim1=1, dim2=2).sum(-1)
            sig = LAM * tr[:, None, None] * torch.eye(3, dtype=du.dtype, device=du.device) + 2 * MU * eps
            a["dv"].copy_(a["jw"][:, None, None] * sig)
        y, _, _ = cycle(fs, g, elast)
        yo = o.apply(g, kind=2, param=np.array([LAM, MU]))
        yf = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
        fs.operator(dg.dOP_ELASTICITY, param=(E0, NU)).mult(torch.as_tensor(g, device="cuda"), yf)
    torch.cuda.synchronize()
    assert np.linalg.norm(y - yo) / np.linalg.norm(yo) < 1e-12
    assert np.linalg.norm(y - yf.cpu().numpy()) / np.linalg.norm(yo) < 1e-12


def test_error_norms_match_numpy():
    """dRulesetIteratorErrorNorms = dNormsUpdate (src/util/util.c:121-144) summed over the points"""
    fs = dg.FS((4, 5, 4), degree=3, perturb=0.1, seed=2)
    g = np.random.default_rng(8).uniform(-1, 1, fs.n)
    it = dg.RulesetIterator(fs)
    it.start(torch.as_tensor(g, device="cuda"))
    a = it.get()
    rng = np.random.default_rng(9)
    eu = rng.standard_normal(a["u"].shape)
    edu = rng.standard_normal(a["du"].shape)
    ue, ge = it.error_norms(torch.as_tensor(eu, device="cuda"), torch.as_tensor(edu, device="cuda"))
    jw, u, du = a["jw"].cpu().numpy(), a["u"].cpu().numpy(), a["du"].cpu().numpy()
    r = eu - u
    gr = np.sqrt(((edu - du) ** 2).sum(-1))
    np.testing.assert_allclose(ue, [(np.abs(r) * jw[:, None]).sum(), np.sqrt((r ** 2 * jw[:, None]).sum()), np.abs(r).max()],
                               rtol=1e-12)
    np.testing.assert_allclose(ge, [(gr * jw[:, None]).sum(), np.sqrt((gr ** 2 * jw[:, None]).sum()), gr.max()], rtol=1e-12)


def test_error_norms_of_an_exactly_represented_solution():
    """u = x(1-x) y(1-y) z(1-z) lies in the p=2 space on an unperturbed mesh: errors at rounding level"""
    npoints = (4, 4, 5)
    fs = dg.FS(npoints, degree=2, perturb=0.0, seed=1)
    o = po.FS(*npoints, degree=2, perturb=0.0, seed=1)
    em, xs, ce = o.emap(), o.xstart(), o.coords_expanded()
    gll = po.lobatto(3)[0]
    f = lambda X: X[0] * (1 - X[0]) * X[1] * (1 - X[1]) * X[2] * (1 - X[2])
    g = np.zeros(fs.n)
    for e in range(o.nelem):
        lo, hi = ce[e].min(0), ce[e].max(0)
        for loc in range(27):
            d = em[xs[e] + loc]
            if d < fs.n:
                ijk = (loc // 9, (loc // 3) % 3, loc % 3)
                g[d] = f([lo[k] + (1 + gll[ijk[k]]) / 2 * (hi[k] - lo[k]) for k in range(3)])
    it = dg.RulesetIterator(fs)
    it.start(torch.as_tensor(g, device="cuda"))
    a = it.get()
    X = a["x"].cpu().numpy()
    eu = f(X.T)[:, None]
    edu = np.stack([(1 - 2 * X[:, 0]) * X[:, 1] * (1 - X[:, 1]) * X[:, 2] * (1 - X[:, 2]),
                    X[:, 0] * (1 - X[:, 0]) * (1 - 2 * X[:, 1]) * X[:, 2] * (1 - X[:, 2]),
                    X[:, 0] * (1 - X[:, 0]) * X[:, 1] * (1 - X[:, 1]) * (1 - 2 * X[:, 2])], -1)[:, None, :]
    ue, ge = it.error_norms(torch.as_tensor(eu, device="cuda"), torch.as_tensor(edu, device="cuda"))
    assert ue[2] < 1e-15 and ge[2] < 1e-13 and ue[1] < 1e-15


@pytest.mark.parametrize("p,bs", [(2, 1), (3, 1), (4, 1), (6, 3)])
def test_sparse_rule_iterator(p, bs):
    """SPARSE rule (2 Gauss points per GLL sub-interval, (2p)^3 per element): the mesh volume on a perturbed mesh
    (the trilinear det J is integrated exactly), and on an affine mesh the integrals of |u|^2 and |grad u|^2 of a
    linear field agree with the FAST rule's (both rules are exact there); the stiffness energy identity holds.
    Degree 6 with three components: 12^3 points per element, applied one component at a time."""
    npts = (4, 3, 5)
    fs = dg.FS(npts, degree=p, perturb=0.1, seed=p, bs=bs)
    it = dg.RulesetIterator(fs, method=dg.SPARSE)
    it.start(None)
    a = it.get()
    assert a["jw"].numel() == fs.nelem * (2 * p) ** 3
    assert abs(float(a["jw"].sum()) - 1.0) < 1e-13
    o = po.FS(*npts, degree=p, perturb=0.0, seed=p, dirichlet_mask=0)
    fs = dg.FS(npts, degree=p, perturb=0.0, seed=p, dirichlet=(), bs=bs)
    em, xs, ce = o.emap(), o.xstart(), o.coords_expanded()
    gll = po.lobatto(p + 1)[0]
    coef = np.array([[0.3, -1.1, 0.7, 0.2], [-0.4, 0.5, 0.9, -0.1], [1.3, 0.2, -0.6, 0.4]])[:bs]
    f = lambda X: np.stack([c[0] * X[0] + c[1] * X[1] + c[2] * X[2] + c[3] for c in coef], -1)
    g = np.zeros(fs.n * bs)
    P = p + 1
    for e in range(o.nelem):
        lo, hi = ce[e].min(0), ce[e].max(0)
        for loc in range(P ** 3):
            ijk = (loc // (P * P), (loc // P) % P, loc % P)
            node = em[xs[e] + loc]
            g[node * bs:(node + 1) * bs] = f([lo[k] + (1 + gll[ijk[k]]) / 2 * (hi[k] - lo[k]) for k in range(3)])
    vals = {}
    for m in (dg.FAST, dg.SPARSE):
        it = dg.RulesetIterator(fs, method=m)
        it.start(torch.as_tensor(g, device="cuda"))
        a = it.get()
        vals[m] = (float((a["jw"][:, None] * a["u"] ** 2).sum()), float((a["jw"][:, None, None] * a["du"] ** 2).sum()))
        if m == dg.SPARSE:
            np.testing.assert_allclose(a["u"].cpu().numpy(), f(a["x"].cpu().numpy().T), rtol=0, atol=1e-13)
            a["dv"].copy_(a["jw"][:, None, None] * a["du"])
            it.commit(dg.INSERT_VALUES, use_v=False, use_dv=True)
            y = torch.zeros(fs.n * bs, dtype=torch.float64, device="cuda")
            it.finish(y)
            torch.cuda.synchronize()
            assert abs(g @ y.cpu().numpy() - vals[m][1]) < 1e-12 * abs(vals[m][1])
    np.testing.assert_allclose(vals[dg.SPARSE], vals[dg.FAST], rtol=1e-13)


@pytest.mark.parametrize("bs", [1, 3])
def test_sparse_rule_mixed_orders(bs):
    """SPARSE rules on a mixed-order space (per-element degrees 1..6, each element with the SPARSE rule of its own
    orders, as fsruleset.c:30-36 asks element by element): weights, values and gradients at every element's points
    against the oracle's tensor contraction with that element's SPARSE points and basis, the mesh volume, and the
    refusal of patch assembly (its patches are the sub-cells of one degree)"""
    npts = (4, 3, 5)
    ne = 3 * 2 * 4
    ed = np.random.default_rng(7 + bs).integers(1, 7, size=ne).astype(np.int32)
    fs = dg.FS(npts, degree=3, perturb=0.1, seed=3, bs=bs, elem_degree=ed, dirichlet=())
    g = torch.as_tensor(np.random.default_rng(bs).uniform(-1, 1, fs.n * bs), device="cuda")
    it = dg.RulesetIterator(fs, method=dg.SPARSE)
    it.start(g)
    a = it.get()
    qe = (2 * ed.astype(np.int64)) ** 3
    assert a["jw"].numel() == int(qe.sum())
    assert abs(float(a["jw"].sum()) - 1.0) < 1e-13
    xexp = torch.zeros(fs.nexp * bs, dtype=torch.float64, device="cuda")
    fs.global_to_expanded(g, xexp)
    torch.cuda.synchronize()
    xexp = xexp.cpu().numpy()
    _, xs = fs.emap()
    u, du, dx, jw = (a[k].cpu().numpy() for k in ("u", "du", "dx", "jw"))
    qoff = np.concatenate([[0], np.cumsum(qe)])
    efs_of = {}
    for e in range(ne):
        p = int(ed[e])
        if p not in efs_of:
            efs = fs.jac.efs(p, method=dg.SPARSE)
            assert efs.Q == [2 * p] * 3
            x1, w1 = efs.points[:2 * p], efs.weights[:2 * p]
            interp, deriv, _, _ = po.tensor_basis(p + 1, x1)
            efs_of[p] = (interp, deriv, np.einsum("i,j,k->ijk", w1, w1, w1).ravel())
        interp, deriv, w = efs_of[p]
        q = slice(qoff[e], qoff[e + 1])
        jinv = np.linalg.inv(dx[q])
        np.testing.assert_allclose(jw[q], w * np.linalg.det(dx[q]), rtol=1e-13, atol=0)
        xe = xexp[xs[e] * bs:(xs[e] + (p + 1) ** 3) * bs]
        for amode, got in ((dg.dAPPLY_INTERP, u[q]), (dg.dAPPLY_GRAD, du[q])):
            ref = po.efs_apply_hex([p + 1] * 3, [2 * p] * 3, [interp] * 3, [deriv] * 3, jinv.ravel(), bs, xe, amode)
            assert np.linalg.norm(got.ravel() - ref) <= 1e-13 * np.linalg.norm(ref), (e, p, amode)
    L = dg.lib()
    P, rc, bi, bd = ctypes.c_int32(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    NULL = ctypes.c_void_p(0)
    assert L.dRulesetIteratorGetPatchAssembly(it.h, NULL, NULL, NULL, NULL, ctypes.byref(P), ctypes.byref(rc), ctypes.byref(bi),
                                              ctypes.byref(bd)) != 0
