"""St. Venant-Kirchhoff elasticity (src/fs/tests/elast.c:224-309): the function and the Jacobian at a stashed
state on the device against the oracle, the Jacobian as the derivative of the function, the linear limit
F = I, and a Newton-Krylov solve preconditioned by the blocked Q1 matrix."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

E0, NU = 1.0, 0.3
LAM, MU = E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))
PAR = np.array([LAM, MU])


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def setup(degree=3, seed=1, npoints=(4, 4, 4)):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=seed, bs=3)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=seed, bs=3)
    g = np.random.default_rng(seed).uniform(-0.05, 0.05, fs.n * 3)
    return fs, o, g


@pytest.mark.parametrize("degree", [2, 3, 5])
def test_function_and_jacobian_match_oracle(degree):
    fs, o, g = setup(degree=degree, seed=degree)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    y = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    op.elasticity_function(dev(g), y)
    assert rel(host(y), o.apply(g, kind=4, param=PAR)) < 1e-12
    d = np.random.default_rng(7).uniform(-1, 1, fs.n * 3)
    jd = torch.zeros_like(y)
    op.mult(dev(d), jd)
    assert rel(host(jd), o.apply(d, kind=5, qdata=o.elast_state(g), param=PAR)) < 1e-12


def test_jacobian_is_derivative_and_linear_limit():
    fs, o, g = setup(degree=3, seed=4)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    d = np.random.default_rng(5).uniform(-1, 1, fs.n * 3)
    h = 1e-6
    yp, ym = (torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda") for _ in range(2))
    op.elasticity_function(dev(g + h * d), yp)
    op.elasticity_function(dev(g - h * d), ym)
    fd = (host(yp) - host(ym)) / (2 * h)
    op.elasticity_state(dev(g))
    jd = torch.zeros_like(yp)
    op.mult(dev(d), jd)
    assert rel(fd, host(jd)) < 1e-6
    # zero state: no force, and the Jacobian is linear elasticity; resetting the state restores it
    z = torch.zeros_like(yp)
    op.elasticity_function(dev(0 * g), z)
    assert float(torch.linalg.norm(z)) == 0.0
    lin, j0 = torch.zeros_like(yp), torch.zeros_like(yp)
    fs.operator(dg.dOP_ELASTICITY, param=(E0, NU)).mult(dev(d), lin)
    op.mult(dev(d), j0)
    assert rel(host(j0), host(lin)) < 1e-14
    op.elasticity_state(dev(g))
    op.elasticity_state(None)
    op.mult(dev(d), j0)
    assert rel(host(j0), host(lin)) < 1e-15


def test_newton_krylov_large_deformation():
    fs, o, _ = setup(degree=3, seed=6, npoints=(5, 5, 5))
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    m = fs.matrix()
    m.assemble(kind=dg.dOP_ELASTICITY, param=(E0, NU))  # linear-elasticity Q1 as the preconditioner
    b = dev(np.random.default_rng(0).uniform(-1, 1, fs.n * 3) * 2e-3)
    u = torch.zeros_like(b)
    F = torch.zeros_like(b)
    op.elasticity_function(u, F)
    F -= b
    f0 = float(torch.linalg.norm(F))
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, restart=30)
    for k in range(12):
        du = torch.zeros_like(u)
        ksp.solve(-F, du, rtol=1e-6, maxit=500)
        u += du
        op.elasticity_function(u, F)  # also the state of the next Jacobian
        F -= b
        if float(torch.linalg.norm(F)) <= 1e-9 * f0:
            break
    assert float(torch.linalg.norm(F)) <= 1e-9 * f0 and k <= 6
    r = o.apply(host(u), kind=4, param=PAR) - host(b)
    assert np.linalg.norm(r) <= 1e-8 * f0
    assert float(torch.linalg.norm(u)) > 0


def test_reference_elast_target_through_the_product():
    """the reference's elast-e0-b3-g01 target (src/fs/tests/CMakeLists.txt:58; the problem and its oracle side are in
    tests/test_oracle_ellip_elast_golden.py) through the product: the exact solution's Dirichlet values committed to the
    space (dFSInhomogeneousDirichletCommit), the body force integrated by the dRulesetIterator, and
    dOperatorElasticityFunction at zero, whose dFS_INHOMOGENEOUS expansion is ElastFunction's (elast.c:293): ||F(0)|| is
    the printed first SNES function norm 14965.9 to six digits, and the residual vector is the oracle's"""
    import test_oracle_ellip_elast_golden as G
    name = "elast_e0_b3_g01"
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    O = G.Problem(*G.CASES[name])
    fs = dg.FS((5, 5, 5), degree=3, box=G.BOX, perturb=0.0, seed=1, bs=3)
    assert (fs.n, fs.nc) == (O.fs.n, O.fs.nc)
    fs.dirichlet_commit(dev(np.concatenate([O.s, O.dc])))
    it = dg.RulesetIterator(fs)
    it.start(None)
    a = it.get()
    np.testing.assert_allclose(a["x"].cpu().numpy(), O.fs.qpt_coords(), rtol=0, atol=1e-14)
    a["v"].copy_(a["jw"][:, None] * dev(O.fq))
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    b = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    it.finish(b)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    y = torch.zeros_like(b)
    op.elasticity_function(torch.zeros_like(b), y)
    F0 = host(y) - host(b)
    assert abs(np.linalg.norm(F0) - ref["fnorm0"][0]) < 3e-6 * ref["fnorm0"][0], np.linalg.norm(F0)
    assert rel(F0, O.F(np.zeros(fs.n * 3))) < 1e-12
    # the Jacobian at that state (F from the inhomogeneous expansion) against the oracle's at the same state
    d = np.random.default_rng(3).uniform(-1, 1, fs.n * 3)
    jd = torch.zeros_like(b)
    op.mult(dev(d), jd)
    assert rel(host(jd), O.fs.apply(d, kind=5, qdata=O.qdata(np.zeros(fs.n * 3)), param=PAR)) < 1e-12
