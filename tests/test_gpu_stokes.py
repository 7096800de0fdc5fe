"""Stokes (src/fs/tests/stokes.c) on the device: every block apply (A with and without the penalty, Bt, B,
coupled) against the oracle, the block-preconditioned FGMRES solve of a manufactured problem (divergence-free
velocity vanishing on the walls, zero-mean pressure) converging at the Taylor-Hood rates, and the power-law
rheology: the nonlinear function, the Jacobian at its state, and Newton recovering a discrete solution."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


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


def spaces(M, k, codim, seed=1, perturb=0.1):
    fsu = dg.FS((M + 1,) * 3, degree=k, perturb=perturb, seed=seed, bs=3)
    fsp = dg.FS(None, degree=k - codim, bs=1, dirichlet=(), mesh_of=fsu)
    return fsu, fsp


@pytest.mark.parametrize("k,codim,nu", [(3, 2, 0.0), (2, 1, 0.3), (4, 1, 0.0), (6, 2, 0.2)])
def test_blocks_match_oracle(k, codim, nu):
    M = 3
    fsu, fsp = spaces(M, k, codim, seed=k)
    ou = po.FS(M + 1, M + 1, M + 1, degree=k, perturb=0.1, seed=k, bs=3, dirichlet_mask=7)
    op = po.FS(M + 1, M + 1, M + 1, degree=k - codim, perturb=0.1, seed=k, bs=1, dirichlet_mask=0)
    rheo = (1.7, 1.0, 2.0, nu)
    st = dg.Stokes(fsu, fsp, rheo)
    rng = np.random.default_rng(k)
    xu, xp = rng.uniform(-1, 1, fsu.n * 3), rng.uniform(-1, 1, fsp.n)
    yu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
    yp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    st.mult(dg.dSTOKES_MULT_A, xu=dev(xu), yu=yu)
    assert rel(host(yu), po.stokes_apply(ou, op, 0, rheo, xu=xu)[0]) < 1e-12
    st.mult(dg.dSTOKES_MULT_BT, xp=dev(xp), yu=yu)
    assert rel(host(yu), po.stokes_apply(ou, op, 1, rheo, xp=xp)[0]) < 1e-12
    st.mult(dg.dSTOKES_MULT_B, xu=dev(xu), yp=yp)
    assert rel(host(yp), po.stokes_apply(ou, op, 2, rheo, xu=xu)[1]) < 1e-12
    st.mult(dg.dSTOKES_MULT_COUPLED, xu=dev(xu), xp=dev(xp), yu=yu, yp=yp)
    cu, cp = po.stokes_apply(ou, op, 3, rheo, xu=xu, xp=xp)
    assert rel(host(yu), cu) < 1e-12 and rel(host(yp), cp) < 1e-12


def test_errors():
    fsu, fsp = spaces(2, 3, 2)
    with pytest.raises(dg.DohpError):
        dg.Stokes(fsu, fsp, (1.0, 1.0, 1.0, 0.0))  # the power law needs p > 1
    with pytest.raises(dg.DohpError):
        dg.Stokes(fsu, fsp, (1.0, 0.0, 1.5, 0.0))  # and a positive regularisation when p != 2
    other = dg.FS((3, 3, 3), degree=1, bs=1, dirichlet=())
    with pytest.raises(dg.DohpError):
        dg.Stokes(fsu, other)  # not the same mesh
    with pytest.raises(dg.DohpError):
        dg.Stokes(fsu, dg.FS(None, degree=1, bs=1, mesh_of=fsu))  # pressure with Dirichlet sets


def exact(x, eta):
    """u = (psi_y, -psi_x, 0), psi = sin^2(pi x) sin^2(pi y) sin(pi z); p = cos(pi x) cos(pi y) cos(pi z);
    f = -div(eta Du) + grad p = -(eta/2) lap u + grad p (div u = 0)"""
    x = x.detach().clone().requires_grad_(True)
    pi = np.pi
    sx, sy, sz = torch.sin(pi * x[:, 0]), torch.sin(pi * x[:, 1]), torch.sin(pi * x[:, 2])
    cx, cy = torch.cos(pi * x[:, 0]), torch.cos(pi * x[:, 1])
    u = [sx ** 2 * 2 * pi * sy * cy * sz, -2 * pi * sx * cx * sy ** 2 * sz, torch.zeros_like(sx)]
    p = torch.cos(pi * x[:, 0]) * torch.cos(pi * x[:, 1]) * torch.cos(pi * x[:, 2])
    f = []
    for i in range(3):
        lap = torch.zeros_like(sx)
        if i < 2:
            g = torch.autograd.grad(u[i].sum(), x, create_graph=True)[0]
            for j in range(3):
                lap = lap + torch.autograd.grad(g[:, j].sum(), x, retain_graph=True)[0][:, j]
        gp = torch.autograd.grad(p.sum(), x, retain_graph=True)[0][:, i]
        f.append(-0.5 * eta * lap + gp)
    return (torch.stack([v.detach() for v in u], 1), p.detach(), torch.stack([v.detach() for v in f], 1))


def manufactured(M, k, codim, eta=1.0):
    fsu, fsp = spaces(M, k, codim, seed=7)
    st = dg.Stokes(fsu, fsp, (eta, 1.0, 2.0, 0.0))
    it = dg.RulesetIterator(fsu)
    it.start(None)
    a = it.get()
    _, _, f = exact(a["x"], eta)
    a["v"].copy_(a["jw"][:, None] * f)
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    bu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
    it.finish(bu)
    bp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
    xu, xp = torch.zeros_like(bu), torch.zeros_like(bp)
    its, rn = st.solve(bu, bp, xu, xp, rtol=1e-10, maxit=1000)
    # velocity error
    it.start(xu)
    a = it.get()
    ue, _, _ = exact(a["x"], eta)
    uerr, _ = it.error_norms(ue.contiguous(), None)
    # pressure error modulo constants
    ip = dg.RulesetIterator(fsp)
    ip.start(xp)
    b = ip.get()
    _, pe, _ = exact(b["x"], eta)
    e = b["u"][:, 0] - pe
    e = e - (b["jw"] * e).sum() / b["jw"].sum()
    perr = float(torch.sqrt((b["jw"] * e ** 2).sum()))
    return uerr[1], perr, its, abs(float(xp.sum()))


def test_manufactured_taylor_hood_converges():
    eu4, ep4, its4, m4 = manufactured(4, 3, 1)
    eu8, ep8, its8, m8 = manufactured(8, 3, 1)
    assert m4 < 1e-10 and m8 < 1e-10  # zero-mean pressure returned
    assert eu8 < 1e-3 and ep8 < 1e-2
    assert eu4 / eu8 > 10 and ep4 / ep8 > 5, (eu4, eu8, ep4, ep8)  # h^4 velocity, h^3 pressure at k = 3
    assert its8 < 2 * its4 + 20, (its4, its8)  # the block preconditioner keeps the count nearly mesh-independent


@pytest.mark.parametrize("k,codim", [(3, 2), (2, 1)])
def test_power_law_function_and_jacobian_match_oracle(k, codim):
    """p = 4/3 (Glen n = 3): the Jacobian at the zero state, the function (StokesFunction without forcing) at a
    random state, and the A / coupled Jacobian at that state (StokesPointwiseJacobian(_A)) against the oracle"""
    M = 3
    fsu, fsp = spaces(M, k, codim, seed=10 + k)
    ou = po.FS(M + 1, M + 1, M + 1, degree=k, perturb=0.1, seed=10 + k, bs=3, dirichlet_mask=7)
    op = po.FS(M + 1, M + 1, M + 1, degree=k - codim, perturb=0.1, seed=10 + k, bs=1, dirichlet_mask=0)
    rheo = (1.3, 0.7, 4.0 / 3.0, 0.2)
    st = dg.Stokes(fsu, fsp, rheo)
    rng = np.random.default_rng(20 + k)
    su, sp = 2.0 * rng.standard_normal(fsu.n * 3), rng.standard_normal(fsp.n)
    vu, vp = rng.standard_normal(fsu.n * 3), rng.standard_normal(fsp.n)
    yu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
    yp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    st.mult(dg.dSTOKES_MULT_A, xu=dev(vu), yu=yu)  # no state yet: eta = B (eps^2/2)^((p-2)/2)
    assert rel(host(yu), po.stokes_apply(ou, op, 0, rheo, xu=vu)[0]) < 1e-12
    st.function(dev(su), dev(sp), yu, yp)
    fu, fp = po.stokes_apply(ou, op, 4, rheo, xu=su, xp=sp)
    assert rel(host(yu), fu) < 1e-12 and rel(host(yp), fp) < 1e-12
    st.mult(dg.dSTOKES_MULT_A, xu=dev(vu), yu=yu)
    assert rel(host(yu), po.stokes_apply(ou, op, 0, rheo, xu=vu, state=su)[0]) < 1e-12
    st.mult(dg.dSTOKES_MULT_COUPLED, xu=dev(vu), xp=dev(vp), yu=yu, yp=yp)
    cu, cp = po.stokes_apply(ou, op, 3, rheo, xu=vu, xp=vp, state=su)
    assert rel(host(yu), cu) < 1e-12 and rel(host(yp), cp) < 1e-12
    st.mult(dg.dSTOKES_MULT_BT, xp=dev(vp), yu=yu)  # the pressure blocks do not depend on the state
    assert rel(host(yu), po.stokes_apply(ou, op, 1, rheo, xp=vp)[0]) < 1e-12


def test_power_law_newton_recovers_a_discrete_solution():
    """x* = the Newtonian solution of the manufactured forcing (scaled to strain rates of order one); b = N(x*) for
    the power law p = 4/3, eps = 0.5 (viscosity varying between about 0.7 and 2); Newton from zero with the
    block-preconditioned FGMRES (one Q1 multigrid V-cycle on the velocity block) returns x*"""
    fsu, fsp = spaces(4, 3, 2, seed=7)
    lin = dg.Stokes(fsu, fsp, (1.0, 1.0, 2.0, 0.0))
    it = dg.RulesetIterator(fsu)
    it.start(None)
    a = it.get()
    _, _, f = exact(a["x"], 1.0)
    a["v"].copy_(0.1 * a["jw"][:, None] * f)
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    bu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
    it.finish(bu)
    bp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
    xs_u, xs_p = torch.zeros_like(bu), torch.zeros_like(bp)
    lin.solve(bu, bp, xs_u, xs_p, rtol=1e-12, maxit=2000)
    pl = dg.Stokes(fsu, fsp, (1.0, 0.5, 4.0 / 3.0, 0.0))
    b2u, b2p = torch.zeros_like(bu), torch.zeros_like(bp)
    pl.function(xs_u, xs_p, b2u, b2p)
    xu, xp = torch.zeros_like(bu), torch.zeros_like(bp)
    k, fn, li = pl.newton(b2u, b2p, xu, xp, rtol=1e-11, lin_rtol=1e-6, lin_maxit=1000, max_it=40)
    assert fn[-1] <= 1e-11 * fn[0], (k, fn, li)
    assert 2 <= k <= 25, (k, fn)
    ru = float(torch.linalg.norm(xu - xs_u) / torch.linalg.norm(xs_u))
    rp = float(torch.linalg.norm(xp - xs_p) / torch.linalg.norm(xs_p))
    assert ru < 1e-7 and rp < 1e-6, (ru, rp, k, fn)
    assert abs(float(xp.sum())) < 1e-10


def test_reference_stokes_targets_through_the_product():
    """the reference's two Stokes targets (src/fs/tests/CMakeLists.txt:62-70; the problem and the oracle side are in
    tests/test_oracle_stokes_golden.py) through the product: Dirichlet values of the exact solution committed to the
    velocity space, the forcing integrated by the iterator (velocity) and dStokesIntegratePressure on the same rule,
    dStokesFunction and the Jacobian at its state reproduce the printed residual norms to six digits, and
    dStokesNewtonSolve's solution reproduces the printed error norms"""
    import test_oracle_stokes_golden as G
    here = os.path.dirname(os.path.abspath(__file__))
    for name, rheo in sorted(G.CASES.items()):
        ref = np.load(os.path.join(here, "golden", name + ".npz"))
        O = G.Problem(rheo)
        fsu = dg.FS((5, 5, 5), degree=3, box=G.BOX, perturb=0.0, seed=1, bs=3)
        fsp = dg.FS(None, degree=2, bs=1, dirichlet=(), mesh_of=fsu)
        assert (fsu.n, fsu.nc, fsp.n) == (O.fu.n, O.fu.nc, O.fp.n)
        nu3 = O.nu3
        fsu.dirichlet_commit(dev(np.concatenate([O.s[:nu3], O.ud])))
        st = dg.Stokes(fsu, fsp, rheo)
        it = dg.RulesetIterator(fsu)
        it.start(None)
        a = it.get()
        np.testing.assert_allclose(a["x"].cpu().numpy(), O.xq, rtol=0, atol=1e-14)
        a["v"].copy_(a["jw"][:, None] * dev(O.fq))
        it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
        bu = torch.zeros(nu3, dtype=torch.float64, device="cuda")
        it.finish(bu)
        bp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
        st.integrate_pressure(dev(O.fpq), bp)
        yu, yp = torch.zeros_like(bu), torch.zeros_like(bp)

        def F(x):
            st.function(dev(x[:nu3]), dev(x[nu3:]), yu, yp)
            return np.concatenate([host(yu) - host(bu), host(yp) - host(bp)])

        rel = lambda a, b: abs(a - b) / abs(b)
        F0 = F(np.zeros_like(O.s))
        assert rel(np.linalg.norm(F0), ref["fnorm0"][0]) < 3e-6, name
        Fs = F(O.s)  # leaves the state at s
        assert rel(np.linalg.norm(Fs), ref["residual_exact"][0]) < 3e-6, name
        np.testing.assert_allclose(Fs, O.F(O.s), rtol=0, atol=1e-12 * np.linalg.norm(Fs))
        st.mult(dg.dSTOKES_MULT_COUPLED, xu=dev(O.s[:nu3]), xp=dev(O.s[nu3:]), yu=yu, yp=yp)
        lin = np.concatenate([host(yu), host(yp)]) + F0
        assert rel(np.linalg.norm(lin), ref["linear_residual_exact"][0]) < 3e-6, name
        # the solve: from zero for the linear (Newtonian) target, from the interpolant for the power law
        x0 = np.zeros_like(O.s) if rheo[2] == 2.0 else O.s
        xu, xp = dev(x0[:nu3]), dev(x0[nu3:])
        k, fn, li = st.newton(bu, bp, xu, xp, rtol=1e-9, atol=1e-12, lin_rtol=1e-9, lin_maxit=3000, max_it=20)
        assert fn[-1] <= max(1e-9 * fn[0], 1e-12), (name, k, fn, li)
        x = np.concatenate([host(xu), host(xp)])
        assert np.linalg.norm(O.F(x)) < 1e-8, name  # the oracle's residual of the product's solution
        got = O.norms(x)
        for key in ("interpolation", "velocity", "gradient", "pressure"):
            np.testing.assert_allclose(got[key], ref[key], rtol=0.012, err_msg=name + " " + key)
