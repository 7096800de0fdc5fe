"""p-Laplacian (src/fs/tests/ellip.c:333-536): store, function, matrix-free Jacobian, Q1-embedded Jacobian
and Newton-Krylov on the device, against the oracle on the same seeded meshes and states."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

P, EPS = 1.5, 1e-6


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


def setup(npoints=(4, 5, 4), degree=3, seed=1):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=seed)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=seed)
    g = np.random.default_rng(seed).uniform(-1, 1, fs.n)
    return fs, o, g


@pytest.mark.parametrize("pe,degree", [(1.5, 3), (1.5, 6), (1.2, 4), (2.0, 2)])
def test_stash_and_jacobian_match_oracle(pe, degree):
    fs, o, g = setup(degree=degree, seed=degree)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    op.plap_stash(dev(g), pe, EPS)
    st = torch.zeros(fs.nq * 4, dtype=torch.float64, device="cuda")
    op.get_qdata(st)
    sto = o.plap_stash(g, pe, EPS)
    assert rel(host(st), sto) < 1e-13
    x = np.random.default_rng(7).uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(dev(x), y)
    yo = o.apply(x, kind=1, qdata=sto)
    assert rel(host(y), yo) < 1e-12


def test_exponent_outside_range_is_an_error():
    """The store's sqrt(-eta') (ellip.c:339) is real only for p <= 2; the oracle gives NaN there."""
    fs, o, g = setup(degree=2, seed=9)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    for pe in (3.0, 1.0):
        with pytest.raises(dg.DohpError):
            op.plap_stash(dev(g), pe, EPS)
    with pytest.raises(dg.DohpError):
        op.mult(dev(g), torch.zeros(fs.n, dtype=torch.float64, device="cuda"))  # no stash yet
    assert np.isnan(o.plap_stash(g, 3.0, EPS)).any()


def test_set_quadrature_data_path():
    fs, o, g = setup(seed=2)
    sto = o.plap_stash(g, P, EPS)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    op.set_qdata(dev(sto))
    x = np.random.default_rng(3).uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(dev(x), y)
    assert rel(host(y), o.apply(x, kind=1, qdata=sto)) < 1e-12


def test_function_matches_oracle():
    """EllipFunction's Dv = w eta Du is the Jacobian q-function with s = 0."""
    fs, o, g = setup(degree=4, seed=3)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.plap_function(dev(g), P, EPS, y)
    st = o.plap_stash(g, P, EPS).reshape(-1, 4).copy()
    st[:, 1:] = 0
    assert rel(host(y), o.apply(g, kind=1, qdata=st.ravel())) < 1e-12


def test_jacobian_is_derivative_of_function():
    """(N(g + h d) - N(g - h d)) / 2h -> J(g) d (central difference, FP64)."""
    fs, o, g = setup(degree=3, seed=4)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    d = np.random.default_rng(5).uniform(-1, 1, fs.n)
    h = 1e-5
    yp = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    ym = torch.zeros_like(yp)
    op.plap_function(dev(g + h * d), P, EPS, yp)
    op.plap_function(dev(g - h * d), P, EPS, ym)
    fd = (host(yp) - host(ym)) / (2 * h)
    op.plap_stash(dev(g), P, EPS)
    jd = torch.zeros_like(yp)
    op.mult(dev(d), jd)
    assert rel(fd, host(jd)) < 1e-7


@pytest.mark.parametrize("quirk", [1, 0])
def test_q1_plap_matches_oracle(quirk):
    fs, o, g = setup(degree=3, seed=5)
    m = fs.matrix()
    m.assemble_plap(dev(g), P, EPS, quirk=quirk)
    rp, col, val = m.csr_host()
    rpo, colo, valo = o.q1_assemble(kind=1, param=(P, EPS), state=g, quirk=quirk)
    np.testing.assert_array_equal(rp, rpo)
    np.testing.assert_array_equal(col, colo)
    assert np.abs(val - valo).max() < 1e-12 * np.abs(valo).max()


def test_fp32_jacobian_error():
    fs, o, g = setup(degree=6, seed=6)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    op.plap_stash(dev(g), P, EPS)
    x = dev(np.random.default_rng(1).uniform(-1, 1, fs.n))
    y64 = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    y32 = torch.zeros_like(y64)
    op.mult(x, y64)
    op.set_precision(dg.dPREC_FP32)
    op.mult(x, y32)
    e = rel(host(y32), host(y64))
    assert 1e-9 < e < 1e-5


def newton(fs, b, inner_prec, lin_rtol=1e-3):
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    m = fs.matrix()
    u = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    m.assemble_plap(u, P, EPS)
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=inner_prec, restart=30)
    its, fn, li = dg.plap_newton(op, m, ksp, dev(b), u, P, EPS, rtol=1e-8, lin_rtol=lin_rtol)
    return host(u), its, fn, li


def test_newton_fp64_and_mixed_reach_the_oracle_solution():
    fs, o, _ = setup(npoints=(6, 6, 6), degree=3, seed=7)
    b = np.random.default_rng(0).uniform(-1, 1, fs.n)
    u64, its64, fn64, _ = newton(fs, b, dg.dPREC_FP64)
    u32, its32, fn32, _ = newton(fs, b, dg.dPREC_FP32)
    assert fn64[its64] <= 1e-8 * fn64[0] and fn32[its32] <= 1e-8 * fn32[0]
    assert its64 <= 12 and its32 <= 14
    # the oracle's own residual at the GPU solutions
    for u in (u64, u32):
        st = o.plap_stash(u, P, EPS).reshape(-1, 4).copy()
        st[:, 1:] = 0
        r = o.apply(u, kind=1, qdata=st.ravel()) - b
        assert np.linalg.norm(r) <= 1e-7 * fn64[0]
    assert rel(u32, u64) < 1e-6


@pytest.mark.parametrize("name", ["ellip_e0_b3_p16", "ellip_e0_b3_p14"])
def test_reference_ellip_target_through_the_product(name):
    """the reference's ellip-e0-b3-p16 / -p14 targets (src/fs/tests/CMakeLists.txt:50-51; the problem and its oracle
    side are in tests/test_oracle_ellip_elast_golden.py) through the product: the exact solution's Dirichlet values
    committed to the space (dFSInhomogeneousDirichletCommit, as ellip.c:719-724), the forcing integrated by the
    dRulesetIterator, dOperatorPLaplaceFunction at zero (its dFS_INHOMOGENEOUS expansion, as EllipFunction):
    ||F(0)|| is the printed first SNES function norm to six digits, and the residual vector is the oracle's"""
    import test_oracle_ellip_elast_golden as G
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    O = G.Problem(*G.CASES[name])
    pe, eps = O.param
    fs = dg.FS((5, 5, 5), degree=3, box=G.BOX, perturb=0.0, seed=1)
    assert (fs.n, fs.nc) == (O.fs.n, O.fs.nc)
    fs.dirichlet_commit(dev(np.concatenate([O.s, O.dc])))
    it = dg.RulesetIterator(fs)
    it.start(None)
    a = it.get()
    np.testing.assert_allclose(a["x"].cpu().numpy(), O.fs.qpt_coords(), rtol=0, atol=1e-14)
    a["v"].copy_(a["jw"][:, None] * dev(O.fq))
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    b = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    it.finish(b)
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    y = torch.zeros_like(b)
    op.plap_function(torch.zeros_like(b), pe, eps, y)
    F0 = host(y) - host(b)
    assert abs(np.linalg.norm(F0) - ref["fnorm0"][0]) < 3e-6 * ref["fnorm0"][0], np.linalg.norm(F0)
    assert rel(F0, O.F(np.zeros(fs.n))) < 1e-12
