"""Geometric multigrid on the Q1-embedded lattice (dPC_MG_Q1): the configuration-1 solve against the oracle with
a fraction of the Chebyshev-Jacobi iterations, mesh-independent CG iteration counts, a lognormal coefficient with
FGMRES, a p-Laplacian Newton solve, and the refusals (blocked, mixed-order and odd lattices)."""
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


def solve(fs, op, m, b, pc, ksp_type=dg.dKSP_CG, rtol=1e-8, maxit=3000):
    ksp = dg.KSP(op, m, ksp_type=ksp_type, pc=pc)
    x = torch.zeros_like(b)
    its, rn = ksp.solve(b, x, rtol=rtol, maxit=maxit)
    r = torch.empty_like(x)
    op.mult(x, r)
    return its, float(torch.linalg.norm(b - r) / torch.linalg.norm(b)), x


def test_poisson_8_with_multigrid():
    fs = dg.FS((9, 9, 9), degree=4, perturb=0.1, seed=1)
    o = po.FS(9, 9, 9, degree=4, perturb=0.1, seed=1)
    f = np.random.default_rng(0).uniform(-1, 1, fs.n)
    b = torch.as_tensor(o.apply(f, kind=3), device="cuda")
    op, m = fs.operator(), fs.matrix()
    m.assemble()
    its_c, res_c, _ = solve(fs, op, m, b, dg.dPC_CHEBYSHEV_Q1)
    its_m, res_m, x = solve(fs, op, m, b, dg.dPC_MG_Q1)
    assert res_c <= 1.01e-8 and res_m <= 1.01e-8
    assert its_m <= its_c // 2, (its_m, its_c)  # the Q1-embedding bounds what any Q1 solve can give at 8^3
    bo = b.cpu().numpy()
    xo, _, _ = o.cg_solve(bo, o.q1_assemble(), rtol=1e-10, maxit=2000, nthreads=4)
    assert np.linalg.norm(x.cpu().numpy() - xo) / np.linalg.norm(xo) < 1e-6


def test_iterations_do_not_grow_with_the_mesh():
    its = []
    for M in (8, 16, 32):
        fs = dg.FS((M + 1,) * 3, degree=4, perturb=0.1, seed=2)
        b = torch.as_tensor(np.random.default_rng(M).uniform(-1, 1, fs.n), device="cuda")
        op, m = fs.operator(), fs.matrix()
        m.assemble()
        n, res, _ = solve(fs, op, m, b, dg.dPC_MG_Q1)
        assert res <= 1.01e-8
        its.append(n)
    assert its[2] <= its[0] + 10, its


def test_lognormal_fgmres():
    M = 16
    fs = dg.FS((M + 1,) * 3, degree=4, perturb=0.1, seed=1)
    grf = dg.grf_create(64, 2.0, 0.1, 3)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    m = fs.matrix()
    m.assemble(grf=grf)
    b = torch.as_tensor(np.random.default_rng(3).uniform(-1, 1, fs.n), device="cuda")
    its_c, res_c, _ = solve(fs, op, m, b, dg.dPC_CHEBYSHEV_Q1, dg.dKSP_FGMRES)
    its_m, res_m, _ = solve(fs, op, m, b, dg.dPC_MG_Q1, dg.dKSP_FGMRES)
    assert res_c <= 1.01e-8 and res_m <= 1.01e-8
    assert its_m <= its_c // 4, (its_m, its_c)


def test_fp32_cycle_on_a_box_lattice():
    """the FP32 V-cycle (the scalar fine-level stencil product on 32 x 8 node tiles, ragged at every edge of a
    33 x 17 x 25 lattice) inside FGMRES with FP32 inner applies: the same convergence as the FP64 cycle"""
    fs = dg.FS((9, 5, 7), degree=4, perturb=0.1, seed=4)
    b = torch.as_tensor(np.random.default_rng(4).uniform(-1, 1, fs.n), device="cuda")
    op, m = fs.operator(), fs.matrix()
    m.assemble()
    its = {}
    for prec in (dg.dPREC_FP64, dg.dPREC_FP32):
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30, pc=dg.dPC_MG_Q1)
        x = torch.zeros_like(b)
        its[prec], _ = ksp.solve(b, x, rtol=1e-8, maxit=500)
        r = torch.empty_like(x)
        op.mult(x, r)
        assert float(torch.linalg.norm(b - r) / torch.linalg.norm(b)) <= 1.01e-8
    assert its[dg.dPREC_FP32] <= its[dg.dPREC_FP64] + 3, its


def test_plaplace_newton_with_multigrid():
    fs = dg.FS((9, 9, 9), degree=4, perturb=0.1, seed=1)
    b = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, fs.n), device="cuda")
    op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
    m = fs.matrix()
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, pc=dg.dPC_MG_Q1)
    u = torch.zeros_like(b)
    res = dg.plap_newton(op, m, ksp, b, u, 1.5, 1e-6, rtol=1e-8, lin_rtol=1e-3, lin_maxit=200, max_it=40)
    its, fnorm = res[0], res[1]
    assert fnorm[-1] <= 1e-8 * fnorm[0]


def test_blocked_elasticity():
    """the 3 x 3 blocked Q1 elasticity matrix: CG iterations stay flat where Chebyshev-Jacobi's grow"""
    res = {}
    for M in (4, 8, 16):
        fs = dg.FS((M + 1,) * 3, degree=4, perturb=0.1, seed=3, bs=3)
        op = fs.operator(dg.dOP_ELASTICITY, param=(1.0, 0.3))
        m = fs.matrix()
        m.assemble(kind=dg.dOP_ELASTICITY, param=(1.0, 0.3))
        b = torch.as_tensor(np.random.default_rng(M).uniform(-1, 1, fs.n * 3), device="cuda")
        its_m, r_m, _ = solve(fs, op, m, b, dg.dPC_MG_Q1)
        its_c, r_c, _ = solve(fs, op, m, b, dg.dPC_CHEBYSHEV_Q1)
        assert r_m <= 1.01e-8 and r_c <= 1.01e-8
        res[M] = (its_m, its_c)
    assert res[16][0] <= res[4][0] + 15 and res[16][0] < res[16][1] // 3, res


def test_refusals():
    odd = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=1)  # 3 elements x degree 3 = 9 intervals: odd
    op, m = odd.operator(), odd.matrix()
    m.assemble()
    with pytest.raises(dg.DohpError):
        solve(odd, op, m, torch.ones(odd.n, dtype=torch.float64, device="cuda"), dg.dPC_MG_Q1)
