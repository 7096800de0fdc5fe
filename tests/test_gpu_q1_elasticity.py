"""Blocked (bs = 3) Q1-embedded elasticity matrix (ElastJacobian, src/fs/tests/elast.c:343-407, into the
dFSCreateMatrix BAIJ layout with interleaved components): sparsity bit-exact and values within 1e-12 of the
oracle, uniform and mixed-order spaces, reference quirk on and off; CG with Chebyshev-Jacobi on it solves
the matrix-free elasticity problem (ElastShellMatMult) to rtol 1e-8 on the oracle's residual."""
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


@pytest.mark.parametrize("degree,quirk", [(2, 1), (3, 1), (3, 0), (5, 1)])
def test_blocked_q1_matches_oracle(degree, quirk):
    npoints = (4, 4, 3)
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=2, bs=3)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=2, bs=3)
    m = fs.matrix()
    m.assemble(kind=dg.dOP_ELASTICITY, param=(E0, NU), quirk=quirk)
    rp, col, val = m.csr_host()
    rpo, colo, valo = o.q1_assemble(kind=2, param=(LAM, MU), quirk=quirk)
    np.testing.assert_array_equal(rp, rpo)
    np.testing.assert_array_equal(col, colo)
    assert np.abs(val - valo).max() <= 1e-12 * np.abs(valo).max()


def test_nonconforming_space_is_an_error():
    """interpolation-constrained (hp) E rows are not a node map: the Q1-embedded matrix is refused"""
    npoints = (4, 4, 3)
    ed = np.random.default_rng(3).integers(2, 6, size=3 * 3 * 2).astype(np.int32)
    fs = dg.FS(npoints, degree=4, perturb=0.1, seed=2, bs=3, elem_degree=ed)
    with pytest.raises(dg.DohpError, match="conforming"):
        fs.matrix()


def test_elasticity_cg_with_blocked_chebyshev_jacobi():
    npoints = (5, 5, 5)
    fs = dg.FS(npoints, degree=3, perturb=0.1, seed=4, bs=3)
    o = po.FS(*npoints, degree=3, perturb=0.1, seed=4, bs=3)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    m = fs.matrix()
    m.assemble(kind=dg.dOP_ELASTICITY, param=(E0, NU))
    b = np.random.default_rng(0).uniform(-1, 1, fs.n * 3)
    x = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
    its, rn = ksp.solve(torch.as_tensor(b, device="cuda"), x, rtol=1e-8, maxit=2000)
    r = b - o.apply(x.cpu().numpy(), kind=2, param=np.array([LAM, MU]))
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(b)
    # the preconditioner helps: plain CG needs more iterations
    x2 = torch.zeros_like(x)
    its_plain, _ = dg.KSP(op, m, ksp_type=dg.dKSP_CG, pc=dg.dPC_NONE).solve(torch.as_tensor(b, device="cuda"), x2,
                                                                            rtol=1e-8, maxit=5000)
    assert its < its_plain
