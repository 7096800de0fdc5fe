"""The CPU-runnable configuration: Poisson on an 8^3 perturbed mesh, p=4, right-hand side b = int v f_h with
f_h = sum f_i phi_i, f_i ~ U[-1,1] (the mass apply of src/fs/tests/ex1.c:399-430, here through the batched
dRulesetIterator), CG with the Q1-embedded Chebyshev-Jacobi preconditioner to rtol 1e-8 -- on the GPU and in
the oracle, same seeded inputs."""
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


def mass_rhs(fs, f):
    it = dg.RulesetIterator(fs)
    it.start(torch.as_tensor(f, device="cuda"))
    a = it.get()
    a["v"].copy_(a["jw"][:, None] * a["u"])
    it.commit(dg.INSERT_VALUES, use_v=True, use_dv=False)
    b = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    it.finish(b)
    torch.cuda.synchronize()
    return b


def test_poisson_8_end_to_end():
    fs = dg.FS((9, 9, 9), degree=4, perturb=0.1, seed=1)
    o = po.FS(9, 9, 9, degree=4, perturb=0.1, seed=1)
    assert fs.n == 29791
    f = np.random.default_rng(0).uniform(-1, 1, fs.n)
    b = mass_rhs(fs, f)
    bo = o.apply(f, kind=3)
    assert np.linalg.norm(b.cpu().numpy() - bo) / np.linalg.norm(bo) < 1e-12
    op = fs.operator()
    m = fs.matrix()
    m.assemble()
    x = torch.zeros_like(b)
    its, rn = dg.KSP(op, m, ksp_type=dg.dKSP_CG).solve(b, x, rtol=1e-8, maxit=1000)
    xg = x.cpu().numpy()
    assert np.linalg.norm(bo - o.apply(xg)) <= 1.01e-8 * np.linalg.norm(bo)
    xo, its_o, rn_o = o.cg_solve(bo, o.q1_assemble(), rtol=1e-8, maxit=1000, nthreads=4)
    assert its_o > 0 and rn_o <= 1e-8
    assert abs(its - its_o) <= 2
    assert np.linalg.norm(xg - xo) / np.linalg.norm(xo) < 1e-6
