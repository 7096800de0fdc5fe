"""BF16 applies (BF16 storage of geometric factors, inputs, basis tables and Q1 values; FP32 arithmetic and
accumulation) inside FGMRES and Newton: each states its error against the FP64 path, and the solves still
reach the FP64 tolerance on the FP64 residual."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def lognormal(ne, seed, p=4):
    fs = dg.FS((ne + 1,) * 3, degree=p, perturb=0.1, seed=1)
    grf = dg.grf_create(64, 2.0, 0.1, seed)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    m = fs.matrix()
    m.assemble(grf=grf)
    return fs, op, m


@pytest.mark.parametrize("p", [2, 4, 6])
def test_bf16_apply_error(p):
    fs, op, _ = lognormal(6, 3, p=p)
    x = dev(np.random.default_rng(p).uniform(-1, 1, fs.n))
    y = {}
    for prec in (dg.dPREC_FP64, dg.dPREC_FP32, dg.dPREC_BF16):
        op.set_precision(prec)
        y[prec] = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        op.mult(x, y[prec])
    e32, e16 = rel(y[dg.dPREC_FP32], y[dg.dPREC_FP64]), rel(y[dg.dPREC_BF16], y[dg.dPREC_FP64])
    assert e32 < 1e-5 and 1e-4 < e16 < 3e-2 and e16 > 10 * e32


def test_bf16_fgmres_reaches_fp64_tolerance():
    fs, op, m = lognormal(8, 5)
    b = dev(np.random.default_rng(5).uniform(-1, 1, fs.n))
    its = {}
    for prec in (dg.dPREC_FP64, dg.dPREC_BF16):
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30)
        x = torch.zeros_like(b)
        its[prec], _ = ksp.solve(b, x, rtol=1e-8, maxit=3000)
        r = torch.empty_like(x)
        op.mult(x, r)
        assert float(torch.linalg.norm(b - r) / torch.linalg.norm(b)) <= 1.01e-8
    assert its[dg.dPREC_BF16] <= 2 * its[dg.dPREC_FP64]


def test_bf16_newton():
    P, EPS = 1.5, 1e-6
    fs = dg.FS((6, 6, 6), degree=3, perturb=0.1, seed=7)
    b = dev(np.random.default_rng(0).uniform(-1, 1, fs.n))
    res = {}
    for prec in (dg.dPREC_FP64, dg.dPREC_BF16):
        op = fs.operator(dg.dOP_PLAPLACE_JACOBIAN)
        m = fs.matrix()
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, inner_prec=prec, restart=30)
        u = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        its, fn, _ = dg.plap_newton(op, m, ksp, b, u, P, EPS, rtol=1e-8, lin_rtol=1e-3)
        assert fn[its] <= 1e-8 * fn[0]
        res[prec] = u
        # BF16 Jacobian apply error at the solution
        d = dev(np.random.default_rng(1).uniform(-1, 1, fs.n))
        y64, y16 = torch.zeros_like(d), torch.zeros_like(d)
        op.set_precision(dg.dPREC_FP64)
        op.mult(d, y64)
        op.set_precision(dg.dPREC_BF16)
        op.mult(d, y16)
        assert 1e-4 < rel(y16, y64) < 3e-2
    assert rel(res[dg.dPREC_BF16], res[dg.dPREC_FP64]) < 1e-6
