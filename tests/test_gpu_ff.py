"""Float-float (dPREC_FF) applies: FP64-class results from FP32-pipe arithmetic. Uniform diffusion with a
lognormal coefficient, uniform elasticity, and the hp elasticity apply in its per-order, persistent and graph
forms, each against the oracle at the FP64 parity bound (1e-12), and visibly not the FP32 result."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

LAM, MU = 0.3 / (1.3 * 0.4), 1.0 / 2.6


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def apply(op, g, prec):
    op.set_precision(prec)
    y = torch.zeros(len(g), dtype=torch.float64, device="cuda")
    op.mult(torch.as_tensor(g, device="cuda"), y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("p", [2, 4, 7])
def test_uniform_diffusion(p):
    fs = dg.FS((5, 4, 5), degree=p, perturb=0.1, seed=p)
    o = po.FS(5, 4, 5, degree=p, perturb=0.1, seed=p)
    g = np.random.default_rng(p).uniform(-1, 1, fs.n)
    op = fs.operator()
    yo = o.apply(g)
    e_ff = rel(apply(op, g, dg.dPREC_FF), yo)
    e_32 = rel(apply(op, g, dg.dPREC_FP32), yo)
    assert e_ff < 1e-12 and e_32 > 1e-9 and e_ff < 1e-3 * e_32


def test_lognormal_coefficient():
    fs = dg.FS((6, 6, 6), degree=4, perturb=0.1, seed=3)
    grf = dg.grf_create(16, 2.0, 0.1, 5)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    g = np.random.default_rng(1).uniform(-1, 1, fs.n)
    y64 = apply(op, g, dg.dPREC_FP64)
    assert rel(apply(op, g, dg.dPREC_FF), y64) < 1e-12


def test_uniform_elasticity():
    fs = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=2, bs=3)
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=2, bs=3)
    g = np.random.default_rng(2).uniform(-1, 1, fs.n * 3)
    op = fs.operator(dg.dOP_ELASTICITY, param=(1.0, 0.3))
    assert rel(apply(op, g, dg.dPREC_FF), o.apply(g, kind=2, param=np.array([LAM, MU]))) < 1e-12


@pytest.mark.parametrize("launch", [dg.dLAUNCH_PER_ORDER, dg.dLAUNCH_PERSISTENT, dg.dLAUNCH_GRAPH])
def test_hp_elasticity(launch):
    npts = (4, 4, 4)
    ed = np.random.default_rng(5).integers(2, 9, size=27).astype(np.int32)
    fs = dg.FS(npts, degree=4, perturb=0.1, seed=1, bs=3, elem_degree=ed)
    o = po.FS(*npts, degree=4, perturb=0.1, seed=1, bs=3, elem_degree=ed)
    op = fs.operator(dg.dOP_ELASTICITY, param=(1.0, 0.3))
    op.set_launch(launch)
    g = np.random.default_rng(6).uniform(-1, 1, fs.n * 3)
    yo = o.apply(g, kind=2, param=np.array([LAM, MU]))
    for _ in range(2):  # graph form: capture, then replay
        y = apply(op, g, dg.dPREC_FF)
    assert rel(y, yo) < 1e-12
    assert rel(apply(op, g, dg.dPREC_FP64), yo) < 1e-12  # the FP64 graph is a separate capture
