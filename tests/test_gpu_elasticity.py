"""Linear elasticity (ElastPointwiseJacobian at F = I, src/fs/tests/elast.c:256-280) through the fused
three-component element kernel, against the oracle's element loop."""
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
    import os, subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


@pytest.mark.parametrize("npoints,degree", [((3, 3, 3), 1), ((4, 3, 4), 2), ((3, 3, 3), 4), ((3, 2, 3), 6), ((2, 3, 2), 8)])
def test_elasticity_apply_fp64(npoints, degree):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=2, bs=3)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=2, bs=3)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    g = np.random.default_rng(degree).uniform(-1, 1, fs.n * 3)
    y = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    op.mult(torch.as_tensor(g, device="cuda"), y)
    torch.cuda.synchronize()
    yo = o.apply(g, kind=2, param=np.array([LAM, MU]))
    err = np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo)
    assert err < 1e-12, err


def test_elasticity_apply_fp32():
    fs = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=3, bs=3)
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=3, bs=3)
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    op.set_precision(dg.dPREC_FP32)
    g = np.random.default_rng(0).uniform(-1, 1, fs.n * 3)
    y = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    op.mult(torch.as_tensor(g, device="cuda"), y)
    torch.cuda.synchronize()
    yo = o.apply(g, kind=2, param=np.array([LAM, MU]))
    err = np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo)
    assert err < 1e-5, err


def test_elasticity_rigid_body_modes_in_kernel():
    """Rigid translations/rotations give zero stress: A r = 0 away from the Dirichlet boundary (no Dirichlet)."""
    fs = dg.FS((3, 3, 3), degree=3, perturb=0.1, seed=4, bs=3, dirichlet=())
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    t = np.tile([1.0, -2.0, 0.5], fs.n)
    y = torch.zeros(fs.n * 3, dtype=torch.float64, device="cuda")
    op.mult(torch.as_tensor(t, device="cuda"), y)
    torch.cuda.synchronize()
    assert np.abs(y.cpu().numpy()).max() < 1e-13
