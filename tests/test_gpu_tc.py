"""BF16 tensor-core element apply (dPREC_BF16 on scalar uniform-order spaces, tcgen05 MMAs with FP32 accumulation in
tensor memory): its error against the FP64 apply stays at the BF16 level for every supported degree and element
count (full and partial element groups), it is deterministic, and it agrees with the oracle's FP64 apply to the same
BF16 tolerance on a lognormal coefficient."""
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


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("p,npts", [(1, (6, 5, 7)), (2, (5, 6, 4)), (3, (9, 8, 7)), (4, (6, 6, 6)), (5, (5, 4, 6)), (6, (4, 5, 5)),
                                    (7, (4, 4, 5))])
def test_tc_apply_error_against_fp64(p, npts):
    fs = dg.FS(npts, degree=p, perturb=0.1, seed=p)
    op = fs.operator()
    x = torch.as_tensor(np.random.default_rng(p).uniform(-1, 1, fs.n), device="cuda")
    y64, y16, y16b = (torch.zeros(fs.n, dtype=torch.float64, device="cuda") for _ in range(3))
    op.mult(x, y64)
    op.set_precision(dg.dPREC_BF16)
    op.mult(x, y16)
    op.mult(x, y16b)
    torch.cuda.synchronize()
    e = rel(y16, y64)
    assert 1e-5 < e < 3e-2, e
    assert torch.equal(y16, y16b)  # deterministic: fixed MMA order, no atomics


def test_tc_apply_lognormal_against_oracle():
    ne, p = 12, 4
    fs = dg.FS((ne + 1,) * 3, degree=p, perturb=0.1, seed=1)
    o = po.FS(ne + 1, ne + 1, ne + 1, degree=p, perturb=0.1, seed=1)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(dg.grf_create(64, 2.0, 0.1, 3), kq)
    op = fs.operator()
    op.set_qdata(kq)
    op.set_precision(dg.dPREC_BF16)
    g = np.random.default_rng(0).uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(torch.as_tensor(g, device="cuda"), y)
    torch.cuda.synchronize()
    yo = o.apply(g, kind=0, qdata=kq.cpu().numpy(), nthreads=os.cpu_count() or 1)
    e = float(np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo))
    assert 1e-5 < e < 3e-2, e
