"""Edge cases on the GPU: a space with no explicit dofs (one degree-1 element, every node on the Dirichlet boundary)
through the operator, the Q1 assembly, CG and FGMRES, the iterator and the restriction; an EFS apply over no
elements; the largest degree on the smallest mesh against the oracle."""
import ctypes
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


def test_space_without_explicit_dofs():
    fs = dg.FS((2, 2, 2), degree=1, seed=1)
    assert fs.n == 0 and fs.nexp == 8
    op = fs.operator()
    x = torch.zeros(1, dtype=torch.float64, device="cuda")[:0]
    y = torch.zeros(1, dtype=torch.float64, device="cuda")[:0]
    op.mult(x, y)
    m = fs.matrix()
    m.assemble()
    for ktype in (dg.dKSP_CG, dg.dKSP_FGMRES):
        its, rn = dg.KSP(op, m, ksp_type=ktype).solve(x, y, rtol=1e-8, maxit=10)
        assert its == 0
    yexp = torch.zeros(fs.nexp, dtype=torch.float64, device="cuda")
    op.mult_expanded(x, yexp)
    assert float(yexp.abs().max()) == 0.0


def test_efs_apply_over_no_elements():
    jac = ctypes.c_void_p()
    L = dg.lib()
    dg.chk(L.dJacobiCreate(ctypes.byref(jac)))
    efs = ctypes.c_void_p()
    deg, rule = (ctypes.c_int32 * 3)(3, 3, 3), (ctypes.c_int32 * 3)(4, 4, 4)
    dg.chk(L.dJacobiGetEFSTensor(jac, deg, ctypes.c_int(0), rule, ctypes.byref(efs)))
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    # INTERP, INSERT_VALUES over zero elements: nothing to do, no error
    dg.chk(L.dEFSApplyBatched(efs, ctypes.c_int32(0), None, ctypes.c_int32(1), ctypes.c_void_p(buf.data_ptr()),
                              ctypes.c_void_p(buf.data_ptr()), ctypes.c_int(dg.dAPPLY_INTERP), ctypes.c_int(dg.INSERT_VALUES), None))
    torch.cuda.synchronize()
    L.dJacobiDestroy(ctypes.byref(jac))


def test_largest_degree_on_one_element_matches_oracle():
    fs = dg.FS((2, 2, 2), degree=8, perturb=0.0, seed=1)
    o = po.FS(2, 2, 2, degree=8, perturb=0.0, seed=1)
    assert fs.n == o.n == 7 ** 3
    x = np.random.default_rng(0).uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    fs.operator().mult(torch.as_tensor(x, device="cuda"), y)
    yo = o.apply(x)
    assert np.linalg.norm(y.cpu().numpy() - yo) <= 1e-12 * np.linalg.norm(yo)
