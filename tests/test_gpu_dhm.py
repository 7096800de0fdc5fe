"""DHM files with device vectors: a space set up on the GPU, two time steps of a device closure vector written and read
back into device memory bit for bit, and the space rebuilt from the file applying the same operator."""
import ctypes
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


def test_device_vectors_round_trip(tmp_path):
    L = dg.lib()
    path = str(tmp_path / "dev.dhm").encode()
    fs = dg.FS((5, 4, 6), degree=3, perturb=0.1, seed=2)
    rng = np.random.default_rng(3)
    xs = [torch.as_tensor(rng.standard_normal(fs.nc), device="cuda") for _ in range(2)]
    v = ctypes.c_void_p()
    dg.chk(L.dViewerDHMOpen(path, ctypes.c_int(1), ctypes.byref(v)))
    dg.chk(L.dFSViewDHM(fs.h, b"u", v))
    for k in range(2):
        dg.chk(L.dViewerDHMSetTime(v, ctypes.c_double(0.1 * (k + 1))))
        dg.chk(L.dVecViewDHM(fs.h, b"field", dg.ptr(xs[k]), ctypes.c_int(1), v))
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    dg.chk(L.dViewerDHMOpen(path, ctypes.c_int(0), ctypes.byref(v)))
    mesh2, fs2 = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSLoadDHM(v, b"u", fs.jac.h, ctypes.byref(mesh2), ctypes.byref(fs2)))
    dg.chk(L.dFSSetUp(fs2))
    for k in range(2):
        dg.chk(L.dViewerDHMSetTimeStep(v, ctypes.c_int32(k)))
        y = torch.zeros(fs.nc, dtype=torch.float64, device="cuda")
        dg.chk(L.dVecLoadDHM(v, b"field", fs2, dg.ptr(y), ctypes.c_int(1)))
        torch.cuda.synchronize()
        assert torch.equal(y, xs[k])
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    # the rebuilt space applies the same operator (same mesh, degrees, boundary sets)
    op1, op2 = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSCreateOperator(fs.h, ctypes.c_int(dg.dOP_DIFFUSION), None, ctypes.byref(op1)))
    dg.chk(L.dFSCreateOperator(fs2, ctypes.c_int(dg.dOP_DIFFUSION), None, ctypes.byref(op2)))
    x = xs[0][:fs.n].contiguous()
    y1, y2 = torch.zeros_like(x), torch.zeros_like(x)
    dg.chk(L.dOperatorMult(op1, dg.ptr(x), dg.ptr(y1)))
    dg.chk(L.dOperatorMult(op2, dg.ptr(x), dg.ptr(y2)))
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    L.dOperatorDestroy(ctypes.byref(op1))
    L.dOperatorDestroy(ctypes.byref(op2))
    L.dFSDestroy(ctypes.byref(fs2))
    L.dMeshDestroy(ctypes.byref(mesh2))
