"""dOperatorMultNoAlloc: the operator apply for callers that cannot let the library allocate.

Callers that own all device memory through their own pool, or that call the operator from a solver
callback running beside other streams (where cudaMalloc/cudaFree may synchronize the device), use this
entry point; its temporary lives in a fixed per-device array instead of memory allocated per call.
This file is collected last so that a run stopping at the first failure has already run every other
test. It passes alone in a fresh process and after the other tests."""
import ctypes

import numpy as np
import pytest

import dohp_gb300 as dg

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import os, subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def no_alloc_mult(op, x, y):
    dg.chk(dg.lib().dOperatorMultNoAlloc(op.h, dg.ptr(x), dg.ptr(y)))


def test_no_alloc_matches_mult_on_two_calls_in_a_row():
    fs = dg.FS((6, 5, 7), degree=3, perturb=0.1, seed=4)
    op = fs.operator(dg.dOP_DIFFUSION)
    kq = torch.zeros(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(dg.grf_create(16, 2.0, 0.1, 3), kq)
    op.set_qdata(kq)
    rng = np.random.default_rng(8)
    xs = [torch.as_tensor(rng.uniform(-1, 1, fs.n), device="cuda") for _ in range(2)]
    ref = []
    for x in xs:  # ordinary entry point (builds the geometric factors on its first call)
        y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        op.mult(x, y)
        ref.append(y)
    for x, yr in zip(xs, ref):  # two no-alloc calls in a row, different inputs
        y = torch.full((fs.n,), float("nan"), dtype=torch.float64, device="cuda")
        no_alloc_mult(op, x, y)
        torch.cuda.synchronize()
        err = (torch.linalg.norm(y - yr) / torch.linalg.norm(yr)).item()
        assert err < 1e-12, err


def test_no_alloc_rejects_spaces_beyond_the_scratch():
    fs = dg.FS((22, 22, 22), degree=4, perturb=0.0)  # 21^3 * 125 = 1,157,625 expanded values > 1,048,576
    op = fs.operator(dg.dOP_DIFFUSION)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    op.mult(x, y)
    with pytest.raises(dg.DohpError, match="fixed scratch"):
        no_alloc_mult(op, x, y)


def test_no_alloc_needs_geometry_from_an_ordinary_call():
    fs = dg.FS((3, 3, 3), degree=2, perturb=0.0)
    op = fs.operator(dg.dOP_DIFFUSION)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DohpError, match="geometric factors"):
        no_alloc_mult(op, x, torch.zeros_like(x))


def test_no_alloc_refuses_reduced_precision_and_hp_spaces():
    # the entry point always applies in FP64: a reduced precision set on the operator is refused, not ignored
    fs = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=2)
    op = fs.operator(dg.dOP_DIFFUSION)
    x = torch.as_tensor(np.random.default_rng(1).uniform(-1, 1, fs.n), device="cuda")
    y = torch.zeros_like(x)
    op.mult(x, y)
    op.set_precision(dg.dPREC_FP32)
    with pytest.raises(dg.DohpError, match="FP64 only"):
        no_alloc_mult(op, x, y)
    op.set_precision(dg.dPREC_FP64)
    y2 = torch.zeros_like(x)
    no_alloc_mult(op, x, y2)
    torch.cuda.synchronize()
    assert (torch.linalg.norm(y2 - y) / torch.linalg.norm(y)).item() < 1e-12
    # per-element orders: refused with a message naming the entry point
    ed = np.random.default_rng(2).integers(2, 5, size=27).astype(np.int32)
    fsh = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=2, elem_degree=ed)
    oph = fsh.operator(dg.dOP_DIFFUSION)
    xh = torch.zeros(fsh.n, dtype=torch.float64, device="cuda")
    oph.mult(xh, torch.zeros_like(xh))
    with pytest.raises(dg.DohpError, match="dOperatorMultNoAlloc: uniform-order spaces only"):
        no_alloc_mult(oph, xh, torch.zeros_like(xh))
