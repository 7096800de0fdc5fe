"""GPU: dEFSApply on the modal dJacobi's element spaces and on tensor spaces over Lobatto rules, through the C ABI.

The modal programs of the reference (src/jacobi/tests/ex2.c: jacobi-2-modal-fast-gauss / -fast-lobatto /
-sparse-gauss) are reproduced on the device: modes weighted by the first primes, INTERP to the rule points, then the
weighted INTERP_TRANSPOSE, against the printed numbers; batched applies with several components against the oracle's
dEFSApply_Modal_All (modaltopo.c:73-126) to 1e-13; the tensor apply on Lobatto rules against the oracle's
dEFSApply_Tensor_Hex."""
import ctypes

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po
from test_jacobi_types_host import (FAST, LOBATTO, PRIMES, SPARSE, get_efs, get_rules, gold, node_weight, order, quad,
                                    set_type)

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

INTERP, INTERP_T, GRAD, GRAD_T = 40001, 40002, 40003, 40004
INSERT, ADD = 1, 2


@pytest.fixture(scope="module")
def L():
    import os, subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    return dg.lib()


@pytest.fixture
def jac(L):
    h = ctypes.c_void_p()
    dg.chk(L.dJacobiCreate(ctypes.byref(h)))
    yield h
    L.dJacobiDestroy(ctypes.byref(h))


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def apply(L, efs, nelem, D, x, y, amode, imode=INSERT, jinv=None):
    dg.chk(L.dEFSApplyBatched(efs, ctypes.c_int32(nelem), dg.ptr(jinv), ctypes.c_int32(D), dg.ptr(x), dg.ptr(y),
                              ctypes.c_int(amode), ctypes.c_int(imode), None))


def rel_err(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name,method,family,rdeg", [("jacobi2_modal_fast_gauss", FAST, None, 6),
                                                     ("jacobi2_modal_fast_lobatto", FAST, LOBATTO, 4),
                                                     ("jacobi2_modal_sparse_gauss", SPARSE, None, 6)])
def test_modal_programs_on_the_device(L, jac, name, method, family, rdeg):
    set_type(L, jac, "modal")
    g = gold(name)
    rules = get_rules(L, quad(L, jac, method, family), [order(rdeg)] * 4)
    efs = get_efs(L, jac, [order(i) for i in range(4)], rules)
    for e in range(4):
        _, w = node_weight(L, rules[e])
        P, Q = [1, 4, 10, 18][e], len(w)
        vals = torch.zeros(Q, dtype=torch.float64, device="cuda")
        apply(L, efs[e], 1, 1, dev(PRIMES[:P]), vals, INTERP)
        v = host(vals)
        ref = g[f"e{e}_values"]
        np.testing.assert_allclose(v, ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())
        modes = torch.full((P,), float("nan"), dtype=torch.float64, device="cuda")
        apply(L, efs[e], 1, 1, dev(v * w), modes, INTERP_T)
        ref = g[f"e{e}_mass_applied"]
        np.testing.assert_allclose(host(modes), ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())


@pytest.mark.parametrize("modal_order,D,method,rdeg", [(0, 1, FAST, 2), (1, 3, FAST, 4), (2, 2, SPARSE, 6), (3, 3, FAST, 8),
                                                       (3, 1, SPARSE, 16)])
def test_modal_batched_against_the_oracle(L, jac, modal_order, D, method, rdeg):
    """nelem elements back to back, every mode, INSERT and ADD; a mapping passed in is not used (as the reference)"""
    set_type(L, jac, "modal")
    (r,) = get_rules(L, quad(L, jac, method), [order(rdeg)])
    (efs,) = get_efs(L, jac, [order(modal_order)], [r])
    pts, _ = node_weight(L, r)
    interp, deriv = po.modal_basis(modal_order, pts)
    Q, P = interp.shape
    ne = 37
    rng = np.random.default_rng(10 * modal_order + D)
    jinv = dev(rng.standard_normal(ne * Q * 9))
    for amode, nin, nout in [(INTERP, P * D, Q * D), (INTERP_T, Q * D, P * D), (GRAD, P * D, Q * D * 3)]:
        xin = rng.standard_normal((ne, nin))
        y0 = rng.standard_normal((ne, nout))
        for imode in (INSERT, ADD):
            y = dev(y0)
            apply(L, efs, ne, D, dev(xin), y, amode, imode, jinv=jinv if imode == ADD else None)
            got = host(y)
            for e in range(ne):
                ref = po.modal_apply(interp, deriv, D, xin[e], amode, imode, out=y0[e].copy())
                assert rel_err(got[e], ref) < 1e-13, (amode, imode, e)
    # GRAD_TRANSPOSE has no modal form; an empty batch launches nothing
    x = torch.zeros(Q * D * 3, dtype=torch.float64, device="cuda")
    y = torch.zeros(P * D, dtype=torch.float64, device="cuda")
    assert L.dEFSApplyBatched(efs, ctypes.c_int32(1), None, ctypes.c_int32(D), dg.ptr(x), dg.ptr(y), ctypes.c_int(GRAD_T),
                              ctypes.c_int(INSERT), None) != 0
    assert b"not implemented" in L.dGetLastError()
    apply(L, efs, 0, D, x, y, INTERP)


@pytest.mark.parametrize("degree,method,rdeg,D", [(2, FAST, 4, 1), (4, FAST, 8, 3), (3, SPARSE, 6, 1), (5, FAST, 6, 2)])
def test_tensor_apply_on_lobatto_rules(L, jac, degree, method, rdeg, D):
    """dEFSApply of GLL tensor spaces on Lobatto rules (FAST: 2 + order/2 points; SPARSE: the Lobatto pair per
    sub-interval), all four modes with a mapping, against the oracle"""
    (r,) = get_rules(L, quad(L, jac, method, LOBATTO), [order(rdeg)])
    (efs,) = get_efs(L, jac, [order(degree)], [r])
    x, _ = po.rule_1d(method, 1, rdeg)
    interp, deriv, _, _ = po.tensor_basis(degree + 1, x)
    nb, nq, ne = (degree + 1) ** 3, len(x) ** 3, 6
    rng = np.random.default_rng(degree + rdeg)
    jinv = rng.standard_normal((ne, nq, 9))
    for amode, nin, nout in [(INTERP, nb * D, nq * D), (GRAD, nb * D, nq * D * 3), (INTERP_T, nq * D, nb * D),
                             (GRAD_T, nq * D * 3, nb * D)]:
        xin = rng.standard_normal((ne, nin))
        y = torch.zeros(ne * nout, dtype=torch.float64, device="cuda")
        apply(L, efs, ne, D, dev(xin), y, amode, jinv=dev(jinv))
        got = host(y).reshape(ne, nout)
        for e in range(ne):
            ref = po.efs_apply_hex([degree + 1] * 3, [len(x)] * 3, [interp] * 3, [deriv] * 3, jinv[e].ravel(), D, xin[e],
                                   amode)
            assert rel_err(got[e], ref) < 1e-13, amode
