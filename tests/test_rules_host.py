"""Host-side dJacobi entry points through the C ABI, on the CPU (no GPU needed): dJacobiGetQuadrature,
dQuadratureGetRules, dRuleGetNodeWeight / GetTensorNodeWeight / GetPatches, dRuleComputePhysical, dJacobiGetEFS,
dEFSGetRule and dEFSGetExplicitSparse, pinned to the reference's own printed tables (jacobi-3-tensor-sparsex-r4/r6,
jacobi-4-tensor-fast/sparse refouts, as extracted into tests/golden) and to the oracle."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
FAST, SPARSE = 0, 1
HEX = 7


def gold(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


@pytest.fixture(scope="module")
def L():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    return dg.lib()


def order(mx, x=0, y=0, z=0):
    """dPolynomialOrder as the four bytes {max, x, y, z} of an int"""
    return np.int32(int.from_bytes(bytes([mx, x, y, z]), "little", signed=True))


@pytest.fixture(scope="module")
def jac(L):
    h = ctypes.c_void_p()
    dg.chk(L.dJacobiCreate(ctypes.byref(h)))
    yield h
    L.dJacobiDestroy(ctypes.byref(h))


def rules(L, jac, method, orders):
    q = ctypes.c_void_p()
    dg.chk(L.dJacobiGetQuadrature(jac, ctypes.c_int(method), ctypes.byref(q)))
    n = len(orders)
    topo = np.full(n, HEX, np.int32)
    ords = np.array(orders, np.int32)
    arr = ctypes.POINTER(ctypes.c_void_p)()
    dg.chk(L.dQuadratureGetRules(q, ctypes.c_int32(n), dg.ptr(topo), dg.ptr(ords), ctypes.byref(arr)))
    out = [ctypes.c_void_p(arr[i]) for i in range(n)]
    dg.chk(L.dFree(arr))
    return out


def efs_on(L, jac, degree, rule):
    topo = np.array([HEX], np.int32)
    ords = np.array([order(degree)], np.int32)
    rl = (ctypes.c_void_p * 1)(rule.value)
    arr = ctypes.POINTER(ctypes.c_void_p)()
    dg.chk(L.dJacobiGetEFS(jac, ctypes.c_int32(1), dg.ptr(topo), dg.ptr(ords), rl, ctypes.byref(arr)))
    e = ctypes.c_void_p(arr[0])
    dg.chk(L.dFree(arr))
    return e


def patches(L, rule):
    npch, psz = ctypes.c_int32(), ctypes.c_int32()
    ind, w = ctypes.POINTER(ctypes.c_int32)(), ctypes.POINTER(ctypes.c_double)()
    dg.chk(L.dRuleGetPatches(rule, ctypes.byref(npch), ctypes.byref(psz), ctypes.byref(ind), ctypes.byref(w)))
    n = npch.value * psz.value
    return npch.value, psz.value, np.ctypeslib.as_array(ind, (n,)).reshape(npch.value, psz.value).copy(), \
        np.ctypeslib.as_array(w, (n,)).reshape(npch.value, psz.value).copy()


def test_fast_and_sparse_rules_match_the_oracle(L, jac):
    for method in (FAST, SPARSE):
        for deg in (2, 4, 6, 8):
            (r,) = rules(L, jac, method, [order(deg)])
            x, w = po.rule_1d(method, 0, deg)
            nn = ctypes.c_int32()
            dg.chk(L.dRuleGetSize(r, None, ctypes.byref(nn)))
            assert nn.value == len(x) ** 3
            coord, wt = np.zeros(nn.value * 3), np.zeros(nn.value)
            dg.chk(L.dRuleGetNodeWeight(r, dg.ptr(coord), dg.ptr(wt)))
            X = np.stack(np.meshgrid(x, x, x, indexing="ij"), -1).reshape(-1, 3)
            W = np.einsum("i,j,k->ijk", w, w, w).ravel()
            np.testing.assert_allclose(coord.reshape(-1, 3), X, rtol=0, atol=1e-15)
            np.testing.assert_allclose(wt, W, rtol=1e-14)
    # anisotropic orders and the rule cache: the same orders give the same rule object
    a = rules(L, jac, FAST, [order(0, 2, 4, 6), order(0, 2, 4, 6)])
    assert a[0].value == a[1].value
    nn = (ctypes.c_int32 * 3)()
    dg.chk(L.dRuleGetTensorNodeWeight(a[0], None, nn, None, None))
    assert list(nn) == [2, 3, 4]


@pytest.mark.parametrize("name,method", [("jacobi4_fast", FAST), ("jacobi4_sparse", SPARSE)])
def test_patch_tables_golden(L, jac, name, method):
    """dRuleGetPatches against the reference's printed patch tables (tensorquad.c:120-169, z-weight index included)"""
    g = gold(name)
    for e in range(4):
        rdeg = (e + 1) * 2 - 2
        (r,) = rules(L, jac, method, [order(rdeg)])
        npch, psz, ind, wt = patches(L, r)
        assert [npch, psz] == list(g[f"e{e}_shape"])
        np.testing.assert_array_equal(ind, g[f"e{e}_indices"])
        np.testing.assert_allclose(wt, g[f"e{e}_weights"], atol=6e-6)


@pytest.mark.parametrize("name,rdeg", [("jacobi3_sparsex_r4", 4), ("jacobi3_sparsex_r6", 6)])
def test_explicit_sparse_golden(L, jac, name, rdeg):
    """dEFSGetExplicitSparse against the reference's printed Q1 sub-cell bases (efstopo.c:660-717, without the 1/h_sub
    factor) and, where patches are not the sub-cells, its element-basis fallback (jacobi.c:611-643)"""
    g = gold(name)
    (r,) = rules(L, jac, SPARSE, [order(rdeg)])
    npch, psz, ind, _ = patches(L, r)
    for e in range(3):
        P = e + 2
        efs = efs_on(L, jac, P - 1, r)
        rr = ctypes.c_void_p()
        dg.chk(L.dEFSGetRule(efs, ctypes.byref(rr)))
        assert rr.value == r.value
        maxP = P ** 3
        eidx = np.zeros(npch * maxP, np.int32)
        bi, bd = np.zeros(npch * psz * maxP), np.zeros(npch * psz * maxP * 3)
        Pout = ctypes.c_int32()
        dg.chk(L.dEFSGetExplicitSparse(efs, ctypes.c_int32(npch), ctypes.c_int32(psz), dg.ptr(np.ascontiguousarray(ind, np.int32)),
                                       None, ctypes.c_int32(0), ctypes.byref(Pout), dg.ptr(eidx), dg.ptr(bi), dg.ptr(bd)))
        Pn = Pout.value
        np.testing.assert_array_equal(ind, g[f"e{e}_qidx"])
        np.testing.assert_array_equal(eidx[:npch * Pn].reshape(npch, Pn), g[f"e{e}_bidx"])
        bi = bi[:npch * psz * Pn].reshape(npch, psz, Pn)
        bd = bd[:npch * psz * Pn * 3].reshape(npch, psz, Pn * 3)
        for p in range(min(4, npch)):
            np.testing.assert_allclose(bi[p], g[f"e{e}_p{p}_interp"], atol=6e-6)
            np.testing.assert_allclose(bd[p], g[f"e{e}_p{p}_deriv"], atol=6e-6)
        # the oracle's restatement, every patch, full precision, with a physical map
        interp, deriv, _, _ = po.tensor_basis(P, po.rule_1d(SPARSE, 0, rdeg)[0])
        cj = np.random.default_rng(e).uniform(-1, 1, (npch * psz, 9))
        oe, oi, od = po.explicit_sparse([P] * 3, [rdeg] * 3, [interp] * 3, [deriv] * 3, npch, psz, ind, cjinv=cj, eoffset=5)
        dg.chk(L.dEFSGetExplicitSparse(efs, ctypes.c_int32(npch), ctypes.c_int32(psz), dg.ptr(np.ascontiguousarray(ind, np.int32)),
                                       dg.ptr(cj), ctypes.c_int32(5), ctypes.byref(Pout), dg.ptr(eidx), dg.ptr(bi), dg.ptr(bd)))
        np.testing.assert_array_equal(eidx[:npch * Pn].reshape(npch, Pn), oe)
        np.testing.assert_allclose(bi.reshape(oi.shape), oi, rtol=0, atol=1e-15)
        np.testing.assert_allclose(bd.reshape(od.shape), od, rtol=0, atol=1e-14)


def test_compute_physical(L, jac):
    (r,) = rules(L, jac, FAST, [order(4)])
    nn = ctypes.c_int32()
    dg.chk(L.dRuleGetSize(r, None, ctypes.byref(nn)))
    n = nn.value
    rng = np.random.default_rng(1)
    J = np.eye(3)[None] * 2 + 0.3 * rng.uniform(-1, 1, (n, 3, 3))
    jinv, jw = np.zeros(n * 9), np.zeros(n)
    dg.chk(L.dRuleComputePhysical(r, dg.ptr(np.ascontiguousarray(J.ravel())), dg.ptr(jinv), dg.ptr(jw)))
    wt = np.zeros(n)
    dg.chk(L.dRuleGetNodeWeight(r, None, dg.ptr(wt)))
    np.testing.assert_allclose(jinv.reshape(n, 3, 3), np.linalg.inv(J), rtol=1e-13, atol=1e-14)
    np.testing.assert_allclose(jw, wt * np.linalg.det(J), rtol=1e-13)
    dg.chk(L.dRuleComputePhysical(r, None, dg.ptr(jinv), dg.ptr(jw)))
    np.testing.assert_array_equal(jinv.reshape(n, 3, 3), np.broadcast_to(np.eye(3), (n, 3, 3)))
    np.testing.assert_array_equal(jw, wt)
    J[3] = np.diag([1.0, 1.0, -1.0])  # a negative determinant is an error, not an abort
    assert L.dRuleComputePhysical(r, dg.ptr(np.ascontiguousarray(J.ravel())), dg.ptr(jinv), dg.ptr(jw)) != 0
    assert b"Negative Jacobian" in L.dGetLastError()


def test_errors(L, jac):
    q = ctypes.c_void_p()
    assert L.dJacobiGetQuadrature(jac, ctypes.c_int(7), ctypes.byref(q)) != 0
    dg.chk(L.dJacobiGetQuadrature(jac, ctypes.c_int(FAST), ctypes.byref(q)))
    arr = ctypes.POINTER(ctypes.c_void_p)()
    tet = np.array([6], np.int32)
    assert L.dQuadratureGetRules(q, ctypes.c_int32(1), dg.ptr(tet), dg.ptr(np.array([order(2)], np.int32)), ctypes.byref(arr)) != 0
    assert b"hexahedra only" in L.dGetLastError()
