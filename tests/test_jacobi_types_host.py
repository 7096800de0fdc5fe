"""The reference's jacobi test programs through the product's C ABI on the CPU (no GPU needed): the modal dJacobi
type (dJacobiSetType "modal", P-discontinuous bases of orders 0..3), the Lobatto point family of the tensor
quadrature (dQuadratureTensorSetGaussFamily) and explicit element bases (dEFSGetExplicit), pinned to the printed
matrices of jacobi-3-tensor-gauss / -lobatto / jacobi-3-modal-gauss and the printed values of jacobi-2-modal-*
(src/jacobi/tests/ex2.c, ex3.c; refout files extracted into tests/golden) and to the oracle."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
FAST, SPARSE = 0, 1
HEX = 7
LEGENDRE, LOBATTO, RADAU = 0, 1, 2
P_CONFORMING, P_DISCONTINUOUS = 0, 1
PRIMES = np.array([2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71], float)


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


@pytest.fixture
def jac(L):
    h = ctypes.c_void_p()
    dg.chk(L.dJacobiCreate(ctypes.byref(h)))
    yield h
    L.dJacobiDestroy(ctypes.byref(h))


def quad(L, jac, method, family=None):
    q = ctypes.c_void_p()
    dg.chk(L.dJacobiGetQuadrature(jac, ctypes.c_int(method), ctypes.byref(q)))
    if family is not None:
        dg.chk(L.dQuadratureTensorSetGaussFamily(q, ctypes.c_int(family)))
    return q


def get_rules(L, q, orders):
    n = len(orders)
    arr = ctypes.POINTER(ctypes.c_void_p)()
    topo, ords = np.full(n, HEX, np.int32), np.array(orders, np.int32)  # alive for the call
    dg.chk(L.dQuadratureGetRules(q, ctypes.c_int32(n), dg.ptr(topo), dg.ptr(ords), ctypes.byref(arr)))
    out = [ctypes.c_void_p(arr[i]) for i in range(n)]
    dg.chk(L.dFree(arr))
    return out


def get_efs(L, jac, degrees, rules):
    n = len(degrees)
    rl = (ctypes.c_void_p * n)(*[r.value for r in rules])
    arr = ctypes.POINTER(ctypes.c_void_p)()
    topo, degs = np.full(n, HEX, np.int32), np.array(degrees, np.int32)
    dg.chk(L.dJacobiGetEFS(jac, ctypes.c_int32(n), dg.ptr(topo), dg.ptr(degs), rl, ctypes.byref(arr)))
    out = [ctypes.c_void_p(arr[i]) for i in range(n)]
    dg.chk(L.dFree(arr))
    return out


def node_weight(L, rule):
    nn = ctypes.c_int32()
    dg.chk(L.dRuleGetSize(rule, None, ctypes.byref(nn)))
    coord, wt = np.zeros(nn.value * 3), np.zeros(nn.value)
    dg.chk(L.dRuleGetNodeWeight(rule, dg.ptr(coord), dg.ptr(wt)))
    return coord.reshape(-1, 3), wt


def explicit(L, efs, jinv=None):
    """dEFSGetExplicit, copied out, then dEFSRestoreExplicit"""
    Q, P = ctypes.c_int32(), ctypes.c_int32()
    B, G = ctypes.POINTER(ctypes.c_double)(), ctypes.POINTER(ctypes.c_double)()
    jv = None if jinv is None else np.ascontiguousarray(jinv, np.float64)
    jp = dg.ptr(jv)
    dg.chk(L.dEFSGetExplicit(efs, jp, ctypes.byref(Q), ctypes.byref(P), ctypes.byref(B), ctypes.byref(G)))
    q, p = Q.value, P.value
    bas = np.ctypeslib.as_array(B, (q * p,)).reshape(q, p).copy()
    der = np.ctypeslib.as_array(G, (q * p * 3,)).reshape(q, p, 3).copy()
    dg.chk(L.dEFSRestoreExplicit(efs, jp, ctypes.byref(Q), ctypes.byref(P), ctypes.byref(B), ctypes.byref(G)))
    assert Q.value == 0 and P.value == 0 and not B and not G
    return bas, der


def set_type(L, jac, name):
    dg.chk(L.dJacobiSetType(jac, name.encode()))
    t = ctypes.c_char_p()
    dg.chk(L.dJacobiGetType(jac, ctypes.byref(t)))
    assert t.value == name.encode()


def check_explicit_golden(g, e, bas, der, w):
    """the matrices ex3.c prints (interpolation (Q,P), gradient (Q,3P), mass (P,P)) for element e"""
    q, p = bas.shape
    mass = bas.T @ (w[:, None] * bas)
    np.testing.assert_allclose(mass, g[f"e{e}_mass"], atol=6e-7)
    if f"e{e}_interpolation" in g:
        np.testing.assert_allclose(bas, g[f"e{e}_interpolation"], atol=6e-7)
        np.testing.assert_allclose(der.reshape(q, 3 * p), g[f"e{e}_gradient"], atol=6e-7)
    else:
        h = g[f"e{e}_interpolation_head"]
        np.testing.assert_allclose(bas[:len(h)], h, atol=6e-7)
        np.testing.assert_allclose(der.reshape(q, 3 * p)[:len(h)], g[f"e{e}_gradient_head"], atol=6e-7)


@pytest.mark.parametrize("name,family,rdeg", [("jacobi3_gauss", None, 8), ("jacobi3_lobatto", LOBATTO, 6)])
def test_tensor_explicit_golden(L, jac, name, family, rdeg):
    """ex3.c on the tensor type: basis degrees 1..4 per direction on the FAST rule of degree rdeg (Gauss, or Lobatto
    through dQuadratureTensorSetGaussFamily)"""
    g = gold(name)
    rules = get_rules(L, quad(L, jac, FAST, family), [order(0, rdeg, rdeg, rdeg)] * 4)
    efs = get_efs(L, jac, [order(0, i + 1, i + 1, i + 1) for i in range(4)], rules)
    for e in range(4):
        bas, der = explicit(L, efs[e])
        _, w = node_weight(L, rules[e])
        check_explicit_golden(g, e, bas, der, w)


def test_modal_explicit_golden(L, jac):
    """ex3.c on the modal type (-djac_type modal -rule_degree 6): orders 0..3 on the FAST Gauss rule of degree 6"""
    set_type(L, jac, "modal")
    g = gold("jacobi3_modal_gauss")
    rules = get_rules(L, quad(L, jac, FAST), [order(6)] * 4)
    efs = get_efs(L, jac, [order(i) for i in range(4)], rules)
    for e in range(4):
        dim, inodes, total = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        dg.chk(L.dEFSGetSizes(efs[e], ctypes.byref(dim), ctypes.byref(inodes), ctypes.byref(total)))
        assert (dim.value, inodes.value, total.value) == (3, [1, 4, 10, 18][e], [1, 4, 10, 18][e])
        bas, der = explicit(L, efs[e])
        pts, w = node_weight(L, rules[e])
        check_explicit_golden(g, e, bas, der, w)
        # against the oracle's restatement at full precision; the modal apply ignores a mapping
        oi, od = po.modal_basis(e, pts)
        np.testing.assert_allclose(bas, oi, rtol=0, atol=4e-15)
        np.testing.assert_allclose(der, od, rtol=0, atol=4e-14)
        _, d2 = explicit(L, efs[e], jinv=np.tile(2 * np.eye(3).ravel(), len(pts)))
        np.testing.assert_array_equal(d2, der)


@pytest.mark.parametrize("name,method,family,rdeg", [("jacobi2_modal_fast_gauss", FAST, None, 6),
                                                     ("jacobi2_modal_fast_lobatto", FAST, LOBATTO, 4),
                                                     ("jacobi2_modal_sparse_gauss", SPARSE, None, 6)])
def test_modal_values_golden(L, jac, name, method, family, rdeg):
    """ex2.c's numbers from the product's modal tables: the modes (weights 2, 3, 5, ...) at the rule points and the
    weighted transpose (the Lobatto rule of 4 points does not integrate the cubic modes' products exactly)"""
    set_type(L, jac, "modal")
    g = gold(name)
    rules = get_rules(L, quad(L, jac, method, family), [order(rdeg)] * 4)
    efs = get_efs(L, jac, [order(i) for i in range(4)], rules)
    for e in range(4):
        bas, _ = explicit(L, efs[e])
        _, w = node_weight(L, rules[e])
        vals = bas @ PRIMES[:bas.shape[1]]
        ref = g[f"e{e}_values"]
        np.testing.assert_allclose(vals, ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())
        ref = g[f"e{e}_mass_applied"]
        np.testing.assert_allclose(bas.T @ (w * vals), ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())


def test_lobatto_rules_match_the_oracle(L, jac):
    """FAST Lobatto rules (2 + order/2 points, tensorquad.c:86-89) and SPARSE rules with the Lobatto pair (the ends of
    each GLL sub-interval, two_point_lobatto, tensorquad.c:46-49) against the oracle's restatement"""
    for method in (FAST, SPARSE):
        q = quad(L, jac, method, LOBATTO)
        for deg in (2, 4, 6, 8):
            (r,) = get_rules(L, q, [order(deg)])
            x, w = po.rule_1d(method, 1, deg)
            pts, wt = node_weight(L, r)
            X = np.stack(np.meshgrid(x, x, x, indexing="ij"), -1).reshape(-1, 3)
            np.testing.assert_allclose(pts, X, rtol=0, atol=1e-15)
            np.testing.assert_allclose(wt, np.einsum("i,j,k->ijk", w, w, w).ravel(), rtol=1e-14)


def test_family_applies_to_rules_made_after_the_call(L, jac):
    q = quad(L, jac, FAST)
    (a,) = get_rules(L, q, [order(4)])
    dg.chk(L.dQuadratureTensorSetGaussFamily(q, ctypes.c_int(LOBATTO)))
    (b,) = get_rules(L, q, [order(4)])
    assert a.value != b.value
    assert len(node_weight(L, a)[1]) == 27 and len(node_weight(L, b)[1]) == 64  # 3 Gauss / 4 Lobatto points
    # element spaces on the two rules are distinct and keep their rule
    ea, eb = get_efs(L, jac, [order(2), order(2)], [a, b])
    assert ea.value != eb.value
    for e, r in ((ea, a), (eb, b)):
        rr = ctypes.c_void_p()
        dg.chk(L.dEFSGetRule(e, ctypes.byref(rr)))
        assert rr.value == r.value
    assert L.dQuadratureTensorSetGaussFamily(q, ctypes.c_int(RADAU)) != 0
    assert b"radau" in L.dGetLastError()


def test_tensor_explicit_mapped_by_jinv(L, jac):
    """dEFSGetExplicit with a mapping: derivatives sum_k dphi/dxi_k jinv[q][k][e] (TensorRuleMapping)"""
    (r,) = get_rules(L, quad(L, jac, FAST), [order(0, 4, 6, 2)])
    (efs,) = get_efs(L, jac, [order(0, 2, 3, 1)], [r])
    bas, der = explicit(L, efs)
    jinv = np.random.default_rng(4).uniform(-1, 1, (len(bas), 3, 3))
    _, dm = explicit(L, efs, jinv=jinv.ravel())
    np.testing.assert_allclose(dm, np.einsum("qpk,qke->qpe", der, jinv), rtol=1e-13, atol=1e-14)
    assert bas.shape == (3 * 4 * 2, 3 * 4 * 2)


def test_type_and_family_errors(L, jac):
    assert L.dJacobiSetType(jac, b"nodal") != 0
    assert b"Unable to find requested dJacobi type nodal" in L.dGetLastError()
    dg.chk(L.dJacobiModalSetFamily(jac, ctypes.c_int(P_CONFORMING)))  # tensor type: nothing to do
    set_type(L, jac, "modal")
    dg.chk(L.dJacobiModalSetFamily(jac, ctypes.c_int(P_DISCONTINUOUS)))
    assert L.dJacobiModalSetFamily(jac, ctypes.c_int(P_CONFORMING)) != 0
    assert b"only P-discontinuous" in L.dGetLastError()
    (r,) = get_rules(L, quad(L, jac, FAST), [order(4)])
    rl = (ctypes.c_void_p * 1)(r.value)
    arr = ctypes.POINTER(ctypes.c_void_p)()
    topo, ords = np.array([HEX], np.int32), np.array([order(4)], np.int32)
    assert L.dJacobiGetEFS(jac, ctypes.c_int32(1), dg.ptr(topo), dg.ptr(ords), rl, ctypes.byref(arr)) != 0
    assert b"order 4" in L.dGetLastError()
    (m,) = get_efs(L, jac, [order(2)], [r])
    assert L.dEFSGetTensorNodes(m, None, None, None, None, None, None) != 0
    assert L.dEFSGetTensorTables(m, None, None, None, None, None) != 0
    eidx, bi, bd, Pn = np.zeros(64, np.int32), np.zeros(512), np.zeros(1536), ctypes.c_int32()
    qidx = np.arange(8, dtype=np.int32)
    assert L.dEFSGetExplicitSparse(m, ctypes.c_int32(1), ctypes.c_int32(8), dg.ptr(qidx), None,
                                   ctypes.c_int32(0), ctypes.byref(Pn), dg.ptr(eidx), dg.ptr(bi), dg.ptr(bd)) != 0
    assert b"modal" in L.dGetLastError()
    # a dFS needs the tensor type; back on the tensor type the same dJacobi makes tensor spaces again
    mesh = ctypes.c_void_p()
    npts, box = np.array([3, 3, 3], np.int32), np.array([0, 1, 0, 1, 0, 1], np.float64)
    dg.chk(L.dMeshCreateBlock(dg.ptr(npts), dg.ptr(box), ctypes.c_double(0.0), ctypes.c_uint64(1), ctypes.byref(mesh)))
    fs = ctypes.c_void_p()
    assert L.dFSCreate(mesh, jac, ctypes.byref(fs)) != 0
    assert b"tensor dJacobi" in L.dGetLastError()
    set_type(L, jac, "tensor")
    dg.chk(L.dFSCreate(mesh, jac, ctypes.byref(fs)))
    set_type(L, jac, "modal")
    dg.chk(L.dFSSetDegree(fs, ctypes.c_int32(2), None))
    assert L.dFSBuildSpace(fs) != 0
    assert b"tensor dJacobi" in L.dGetLastError()
    L.dFSDestroy(ctypes.byref(fs))
    L.dMeshDestroy(ctypes.byref(mesh))


def test_tensor_nodes_with_the_reference_signature(L, jac):
    """dEFSGetTensorNodes (jacobi.c:447-455, efstopo.c:260-290): dim, nodes per direction and the element's own GLL
    nodes and weights per direction (jacobi/tests/ex1.c:138 reads them this way)"""
    (r,) = get_rules(L, quad(L, jac, FAST), [order(0, 4, 6, 8)])
    (efs,) = get_efs(L, jac, [order(0, 2, 3, 4)], [r])
    dim, tsize = ctypes.c_int32(), (ctypes.c_int32 * 3)()
    nodes, weights = (ctypes.POINTER(ctypes.c_double) * 3)(), (ctypes.POINTER(ctypes.c_double) * 3)()
    dg.chk(L.dEFSGetTensorNodes(efs, ctypes.byref(dim), tsize, nodes, weights, None, None))
    assert dim.value == 3 and list(tsize) == [3, 4, 5]
    for d, P in enumerate(tsize):
        x, w = po.lobatto(P)
        np.testing.assert_allclose(np.ctypeslib.as_array(nodes[d], (P,)), x, rtol=0, atol=1e-15)
        np.testing.assert_allclose(np.ctypeslib.as_array(weights[d], (P,)), w, rtol=1e-14)
    ms = (ctypes.POINTER(ctypes.c_double) * 3)()
    assert L.dEFSGetTensorNodes(efs, None, None, None, None, ms, None) != 0
    assert b"pass NULL" in L.dGetLastError()


def test_facet_rules_with_the_reference_arguments(L, jac):
    """dQuadratureGetFacetRules (tensorquad.c:309-355): for every side of the hex and isotropic orders, the facet rule's
    points and weights are those of dFSGetFacetRule and of the oracle's restatement; dim 2; cached per (side, orders);
    tensor element spaces and tensor node queries are refused on facet rules; a side out of range is an error"""
    q = quad(L, jac, FAST)
    for order_ in (2, 4, 6):
        sides = np.arange(6, dtype=np.int32)
        topo, ords = np.full(6, HEX, np.int32), np.full(6, order(order_), np.int32)
        arr = ctypes.POINTER(ctypes.c_void_p)()
        dg.chk(L.dQuadratureGetFacetRules(q, ctypes.c_int32(6), dg.ptr(topo), dg.ptr(sides), dg.ptr(ords), ctypes.byref(arr)))
        rules = [ctypes.c_void_p(arr[i]) for i in range(6)]
        dg.chk(L.dFree(arr))
        for side, r in enumerate(rules):
            dim, nn = ctypes.c_int32(), ctypes.c_int32()
            dg.chk(L.dRuleGetSize(r, ctypes.byref(dim), ctypes.byref(nn)))
            assert dim.value == 2 and nn.value == (1 + order_ // 2) ** 2
            pts, w = node_weight(L, r)
            n_ref, w_ref = dg.facet_rule(side, order_)
            np.testing.assert_array_equal(pts, n_ref.reshape(-1, 3))
            np.testing.assert_array_equal(w, w_ref)
            no, wo = po.facet_rule(side, order_)
            np.testing.assert_allclose(pts, no.reshape(-1, 3), rtol=0, atol=1e-15)
            np.testing.assert_allclose(w, wo, rtol=1e-14)
            npch, psz = ctypes.c_int32(), ctypes.c_int32()
            dg.chk(L.dRuleGetPatches(r, ctypes.byref(npch), ctypes.byref(psz), None, None))
            assert (npch.value, psz.value) == (1, nn.value)
        again = ctypes.POINTER(ctypes.c_void_p)()
        dg.chk(L.dQuadratureGetFacetRules(q, ctypes.c_int32(6), dg.ptr(topo), dg.ptr(sides), dg.ptr(ords), ctypes.byref(again)))
        assert [again[i] for i in range(6)] == [r.value for r in rules]
        dg.chk(L.dFree(again))
    assert L.dRuleGetTensorNodeWeight(rules[0], None, None, None, None) != 0
    rl = (ctypes.c_void_p * 1)(rules[0].value)
    topo1, ord1 = np.array([HEX], np.int32), np.array([order(2)], np.int32)
    assert L.dJacobiGetEFS(jac, ctypes.c_int32(1), dg.ptr(topo1), dg.ptr(ord1), rl, ctypes.byref(arr)) != 0
    assert b"facet rules" in L.dGetLastError()
    bad = np.array([6], np.int32)
    assert L.dQuadratureGetFacetRules(q, ctypes.c_int32(1), dg.ptr(topo1), dg.ptr(bad), dg.ptr(ord1), ctypes.byref(arr)) != 0


def test_node_counts(L, jac):
    """dJacobiGetNodeCount (tensor.c:249-281, modal.c:297-310): interior and expanded nodes per entity; against the sizes
    of the element spaces the dJacobi makes and of a built space's closure"""
    topo = np.array([HEX, HEX, 4, 1, 0], np.int32)  # hexahedron, quadrilateral, line, point
    deg = np.array([order(0, 2, 3, 4), order(5), order(0, 3, 2, 2), order(4), order(4)], np.int32)
    ino, xno = np.zeros(5, np.int32), np.zeros(5, np.int32)
    dg.chk(L.dJacobiGetNodeCount(jac, ctypes.c_int32(5), dg.ptr(topo), dg.ptr(deg), dg.ptr(ino), dg.ptr(xno)))
    np.testing.assert_array_equal(ino, [1 * 2 * 3, 4 ** 3, 2 * 1, 3, 1])
    np.testing.assert_array_equal(xno, [3 * 4 * 5, 6 ** 3, 4 * 3, 5, 1])
    (r,) = get_rules(L, quad(L, jac, FAST), [order(10)])
    (efs,) = get_efs(L, jac, [order(5)], [r])
    dim, inodes, total = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    dg.chk(L.dEFSGetSizes(efs, ctypes.byref(dim), ctypes.byref(inodes), ctypes.byref(total)))
    assert (inodes.value, total.value) == (ino[1], xno[1])
    bad, deg1 = np.array([6], np.int32), deg[:1].copy()
    assert L.dJacobiGetNodeCount(jac, ctypes.c_int32(1), dg.ptr(bad), dg.ptr(deg1), None, None) != 0
    set_type(L, jac, "modal")
    mdeg, mtopo = np.array([order(i) for i in range(4)], np.int32), np.full(4, HEX, np.int32)
    dg.chk(L.dJacobiGetNodeCount(jac, ctypes.c_int32(4), dg.ptr(mtopo), dg.ptr(mdeg), dg.ptr(ino), dg.ptr(xno)))
    np.testing.assert_array_equal(ino[:4], [1, 4, 10, 18])
    np.testing.assert_array_equal(xno[:4], [1, 4, 10, 18])
