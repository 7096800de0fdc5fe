"""Pins the CPU oracle against the reference's own golden outputs (refout files turned into fixtures
by tests/golden/make_golden.py) and, where it was built here, against the reference's own polylib and
TensorMult_Hex compiled from source (oracle/_ref)."""
import os

import numpy as np
import pytest

import pyoracle as po

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INTERP, INTERP_T, GRAD, GRAD_T = 40001, 40002, 40003, 40004


def gold(name):
    return np.load(os.path.join(GOLD, name + ".npz"))


# ---------------------------------------------------------------- 1-D rules and bases vs reference polylib
@pytest.mark.parametrize("n", range(2, 13))
def test_gauss_lobatto_vs_reference_polylib(n):
    R = po.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built (reference tree not present)")
    for ours, name in ((po.gauss, "zwgj"), (po.lobatto, "zwglj")):
        x, w = ours(n)
        xr = np.zeros(n); wr = np.zeros(n)
        getattr(R, name)(xr, wr, n, 0.0, 0.0)
        np.testing.assert_allclose(x, xr, rtol=0, atol=2e-15)
        np.testing.assert_allclose(w, wr, rtol=0, atol=2e-15)


@pytest.mark.parametrize("P", range(2, 11))
def test_tensor_basis_vs_reference_polylib(P):
    R = po.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built")
    rx, _ = po.gauss(P + 1)
    interp, deriv, node, _ = po.tensor_basis(P, rx)
    zr = np.zeros(P); wr = np.zeros(P)
    R.zwglj(zr, wr, P, 0.0, 0.0)
    Ir = np.zeros(P * len(rx)); Dc = np.zeros(P * P); DcT = np.zeros(P * P)
    R.Imglj(Ir, zr, rx, P, len(rx), 0.0, 0.0)
    R.Dglj(Dc, DcT, zr, P, 0.0, 0.0)
    Ir = Ir.reshape(len(rx), P)
    np.testing.assert_allclose(interp, Ir, rtol=0, atol=1e-13)
    np.testing.assert_allclose(deriv, Ir @ Dc.reshape(P, P), rtol=0, atol=5e-12 * P * P)


@pytest.mark.parametrize("D", [1, 3])
def test_tensor_mult_vs_reference(D):
    R = po.ref_lib()
    if R is None:
        pytest.skip("oracle/_ref not built")
    rng = np.random.default_rng(3)
    for P, Q in [((2, 2, 2), (3, 3, 3)), ((5, 4, 3), (3, 6, 5)), ((9, 9, 9), (9, 9, 9))]:
        P = np.array(P, np.int32); Q = np.array(Q, np.int32)
        A = [rng.standard_normal(int(Q[i] * P[i])) for i in range(3)]
        x = rng.standard_normal(int(np.prod(P)) * D)
        ptrs, keep = po._ptr_array(A)
        out = np.zeros(int(np.prod(Q)) * D); outr = np.zeros_like(out)
        po.lib().or_tensor_mult_hex(D, P, Q, ptrs, x, out, 1)
        R.ref_tensor_mult_hex(D, P, Q, ptrs, x, outr, 1)
        np.testing.assert_allclose(out, outr, rtol=1e-14, atol=1e-13)


# ---------------------------------------------------------------- explicit bases (jacobi-3-tensor-*)
def explicit(P, family, rule_degree):
    rx, rw = po.rule_1d(0, family, rule_degree)
    interp, deriv, _, _ = po.tensor_basis(P, rx)
    nb, nq = P ** 3, len(rx) ** 3
    bas = np.zeros((nq, nb)); der = np.zeros((nq, nb * 3))
    for i in range(nb):
        e = np.zeros(nb); e[i] = 1
        bas[:, i] = po.efs_apply_hex([P] * 3, [len(rx)] * 3, [interp] * 3, [deriv] * 3, None, 1, e, INTERP)
        der[:, 3 * i:3 * i + 3] = po.efs_apply_hex([P] * 3, [len(rx)] * 3, [interp] * 3, [deriv] * 3, None, 1, e,
                                                   GRAD).reshape(nq, 3)
    w = np.einsum("i,j,k->ijk", rw, rw, rw).ravel()
    mass = bas.T @ (w[:, None] * bas)
    return bas, der, mass


@pytest.mark.parametrize("name,family,rdeg", [("jacobi3_gauss", 0, 8), ("jacobi3_lobatto", 1, 6)])
def test_explicit_bases_golden(name, family, rdeg):
    g = gold(name)
    for e in range(4):
        bas, der, mass = explicit(e + 2, family, rdeg)
        np.testing.assert_allclose(mass, g[f"e{e}_mass"], atol=6e-7)
        if f"e{e}_interpolation" in g:
            np.testing.assert_allclose(bas, g[f"e{e}_interpolation"], atol=6e-7)
            np.testing.assert_allclose(der, g[f"e{e}_gradient"], atol=6e-7)
        else:
            h = g[f"e{e}_interpolation_head"]
            np.testing.assert_allclose(bas[:len(h)], h, atol=6e-7)
            np.testing.assert_allclose(der[:len(h)], g[f"e{e}_gradient_head"], atol=6e-7)


@pytest.mark.parametrize("name,rdeg", [("jacobi3_sparsex_r4", 4), ("jacobi3_sparsex_r6", 6)])
def test_sparse_q1_bases_golden(name, rdeg):
    """Q1 sub-cell bases incl. the missing 1/h_sub factor (efstopo.c:665-706)."""
    g = gold(name)
    rx, rw = po.rule_1d(1, 0, rdeg)
    Q = [len(rx)] * 3
    npatch, psz, ind, _ = po.rule_patches(1, Q, [rw, rw, rw])
    for e in range(3):
        P = e + 2
        interp, deriv, _, _ = po.tensor_basis(P, rx)
        eidx, bi, bd = po.explicit_sparse([P] * 3, Q, [interp] * 3, [deriv] * 3, npatch, psz, ind)
        np.testing.assert_array_equal(ind, g[f"e{e}_qidx"])
        np.testing.assert_array_equal(eidx, g[f"e{e}_bidx"])
        for p in range(min(4, npatch)):
            np.testing.assert_allclose(bi[p], g[f"e{e}_p{p}_interp"], atol=6e-6)
            np.testing.assert_allclose(bd[p], g[f"e{e}_p{p}_deriv"], atol=6e-6)


@pytest.mark.parametrize("name,method", [("jacobi4_fast", 0), ("jacobi4_sparse", 1)])
def test_patch_tables_golden(name, method):
    """dRuleGetPatches (tensorquad.c:120-169) incl. the z-weight index quirk."""
    g = gold(name)
    for e in range(4):
        rdeg = (e + 1) * 2 - 2
        rx, rw = po.rule_1d(method, 0, rdeg)
        npatch, psz, ind, wt = po.rule_patches(method, [len(rx)] * 3, [rw, rw, rw])
        assert [npatch, psz] == list(g[f"e{e}_shape"])
        np.testing.assert_array_equal(ind, g[f"e{e}_indices"])
        np.testing.assert_allclose(wt, g[f"e{e}_weights"], atol=6e-6)


# ---------------------------------------------------------------- interpolation accuracy (jacobi-1)
def exact0(y):
    a, b, c = 0.1, 0.2, 0.3
    x0, x1, x2 = y
    f = np.array([np.sin(x0 - a) * np.cos(-x1 - b) * np.tanh(-x2 - c),
                  np.cos(x0 - a) * np.sin(x1 - b) * np.tanh(-x2 - c),
                  np.sinh(x0 - a) * np.tanh(x1 - b) * np.cosh(x2 - c)])
    dt = lambda t: 1 - np.tanh(t) ** 2
    df = np.array([
        [np.cos(x0 - a) * np.cos(-x1 - b) * np.tanh(-x2 - c), np.sin(x0 - a) * np.sin(-x1 - b) * np.tanh(-x2 - c),
         -np.sin(x0 - a) * np.cos(-x1 - b) * dt(-x2 - c)],
        [-np.sin(x0 - a) * np.sin(x1 - b) * np.tanh(-x2 - c), np.cos(x0 - a) * np.cos(x1 - b) * np.tanh(-x2 - c),
         -np.cos(x0 - a) * np.sin(x1 - b) * dt(-x2 - c)],
        [np.cosh(x0 - a) * np.tanh(x1 - b) * np.cosh(x2 - c), np.sinh(x0 - a) * dt(x1 - b) * np.cosh(x2 - c),
         np.sinh(x0 - a) * np.tanh(x1 - b) * np.sinh(x2 - c)]])
    return f, df


@pytest.mark.parametrize("name,family", [("jacobi1_gauss", 0), ("jacobi1_lobatto", 1)])
def test_interp_errors_golden(name, family):
    """checkInterp (src/jacobi/tests/ex1.c:119-223): D=3 field at GLL nodes -> INTERP/GRAD errors."""
    rows = gold(name)["rows"]
    for _, P, Qn, ez_ref, edz_ref in rows:
        P, Qn = int(P), int(Qn)
        rdeg = 2 * (Qn - 1) if family == 0 else 2 * (Qn - 2)
        rx, rw = po.rule_1d(0, family, rdeg)
        assert len(rx) == Qn
        interp, deriv, node, _ = po.tensor_basis(P, rx)
        f = np.zeros((P, P, P, 3))
        for i in range(P):
            for j in range(P):
                for k in range(P):
                    f[i, j, k] = exact0((node[i], node[j], node[k]))[0]
        g = po.efs_apply_hex([P] * 3, [Qn] * 3, [interp] * 3, [deriv] * 3, None, 3, f.ravel(), INTERP).reshape(-1, 3)
        dg = po.efs_apply_hex([P] * 3, [Qn] * 3, [interp] * 3, [deriv] * 3, None, 3, f.ravel(), GRAD).reshape(-1, 3, 3)
        z = dz = 0.0
        q = 0
        for i in range(Qn):
            for j in range(Qn):
                for k in range(Qn):
                    h, dh = exact0((rx[i], rx[j], rx[k]))
                    w = rw[i] * rw[j] * rw[k]
                    z += np.sum((g[q] - h) ** 2) * w
                    dz += np.sum((dg[q] - dh) ** 2) * w
                    q += 1
        assert float("%.1e" % z) == pytest.approx(ez_ref, rel=0.06, abs=2e-12)
        assert float("%.1e" % dz) == pytest.approx(edz_ref, rel=0.06, abs=2e-10)


# ---------------------------------------------------------------- function space numbering (bu-0)
def test_bu0_expanded_and_closure_golden():
    """bu-0 (src/fs/tests/bu.c): 3x2x2 block, p=2, walls (100) Dirichlet, natural ordering."""
    g = gold("bu0")
    fs = po.FS(3, 2, 2, degree=2, box=(-1, 1, -1, 1, -1, 1), perturb=0.0, dirichlet_mask=1)
    assert (fs.nelem, fs.n, fs.nc, fs.nexp) == (2, 9, 45, 54)
    closure = g["closure"]
    np.testing.assert_array_equal(fs.global_to_expanded(closure[:fs.n]), g["homogeneous"])
    np.testing.assert_array_equal(fs.global_to_expanded(closure[:fs.n], dcache=np.full(fs.nc - fs.n, 10.0)),
                                  g["inhomogeneous"])
    # nodal coordinates of every closure node, through E from the trilinear map of each element's GLL nodes
    node, _ = po.lobatto(3)
    X = fs.coords_expanded()
    em = fs.emap()
    xs = fs.xstart()
    cl = np.full((fs.nc, 3), np.nan)
    for e in range(fs.nelem):
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    s = np.array([node[i], node[j], node[k]])
                    wts = np.array([(1 + (2 * a - 1) * s[0]) * (1 + (2 * b - 1) * s[1]) * (1 + (2 * c - 1) * s[2]) / 8
                                    for a in (0, 1) for b in (0, 1) for c in (0, 1)])
                    cl[em[xs[e] + (i * 3 + j) * 3 + k]] = wts @ X[e]
    np.testing.assert_allclose(cl.ravel(), g["coords"], atol=1e-12)


def test_expand_restrict_adjoint():
    fs = po.FS(4, 3, 5, degree=3, perturb=0.1, seed=7)
    rng = np.random.default_rng(0)
    g = rng.standard_normal(fs.n)
    x = rng.standard_normal(fs.nexp)
    lhs = x @ fs.global_to_expanded(g)
    rhs = g @ fs.expanded_to_global(x)
    assert lhs == pytest.approx(rhs, rel=1e-13)


def test_operator_symmetric_positive():
    fs = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=3)
    rng = np.random.default_rng(1)
    a, b = rng.standard_normal(fs.n), rng.standard_normal(fs.n)
    Aa, Ab = fs.apply(a), fs.apply(b)
    assert a @ Ab == pytest.approx(b @ Aa, rel=1e-12)
    assert a @ Aa > 0


def test_q1_assembly_and_cg_solve():
    fs = po.FS(5, 5, 5, degree=4, perturb=0.1, seed=2)
    csr = fs.q1_assemble()
    rp, col, val = csr
    # symmetric sparsity, <= 27 entries per row, rows sorted
    assert np.all(np.diff(rp) <= 27)
    for i in range(0, fs.n, 37):
        c = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(c) > 0)
    rng = np.random.default_rng(5)
    b = rng.uniform(-1, 1, fs.n)
    x, its, rn = fs.cg_solve(b, csr, rtol=1e-8)
    assert its > 0 and rn <= 1e-8
    r = b - fs.apply(x)
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(b)


def test_sparse_rule_efs_golden():
    """jacobi-3-tensor-sparse-gauss (dEFSView on the SPARSE rule of degree 4, tensorquad.c:32-49, 68-80): the rule's
    points and weights (2 Gauss points in each GLL sub-interval, weight h/2) and the GLL bases of 2..5 nodes at them
    (tensor.c:22-109), to the 5 printed decimals"""
    g = gold("jacobi3_sparse_efs")
    rx, rw = po.rule_1d(1, 0, 4)
    for P in range(2, 6):
        np.testing.assert_allclose(rx, g[f"P{P}_q"], atol=6e-6)
        np.testing.assert_allclose(rw, g[f"P{P}_w"], atol=6e-6)
        interp, deriv, node, _ = po.tensor_basis(P, rx)
        np.testing.assert_allclose(interp, g[f"P{P}_interp"], atol=6e-6)
        np.testing.assert_allclose(deriv, g[f"P{P}_deriv"], atol=6e-6)
        np.testing.assert_allclose(node, g[f"P{P}_node"], atol=6e-6)


# ---------------------------------------------------------------- modal bases (jacobi-2-modal-*, jacobi-3-modal-gauss)
# ex2.c's mode weights: the first primes, one per mode
PRIMES = np.array([2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71], float)


def tensor_points(method, family, rule_degree):
    """rule points [Q][3] (x slowest) and weights of the tensor rule (dRuleGetNodeWeight order)"""
    x, w = po.rule_1d(method, family, rule_degree)
    pts = np.stack(np.meshgrid(x, x, x, indexing="ij"), axis=-1).reshape(-1, 3)
    return pts, np.einsum("i,j,k->ijk", w, w, w).ravel()


@pytest.mark.parametrize("name,method,family,rdeg", [("jacobi2_modal_fast_gauss", 0, 0, 6),
                                                     ("jacobi2_modal_fast_lobatto", 0, 1, 4),
                                                     ("jacobi2_modal_sparse_gauss", 1, 0, 6)])
def test_modal_values_and_mass_golden(name, method, family, rdeg):
    """jacobi-2-modal-* (src/jacobi/tests/ex2.c): modes of orders 0..3 weighted by the first primes, evaluated at the
    rule points (INTERP) and brought back through the weighted INTERP_TRANSPOSE (the mass matrix: the identity where
    the rule integrates the products exactly; the 4-point Lobatto rule does not for the cubic modes), to the 5
    printed digits"""
    g = gold(name)
    pts, w = tensor_points(method, family, rdeg)
    for order in range(4):
        interp, deriv = po.modal_basis(order, pts)
        P = interp.shape[1]
        assert P == [1, 4, 10, 18][order]
        vals = po.modal_apply(interp, deriv, 1, PRIMES[:P], INTERP)
        ref = g[f"e{order}_values"]
        np.testing.assert_allclose(vals, ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())
        back = po.modal_apply(interp, deriv, 1, vals * w, INTERP_T)
        ref = g[f"e{order}_mass_applied"]
        np.testing.assert_allclose(back, ref, rtol=5.1e-5, atol=1e-9 * np.abs(ref).max())


def test_modal_explicit_golden():
    """jacobi-3-modal-gauss (src/jacobi/tests/ex3.c on the modal type, FAST Gauss rule of degree 6): interpolation
    (Q, P), gradient (Q, 3P) and mass (P, P) matrices of the orders 0..3 to the 6 printed decimals; GRAD of each unit
    mode is the gradient column block, as the reference's generic dEFSGetExplicit forms it"""
    g = gold("jacobi3_modal_gauss")
    pts, w = tensor_points(0, 0, 6)
    for order in range(4):
        interp, deriv = po.modal_basis(order, pts)
        P = interp.shape[1]
        grad = np.stack([po.modal_apply(interp, deriv, 1, np.eye(P)[j], GRAD).reshape(-1, 3) for j in range(P)], axis=1)
        np.testing.assert_allclose(interp, g[f"e{order}_interpolation"], atol=6e-7)
        np.testing.assert_allclose(grad.reshape(len(pts), 3 * P), g[f"e{order}_gradient"], atol=6e-7)
        np.testing.assert_allclose(interp.T @ (w[:, None] * interp), g[f"e{order}_mass"], atol=6e-7)


def test_modal_orders_and_modes_refused():
    with pytest.raises(RuntimeError, match="Order 4"):
        po.modal_basis(4, np.zeros((1, 3)))
    interp, deriv = po.modal_basis(2, tensor_points(0, 0, 4)[0])
    with pytest.raises(RuntimeError, match="Apply-mode not implemented"):
        po.modal_apply(interp, deriv, 1, np.zeros(len(interp) * 3), GRAD_T)
