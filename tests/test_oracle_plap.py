"""Oracle p-Laplacian (src/fs/tests/ellip.c:333-536): store, Q1-embedded Jacobian at a state, and a
Newton solve built from the oracle's own pieces (CPU)."""
import numpy as np
import pytest

import pyoracle as po

sp = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")


def test_p2_reduces_to_poisson():
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=1)
    g = np.random.default_rng(0).uniform(-1, 1, o.n)
    st = o.plap_stash(g, 2.0, 1e-6).reshape(-1, 4)
    assert np.all(st[:, 0] == 1.0) and np.all(st[:, 1:] == 0.0)
    rp, col, val = o.q1_assemble(kind=1, param=(2.0, 1e-6), state=g)
    rp0, col0, val0 = o.q1_assemble(kind=0)
    np.testing.assert_array_equal(col, col0)
    assert np.abs(val - val0).max() < 1e-15 * np.abs(val0).max()


def test_q1_jacobian_symmetric_positive():
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=2)
    g = np.random.default_rng(1).uniform(-1, 1, o.n)
    rp, col, val = o.q1_assemble(kind=1, param=(1.5, 1e-6), state=g)
    A = sp.csr_matrix((val, col, rp), shape=(o.n, o.n))
    assert abs(A - A.T).max() < 1e-14 * abs(A).max()
    assert np.linalg.eigvalsh(A.toarray()).min() > 0


def test_stash_store_formula():
    """eta = (eps^2 + |Du|^2/2)^((p-2)/2), |s|^2 = ((2-p)/2) eta |Du|^2 / (eps^2 + |Du|^2/2)."""
    o = po.FS(3, 3, 3, degree=2, perturb=0.1, seed=3)
    g = np.random.default_rng(2).uniform(-1, 1, o.n)
    p, eps = 1.5, 1e-3
    st = o.plap_stash(g, p, eps).reshape(-1, 4)
    eta, s2 = st[:, 0], (st[:, 1:] ** 2).sum(1)
    espg = eta ** (2 / (p - 2))
    du2 = 2 * (espg - eps * eps)
    np.testing.assert_allclose(s2, (2 - p) / 2 * eta * du2 / espg, rtol=1e-9, atol=1e-14)


def test_oracle_newton_converges():
    o = po.FS(5, 5, 5, degree=2, perturb=0.1, seed=4)
    p, eps = 1.5, 1e-6
    b = np.random.default_rng(0).uniform(-1, 1, o.n)

    def F(u):
        st = o.plap_stash(u, p, eps).reshape(-1, 4)
        s0 = st.copy()
        s0[:, 1:] = 0
        return o.apply(u, kind=1, qdata=s0.ravel()) - b, st

    u = np.zeros(o.n)
    r, st = F(u)
    f0 = np.linalg.norm(r)
    for _ in range(20):
        J = spl.LinearOperator((o.n, o.n), matvec=lambda x: o.apply(x, kind=1, qdata=st.ravel()))
        rp, col, val = o.q1_assemble(kind=1, param=(p, eps), state=u)
        M = spl.factorized(sp.csr_matrix((val, col, rp), shape=(o.n, o.n)).tocsc())
        du, info = spl.gmres(J, -r, rtol=1e-6, M=spl.LinearOperator((o.n, o.n), matvec=M), restart=30, maxiter=100)
        assert info == 0
        u = u + du
        r, st = F(u)
        if np.linalg.norm(r) < 1e-8 * f0:
            break
    assert np.linalg.norm(r) < 1e-8 * f0
