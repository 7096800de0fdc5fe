"""dFSMatSetValuesBlockedExpanded (src/fs/interface/fs.c:826-930): element blocks in expanded indices expanded through
E into the Q1-embedded matrix: ADD_VALUES adds exactly the block at the E images of its rows and columns (Dirichlet
rows and columns dropped), INSERT_VALUES overwrites them, the KSP sees the change after dKSPSetOperators, and a target
outside the sparsity pattern is an error."""
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


def entry(rp, col, r, c):
    k = np.nonzero(col[rp[r]:rp[r + 1]] == c)[0]
    return rp[r] + int(k[0]) if len(k) else -1


def test_add_insert_and_pattern():
    p = 2
    fs = dg.FS((4, 4, 4), degree=p, perturb=0.1, seed=2)
    m = fs.matrix()
    m.assemble()
    rp, col, v0 = m.csr_host()
    em, xs = fs.emap()
    N = p + 1
    rng = np.random.default_rng(1)
    for e in (0, 13, 26):  # a corner element (Dirichlet nodes dropped) and interior ones
        # the 8 corners of the element's first Q1 sub-cell, in expanded indices
        idx = np.array([xs[e] + (a * N + b) * N + c for a in (0, 1) for b in (0, 1) for c in (0, 1)], np.int32)
        blk = rng.standard_normal((8, 8))
        m.set_values_expanded(idx, idx, blk, dg.ADD_VALUES)
        _, _, v1 = m.csr_host()
        want = v0.copy()
        for i in range(8):
            for j in range(8):
                r, c = em[idx[i]], em[idx[j]]
                if r < fs.n and c < fs.n:
                    want[entry(rp, col, r, c)] += blk[i, j]
        np.testing.assert_array_equal(v1, want)
        v0 = v1
    blk = rng.standard_normal((8, 8))
    m.set_values_expanded(idx, idx, blk, dg.INSERT_VALUES)
    _, _, v2 = m.csr_host()
    for i in range(8):
        for j in range(8):
            r, c = em[idx[i]], em[idx[j]]
            if r < fs.n and c < fs.n:
                assert v2[entry(rp, col, r, c)] == blk[i, j]
    # nodes of two far-apart elements do not couple in the Q1 pattern
    far = np.array([xs[0] + N * N * N - 1 - N * N - N - 1, xs[fs.nelem - 1] + N * N + N + 1], np.int32)
    assert em[far[0]] < fs.n and em[far[1]] < fs.n
    with pytest.raises(dg.DohpError, match="sparsity"):
        m.set_values_expanded(far[:1], far[1:], np.ones((1, 1)))


def test_ksp_sees_the_new_values_after_set_operators():
    """a matrix assembled element by element through the expanded entry point (the reference's EllipJacobian loop shape)
    preconditions CG as well as the batched assembly: the same iteration count when the blocks are the batched
    assembly's own values re-added to a zeroed matrix"""
    fs = dg.FS((5, 5, 5), degree=2, perturb=0.1, seed=3)
    op = fs.operator()
    ref = fs.matrix()
    ref.assemble()
    b = torch.as_tensor(np.random.default_rng(2).uniform(-1, 1, fs.n), device="cuda")
    x = torch.zeros_like(b)
    its_ref, _ = dg.KSP(op, ref, ksp_type=dg.dKSP_CG).solve(b, x, rtol=1e-8, maxit=500)
    m = fs.matrix()
    m.assemble()
    ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
    # scale the matrix by 2 through INSERT of 2x every existing entry (row by row from the CSR, expanded indices of
    # each row's and column's first appearance)
    rp, col, v = m.csr_host()
    em, xs = fs.emap()
    first = {}
    for e_idx, c in enumerate(em):
        if c < fs.n and c not in first:
            first[c] = e_idx
    for r in range(fs.n):
        cols = col[rp[r]:rp[r + 1]]
        m.set_values_expanded([first[r]], [first[c] for c in cols], (2 * v[rp[r]:rp[r + 1]])[None, :], dg.INSERT_VALUES)
    chk_rp, chk_col, v2 = m.csr_host()
    np.testing.assert_array_equal(v2, 2 * v)
    ksp.set_operators(op, m)
    x.zero_()
    its2, rn = ksp.solve(b, x, rtol=1e-8, maxit=500)
    assert rn <= 1e-8 and abs(its2 - its_ref) <= 2  # a scaled preconditioner: the same Krylov space
