"""The oracle's hp extension (interpolation-constrained E for per-element orders; the reference errors on
p-nonconforming entities, src/jacobi/impls/tensor/tensor.c:417): conformity and consistency checks."""
import numpy as np
import pytest

import pyoracle as po


def element_trace(fs, xe, e, P, face):
    """values of element e's tensor polynomial on one face at 5x5 reference points (face: axis, side)."""
    axis, side = face
    node, _ = po.lobatto(P)
    pts = np.linspace(-0.9, 0.9, 5)
    U = xe.reshape(P, P, P)
    vals = np.zeros((5, 5))
    for a, s in enumerate(pts):
        for b, t in enumerate(pts):
            ref = [None, None, None]
            ref[axis] = side
            others = [d for d in range(3) if d != axis]
            ref[others[0]], ref[others[1]] = s, t
            L = [po.tensor_basis(P, np.array([ref[d]]))[0][0] for d in range(3)]
            vals[a, b] = np.einsum("i,j,k,ijk->", L[0], L[1], L[2], U)
    return vals


@pytest.mark.parametrize("seed", [1, 2])
def test_hp_expanded_field_is_continuous_across_faces(seed):
    rng = np.random.default_rng(seed)
    ed = rng.integers(2, 9, size=8).astype(np.int32)
    fs = po.FS(3, 3, 3, degree=4, perturb=0.0, seed=1, elem_degree=ed, dirichlet_mask=0)
    g = rng.standard_normal(fs.n)
    x = fs.global_to_expanded(g)
    xs = fs.xstart()
    deg = fs.elem_degree()[:, 0]
    # element index (i*2 + j)*2 + k on the 2x2x2 block; neighbours across x, y and z faces
    for e in range(8):
        i, j, k = e // 4, (e // 2) % 2, e % 2
        for axis in range(3):
            nb = [i, j, k]
            if nb[axis] == 1:
                continue
            nb[axis] += 1
            f = (nb[0] * 2 + nb[1]) * 2 + nb[2]
            ta = element_trace(fs, x[xs[e]:xs[e + 1]], e, deg[e] + 1, (axis, 1.0))
            tb = element_trace(fs, x[xs[f]:xs[f + 1]], f, deg[f] + 1, (axis, -1.0))
            np.testing.assert_allclose(ta, tb, atol=1e-12)


def test_hp_reduces_to_reference_map_when_uniform():
    ed = np.full(27, 3, np.int32)
    a = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=2, elem_degree=ed)
    b = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=2)
    np.testing.assert_array_equal(a.emap(), b.emap())
    p, c, v = a.ecsr()
    assert np.all(np.diff(p) == 1) and np.all(v == 1.0)


def test_hp_operator_symmetric_and_constant_preserving():
    rng = np.random.default_rng(3)
    ed = rng.integers(2, 9, size=27).astype(np.int32)
    fs = po.FS(4, 4, 4, degree=4, perturb=0.1, seed=1, elem_degree=ed)
    one = fs.global_to_expanded(np.ones(fs.n), dcache=np.ones(fs.nc - fs.n))
    assert np.abs(one - 1).max() < 1e-14
    a, b = rng.standard_normal(fs.n), rng.standard_normal(fs.n)
    Aa, Ab = fs.apply(a), fs.apply(b)
    assert a @ Ab == pytest.approx(b @ Aa, rel=1e-12)
