"""The oracle's Stokes blocks (src/fs/tests/stokes.c restated) pinned by structure: the coupled apply is A + Bt
and B, Bt is the adjoint of B, A is symmetric positive, constants are the pressure null space with Dirichlet
walls, the penalty adds lambda int (div u)^2, and B of a linear field integrates its divergence."""
import numpy as np

import pyoracle as po


def pair(k=3, codim=2, npts=(4, 4, 5), dirichlet=7, seed=1):
    fu = po.FS(*npts, degree=k, perturb=0.1, seed=seed, bs=3, dirichlet_mask=dirichlet)
    fp = po.FS(*npts, degree=k - codim, perturb=0.1, seed=seed, bs=1, dirichlet_mask=0)
    return fu, fp


def test_block_structure():
    fu, fp = pair()
    rng = np.random.default_rng(0)
    xu, yu, xp = rng.standard_normal(fu.n * 3), rng.standard_normal(fu.n * 3), rng.standard_normal(fp.n)
    A, _ = po.stokes_apply(fu, fp, 0, xu=xu)
    Ay, _ = po.stokes_apply(fu, fp, 0, xu=yu)
    Bt, _ = po.stokes_apply(fu, fp, 1, xp=xp)
    _, B = po.stokes_apply(fu, fp, 2, xu=xu)
    Cu, Cp = po.stokes_apply(fu, fp, 3, xu=xu, xp=xp)
    s = np.linalg.norm(Cu)
    assert np.linalg.norm(Cu - A - Bt) < 1e-14 * s and np.linalg.norm(Cp - B) < 1e-14 * np.linalg.norm(B)
    assert abs(xp @ B - xu @ Bt) < 1e-13 * abs(xp @ B)
    assert abs(yu @ A - xu @ Ay) < 1e-13 * abs(yu @ A) and xu @ A > 0
    Bt1, _ = po.stokes_apply(fu, fp, 1, xp=np.ones(fp.n))
    assert np.abs(Bt1).max() < 1e-13


def test_penalty_is_lambda_div_squared():
    fu, fp = pair(k=2, codim=1, seed=3)
    xu = np.random.default_rng(1).standard_normal(fu.n * 3)
    nu = 0.3
    lam = nu / (1 - 2 * nu)
    A0, _ = po.stokes_apply(fu, fp, 0, rheo=(1.0, 1.0, 2.0, 0.0), xu=xu)
    A1, _ = po.stokes_apply(fu, fp, 0, rheo=(1.0, 1.0, 2.0, nu), xu=xu)
    # (A1 - A0) = lam D^T W D with D the divergence at the points; xu.(A1 - A0).xu = lam int (div u)^2 >= 0, and
    # B with the penalty-free coupled apply does not change
    d = xu @ (A1 - A0)
    assert d > 0
    Cu0, _ = po.stokes_apply(fu, fp, 3, rheo=(1.0, 1.0, 2.0, 0.0), xu=xu, xp=np.zeros(fp.n))
    Cu1, _ = po.stokes_apply(fu, fp, 3, rheo=(1.0, 1.0, 2.0, nu), xu=xu, xp=np.zeros(fp.n))
    np.testing.assert_array_equal(Cu0, Cu1)
    # viscosity scales A linearly
    A2, _ = po.stokes_apply(fu, fp, 0, rheo=(2.5, 1.0, 2.0, 0.0), xu=xu)
    np.testing.assert_allclose(A2, 2.5 * A0, rtol=1e-13, atol=1e-13 * np.abs(A0).max())


def test_divergence_of_a_linear_field():
    """no Dirichlet sets: u = M x + c is in the space, div u = tr M, so sum_i (B u)_i = -tr(M) |Omega| = -tr M"""
    fu, fp = pair(k=2, codim=1, dirichlet=0, seed=5)
    M = np.array([[0.3, 1.0, -0.2], [0.5, -1.1, 0.4], [0.0, 0.7, 2.0]])
    c = np.array([0.1, -0.3, 0.2])
    # nodal coordinates of the velocity space (vertices of the unperturbed boundary and the trilinear map)
    ce, xs, ed, em = fu.coords_expanded(), fu.xstart(), fu.elem_degree(), fu.emap()
    g = np.zeros(fu.n * 3)
    gll = po.lobatto(3)[0]
    for e in range(fu.nelem):
        loc = 0
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    xi = (gll[i], gll[j], gll[k])
                    x = sum(np.prod([(1 + (2 * ((t >> (2 - a)) & 1) - 1) * xi[a]) / 2 for a in range(3)]) * ce[e, t]
                            for t in range(8))
                    r = em[xs[e] + loc]
                    if r >= 0:
                        g[3 * r:3 * r + 3] = M @ x + c
                    loc += 1
    _, B = po.stokes_apply(fu, fp, 2, xu=g)
    assert abs(B.sum() + np.trace(M)) < 1e-12


def test_function_is_the_coupled_apply_when_newtonian():
    """p = 2: eta = B whatever the state, so the function is the penalty-free coupled Jacobian"""
    fu, fp = pair(k=3, codim=1, seed=2)
    rng = np.random.default_rng(4)
    xu, xp = rng.standard_normal(fu.n * 3), rng.standard_normal(fp.n)
    rheo = (1.6, 0.5, 2.0, 0.25)
    Fu, Fp = po.stokes_apply(fu, fp, 4, rheo=rheo, xu=xu, xp=xp)
    Cu, Cp = po.stokes_apply(fu, fp, 3, rheo=rheo, xu=xu, xp=xp)
    np.testing.assert_allclose(Fu, Cu, rtol=0, atol=1e-14 * np.abs(Cu).max())
    np.testing.assert_array_equal(Fp, Cp)


def test_power_law_jacobian_is_the_derivative_of_the_function():
    """shear-thinning power law (p = 4/3, Glen n = 3): the Jacobian at the state x (the store eta, eta', Du of
    StokesPointwiseComputeStore) is the derivative of the function, checked by central differences; its A block
    stays symmetric positive (eta (p - 1) > 0 along the state's own direction)"""
    fu, fp = pair(k=2, codim=1, seed=6)
    rng = np.random.default_rng(8)
    xu, xp = 2.0 * rng.standard_normal(fu.n * 3), rng.standard_normal(fp.n)
    vu, vp = rng.standard_normal(fu.n * 3), rng.standard_normal(fp.n)
    rheo = (1.3, 0.7, 4.0 / 3.0, 0.0)
    h = 1e-5
    Fpu, Fpp = po.stokes_apply(fu, fp, 4, rheo=rheo, xu=xu + h * vu, xp=xp + h * vp)
    Fmu, Fmp = po.stokes_apply(fu, fp, 4, rheo=rheo, xu=xu - h * vu, xp=xp - h * vp)
    Ju, Jp = po.stokes_apply(fu, fp, 3, rheo=rheo, xu=vu, xp=vp, state=xu)
    du, dp = (Fpu - Fmu) / (2 * h), (Fpp - Fmp) / (2 * h)
    assert np.linalg.norm(du - Ju) < 1e-7 * np.linalg.norm(Ju)
    assert np.linalg.norm(dp - Jp) < 1e-9 * np.linalg.norm(Jp)
    # the Jacobian really depends on the state: at the zero state it differs
    J0u, _ = po.stokes_apply(fu, fp, 3, rheo=rheo, xu=vu, xp=vp)
    assert np.linalg.norm(J0u - Ju) > 1e-2 * np.linalg.norm(Ju)
    Au, _ = po.stokes_apply(fu, fp, 0, rheo=rheo, xu=vu, state=xu)
    Aw, _ = po.stokes_apply(fu, fp, 0, rheo=rheo, xu=xu, state=xu)
    assert abs(xu @ Au - vu @ Aw) < 1e-12 * abs(vu @ Au) and vu @ Au > 0 and xu @ Aw > 0
