"""Oracle St. Venant-Kirchhoff (src/fs/tests/elast.c:224-280): the Jacobian at the stashed F is the derivative of
the function, and F = I gives linear elasticity (CPU)."""
import numpy as np

import pyoracle as po

E0, NU = 1.0, 0.3
PAR = np.array([E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))])


def test_jacobian_is_derivative_of_function():
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=1, bs=3)
    g = np.random.default_rng(0).uniform(-0.05, 0.05, o.n * 3)
    d = np.random.default_rng(1).uniform(-1, 1, o.n * 3)
    h = 1e-6
    fd = (o.apply(g + h * d, kind=4, param=PAR) - o.apply(g - h * d, kind=4, param=PAR)) / (2 * h)
    jd = o.apply(d, kind=5, qdata=o.elast_state(g), param=PAR)
    assert np.linalg.norm(fd - jd) <= 1e-8 * np.linalg.norm(jd)


def test_identity_state_is_linear_elasticity():
    o = po.FS(3, 4, 3, degree=2, perturb=0.1, seed=2, bs=3)
    d = np.random.default_rng(3).uniform(-1, 1, o.n * 3)
    F0 = o.elast_state(np.zeros(o.n * 3))
    assert np.all(F0.reshape(-1, 9)[:, [0, 4, 8]] == 1.0)
    np.testing.assert_array_equal(o.apply(d, kind=5, qdata=F0, param=PAR), o.apply(d, kind=2, param=PAR))
    assert np.all(o.apply(np.zeros(o.n * 3), kind=4, param=PAR) == 0)
