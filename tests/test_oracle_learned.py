"""The U-Net oracle's gradient is the derivative of its loss (central differences, float64)."""
import numpy as np

import unet_oracle as uo


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = (7, 6, 7)
    w = np.concatenate([np.concatenate([rng.standard_normal(co * ci * 27) * np.sqrt(2.0 / (ci * 27)),
                                        rng.standard_normal(co) * 0.1]) for _, ci, co, _, _ in uo.LAYERS])
    x = rng.standard_normal((2, 2) + dims)
    t = rng.standard_normal((2, 1) + dims)
    mask = np.zeros(dims, bool)
    mask[1:-1, 1:-1, 1:-1] = True
    loss, g, _ = uo.loss_grad(w, x, t, mask)
    # probe parameters of every layer (weights and biases)
    idx, o = [], 0
    for _, ci, co, _, _ in uo.LAYERS:
        idx += [o + int(rng.integers(co * ci * 27)), o + co * ci * 27 + int(rng.integers(co))]
        o += co * ci * 27 + co
    h = 1e-6
    for i in idx:
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (uo.loss_grad(wp, x, t, mask)[0] - uo.loss_grad(wm, x, t, mask)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-3 * np.abs(g).max()), (i, fd, g[i])


def test_interpolation_adjoint_and_shapes():
    rng = np.random.default_rng(1)
    c = rng.standard_normal((1, 3, 4, 5, 3))
    f = rng.standard_normal((1, 3, 7, 9, 5))
    assert abs((uo.up(c, (7, 9, 5)) * f).sum() - (c * uo.up_bwd(f, (4, 5, 3))).sum()) < 1e-12
    assert uo.coarsen((65, 65, 65)) == (33, 33, 33) and uo.coarsen((33, 33, 33)) == (17, 17, 17)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159], np.float32)
    r = uo.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert abs(r[3] - -3.140625) < 1e-7
