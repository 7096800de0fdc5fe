"""CPU oracle (test infrastructure only) for the learned coarse correction's network: the same 3-level
3-D U-Net as dohp_gb300/csrc/unet.cu, restated in numpy float64 -- forward, mean-squared-error loss over
interior vertices, and the full parameter gradient by the chain rule. There is no reference source for this
part (the reference has no learned component); the restatement is pinned by finite differences
(tests/test_oracle_learned.py) and checks the GPU kernels (tests/test_gpu_learned.py).

Layout: activations [B][C][X][Y][Z] (Z fastest); weights per layer W[co][ci][3][3][3] then bias[co], layers in
the order C1A C1B D1 C2A D2 C3A C3B U2 C2B U1 C1C OUT; convolutions pad 1, stride 1 or 2; up blocks
convolve on the coarse grid, interpolate trilinearly (vertex-centred, corners aligned) and add the skip.
"""
import numpy as np

LAYERS = [("C1A", 2, 16, 1, 0), ("C1B", 16, 16, 1, 0), ("D1", 16, 32, 2, 0), ("C2A", 32, 32, 1, 1),
          ("D2", 32, 64, 2, 1), ("C3A", 64, 64, 1, 2), ("C3B", 64, 64, 1, 2), ("U2", 64, 32, 1, 2),
          ("C2B", 32, 32, 1, 1), ("U1", 32, 16, 1, 1), ("C1C", 16, 16, 1, 0), ("OUT", 16, 1, 1, 0)]


def coarsen(d):
    return tuple((v - 1) // 2 + 1 for v in d)


def nparams():
    return sum(co * ci * 27 + co for _, ci, co, _, _ in LAYERS)


def unpack(w):
    """flat parameter vector -> {name: (W [co][ci][27], b [co])}"""
    out, o = {}, 0
    for name, ci, co, _, _ in LAYERS:
        W = w[o:o + co * ci * 27].reshape(co, ci, 27)
        o += co * ci * 27
        out[name] = (W, w[o:o + co])
        o += co
    return out


def bf16_round(a):
    """round float32 values to bfloat16 (nearest even), returned as float32"""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _shifted(xp, a, b, c, s, dout):
    return xp[..., a:a + s * (dout[0] - 1) + 1:s, b:b + s * (dout[1] - 1) + 1:s, c:c + s * (dout[2] - 1) + 1:s]


def conv(x, W, bias, s, dout):
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))
    y = np.zeros((x.shape[0], W.shape[0]) + tuple(dout))
    for t in range(27):
        a, b, c = t // 9, (t // 3) % 3, t % 3
        y += np.einsum("oi,nixyz->noxyz", W[:, :, t], _shifted(xp, a, b, c, s, dout))
    return y + bias[None, :, None, None, None]


def conv_bwd(x, W, gy, s):
    dout = gy.shape[2:]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))
    gxp = np.zeros_like(xp)
    gW = np.zeros_like(W)
    for t in range(27):
        a, b, c = t // 9, (t // 3) % 3, t % 3
        gW[:, :, t] = np.einsum("noxyz,nixyz->oi", gy, _shifted(xp, a, b, c, s, dout))
        _shifted(gxp, a, b, c, s, dout)[...] += np.einsum("oi,noxyz->nixyz", W[:, :, t], gy)
    return gxp[:, :, 1:-1, 1:-1, 1:-1], gW, gy.sum(axis=(0, 2, 3, 4))


def interp_matrix(lf, lc):
    """tent weights of coarse i at fine f, positions f (lc-1)/(lf-1)"""
    M = np.zeros((lf, lc))
    for f in range(lf):
        pos = f * (lc - 1) / (lf - 1) if lc > 1 else 0.0
        for i in range(lc):
            M[f, i] = max(0.0, 1.0 - abs(pos - i)) if lc > 1 else 1.0
    return M


def up(x, df):
    dc = x.shape[2:]
    Ix, Iy, Iz = (interp_matrix(df[k], dc[k]) for k in range(3))
    return np.einsum("fi,gj,hk,ncijk->ncfgh", Ix, Iy, Iz, x)


def up_bwd(g, dc):
    df = g.shape[2:]
    Ix, Iy, Iz = (interp_matrix(df[k], dc[k]) for k in range(3))
    return np.einsum("fi,gj,hk,ncfgh->ncijk", Ix, Iy, Iz, g)


def relu(a):
    return np.maximum(a, 0.0)


# the layers the product runs on the tensor cores when they are enabled (stride 1, 16 or 32 channels in and out):
# their input activations (forward) and incoming gradients (data gradient) are rounded to bf16
TC_LAYERS = {name for name, ci, co, s, _ in LAYERS if s == 1 and ci in (16, 32) and co in (16, 32)}


def _rnd(a, name, tc):
    return bf16_round(a).astype(np.float64) if tc and name in TC_LAYERS else a


def forward(w, x, dims, tc=False):
    """w flat float64 (already bf16-rounded weights), x [B][2][dims] -> (y [B][1][dims], activations); tc: the
    inputs of the tensor-core layers rounded to bf16"""
    P = unpack(np.asarray(w, np.float64))
    d0 = tuple(dims)
    d1 = coarsen(d0)
    d2 = coarsen(d1)
    A = {"X0": np.asarray(x, np.float64)}

    def cv(name, a, s, d):
        return conv(_rnd(a, name, tc), *P[name], s, d)

    A["H1"] = relu(cv("C1A", A["X0"], 1, d0))
    A["A1"] = relu(cv("C1B", A["H1"], 1, d0))
    A["H2"] = relu(cv("D1", A["A1"], 2, d1))
    A["A2"] = relu(cv("C2A", A["H2"], 1, d1))
    A["H3"] = relu(cv("D2", A["A2"], 2, d2))
    A["H3B"] = relu(cv("C3A", A["H3"], 1, d2))
    A["A3"] = relu(cv("C3B", A["H3B"], 1, d2))
    A["W2"] = relu(cv("U2", A["A3"], 1, d2))
    A["S2"] = up(A["W2"], d1) + A["A2"]
    A["B2"] = relu(cv("C2B", A["S2"], 1, d1))
    A["W1"] = relu(cv("U1", A["B2"], 1, d1))
    A["S1"] = up(A["W1"], d0) + A["A1"]
    A["B1"] = relu(cv("C1C", A["S1"], 1, d0))
    A["Y"] = cv("OUT", A["B1"], 1, d0)
    return A["Y"], A


def loss_grad(w, x, t, mask, tc=False):
    """MSE over interior vertices (mask [dims] bool) and its gradient w.r.t. the flat parameters; tc: the
    tensor-core layers' forward inputs, and the activations and incoming gradients of their data and weight
    gradients, rounded to bf16 (their bias gradients sum the unrounded incoming gradients)"""
    dims = x.shape[2:]
    B = x.shape[0]
    nint = int(mask.sum())
    y, A = forward(w, x, dims, tc)
    m = mask[None, None].astype(np.float64)
    d = (y - t) * m
    loss = float((d ** 2).sum() / (B * nint))
    G = {}
    P = unpack(np.asarray(w, np.float64))

    def step(name, xin, g, s):
        gx, gW, gb = conv_bwd(xin, P[name][0], g, s)
        if tc and name in TC_LAYERS:  # data and weight gradients from bf16 operands; the bias gradient from g itself
            gx, gW, _ = conv_bwd(_rnd(xin, name, tc), P[name][0], _rnd(g, name, tc), s)
        G[name] = (gW, gb)
        return gx

    g = 2.0 * d / (B * nint)
    g = step("OUT", A["B1"], g, 1) * (A["B1"] > 0)
    gs1 = step("C1C", A["S1"], g, 1)
    ga1 = gs1.copy()
    g = up_bwd(gs1, A["W1"].shape[2:]) * (A["W1"] > 0)
    g = step("U1", A["B2"], g, 1) * (A["B2"] > 0)
    gs2 = step("C2B", A["S2"], g, 1)
    ga2 = gs2.copy()
    g = up_bwd(gs2, A["W2"].shape[2:]) * (A["W2"] > 0)
    g = step("U2", A["A3"], g, 1) * (A["A3"] > 0)
    g = step("C3B", A["H3B"], g, 1) * (A["H3B"] > 0)
    g = step("C3A", A["H3"], g, 1) * (A["H3"] > 0)
    ga2 = ga2 + step("D2", A["A2"], g, 2)
    g = step("C2A", A["H2"], ga2 * (A["A2"] > 0), 1) * (A["H2"] > 0)
    ga1 = ga1 + step("D1", A["A1"], g, 2)
    g = step("C1B", A["H1"], ga1 * (A["A1"] > 0), 1) * (A["H1"] > 0)
    step("C1A", A["X0"], g, 1)
    flat = np.concatenate([np.concatenate([G[name][0].ravel(), G[name][1]]) for name, *_ in LAYERS])
    return loss, flat, y
