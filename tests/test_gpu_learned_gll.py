"""Learned correction on the GLL lattice (the lattice of the Q1-embedded matrix): the injection transfer operators
against an independent construction from the oracle's E map, the network on the whole lattice against the numpy
oracle, training windows that are exact windows of the whole-lattice pairs, and a trained window network inside
FGMRES (the FP64 true residual reaches the tolerance; the correction is kept or dropped by the restart test)."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po
import unet_oracle as uo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GLL = dg.LEARNED_GRID_GLL


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def rounded(w):
    out, o = np.asarray(w, np.float64).copy(), 0
    for _, ci, co, _, _ in uo.LAYERS:
        out[o:o + co * ci * 27] = uo.bf16_round(w[o:o + co * ci * 27])
        o += co * ci * 27 + co
    return out


def test_injection_onto_the_gll_lattice():
    """R r puts every explicit dof at its GLL node ((e p + a, ...) for element e, local node a); P R r = r"""
    M, p = 4, 3
    fs = dg.FS((M + 1,) * 3, degree=p, perturb=0.1, seed=4)
    o = po.FS(M + 1, M + 1, M + 1, degree=p, perturb=0.1, seed=4)
    net = dg.Learned(fs, grid=GLL)
    L = M * p + 1
    assert net.dims == (L, L, L)
    r = np.random.default_rng(2).standard_normal(fs.n)
    rc = torch.zeros(L ** 3, dtype=torch.float64, device="cuda")
    z = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    net.restrict(dev(r), rc)
    net.prolong(rc, z)
    torch.cuda.synchronize()
    rcc = rc.cpu().numpy()
    np.testing.assert_array_equal(z.cpu().numpy(), r)
    # independent: corner 0 of each element from its coordinates on the unit box, local node offsets
    em, xs, ce = o.emap(), o.xstart(), o.coords_expanded()
    ref = np.zeros(L ** 3)
    for e in range(o.nelem):
        c0 = np.rint(ce[e][0] * M).astype(int) * p
        for loc in range(xs[e + 1] - xs[e]):
            d = em[xs[e] + loc]
            if d >= fs.n:
                continue
            a, b, c = loc // (p + 1) ** 2, (loc // (p + 1)) % (p + 1), loc % (p + 1)
            ref[((c0[0] + a) * L + c0[1] + b) * L + c0[2] + c] = r[d]
    np.testing.assert_array_equal(rcc, ref)
    assert np.count_nonzero(rcc) == fs.n


def test_whole_lattice_forward_matches_oracle():
    fs = dg.FS((3, 3, 3), degree=4, seed=1)
    net = dg.Learned(fs, seed=3, grid=GLL)
    assert net.dims == (9, 9, 9)
    x = np.random.default_rng(0).standard_normal((1, 2) + net.dims).astype(np.float32)
    y = torch.zeros((1, 1) + net.dims, dtype=torch.float32, device="cuda")
    net.forward(dev(x), y)
    yo, _ = uo.forward(rounded(net.get_weights()), x.astype(np.float64), net.dims, tc=True)
    assert np.linalg.norm(y.cpu().numpy() - yo) / np.linalg.norm(yo) < 5e-3  # BF16 rounding flips, as the vertex test


def lognormal(ne, field_seed, p=4):
    fs = dg.FS((ne + 1,) * 3, degree=p, perturb=0.1, seed=1)
    grf = dg.grf_create(64, 2.0, 0.1, field_seed)
    kq = torch.empty(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    op = fs.operator()
    op.set_qdata(kq)
    m = fs.matrix()
    m.assemble(grf=grf)
    return fs, op, m, grf


def test_windows_are_windows_of_the_whole_lattice_pairs():
    """the same deterministic CG recorded by a window network and a whole-lattice network: every window pair is
    the whole-lattice pair cut at its origin (origins multiples of 4 inside the lattice)"""
    ne = 4
    fs, op, m, grf = lognormal(ne, 21)
    b = dev(np.random.default_rng(21).uniform(-1, 1, fs.n))
    nets = {}
    for crop in (9, 0):
        net = dg.Learned(fs, seed=5, grid=GLL, crop=crop)
        net.set_field(grf)
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
        assert net.collect(ksp, b, rtol=1e-10, every=2, max_pairs=12) == 12
        nets[crop] = net
    L = net.dims[0]
    seen = set()
    for p in range(12):
        org, wi, wt = nets[9].pair(p)
        o2, fi, ft = nets[0].pair(p)
        assert o2 == (0, 0, 0) and fi.shape == (L,) * 3 and wi.shape == (9, 9, 9)
        assert all(c % 4 == 0 and 0 <= c <= L - 9 for c in org)
        sl = tuple(slice(c, c + 9) for c in org)
        np.testing.assert_array_equal(wi, fi[sl])
        np.testing.assert_array_equal(wt, ft[sl])
        seen.add(org)
    assert len(seen) > 1


def test_window_training_and_fgmres():
    """a network trained on 17^3 windows of a 33^3 GLL lattice, applied to the whole lattice inside FGMRES: the
    loss falls, the FP64 true residual reaches 1e-8 whatever the network does, and the plain preconditioner judges
    the correction (paired trial cycles from the same iterate)"""
    ne = 8
    fs0, _, _, _ = lognormal(ne, 31)
    net = dg.Learned(fs0, seed=7, grid=GLL, crop=17)
    for seed in (31, 32, 33):
        fs, op, m, grf = lognormal(ne, seed)
        net.set_field(grf)
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_CG)
        b = dev(np.random.default_rng(seed).uniform(-1, 1, fs.n))
        net.collect(ksp, b, rtol=1e-10, every=1, max_pairs=80)
    assert net.npairs >= 200
    losses = net.train(epochs=20, batch=8, lr=1e-3, seed=1)
    assert losses[-1] < 0.7 * losses[0]
    fs, op, m, grf = lognormal(ne, 99)
    net.set_field(grf)
    b = dev(np.random.default_rng(99).uniform(-1, 1, fs.n))
    res = {}
    for name, n in (("plain", None), ("learned", net)):
        ksp = dg.KSP(op, m, ksp_type=dg.dKSP_FGMRES, restart=30)
        if n is not None:
            ksp.set_learned(n)
        x = torch.zeros_like(b)
        its, _ = ksp.solve(b, x, rtol=1e-8, maxit=3000)
        r = torch.empty_like(x)
        op.mult(x, r)
        res[name] = (its, float(torch.linalg.norm(b - r) / torch.linalg.norm(b)), ksp.stats())
    assert res["plain"][1] <= 1.01e-8 and res["learned"][1] <= 1.01e-8
    assert net.stats()[0] > 0 and net.stats()[1] == 0
    _, rejects, active = res["learned"][2]
    if active:  # kept: it beat its plain trial cycles; the trials' extra cycles are the price of the judgement
        assert res["learned"][0] <= res["plain"][0] + 2 * 30, res
    else:  # dropped after its paired trials against plain cycles, which keep the better iterate: at most the two
        # corrected trial cycles (and a partial cycle) more than the plain solve
        assert rejects >= 1 and res["learned"][0] <= res["plain"][0] + 3 * 30, res


def test_refusals():
    fs = dg.FS((5, 5, 5), degree=2, seed=1)
    for grid, crop in ((GLL, 8), (GLL, 5), (dg.LEARNED_GRID_VERTEX, 9), (7, 0)):
        with pytest.raises(dg.DohpError):
            dg.Learned(fs, grid=grid, crop=crop)
