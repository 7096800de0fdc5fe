"""GPU: the reference's projection program (src/fs/tests/ex1.c, the fs-mf-projection-* / fs-mf-op-proj-1 targets) on its
hand-built two-hex mesh (dMeshCreateFromConnectivity), through the product's device expand / restrict and batched
dRulesetIterator, against the printed numbers: useFS's sums, the first SNES function norm (the projection residual at
zero) and, after solving the projection, the pointwise value and gradient residual norms (ProjResidualNorms,
ex1.c:484-530); fs-mf-projection-v3 prints the same numbers as -v1. The operator apply on the hand-built meshes of
ex1.c and fsex4.c against the oracle's (its own mesh from the same entities) at 1e-12."""
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FAST, SPARSE = 0, 1


def gold(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def ex1_space(degree):
    hm = gold("hex_meshes")
    mesh = dg.Mesh(hm["ex1_vtx_parametric"], hm["ex1_econn"], hm["ex1_fconn"], hm["ex1_rconn"])
    return dg.FS(None, degree=degree, dirichlet=(), mesh=mesh)


def exact0(x, a, b, c):
    """exact_0_function / exact_0_gradient of ex1.c:34-48"""
    X, Y, Z = x[:, 0], x[:, 1], x[:, 2]
    f = torch.sin(X) * torch.cosh(b * Y) + torch.cos(a * X) * torch.exp(Y) + torch.sinh(Y) * torch.tanh(c * Z)
    df = torch.stack([torch.cos(X) * torch.cosh(b * Y) - a * torch.sin(a * X) * torch.exp(Y),
                      torch.sin(X) * b * torch.sinh(b * Y) + torch.cos(a * X) * torch.exp(Y) + torch.cosh(Y) * torch.tanh(c * Z),
                      torch.sinh(Y) * c * (1.0 - torch.tanh(c * Z) ** 2)], dim=1)
    return f, df


def residual(it, fs, u, freq):
    """ProjResidual3 (ex1.c:398-427): F(u) = int phi (u - f) over the ruleset"""
    it.start(u)
    q = it.get()
    f, _ = exact0(q["x"], *freq)
    q["v"][:, 0] = (q["u"][:, 0] - f) * q["jw"]
    it.commit(use_v=True, use_dv=False)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    it.finish(y)
    return y


@pytest.mark.parametrize("name,degree,method,freq", [("fs_mf_projection_v1", 5, FAST, (1.0, 1.0, 1.0)),
                                                     ("fs_mf_projection_v3_sparse", 5, SPARSE, (1.0, 1.0, 1.0)),
                                                     ("fs_mf_op_proj_1", 6, FAST, (2.0, 2.0, 2.0))])
def test_ex1_projection(name, degree, method, freq):
    g = gold(name)
    fs = ex1_space(degree)
    assert [fs.nexp, fs.n] == list(g["sizes"])
    # useFS (ex1.c:199-238): x = 1 on the expanded nodes, g = E^T x, y = E g
    x = torch.ones(fs.nexp, dtype=torch.float64, device="cuda")
    gv = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    fs.expanded_to_global(x, gv)
    y = torch.zeros_like(x)
    fs.global_to_expanded(gv, y)
    sums = [x.sum().item(), gv.sum().item(), y.sum().item()]
    np.testing.assert_allclose(sums, g["sums"], rtol=1e-14)
    # the first SNES function norm: ||F(0)||
    it = dg.RulesetIterator(fs, method)
    zero = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    F0 = residual(it, fs, zero, freq)
    np.testing.assert_allclose(torch.linalg.norm(F0).item(), g["snes"][0], rtol=2e-6)
    # the projection: M u = -F(0) with M u = F(u) - F(0), conjugate gradients to 1e-13
    b = -F0
    u = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rr = torch.dot(r, r)
    for _ in range(4 * fs.n):
        Mp = residual(it, fs, p, freq) - F0
        alpha = rr / torch.dot(p, Mp)
        u += alpha * p
        r -= alpha * Mp
        rr_new = torch.dot(r, r)
        if rr_new.sqrt().item() <= 1e-13 * torch.linalg.norm(b).item():
            break
        p = r + (rr_new / rr) * p
        rr = rr_new
    assert torch.linalg.norm(residual(it, fs, u, freq)).item() < 1e-11  # the reference's SNES stopping norm
    # ProjResidualNorms: 1-, 2- and sup-norms of u - f and of |grad u - grad f|^2 over the ruleset
    it.start(u)
    q = it.get()
    f, df = exact0(q["x"], *freq)
    rv = (q["u"][:, 0] - f).abs()
    gr = ((q["du"][:, 0, :] - df) ** 2).sum(dim=1)
    jw = q["jw"]
    pw = [(rv * jw).sum().item(), torch.sqrt((rv ** 2 * jw).sum()).item(), rv.max().item()]
    gw = [(gr * jw).sum().item(), torch.sqrt((gr ** 2 * jw).sum()).item(), gr.max().item()]
    np.testing.assert_allclose(pw, g["pointwise"], rtol=6e-3)
    np.testing.assert_allclose(gw, g["gradient"], rtol=6e-3)


@pytest.mark.parametrize("prefix,vtx", [("ex1_", "ex1_vtx_parametric"), ("fsex4_", "fsex4_vtx")])
def test_operator_apply_against_the_oracle(prefix, vtx):
    """EllipShellMatMult / ElastShellMatMult on meshes given by their entities (no boundary sets): diffusion at
    degrees 1, 3, 6, 8 and with per-element degrees 2..8 (the hp form), linear elasticity at degree 3, each against
    the oracle's apply of the same input at 1e-12"""
    hm = gold("hex_meshes")
    conn = (hm[vtx], hm[prefix + "econn"], hm[prefix + "fconn"], hm[prefix + "rconn"])
    mesh = dg.Mesh(*conn)
    rng = np.random.default_rng(5)
    nr = len(conn[3]) // 8

    def check(fs, o, op, kind=0, param=None):
        x = rng.uniform(-1, 1, fs.n * fs.bs)
        y = torch.zeros(fs.n * fs.bs, dtype=torch.float64, device="cuda")
        op.mult(torch.as_tensor(x, device="cuda"), y)
        torch.cuda.synchronize()
        ref = o.apply(x, kind=kind, param=param)
        err = np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err < 1e-12, err

    for degree in (1, 3, 6, 8):
        fs = dg.FS(None, degree=degree, dirichlet=(), mesh=mesh)
        check(fs, po.FS(0, 0, 0, degree=degree, conn=conn), fs.operator())
    ed = rng.integers(2, 9, size=nr).astype(np.int32)
    fs = dg.FS(None, degree=8, dirichlet=(), mesh=mesh, elem_degree=ed)
    check(fs, po.FS(0, 0, 0, degree=8, elem_degree=ed, conn=conn), fs.operator())
    E0, NU = 1.0, 0.3
    fs = dg.FS(None, degree=3, bs=3, dirichlet=(), mesh=mesh)
    check(fs, po.FS(0, 0, 0, degree=3, bs=3, conn=conn), fs.operator(dg.dOP_ELASTICITY, param=(E0, NU)), kind=2,
          param=np.array([E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))]))
