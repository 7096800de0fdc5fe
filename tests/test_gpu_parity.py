"""GPU parity: the product's CUDA path (through the C ABI) against the CPU oracle on identical seeded
meshes and fields. Integer maps bit-exact; FP64 applies within 1e-12 relative."""
import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-12


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def rel_err(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def _built():
    import os, subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


CASES = [((3, 3, 3), 1), ((4, 3, 5), 2), ((4, 4, 4), 3), ((5, 4, 4), 4), ((3, 4, 3), 5), ((3, 3, 3), 6), ((3, 3, 2), 7),
         ((2, 3, 3), 8)]


@pytest.mark.parametrize("npoints,degree", CASES)
def test_expand_restrict(npoints, degree):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=3)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=3)
    em, xs = fs.emap()
    np.testing.assert_array_equal(em, o.emap())
    rng = np.random.default_rng(0)
    g = rng.standard_normal(fs.n)
    x = torch.zeros(fs.nexp, dtype=torch.float64, device="cuda")
    fs.global_to_expanded(dev(g), x)
    np.testing.assert_array_equal(host(x), o.global_to_expanded(g))
    xe = rng.standard_normal(fs.nexp)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    fs.expanded_to_global(dev(xe), y)
    np.testing.assert_array_equal(host(y), o.expanded_to_global(xe))  # same summation order as E^T


def test_inhomogeneous_expand():
    fs = dg.FS((4, 4, 3), degree=3, perturb=0.0)
    o = po.FS(4, 4, 3, degree=3, perturb=0.0)
    rng = np.random.default_rng(1)
    cl = rng.standard_normal(fs.nc)
    fs.dirichlet_commit(dev(cl))
    x = torch.zeros(fs.nexp, dtype=torch.float64, device="cuda")
    fs.global_to_expanded(dev(cl[:fs.n]), x, inhomogeneous=True)
    np.testing.assert_array_equal(host(x), o.global_to_expanded(cl[:fs.n], dcache=cl[fs.n:]))


@pytest.mark.parametrize("npoints,degree", CASES)
def test_diffusion_apply_fp64(npoints, degree):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=5)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=5)
    op = fs.operator(dg.dOP_DIFFUSION)
    rng = np.random.default_rng(2)
    g = rng.uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(dev(g), y)
    yo = o.apply(g)
    assert rel_err(host(y), yo) < RTOL_FP64


def test_diffusion_apply_with_coefficient():
    fs = dg.FS((5, 5, 5), degree=4, perturb=0.1, seed=7)
    o = po.FS(5, 5, 5, degree=4, perturb=0.1, seed=7)
    nq, _ = o.num_qpts()
    assert nq == fs.nq
    grf = dg.grf_create(32, 2.0, 0.1, 9)
    kq = torch.zeros(fs.nq, dtype=torch.float64, device="cuda")
    fs.lognormal(grf, kq)
    xq = o.qpt_coords()
    ko = np.exp([po.grf_eval(grf, x) for x in xq])
    assert rel_err(host(kq), ko) < 1e-13
    op = fs.operator(dg.dOP_DIFFUSION)
    op.set_qdata(kq)
    g = np.random.default_rng(3).uniform(-1, 1, fs.n)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(dev(g), y)
    assert rel_err(host(y), o.apply(g, qdata=host(kq))) < RTOL_FP64


def test_apply_deterministic_and_host_form():
    fs = dg.FS((6, 6, 6), degree=4, perturb=0.1, seed=2)
    op = fs.operator()
    g = np.random.default_rng(4).uniform(-1, 1, fs.n)
    y1 = torch.zeros(fs.n, dtype=torch.float64, device="cuda"); y2 = torch.zeros_like(y1)
    op.mult(dev(g), y1)
    op.mult(dev(g), y2)
    assert torch.equal(y1, y2)
    yh = np.zeros(fs.n)
    op.mult_host(np.ascontiguousarray(g), yh)
    np.testing.assert_array_equal(yh, host(y1))


@pytest.mark.parametrize("hp", [False, True])
def test_host_form_with_overlapped_copies(hp):
    """spaces large enough for the chunked restriction whose blocks are copied back while the next is restricted:
    bit-identical to the device apply (uniform diffusion, and hp elasticity in the graph form)"""
    if hp:
        ed = np.random.default_rng(8).integers(2, 9, size=12 ** 3).astype(np.int32)
        fs = dg.FS((13, 13, 13), degree=4, perturb=0.1, seed=3, bs=3, elem_degree=ed)
        op = fs.operator(dg.dOP_ELASTICITY, param=(1.0, 0.3))
        op.set_launch(dg.dLAUNCH_GRAPH)
    else:
        fs = dg.FS((25, 25, 25), degree=4, perturb=0.1, seed=3)
        op = fs.operator()
    N = fs.n * fs.bs
    assert N >= 4 * 65536
    g = np.random.default_rng(9).uniform(-1, 1, N)
    y = torch.zeros(N, dtype=torch.float64, device="cuda")
    for _ in range(2):
        op.mult(dev(g), y)
    yh = np.zeros(N)
    for _ in range(2):
        op.mult_host(np.ascontiguousarray(g), yh)
    np.testing.assert_array_equal(yh, host(y))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 6])
@pytest.mark.parametrize("quirk", [1, 0])
def test_q1_assembly(degree, quirk):
    npoints = (4, 3, 4)
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=11)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=11)
    J = fs.matrix()
    J.assemble(quirk=quirk)
    rp, col, val = J.csr_host()
    orp, ocol, oval = o.q1_assemble(quirk=quirk)
    np.testing.assert_array_equal(rp, orp)  # bit-exact sparsity
    np.testing.assert_array_equal(col, ocol)
    assert rel_err(val, oval) < RTOL_FP64


def test_q1_assembly_lognormal():
    fs = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=12)
    o = po.FS(4, 4, 4, degree=3, perturb=0.1, seed=12)
    grf = dg.grf_create(16, 2.0, 0.1, 5)
    J = fs.matrix()
    J.assemble(grf=grf)
    _, _, val = J.csr_host()
    _, _, oval = o.q1_assemble(grf=grf)
    assert rel_err(val, oval) < 1e-12


def test_cg_chebyshev_q1_reaches_rtol():
    """config-1 shape at reduced size: Poisson, perturbed mesh, p=4, f ~ U[-1,1], CG + Q1 Chebyshev-Jacobi."""
    fs = dg.FS((5, 5, 5), degree=4, perturb=0.1, seed=1)
    o = po.FS(5, 5, 5, degree=4, perturb=0.1, seed=1)
    op = fs.operator()
    J = fs.matrix()
    J.assemble()
    ksp = dg.KSP(op, J, pc=dg.dPC_CHEBYSHEV_Q1, cheb_degree=3)
    b = np.random.default_rng(6).uniform(-1, 1, fs.n)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    its, rn = ksp.solve(dev(b), x, rtol=1e-8, maxit=500)
    assert rn <= 1e-8
    r = b - o.apply(host(x))  # true residual with the oracle's own apply
    assert np.linalg.norm(r) <= 1.05e-8 * np.linalg.norm(b)
    _, its_o, _ = o.cg_solve(b, o.q1_assemble(), rtol=1e-8)
    assert abs(its - its_o) <= 2


INTERP, INTERP_T, GRAD, GRAD_T = 40001, 40002, 40003, 40004


# (6, 3, 22) and (8, 3, 30): 12 and 16 points per direction, too many for all three components' buffers in shared
# memory at once, so the kernel runs one component per pass
@pytest.mark.parametrize("degree,D,order", [(1, 1, None), (3, 1, None), (4, 3, None), (7, 1, None), (8, 3, None),
                                            (6, 3, 22), (8, 3, 30)])
def test_efs_apply_batched(degree, D, order):
    order = order or 2 * degree
    jac = dg.Jacobi()
    efs = jac.efs(degree, rule_order=[order] * 3)
    P, Q = efs.P, efs.Q
    nb, nq, ne = int(np.prod(P)), int(np.prod(Q)), 5
    rng = np.random.default_rng(degree)
    x, _ = po.rule_1d(0, 0, order)
    assert Q == [len(x)] * 3
    interp, deriv, _, _ = po.tensor_basis(degree + 1, x)
    jinv = rng.standard_normal((ne, nq, 9))
    for amode, nin, nout in [(INTERP, nb * D, nq * D), (GRAD, nb * D, nq * D * 3), (INTERP_T, nq * D, nb * D), (GRAD_T, nq * D * 3, nb * D)]:
        xin = rng.standard_normal((ne, nin))
        out = torch.zeros(ne * nout, dtype=torch.float64, device="cuda")
        efs.apply(ne, dev(jinv), D, dev(xin), out, amode)
        got = host(out).reshape(ne, nout)
        for e in range(ne):
            ref = po.efs_apply_hex([degree + 1] * 3, [len(x)] * 3, [interp] * 3, [deriv] * 3, jinv[e].ravel(), D, xin[e], amode)
            assert rel_err(got[e], ref) < 1e-13, amode


def test_negative_jacobian_is_an_error():
    fs = dg.FS((3, 3, 3), degree=2, box=(1, 0, 0, 1, 0, 1), perturb=0.0)  # mirrored box: det J < 0
    op = fs.operator()
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DohpError, match="Negative Jacobian"):
        op.mult(x, torch.zeros_like(x))


def _poisson_setup(npoints=(6, 6, 6), degree=4, seed=1):
    fs = dg.FS(npoints, degree=degree, perturb=0.1, seed=seed)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=seed)
    op = fs.operator()
    J = fs.matrix()
    J.assemble()
    b = np.random.default_rng(seed).uniform(-1, 1, fs.n)
    return fs, o, op, J, b


def test_fp32_apply_accuracy():
    fs, o, op, _, b = _poisson_setup()
    op.set_precision(dg.dPREC_FP32)
    y = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    op.mult(dev(b), y)
    err = rel_err(host(y), o.apply(b))
    assert 1e-9 < err < 1e-5, err  # FP32 element arithmetic, FP64 restriction


@pytest.mark.parametrize("inner", [0, 1])
def test_fgmres_reaches_rtol(inner):
    """FGMRES(30) with Q1 Chebyshev-Jacobi; inner=1: FP32 operator applies and FP32 preconditioner inside
    each cycle, FP64 residual at every restart and FP64 orthogonalisation (mixed precision)."""
    fs, o, op, J, b = _poisson_setup()
    ksp = dg.KSP(op, J, ksp_type=dg.dKSP_FGMRES, pc=dg.dPC_CHEBYSHEV_Q1, cheb_degree=3, inner_prec=inner, restart=30)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    its, rn = ksp.solve(dev(b), x, rtol=1e-8, maxit=400)
    assert rn <= 1e-8
    r = b - o.apply(host(x))
    assert np.linalg.norm(r) <= 1.05e-8 * np.linalg.norm(b)


def test_fgmres_deterministic():
    fs, o, op, J, b = _poisson_setup((5, 5, 5), 3)
    xs = []
    for _ in range(2):
        ksp = dg.KSP(op, J, ksp_type=dg.dKSP_FGMRES, inner_prec=1)
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        ksp.solve(dev(b), x, rtol=1e-8)
        xs.append(host(x))
    np.testing.assert_array_equal(xs[0], xs[1])
