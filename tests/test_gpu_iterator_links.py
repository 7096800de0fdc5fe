"""The reference's multi-link iterator API through the C ABI (include/dohpfs.h:97-128, src/fs/interface/fsrulesetit.c):
dFSGetPreferredQuadratureRuleSet, dFSGetCoordinateFS, dRulesetCreateIterator, dRulesetIteratorAddFS, AddStash /
GetStash, the varargs Start / GetPatchApplied / CommitPatchApplied, HasPatch / NextPatch, GetPatchAssembly and Finish.

* a velocity (bs 3, degree 3) and a pressure (bs 1, degree 2) link on the velocity's ruleset, as the reference's
  Stokes iterator: values and gradients of both links against the oracle's element loop at those points, committed
  integrals against one-link iterators;
* ElastFunction's loop (elast.c:282-309: coordinates, field and a per-point stash in one traversal) driven through
  the varargs calls with the q-function in torch, against dOperatorElasticityFunction, and the stash read back by a
  second traversal (ElastShellMatMult's loop, elast.c:311-341) against dOperatorMult at that state;
* GetPatchAssembly's batched Q1 sub-cell bases against the host dEFSGetExplicitSparse with the element's inverse
  Jacobians."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

E0, NU = 1.0, 0.3
LAM, MU = E0 * NU / ((1 + NU) * (1 - 2 * NU)), E0 / (2 * (1 + NU))
NULL = ctypes.c_void_p(0)


@pytest.fixture(scope="module", autouse=True)
def _built():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    dg.lib()


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


def view(addr, shape):
    return torch.as_tensor(dg._DeviceArray(addr.value if hasattr(addr, "value") else addr, shape), device="cuda")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_iterator(fs, method=dg.FAST, extra=()):
    L = dg.lib()
    rs, cfs, it = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSGetPreferredQuadratureRuleSet(fs.h, ctypes.c_int(method), ctypes.byref(rs)))
    dg.chk(L.dFSGetCoordinateFS(fs.h, ctypes.byref(cfs)))
    dg.chk(L.dRulesetCreateIterator(rs, cfs, ctypes.byref(it)))
    dg.chk(L.dRulesetDestroy(ctypes.byref(rs)))  # the iterator keeps its own reference
    for f in (fs,) + tuple(extra):
        dg.chk(L.dRulesetIteratorAddFS(it, f.h))
    return it


def test_two_field_links_on_one_ruleset():
    L = dg.lib()
    fsu = dg.FS((4, 4, 3), degree=3, perturb=0.1, seed=3, bs=3)
    fsp = dg.FS(None, degree=2, bs=1, dirichlet=(), mesh_of=fsu)
    ou = po.FS(4, 4, 3, degree=3, perturb=0.1, seed=3, bs=3)
    op_ = po.FS(4, 4, 3, degree=2, perturb=0.1, seed=3, bs=1, dirichlet_mask=0)
    rng = np.random.default_rng(5)
    gu, gp = rng.uniform(-1, 1, fsu.n * 3), rng.uniform(-1, 1, fsp.n)
    it = make_iterator(fsu, extra=(fsp,))
    yu = torch.zeros(fsu.n * 3, dtype=torch.float64, device="cuda")
    yp = torch.zeros(fsp.n, dtype=torch.float64, device="cuda")
    xu, xp = dev(gu), dev(gp)
    dg.chk(L.dRulesetIteratorStart(it, NULL, NULL, dg.ptr(xu), ctypes.c_int(dg.dFS_HOMOGENEOUS), dg.ptr(yu), ctypes.c_int(0),
                                   dg.ptr(xp), ctypes.c_int(dg.dFS_HOMOGENEOUS), dg.ptr(yp), ctypes.c_int(0)))
    assert L.dRulesetIteratorHasPatch(it) == 1
    Q, jw = ctypes.c_int32(), ctypes.c_void_p()
    x, dx = ctypes.c_void_p(), ctypes.c_void_p()
    pu = [ctypes.c_void_p() for _ in range(4)]
    pp = [ctypes.c_void_p() for _ in range(4)]
    dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), ctypes.byref(x), ctypes.byref(dx), NULL, NULL,
                                             *[ctypes.byref(p) for p in pu], *[ctypes.byref(p) for p in pp]))
    n = Q.value
    assert n == fsu.nelem * 4 ** 3  # the velocity's FAST rule: 4 Gauss points per direction
    u, du = view(pu[0], (n, 3)), view(pu[1], (n, 3, 3))
    p, dp = view(pp[0], (n, 1)), view(pp[1], (n, 1, 3))
    # oracle: both spaces evaluated at the velocity's points (degree 3 rule) with their own bases
    uo, duo, jwo = ou.eval_points(gu)
    po_, dpo, _ = op_.eval_points(gp, rule_deg=3)
    torch.cuda.synchronize()
    np.testing.assert_allclose(view(jw, (n,)).cpu().numpy(), jwo, rtol=1e-13)
    np.testing.assert_allclose(u.cpu().numpy(), uo, rtol=0, atol=1e-13)
    np.testing.assert_allclose(du.cpu().numpy(), duo, rtol=0, atol=1e-12)
    np.testing.assert_allclose(p.cpu().numpy(), po_, rtol=0, atol=1e-13)
    np.testing.assert_allclose(dp.cpu().numpy(), dpo, rtol=0, atol=1e-12)
    # a coupled residual: v_u = jw p (momentum), dv_p = jw du[:, 0, :] (continuity-like), committed in one call
    vu, dvp = view(pu[2], (n, 3)), view(pp[3], (n, 1, 3))
    jwt = view(jw, (n,))
    vu.copy_(jwt[:, None] * p.expand(n, 3))
    dvp.copy_(jwt[:, None, None] * du[:, :1, :])
    dg.chk(L.dRulesetIteratorCommitPatchApplied(it, ctypes.c_int(dg.INSERT_VALUES), NULL, NULL, pu[2], NULL, NULL, pp[3]))
    dg.chk(L.dRulesetIteratorNextPatch(it))
    assert L.dRulesetIteratorHasPatch(it) == 0
    dg.chk(L.dRulesetIteratorFinish(it))
    torch.cuda.synchronize()
    # the same integrals by one-link iterators of the oracle: int phi_u . (p, p, p) and int grad q . grad u_x
    Vu = (jwo[:, None] * np.repeat(po_, 3, axis=1)).ravel()
    eu = np.zeros(fsu.n * 3)
    # test functions: y_u[i] = sum_q v(q) . phi_i(q); check through linearity against random directions
    for k in range(3):
        d = np.random.default_rng(10 + k).uniform(-1, 1, fsu.n * 3)
        ud, _, _ = ou.eval_points(d)
        assert abs(d @ yu.cpu().numpy() - (ud.ravel() @ Vu)) < 1e-11 * max(1.0, abs(ud.ravel() @ Vu))
        q = np.random.default_rng(20 + k).uniform(-1, 1, fsp.n)
        _, dq, _ = op_.eval_points(q, rule_deg=3)
        ref = float((jwo[:, None] * dq[:, 0, :] * duo[:, 0, :]).sum())
        assert abs(q @ yp.cpu().numpy() - ref) < 1e-11 * max(1.0, abs(ref))
    del eu
    dg.chk(L.dRulesetIteratorDestroy(ctypes.byref(it)))


def svk_pointwise(du, w, lam, mu):
    """ElastPointwiseFunction (elast.c:256-266) in torch: F = I + Du, E = (F^T F - I)/2, S = lam tr(E) I + 2 mu E,
    dv = w F S; returns (dv, F)"""
    n = du.shape[0]
    I = torch.eye(3, dtype=du.dtype, device=du.device).expand(n, 3, 3)
    F = I + du
    E = 0.5 * (F.transpose(1, 2) @ F - I)
    tr = E.diagonal(dim1=1, dim2=2).sum(1)
    S = lam * tr[:, None, None] * I + 2 * mu * E
    return w[:, None, None] * (F @ S), F, S


def test_elast_function_loop_with_stash_then_shell_mult():
    L = dg.lib()
    fs = dg.FS((4, 4, 4), degree=3, perturb=0.1, seed=2, bs=3)
    rng = np.random.default_rng(2)
    g = rng.uniform(-0.05, 0.05, fs.n * 3)
    it = make_iterator(fs)
    dg.chk(L.dRulesetIteratorAddStash(it, ctypes.c_int32(0), ctypes.c_int32(9 * 8)))  # F per point, as struct ElastStore
    # ElastFunction: Start(it, Coords, INHOMOGENEOUS, NULL, gx, INHOMOGENEOUS, gy, INHOMOGENEOUS)
    xg = dev(g)
    y = torch.zeros_like(xg)
    dg.chk(L.dRulesetIteratorStart(it, NULL, NULL, dg.ptr(xg), ctypes.c_int(dg.dFS_INHOMOGENEOUS), dg.ptr(y), ctypes.c_int(1)))
    Q, jw = ctypes.c_int32(), ctypes.c_void_p()
    x, dx = ctypes.c_void_p(), ctypes.c_void_p()
    p = [ctypes.c_void_p() for _ in range(4)]
    while L.dRulesetIteratorHasPatch(it):
        dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), ctypes.byref(x), ctypes.byref(dx), NULL, NULL,
                                                 *[ctypes.byref(q) for q in p]))
        st = ctypes.c_void_p()
        dg.chk(L.dRulesetIteratorGetStash(it, None, ctypes.byref(st)))
        n = Q.value
        dv, F, _ = svk_pointwise(view(p[1], (n, 3, 3)), view(jw, (n,)), LAM, MU)
        view(p[3], (n, 3, 3)).copy_(dv)
        view(st, (n, 9)).copy_(F.reshape(n, 9))
        dg.chk(L.dRulesetIteratorCommitPatchApplied(it, ctypes.c_int(dg.INSERT_VALUES), NULL, NULL, NULL, p[3]))
        dg.chk(L.dRulesetIteratorNextPatch(it))
    dg.chk(L.dRulesetIteratorFinish(it))
    op = fs.operator(dg.dOP_ELASTICITY, param=(E0, NU))
    yr = torch.zeros_like(y)
    op.elasticity_function(xg, yr)  # also leaves the state of g for the Jacobian
    torch.cuda.synchronize()
    assert rel(y.cpu().numpy(), yr.cpu().numpy()) < 1e-12
    # ElastShellMatMult: a second traversal reads the stash (F at each point) and applies ElastPointwiseJacobian
    d = dev(rng.uniform(-1, 1, fs.n * 3))
    yj = torch.zeros_like(d)
    dg.chk(L.dRulesetIteratorStart(it, NULL, NULL, dg.ptr(d), ctypes.c_int(dg.dFS_HOMOGENEOUS), dg.ptr(yj), ctypes.c_int(0)))
    dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), NULL, NULL, NULL, NULL, *[ctypes.byref(q) for q in p]))
    st = ctypes.c_void_p()
    dg.chk(L.dRulesetIteratorGetStash(it, None, ctypes.byref(st)))
    n = Q.value
    F = view(st, (n, 3, 3))
    dF = view(p[1], (n, 3, 3))
    w = view(jw, (n,))
    I = torch.eye(3, dtype=F.dtype, device=F.device).expand(n, 3, 3)
    E = 0.5 * (F.transpose(1, 2) @ F - I)
    S = LAM * E.diagonal(dim1=1, dim2=2).sum(1)[:, None, None] * I + 2 * MU * E
    dE = 0.5 * (F.transpose(1, 2) @ dF + dF.transpose(1, 2) @ F)
    dS = LAM * dE.diagonal(dim1=1, dim2=2).sum(1)[:, None, None] * I + 2 * MU * dE
    view(p[3], (n, 3, 3)).copy_(w[:, None, None] * (dF @ S + F @ dS))
    dg.chk(L.dRulesetIteratorCommitPatchApplied(it, ctypes.c_int(dg.INSERT_VALUES), NULL, NULL, NULL, p[3]))
    dg.chk(L.dRulesetIteratorNextPatch(it))
    dg.chk(L.dRulesetIteratorFinish(it))
    yo = torch.zeros_like(d)
    op.mult(d, yo)
    torch.cuda.synchronize()
    assert rel(yj.cpu().numpy(), yo.cpu().numpy()) < 1e-12
    # committing an array the iterator did not hand out is an error (the reference forbids moving v / dv)
    other = torch.zeros(n * 9, dtype=torch.float64, device="cuda")
    dg.chk(L.dRulesetIteratorStart(it, NULL, NULL, dg.ptr(d), ctypes.c_int(0), dg.ptr(yj), ctypes.c_int(0)))
    dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), NULL, NULL, NULL, NULL, *[ctypes.byref(q) for q in p]))
    assert L.dRulesetIteratorCommitPatchApplied(it, ctypes.c_int(1), NULL, NULL, NULL, dg.ptr(other)) != 0
    dg.chk(L.dRulesetIteratorFinish(it))
    dg.chk(L.dRulesetIteratorDestroy(ctypes.byref(it)))


def test_patch_assembly_matches_host_explicit_sparse():
    L = dg.lib()
    p = 3
    fs = dg.FS((3, 4, 3), degree=p, perturb=0.1, seed=6)
    it = make_iterator(fs, method=dg.SPARSE)
    dg.chk(L.dRulesetIteratorStart(it, NULL, NULL, NULL, NULL))
    Q, jw = ctypes.c_int32(), ctypes.c_void_p()
    dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL))
    P, rc, bi, bd = ctypes.c_int32(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dRulesetIteratorGetPatchAssembly(it, NULL, NULL, NULL, NULL, ctypes.byref(P), ctypes.byref(rc), ctypes.byref(bi),
                                              ctypes.byref(bd)))
    assert P.value == 8
    ne, npch = fs.nelem, p ** 3
    torch.cuda.synchronize()
    rowcol = torch.as_tensor(dg._DeviceArray(rc.value, (ne * npch * 8 // 2,)), device="cuda").cpu().numpy().view(np.int32)
    interp = view(bi, (ne, npch, 8, 8)).cpu().numpy()
    deriv = view(bd, (ne, npch, 8, 8, 3)).cpu().numpy()
    # the element's inverse Jacobians at its SPARSE points (element-natural), from the coordinate link's gradient
    dx = ctypes.c_void_p()
    dg.chk(L.dRulesetIteratorGetPatchApplied(it, ctypes.byref(Q), ctypes.byref(jw), NULL, ctypes.byref(dx), NULL, NULL, NULL, NULL,
                                             NULL, NULL))
    qe = (2 * p) ** 3
    jinv = np.linalg.inv(view(dx, (ne, qe, 3, 3)).cpu().numpy())
    _, xs = fs.emap()
    efs = fs.jac.efs(p, method=dg.SPARSE)
    r = ctypes.c_void_p()
    dg.chk(L.dEFSGetRule(efs.h, ctypes.byref(r)))
    npc, psz, ind, wt = ctypes.c_int32(), ctypes.c_int32(), ctypes.POINTER(ctypes.c_int32)(), ctypes.POINTER(ctypes.c_double)()
    dg.chk(L.dRuleGetPatches(r, ctypes.byref(npc), ctypes.byref(psz), ctypes.byref(ind), ctypes.byref(wt)))
    assert (npc.value, psz.value) == (npch, 8)
    qidx = np.ctypeslib.as_array(ind, (npch * 8,)).copy()
    for e in range(ne):
        Pn = ctypes.c_int32()
        eidx = np.zeros(npch * 8, np.int32)
        hi, hd = np.zeros(npch * 64), np.zeros(npch * 192)
        cj = np.ascontiguousarray(jinv[e].reshape(-1))
        dg.chk(L.dEFSGetExplicitSparse(efs.h, ctypes.c_int32(npch), ctypes.c_int32(8), dg.ptr(qidx), dg.ptr(cj), ctypes.c_int32(int(xs[e])),
                                       ctypes.byref(Pn), dg.ptr(eidx), dg.ptr(hi), dg.ptr(hd)))
        np.testing.assert_array_equal(rowcol.reshape(ne, npch * 8)[e], eidx)
        np.testing.assert_allclose(interp[e].ravel(), hi, rtol=0, atol=1e-15)
        np.testing.assert_allclose(deriv[e].ravel(), hd, rtol=1e-10, atol=1e-10)
    dg.chk(L.dRulesetIteratorFinish(it))
    dg.chk(L.dRulesetIteratorDestroy(ctypes.byref(it)))
