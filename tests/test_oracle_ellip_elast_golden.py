"""The oracle's p-Laplacian and St. Venant-Kirchhoff paths pinned to the reference's own outputs for its ellip and
elast test targets (src/fs/tests/CMakeLists.txt:49-58; expected output src/fs/tests/refout/ellip-e0-*.refout and
elast-e0-b3-g01.refout, extracted into tests/golden/ by make_golden.py): exact solution 0 of each program on the
default block mesh (5^3 vertices on [-1,1]^3, src/fs/mesh/interface/genblock.c:169) with Dirichlet values on all
walls (sets 100, 200, 300).

  ellip-e0-b{1,3}-p16, -b3-p14: u = cos(a x) exp(b y) sin(c z), (a, b, c) = (1.6, 1.7, 1.8) (ellip.c:42-57), the
    p-Laplacian with eps = 1 (ellip.c:153-161) at p = 1.6 / 1.4, degree 1 or 3;
  ellip-e0-b3-p17-lam1-sse: the same solution with (a, b, c) = (1, 1, 1) (ellip.c:199), p = 1.7, degree 3 and the
    Bratu term lambda e^u with lambda = 1 (ellip.c:341, 363, 375), which the forcing does not include (the discrete
    solution then differs from the exact one by about 0.4);
  elast-e0-b3-g01: ElastExact_0 (elastexact.py:74-79), (a, b, c) = (0.98, 1.01, 1.01), E = 1, nu = 0.3
    (elast.c:91-96, 99-110), degree 3.

The forcing of each is the strong residual of the program's weak form, written here with sympy from the exact
solution (ellip.c:42-48: f = -div(eta grad u), eta = (eps^2 + |grad u|^2 / 2)^((p-2)/2); elastexact.py:14-25 with
the conversion of dohpexact.py:115-134: f = -div(F S)). Without a solve: ||F(0)||, the first SNES function norm
(six printed digits). After solving to roundoff (exact Jacobians from the oracle's applies at the stored state,
chord iteration from the interpolant): the interpolation residual and the pointwise solution and gradient error
norms (ellip.c:538-566, 750-757; elast.c:409-438, 539-546; three printed digits)."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

import pyoracle as po
from test_oracle_stokes_golden import BOX, closure_coords, columns

sp = pytest.importorskip("sympy")
HERE = os.path.dirname(os.path.abspath(__file__))
X = sp.symbols("x0:3")


def ellip_exact(a, b, c, pe, eps):
    x, y, z = X
    u = sp.cos(a * x) * sp.exp(b * y) * sp.sin(c * z)
    g = [sp.diff(u, v) for v in X]
    eta = (eps ** 2 + sum(t ** 2 for t in g) / 2) ** ((pe - 2) / 2)
    f = -sum(sp.diff(eta * g[i], X[i]) for i in range(3))
    return sp.lambdify(X, [[u], [f], g], "numpy")


def elast_exact(a, b, c, lam, mu):
    x, y, z = X
    u = sp.Matrix([sp.cos(a * x) * sp.exp(b * y) * z + sp.sin(c * z), sp.sin(a * x) * sp.tanh(b * y) + x * sp.cosh(c * z),
                   sp.exp(a * x) * sp.sinh(b * y) + y * sp.log(1 + (c * z) ** 2)])
    H = u.jacobian(X)
    F = sp.eye(3) + H
    E = (F.T * F - sp.eye(3)) / 2
    P = F * (lam * E.trace() * sp.eye(3) + 2 * mu * E)  # first Piola-Kirchhoff stress
    f = [-sum(sp.diff(P[i, j], X[j]) for j in range(3)) for i in range(3)]
    return sp.lambdify(X, [list(u), f, list(H)], "numpy")


NU = 0.3
LAM, MU = NU / ((1 + NU) * (1 - 2 * NU)), 1 / (2 * (1 + NU))  # ElastSetMaterial (elast.c:91-96), E = 1
CASES = {  # name: (degree, bs, function kind, param, exact)
    "ellip_e0_b1_p16": (1, 1, 6, (1.6, 1.0), lambda: ellip_exact(1.6, 1.7, 1.8, 1.6, 1.0)),
    "ellip_e0_b3_p16": (3, 1, 6, (1.6, 1.0), lambda: ellip_exact(1.6, 1.7, 1.8, 1.6, 1.0)),
    "ellip_e0_b3_p14": (3, 1, 6, (1.4, 1.0), lambda: ellip_exact(1.6, 1.7, 1.8, 1.4, 1.0)),
    "ellip_e0_b3_p17_lam1": (3, 1, 7, (1.7, 1.0, 1.0), lambda: ellip_exact(1.0, 1.0, 1.0, 1.7, 1.0)),
    "elast_e0_b3_g01": (3, 3, 4, (LAM, MU), lambda: elast_exact(0.98, 1.01, 1.01, LAM, MU)),
}


class Problem:
    def __init__(self, degree, bs, kind, param, exact):
        self.bs, self.kind, self.param = bs, kind, param
        self.fs = po.FS(5, 5, 5, degree=degree, box=BOX, perturb=0.0, seed=1, bs=bs, dirichlet_mask=7)
        f = exact()
        Xc = closure_coords(self.fs, degree + 1)
        U = columns(f(*Xc.T)[0], len(Xc))
        self.s = U[:self.fs.n].ravel()
        self.dc = U[self.fs.n:].ravel()
        xq = self.fs.qpt_coords()
        r = f(*xq.T)
        nq = len(xq)
        self.fq = columns(r[1], nq)
        self.ue, self.due = columns(r[0], nq), columns(r[2], nq).reshape(nq, bs, 3)

    def F(self, x):
        return self.fs.function(x, self.kind, self.param, dcache=self.dc, fq=self.fq)

    def qdata(self, x):
        """the Jacobian's store at the state x with the Dirichlet values: [eta, sqrt(-eta') Du] of
        EllipPointwiseComputeStore (ellip.c:333-342), or the deformation gradient I + Du (elast.c:224-225)"""
        u, du, _ = self.fs.eval_points(x, self.dc)
        if self.kind in (6, 7):
            pe, eps = self.param[:2]
            g = du[:, 0, :]
            espg = eps ** 2 + 0.5 * (g ** 2).sum(1)
            eta = espg ** ((pe - 2) / 2)
            st = [eta[:, None], np.sqrt(-(pe - 2) / 2 * eta / espg)[:, None] * g]
            if self.kind == 7:  # lambda e^u, the Bratu term's Jacobian coefficient (ellip.c:341)
                st.append(self.param[2] * np.exp(u[:, :1]))
            return np.concatenate(st, 1).ravel()
        return (np.eye(3)[None] + du).reshape(-1)

    def jacobian(self, x):
        n = self.s.size
        qd = self.qdata(x)
        kind = {6: 1, 7: 8, 4: 5}[self.kind]
        J = np.zeros((n, n))
        e = np.zeros(n)
        for j in range(n):
            e[j] = 1
            J[:, j] = self.fs.apply(e, kind=kind, qdata=qd, param=self.param)
            e[j] = 0
        return J

    def solve(self):
        """chord iteration from the interpolant of the exact solution with the Jacobian there; with the Bratu term the
        discrete solution is far from that interpolant, so Newton steps (Jacobian at the iterate) come first"""
        n = self.s.size
        x = self.s.copy()
        F0 = max(1.0, np.linalg.norm(self.F(np.zeros(n))))
        newton = 6 if self.kind == 7 else 0
        for _ in range(newton):
            x = x - np.linalg.solve(self.jacobian(x), self.F(x))
        lu = sl.lu_factor(self.jacobian(x))
        for _ in range(40):
            Fx = self.F(x)
            if np.linalg.norm(Fx) < 1e-12 * F0:
                break
            x = x - sl.lu_solve(lu, Fx)
        return x

    def norms(self, x):
        d = x - self.s
        n = d.size // self.bs  # dNormsAlgebraicScaled divides by the number of blocks (util.c:155-171)
        out = {"interpolation": np.array([np.abs(d).sum() / n, np.linalg.norm(d) / np.sqrt(n), np.abs(d).max()])}
        uh, duh, jw = self.fs.eval_points(x, self.dc)
        e = self.ue - uh
        out["solution"] = np.array([(np.abs(e).sum(1) * jw).sum(), np.sqrt(((e ** 2).sum(1) * jw).sum()), np.abs(e).max()])
        g = np.sqrt(((self.due - duh) ** 2).sum(2))
        out["gradient"] = np.array([(g * jw[:, None]).sum(), np.sqrt((g ** 2 * jw[:, None]).sum()), g.max()])
        return out


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    g = np.load(os.path.join(HERE, "golden", request.param + ".npz"))
    return request.param, Problem(*CASES[request.param]), {k: g[k] for k in g}


def test_first_function_norm(case):
    name, P, ref = case
    got = np.linalg.norm(P.F(np.zeros_like(P.s)))
    assert abs(got - ref["fnorm0"][0]) < 3e-6 * ref["fnorm0"][0], (name, got)


def test_solution_error_norms(case):
    name, P, ref = case
    got = P.norms(P.solve())
    for key in ("interpolation", "solution", "gradient"):
        np.testing.assert_allclose(got[key], ref[key], rtol=0.006, err_msg=name + " " + key)  # the printed digits


def morph(v, morph, twist, stretch=0.0):
    """the vertex map of ellip.c:173-181 (-morph, -twist, -stretch)"""
    x, y, z = v.T
    return np.stack([np.cos(twist * z) * x + np.sin(twist * z) * y, -np.sin(twist * z) * x + np.cos(twist * z) * y,
                     -1 + (z + 1) * (1 + morph * ((x + 1) ** 2 + (y + 1) ** 2)) + stretch * z], 1)


def test_morphed_mesh_cg_history_and_errors():
    """ellip-morph (src/fs/tests/CMakeLists.txt:55: -morph 1 -twist 0.4, p = 2, exact 0 with a = b = c = 1, degree 3,
    one Newton step solved by CG preconditioned with the LU of the Q1-embedded matrix): on the twisted, non-affine
    mesh the first linear solve's preconditioned residual history (KSPSolve_CG, preconditioned norm) is reproduced
    to the six printed digits through all 20 printed iterations, which pins the matrix-free apply, the Q1-embedded
    assembly with the reference's quirks (the variant without them differs in the fourth digit) and the Dirichlet
    handling; the solution's error norms match the printed ones"""
    import scipy.sparse as ssp
    import scipy.sparse.linalg as sla
    g = np.load(os.path.join(HERE, "golden", "ellip_morph.npz"))
    P = Problem.__new__(Problem)
    P.bs, P.kind, P.param = 1, 6, (2.0, 1.0)
    P.fs = po.FS(5, 5, 5, degree=3, box=BOX, perturb=0.0, seed=1, bs=1, dirichlet_mask=7)
    P.fs.set_vertex_coords(morph(P.fs.vertex_coords(), 1.0, 0.4))
    f = ellip_exact(1.0, 1.0, 1.0, 2.0, 1.0)
    Xc = closure_coords(P.fs, 4)
    U = columns(f(*Xc.T)[0], len(Xc))
    P.s, P.dc = U[:P.fs.n].ravel(), U[P.fs.n:].ravel()
    xq = P.fs.qpt_coords()
    r = f(*xq.T)
    P.fq = columns(r[1], len(xq))
    P.ue, P.due = columns(r[0], len(xq)), columns(r[2], len(xq)).reshape(-1, 1, 3)
    n = P.fs.n
    b = -P.F(np.zeros(n))
    lus = {}
    for quirk in (1, 0):
        rp, ci, val = P.fs.q1_assemble(kind=0, quirk=quirk)
        lus[quirk] = sla.splu(ssp.csr_matrix((val, ci, rp), shape=(n, n)).tocsc())
    ref = g["ksp_first_solve"]
    assert abs(np.linalg.norm(lus[0].solve(b)) - ref[0]) > 1e-4 * ref[0]  # the quirk matters at this precision
    lu = lus[1]
    x, rr = np.zeros(n), b.copy()
    z = lu.solve(rr)
    norms = [np.linalg.norm(z)]
    beta = z @ rr
    p = z.copy()
    for it in range(200):
        w = P.fs.apply(p, kind=0)
        a = beta / (p @ w)
        x += a * p
        rr -= a * w
        z = lu.solve(rr)
        norms.append(np.linalg.norm(z))
        if norms[-1] < 1e-13 * norms[0]:
            break
        bnew = z @ rr
        p = z + (bnew / beta) * p
        beta = bnew
    np.testing.assert_allclose(norms[:len(ref)], ref, rtol=6e-6)
    got = P.norms(x)
    for key in ("interpolation", "solution", "gradient"):
        np.testing.assert_allclose(got[key], g[key], rtol=0.006, err_msg=key)


def ellip_exact3(a, b, c, pe, eps):
    """exact solution 3 of ellip.c:91-104, u = a x^3 + b y^2 z + c (1 - z^2) x, with its p-Laplacian forcing"""
    x, y, z = X
    u = a * x ** 3 + b * y ** 2 * z + c * (1 - z ** 2) * x
    g = [sp.diff(u, v) for v in X]
    eta = (eps ** 2 + sum(t ** 2 for t in g) / 2) ** ((pe - 2) / 2)
    f = -sum(sp.diff(eta * g[i], X[i]) for i in range(3))
    return sp.lambdify(X, [[u], [f], g], "numpy")


def test_morphed_mesh_newton_step():
    """ellip-morph-qfast (src/fs/tests/CMakeLists.txt:56: -morph 0.5 -twist 0.1, p = 1.9, exact 3, one Newton step
    with the Jacobian assembled on the FAST rule, so that Richardson with its LU converges in one iteration): the
    Newton step's norm ||J(0)^-1 F(0)|| (the printed first preconditioned residual), and after the step the
    algebraic residual ||F(x1)|| (scaled norms), the interpolation residual and the error norms, all at a state far
    from the solution (the Jacobian at the Dirichlet lift)"""
    g = np.load(os.path.join(HERE, "golden", "ellip_morph_qfast.npz"))
    P = Problem.__new__(Problem)
    P.bs, P.kind, P.param = 1, 6, (1.9, 1.0)
    P.fs = po.FS(5, 5, 5, degree=3, box=BOX, perturb=0.0, seed=1, bs=1, dirichlet_mask=7)
    P.fs.set_vertex_coords(morph(P.fs.vertex_coords(), 0.5, 0.1))
    f = ellip_exact3(1.0, 1.0, 1.0, 1.9, 1.0)
    Xc = closure_coords(P.fs, 4)
    U = columns(f(*Xc.T)[0], len(Xc))
    P.s, P.dc = U[:P.fs.n].ravel(), U[P.fs.n:].ravel()
    xq = P.fs.qpt_coords()
    r = f(*xq.T)
    P.fq = columns(r[1], len(xq))
    P.ue, P.due = columns(r[0], len(xq)), columns(r[2], len(xq)).reshape(-1, 1, 3)
    n = P.fs.n
    x0 = np.zeros(n)
    F0 = P.F(x0)
    qd = P.qdata(x0)
    J = np.zeros((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = 1
        J[:, j] = P.fs.apply(e, kind=1, qdata=qd, param=P.param)
        e[j] = 0
    dx = -np.linalg.solve(J, F0)
    assert abs(np.linalg.norm(dx) - g["ksp_first_solve"][0]) < 6e-6 * g["ksp_first_solve"][0]
    x1 = x0 + dx
    F1 = P.F(x1)
    alg = np.array([np.abs(F1).sum() / n, np.linalg.norm(F1) / np.sqrt(n), np.abs(F1).max()])
    np.testing.assert_allclose(alg, g["algebraic"], rtol=0.006)
    got = P.norms(x1)
    for key in ("interpolation", "solution", "gradient"):
        np.testing.assert_allclose(got[key], g[key], rtol=0.006, err_msg=key)


def gmres_history(apply, prec, b, steps):
    """left-preconditioned GMRES residual norms ||B (b - A x_k)|| over the first steps Arnoldi steps (KSPGMRES with
    the preconditioned norm, zero initial guess; the minimal residual of each Krylov space, computed here by
    least squares on the Arnoldi relation with twice-orthogonalised vectors)"""
    r0 = prec(b)
    beta = np.linalg.norm(r0)
    V, H, norms = [r0 / beta], np.zeros((steps + 1, steps)), [beta]
    for k in range(steps):
        w = prec(apply(V[k]))
        for _ in range(2):
            for j in range(k + 1):
                c = V[j] @ w
                H[j, k] += c
                w = w - c * V[j]
        H[k + 1, k] = np.linalg.norm(w)
        V.append(w / H[k + 1, k])
        e1 = np.zeros(k + 2)
        e1[0] = beta
        y = np.linalg.lstsq(H[:k + 2, :k + 1], e1, rcond=None)[0]
        norms.append(np.linalg.norm(e1 - H[:k + 2, :k + 1] @ y))
    return np.array(norms)


@pytest.mark.parametrize("name", ["ellip_e0_b1_p16", "ellip_e0_b3_p16", "ellip_e0_b3_p14"])
def test_first_newton_linear_solve_history(name):
    """the first Newton step's linear solve of the ellip targets (GMRES preconditioned with the LU of the Q1-embedded
    p-Laplacian Jacobian, EllipJacobian ellip.c:474-536, at the state zero with the exact Dirichlet values; the
    operator the matrix-free Jacobian there): the printed preconditioned residual norms, to six digits"""
    import scipy.sparse as ssp
    import scipy.sparse.linalg as sla
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    P = Problem(*CASES[name])
    n = P.fs.n
    x0 = np.zeros(n)
    F0 = P.F(x0)
    rp, ci, val = P.fs.q1_assemble(kind=1, param=P.param, quirk=1, state=x0, state_dcache=P.dc)
    lu = sla.splu(ssp.csr_matrix((val, ci, rp), shape=(n, n)).tocsc())
    qd = P.qdata(x0)
    ref = g["ksp_first_solve"]
    got = gmres_history(lambda v: P.fs.apply(v, kind=1, qdata=qd, param=P.param), lu.solve, -F0, min(len(ref) - 1, n - 1))
    np.testing.assert_allclose(got[:len(ref)], ref[:len(got)], rtol=6e-6)
