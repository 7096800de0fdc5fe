"""The oracle's Stokes path pinned to the reference's own outputs for its two Stokes test targets
(src/fs/tests/CMakeLists.txt:62-70; expected output src/fs/tests/refout/stokes-q3q2-{scr,fgmres}.refout, extracted
into tests/golden/ by make_golden.py): the Exact1 manufactured solution (src/fs/tests/stokesexact.py:94-101) on the
default block mesh (5^3 vertices on [-1,1]^3, src/fs/mesh/interface/genblock.c:169), Q3 velocity with Dirichlet
walls (sets 100, 200, 300, stokes.c:114-116) and continuous Q2 pressure (-pressure_codim 1), at the Newtonian
rheology (B = eps = 1, p = 2) and at the power law p = 1.2, eps = 0.1.

Without a solve (six printed digits): ||F(s)|| at the nodal interpolant s of the exact solution, ||J(s) s + F(0)||
and ||F(0)|| (stokes.c:1121-1135; the SNES starts from zero). After solving the discrete system to roundoff (dense
Jacobian from the oracle's applies, bordered by the pressure constant): the interpolation residual and the pointwise
velocity, gradient and pressure error norms (stokes.c:835-885, 1161-1169; three printed digits, and the reference's
solves stop at their tolerances, so the last digit may differ by that)."""
import os

import numpy as np
import pytest
import scipy.linalg as sl

import pyoracle as po

sp = pytest.importorskip("sympy")
HERE = os.path.dirname(os.path.abspath(__file__))
BOX = (-1, 1, -1, 1, -1, 1)


def exact1(B, eps, pe):
    """Exact1 (a = b = c = scale = 1) and its forcing, the strong residual of the weak form
    eta(Du) Dv:Du - q div u - p div v (StokesExact.weak_homogeneous, stokesexact.py:14-21; eta of the power law,
    stokesexact.py:11-13; the weak-to-strong conversion of dohpexact.py:115-134): fu = -div(eta Du) + grad p,
    fp = -div u. Returns numpy functions of (x, y, z) -> [u (3), p, fu (3), fp, du (9, row-major d u_i / d x_j)]."""
    X = sp.symbols("x0:3")
    xx, yy, zz = [sp.pi * s / 2 for s in X]
    u = sp.Matrix([sp.sin(xx) * sp.sin(yy) * sp.sin(zz) / 3, -sp.cos(xx) * sp.cos(yy) * sp.sin(zz) / 3,
                   -2 * sp.cos(xx) * sp.sin(yy) * sp.cos(zz) / 3])
    p = 1 + sp.cos(xx) * sp.sin(yy) * sp.sin(zz)
    du = u.jacobian(X)
    Du = (du + du.T) / 2
    gamma = sum(Du[i, j] ** 2 for i in range(3) for j in range(3)) / 2
    eta = B if pe == 2 else B * (sp.Rational(1, 2) * eps ** 2 + gamma) ** ((pe - 2) / 2)
    S = eta * Du - p * sp.eye(3)
    fu = [-sum(sp.diff(S[i, j], X[j]) for j in range(3)) for i in range(3)]
    fp = -du.trace()
    return sp.lambdify(X, [list(u), p, fu, fp, list(du)], "numpy")


def columns(vals, n):
    return np.stack([np.broadcast_to(np.asarray(v, np.float64), (n,)) for v in vals], 1)


def closure_coords(fs, P):
    """physical coordinates of every closure node (explicit, then Dirichlet) from the trilinear element maps"""
    ce, xs, em = fs.coords_expanded(), fs.xstart(), fs.emap()
    g = po.lobatto(P)[0]
    X = np.full((fs.nc, 3), np.nan)
    t = np.arange(8)
    sgn = np.stack([2 * ((t >> (2 - a)) & 1) - 1 for a in range(3)], 1)  # vertex t's side along each axis
    loc = 0
    ref = np.array([(g[i], g[j], g[k]) for i in range(P) for j in range(P) for k in range(P)])
    phi = np.prod((1 + ref[:, None, :] * sgn[None, :, :]) / 2, axis=2)  # [P^3, 8] trilinear weights
    for e in range(fs.nelem):
        X[em[xs[e]:xs[e] + P ** 3]] = phi @ ce[e]
    assert not np.isnan(X).any()
    return X


class Problem:
    def __init__(self, rheo):
        self.rheo = rheo
        self.fu = po.FS(5, 5, 5, degree=3, box=BOX, perturb=0.0, seed=1, bs=3, dirichlet_mask=7)
        self.fp = po.FS(5, 5, 5, degree=2, box=BOX, perturb=0.0, seed=1, bs=1, dirichlet_mask=0)
        f = exact1(*rheo[:3])
        Xu, Xp = closure_coords(self.fu, 4), closure_coords(self.fp, 3)
        U = columns(f(*Xu.T)[0], len(Xu))
        Pn = columns([f(*Xp.T)[1]], len(Xp))[:, 0]
        self.xq = self.fu.qpt_coords()
        r = f(*self.xq.T)
        nq = len(self.xq)
        self.fq, self.fpq = columns(r[2], nq), columns([r[3]], nq)[:, 0]
        self.ue, self.pe, self.due = columns(r[0], nq), columns([r[1]], nq)[:, 0], columns(r[4], nq).reshape(nq, 3, 3)
        self.nu3 = self.fu.n * 3
        self.ud = U[self.fu.n:].ravel()
        self.s = np.concatenate([U[:self.fu.n].ravel(), Pn])  # the interpolant (global part)

    def F(self, x):
        return np.concatenate(po.stokes_function(self.fu, self.fp, self.rheo, x[:self.nu3], x[self.nu3:], udir=self.ud,
                                                 fq=self.fq, fpq=self.fpq))

    def J(self, state, v):
        a, b = po.stokes_apply(self.fu, self.fp, 3, self.rheo, xu=v[:self.nu3], xp=v[self.nu3:], state=state[:self.nu3],
                               state_dir=self.ud)
        return np.concatenate([a, b])

    def bordered_lu(self, state):
        """[J(state) c; c^T 0] with c the pressure constant (the null space with Dirichlet walls)"""
        n = self.s.size
        A = np.zeros((n + 1, n + 1))
        e = np.zeros(n)
        for j in range(n):
            e[j] = 1
            A[:n, j] = self.J(state, e)
            e[j] = 0
        A[self.nu3:n, n] = A[n, self.nu3:n] = 1
        return sl.lu_factor(A)

    def solve(self):
        """Newton's chord iteration from the interpolant with the Jacobian there (quadratic closeness makes it
        converge in a few steps), to ||F|| at roundoff"""
        lu = self.bordered_lu(self.s)
        x = self.s.copy()
        for _ in range(40):
            Fx = self.F(x)
            if np.linalg.norm(Fx) < 1e-13:
                break
            x = x + sl.lu_solve(lu, np.concatenate([-Fx, [0.0]]))[:-1]
        assert np.linalg.norm(self.F(x)) < 1e-12
        return x

    def norms(self, x):
        """stokes.c:1161-1169: interpolation residual (dNormsAlgebraicScaled, util.c:155-171, of x - s with the
        pressure constant removed from both) and StokesErrorNorms (pressure shifted by the volume mean of the
        difference; dNormsUpdate, util.c:119-142)"""
        nu3 = self.nu3
        a, b = x.copy(), self.s.copy()
        a[nu3:] -= a[nu3:].mean()
        b[nu3:] -= b[nu3:].mean()
        d = a - b
        n = d.size
        out = {"interpolation": np.array([np.abs(d).sum() / n, np.linalg.norm(d) / np.sqrt(n), np.abs(d).max()])}
        uh, duh, jw = self.fu.eval_points(x[:nu3], self.ud)
        ph = self.fp.eval_points(x[nu3:], rule_deg=3)[0][:, 0]  # the pressure at the velocity's FAST points
        e = self.ue - uh
        out["velocity"] = np.array([(np.abs(e).sum(1) * jw).sum(), np.sqrt(((e ** 2).sum(1) * jw).sum()), np.abs(e).max()])
        g = np.sqrt(((self.due - duh) ** 2).sum(2))
        out["gradient"] = np.array([(g * jw[:, None]).sum(), np.sqrt((g ** 2 * jw[:, None]).sum()), g.max()])
        shift = ((self.pe - ph) * jw).sum() / jw.sum()
        ep = self.pe - shift - ph
        out["pressure"] = np.array([(np.abs(ep) * jw).sum(), np.sqrt((ep ** 2 * jw).sum()), np.abs(ep).max()])
        return out


CASES = {"stokes_q3q2_scr": (1.0, 1.0, 2.0, 0.0), "stokes_q3q2_fgmres": (1.0, 0.1, 1.2, 0.0)}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    g = np.load(os.path.join(HERE, "golden", request.param + ".npz"))
    return Problem(CASES[request.param]), {k: g[k] for k in g}


def test_residuals_at_the_exact_solution(case):
    P, ref = case
    rel = lambda a, b: abs(a - b) / abs(b)
    assert rel(np.linalg.norm(P.F(P.s)), ref["residual_exact"][0]) < 3e-6
    lin = P.J(P.s, P.s) + P.F(np.zeros_like(P.s))  # the Jacobian at s (state with the Dirichlet values) times s
    assert rel(np.linalg.norm(lin), ref["linear_residual_exact"][0]) < 3e-6
    assert rel(np.linalg.norm(P.F(np.zeros_like(P.s))), ref["fnorm0"][0]) < 3e-6


def test_solution_error_norms(case):
    P, ref = case
    got = P.norms(P.solve())
    for key in ("interpolation", "velocity", "gradient", "pressure"):
        np.testing.assert_allclose(got[key], ref[key], rtol=0.012, err_msg=key)
