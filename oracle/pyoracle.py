"""ctypes binding for the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``. The product package (dohp_gb300)
never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libdohpref.so")

_lib = None
_ref = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def build(quiet=True, refdir=None):
    """Compile the oracle, and oracle/_ref from the dohp source tree at refdir (or $DOHP_REF_DIR) when given."""
    refdir = refdir or os.environ.get("DOHP_REF_DIR", "")
    out = subprocess.run(["make", "-C", HERE, "REFDIR=" + refdir], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.or_gauss.argtypes = [ctypes.c_int, _f64p, _f64p]
        L.or_lobatto.argtypes = [ctypes.c_int, _f64p, _f64p]
        L.or_tensor_basis.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.or_rule_1d.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, _f64p]
        L.or_rule_patches.argtypes = [ctypes.c_int, _i32p, _f64p, _f64p, _f64p, ctypes.POINTER(ctypes.c_int), _i32p, _f64p]
        L.or_tensor_mult_hex.argtypes = [ctypes.c_int, _i32p, _i32p, ctypes.c_void_p, _f64p, _f64p, ctypes.c_int]
        L.or_efs_apply_hex.argtypes = [_i32p, _i32p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       _f64p, _f64p, ctypes.c_int, ctypes.c_int]
        L.or_explicit_sparse_hex.argtypes = [ctypes.c_int] * 5 + [_i32p, ctypes.c_void_p, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int), _i32p, _f64p, _f64p]
        L.or_explicit_sparse.argtypes = [_i32p, _i32p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                         _i32p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _i32p,
                                         _f64p, _f64p]
        L.or_modal_count.argtypes = [ctypes.c_int]
        L.or_modal_basis.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p]
        L.or_modal_apply.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, _f64p, ctypes.c_int, _f64p, _f64p, ctypes.c_int,
                                     ctypes.c_int]
        L.or_fs_create.restype = ctypes.c_void_p
        L.or_fs_create.argtypes = [ctypes.c_int] * 3 + [_f64p, ctypes.c_double, ctypes.c_uint64, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.or_fs_destroy.argtypes = [ctypes.c_void_p]
        L.or_fs_create_conn.restype = ctypes.c_void_p
        L.or_fs_create_conn.argtypes = [ctypes.c_int, _f64p, ctypes.c_int, _i32p, ctypes.c_int, _i32p, ctypes.c_int, _i32p,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        L.or_fs_adjacency.restype = ctypes.POINTER(ctypes.c_int32)
        L.or_fs_adjacency.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.or_last_error.restype = ctypes.c_char_p
        L.or_fs_sizes.argtypes = [ctypes.c_void_p, _i64p]
        for name in ("or_fs_emap", "or_fs_xstart", "or_fs_elem_degree"):
            getattr(L, name).restype = ctypes.POINTER(ctypes.c_int32)
            getattr(L, name).argtypes = [ctypes.c_void_p]
        for name in ("or_fs_coords_expanded", "or_fs_vertex_coords"):
            getattr(L, name).restype = ctypes.POINTER(ctypes.c_double)
            getattr(L, name).argtypes = [ctypes.c_void_p]
        L.or_fs_ecsr.restype = ctypes.c_int64
        L.or_fs_ecsr.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.POINTER(ctypes.c_int64)),
                                 ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)), ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        L.or_fs_entity_info.argtypes = [ctypes.c_void_p, _i32p, _i32p, _i32p, _i32p]
        L.or_fs_global_to_expanded.argtypes = [ctypes.c_void_p, _f64p, ctypes.c_void_p, _f64p]
        L.or_fs_expanded_to_global.argtypes = [ctypes.c_void_p, _f64p, _f64p, ctypes.c_int]
        L.or_operator_apply.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, _f64p, _f64p,
                                        ctypes.c_int]
        L.or_fs_num_qpts.restype = ctypes.c_int64
        L.or_fs_num_qpts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.or_fs_qpt_coords.argtypes = [ctypes.c_void_p, _f64p]
        L.or_plap_stash.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _f64p, _f64p]
        L.or_plap_stash_mt.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _f64p, _f64p, ctypes.c_int]
        L.or_q1_assemble.restype = ctypes.c_int64
        L.or_q1_assemble.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     _i32p, ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                     ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        L.or_q1_assemble_plap_dir.restype = ctypes.c_int64
        L.or_q1_assemble_plap_dir.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _f64p, _f64p, ctypes.c_int,
                                              _i32p, ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                              ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        L.or_q1_assemble_plap.restype = ctypes.c_int64
        L.or_q1_assemble_plap.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _f64p, ctypes.c_int,
                                          _i32p, ctypes.POINTER(ctypes.POINTER(ctypes.c_int32)),
                                          ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        L.or_free.argtypes = [ctypes.c_void_p]
        L.or_elast_state.argtypes = [ctypes.c_void_p, _f64p, _f64p]
        L.or_grf_make.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_uint64, _f64p]
        L.or_grf_eval.restype = ctypes.c_double
        L.or_grf_eval.argtypes = [_f64p, _f64p]
        L.or_csr_mult.argtypes = [ctypes.c_int64, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.or_cg_solve.restype = ctypes.c_int
        L.or_cg_solve.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, _i32p, _i32p, _f64p,
                                  ctypes.c_int, _f64p, _f64p, ctypes.c_double, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.or_facet_rule.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, _f64p]
        L.or_facet_count.restype = ctypes.c_int64
        L.or_facet_count.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.or_facet_points.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, _f64p, _f64p, _f64p, _f64p]
        L.or_facet_commit.argtypes = [ctypes.c_void_p, ctypes.c_int, _f64p, _f64p, ctypes.c_int]
        L.or_stokes_apply.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _f64p] + [ctypes.c_void_p] * 5
        L.or_fs_set_vertex_coords.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.or_operator_function.argtypes = [ctypes.c_void_p, ctypes.c_int, _f64p, _f64p, ctypes.c_void_p, ctypes.c_void_p,
                                           _f64p, ctypes.c_int]
        L.or_fs_eval_points.argtypes = [ctypes.c_void_p, ctypes.c_int, _f64p] + [ctypes.c_void_p] * 4
        L.or_stokes_function.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _f64p] + [ctypes.c_void_p] * 7
        L.or_stokes_apply_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _f64p] + [ctypes.c_void_p] * 6
        _lib = L
    return _lib


def ref_lib():
    """The reference's own polylib/TensorMult compiled from source, or None when not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        R = ctypes.CDLL(REF_PATH)
        for name in ("zwgj", "zwglj"):
            getattr(R, name).argtypes = [_f64p, _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        R.Imglj.argtypes = [_f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        R.Dglj.argtypes = [_f64p, _f64p, _f64p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        R.ref_tensor_mult_hex.argtypes = [ctypes.c_int, _i32p, _i32p, ctypes.c_void_p, _f64p, _f64p, ctypes.c_int]
        _ref = R
    return _ref


def gauss(n):
    x = np.zeros(n); w = np.zeros(n)
    lib().or_gauss(n, x, w)
    return x, w


def lobatto(n):
    x = np.zeros(n); w = np.zeros(n)
    lib().or_lobatto(n, x, w)
    return x, w


def tensor_basis(P, rcoord):
    rcoord = np.ascontiguousarray(rcoord, dtype=np.float64)
    Q = len(rcoord)
    interp = np.zeros(Q * P); deriv = np.zeros(Q * P); node = np.zeros(max(P, 1)); weight = np.zeros(max(P, 1))
    rc = lib().or_tensor_basis(P, Q, rcoord, interp, deriv, node, weight)
    if rc:
        raise RuntimeError(lib().or_last_error().decode())
    return interp.reshape(Q, P), deriv.reshape(Q, P), node, weight


def rule_1d(method, family, order):
    x = np.zeros(128); w = np.zeros(128)
    n = lib().or_rule_1d(method, family, order, x, w)
    if n < 0:
        raise RuntimeError(lib().or_last_error().decode())
    return x[:n].copy(), w[:n].copy()


def rule_patches(method, Q, w):
    Q = np.asarray(Q, dtype=np.int32)
    nq = int(np.prod(Q))
    ind = np.zeros(nq, dtype=np.int32); wt = np.zeros(nq)
    ps = ctypes.c_int()
    npatch = lib().or_rule_patches(method, Q, w[0], w[1], w[2], ctypes.byref(ps), ind, wt)
    return npatch, ps.value, ind.reshape(npatch, ps.value), wt.reshape(npatch, ps.value)


def _ptr_array(arrs):
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in arrs]
    ptrs = (ctypes.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
    return ptrs, keep


def efs_apply_hex(P, Q, interp, deriv, jinv, D, x, amode, imode=1, out=None):
    P = np.asarray(P, dtype=np.int32); Q = np.asarray(Q, dtype=np.int32)
    ip, k1 = _ptr_array(interp)
    dp, k2 = _ptr_array(deriv)
    nq = int(np.prod(Q)); nb = int(np.prod(P))
    size = {40001: nq * D, 40002: nb * D, 40003: nq * D * 3, 40004: nb * D}[amode]
    if out is None:
        out = np.zeros(size)
    jinv_c = None if jinv is None else np.ascontiguousarray(jinv, dtype=np.float64)
    rc = lib().or_efs_apply_hex(P, Q, ip, dp, None if jinv_c is None else jinv_c.ctypes.data, D,
                                np.ascontiguousarray(x, dtype=np.float64), out, amode, imode)
    if rc:
        raise RuntimeError(lib().or_last_error().decode())
    return out


def modal_basis(order, rcoord):
    """Modal (P-discontinuous) hexahedral basis of an order 0..3 at the points rcoord [Q][3]
    (modal.c:45-240): interp [Q][P], deriv [Q][P][3]."""
    rcoord = np.ascontiguousarray(rcoord, dtype=np.float64).reshape(-1, 3)
    Q = len(rcoord)
    P = lib().or_modal_count(order)
    if P < 0:
        raise RuntimeError(lib().or_last_error().decode())
    interp = np.zeros(Q * P); deriv = np.zeros(Q * P * 3)
    lib().or_modal_basis(order, Q, rcoord, interp, deriv)
    return interp.reshape(Q, P), deriv.reshape(Q, P, 3)


def modal_apply(interp, deriv, D, x, amode, imode=1, out=None):
    """dEFSApply_Modal_All (modaltopo.c:73-126) for one element"""
    Q, P = interp.shape
    size = {40001: Q * D, 40002: P * D, 40003: Q * D * 3}.get(amode, 1)
    if out is None:
        out = np.zeros(size)
    rc = lib().or_modal_apply(P, Q, np.ascontiguousarray(interp, dtype=np.float64),
                              np.ascontiguousarray(deriv, dtype=np.float64), D,
                              np.ascontiguousarray(x, dtype=np.float64), out, amode, imode)
    if rc:
        raise RuntimeError(lib().or_last_error().decode())
    return out


def explicit_sparse(P, Q, interp, deriv, npatches, Qp, qidx, cjinv=None, eoffset=0):
    P = np.asarray(P, dtype=np.int32); Q = np.asarray(Q, dtype=np.int32)
    ip, k1 = _ptr_array(interp)
    dp, k2 = _ptr_array(deriv)
    maxP = int(np.prod(P))
    eidx = np.zeros(npatches * maxP, np.int32)
    oi = np.zeros(npatches * Qp * maxP); od = np.zeros(npatches * Qp * maxP * 3)
    Pout = ctypes.c_int()
    cj = None if cjinv is None else np.ascontiguousarray(cjinv, dtype=np.float64)
    rc = lib().or_explicit_sparse(P, Q, ip, dp, npatches, Qp, np.ascontiguousarray(qidx, dtype=np.int32).ravel(),
                                  None if cj is None else cj.ctypes.data, eoffset, ctypes.byref(Pout), eidx, oi, od)
    if rc:
        raise RuntimeError(lib().or_last_error().decode())
    Pn = Pout.value
    return (eidx[:npatches * Pn].reshape(npatches, Pn), oi[:npatches * Qp * Pn].reshape(npatches, Qp, Pn),
            od[:npatches * Qp * Pn * 3].reshape(npatches, Qp, Pn * 3))


class FS:
    """Oracle function space on a structured block mesh (see oracle.h or_fs_create)."""

    def __init__(self, nx, ny, nz, degree=4, box=(0, 1, 0, 1, 0, 1), perturb=0.1, seed=1, bs=1,
                 dirichlet_mask=7, elem_degree=None, conn=None):
        """conn: (vtx [nv][3], econn [ne][2], fconn [nf][4], hconn [nr][8]) for a mesh given by its entities
        (or_fs_create_conn, no boundary sets); nx, ny, nz, box, perturb, seed and dirichlet_mask are then unused"""
        L = lib()
        ed = None
        self._ed = None
        if elem_degree is not None:
            self._ed = np.ascontiguousarray(elem_degree, dtype=np.int32)
            ed = self._ed.ctypes.data
        if conn is not None:
            v = np.ascontiguousarray(conn[0], np.float64).reshape(-1, 3)
            e, f, r = [np.ascontiguousarray(c, np.int32).ravel() for c in conn[1:]]
            self.h = L.or_fs_create_conn(len(v), v, len(e) // 2, e, len(f) // 4, f, len(r) // 8, r, degree, ed, bs)
        else:
            self.h = L.or_fs_create(nx, ny, nz, np.asarray(box, dtype=np.float64), perturb, seed, degree, ed, bs,
                                    dirichlet_mask)
        if not self.h:
            raise RuntimeError("oracle fs: " + L.or_last_error().decode())
        s = np.zeros(8, dtype=np.int64)
        L.or_fs_sizes(self.h, s)
        self.nelem, self.n, self.nc, self.nexp, self.bs, self.nv, self.ne, self.nf = [int(v) for v in s]
        self.nents = self.nv + self.ne + self.nf + self.nelem

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_fs_destroy(self.h)
            self.h = None

    def emap(self):
        return np.ctypeslib.as_array(lib().or_fs_emap(self.h), shape=(self.nexp,)).copy()

    def adjacency(self):
        """(adjoff, adjind, adjperm) as dMeshGetAdjacency"""
        ai, ap = ctypes.POINTER(ctypes.c_int32)(), ctypes.POINTER(ctypes.c_int32)()
        ao = lib().or_fs_adjacency(self.h, ctypes.byref(ai), ctypes.byref(ap))
        adjoff = np.ctypeslib.as_array(ao, shape=(self.nents + 1,)).copy()
        na = int(adjoff[-1])
        return adjoff, np.ctypeslib.as_array(ai, shape=(na,)).copy(), np.ctypeslib.as_array(ap, shape=(na,)).copy()

    def ecsr(self):
        p = ctypes.POINTER(ctypes.c_int64)(); c = ctypes.POINTER(ctypes.c_int32)(); v = ctypes.POINTER(ctypes.c_double)()
        nnz = lib().or_fs_ecsr(self.h, ctypes.byref(p), ctypes.byref(c), ctypes.byref(v))
        return (np.ctypeslib.as_array(p, shape=(self.nexp + 1,)).copy(), np.ctypeslib.as_array(c, shape=(nnz,)).copy(),
                np.ctypeslib.as_array(v, shape=(nnz,)).copy())

    def xstart(self):
        return np.ctypeslib.as_array(lib().or_fs_xstart(self.h), shape=(self.nelem + 1,)).copy()

    def elem_degree(self):
        return np.ctypeslib.as_array(lib().or_fs_elem_degree(self.h), shape=(self.nelem, 3)).copy()

    def coords_expanded(self):
        return np.ctypeslib.as_array(lib().or_fs_coords_expanded(self.h), shape=(self.nelem, 8, 3)).copy()

    def vertex_coords(self):
        return np.ctypeslib.as_array(lib().or_fs_vertex_coords(self.h), shape=(self.nv, 3)).copy()

    def set_vertex_coords(self, vx):
        """move the vertices (a mesh morph); the expanded coordinates follow"""
        vx = np.ascontiguousarray(vx, dtype=np.float64).reshape(self.nv, 3)
        lib().or_fs_set_vertex_coords(self.h, vx.ctypes.data)

    def entity_info(self):
        o = np.zeros(self.nents, np.int32); g = np.zeros_like(o); gc = np.zeros_like(o); ino = np.zeros_like(o)
        lib().or_fs_entity_info(self.h, o, g, gc, ino)
        return o, g, gc, ino

    def global_to_expanded(self, g, dcache=None):
        x = np.zeros(self.nexp * self.bs)
        dc = None if dcache is None else np.ascontiguousarray(dcache, dtype=np.float64)
        lib().or_fs_global_to_expanded(self.h, np.ascontiguousarray(g, dtype=np.float64),
                                       None if dc is None else dc.ctypes.data, x)
        return x

    def expanded_to_global(self, x, g=None, add=False):
        out = np.zeros(self.n * self.bs) if g is None else np.array(g, dtype=np.float64)
        lib().or_fs_expanded_to_global(self.h, np.ascontiguousarray(x, dtype=np.float64), out, 1 if add else 0)
        return out

    def num_qpts(self):
        qo = np.zeros(self.nelem + 1, np.int32)
        n = lib().or_fs_num_qpts(self.h, qo.ctypes.data)
        return int(n), qo

    def qpt_coords(self):
        nq, _ = self.num_qpts()
        xq = np.zeros(nq * 3)
        lib().or_fs_qpt_coords(self.h, xq)
        return xq.reshape(nq, 3)

    def function(self, g, kind, param, dcache=None, fq=None, nthreads=1):
        """or_operator_function: EllipFunction (kind 6, param (p, eps); kind 7 with the Bratu term, param (p, eps, lambda))
        or ElastFunction (kind 4, param (lambda, mu))
        with the Dirichlet values dcache and the body force fq at qpt_coords()"""
        y = np.zeros(self.n * self.bs)
        keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (dcache, fq)]
        if lib().or_operator_function(self.h, kind, np.asarray(param, np.float64), np.ascontiguousarray(g, np.float64),
                                      *[None if a is None else a.ctypes.data for a in keep], y, nthreads):
            raise RuntimeError(lib().or_last_error().decode())
        return y

    def eval_points(self, g, dcache=None, rule_deg=0):
        """(u [nq, bs], du [nq, bs, 3], jw [nq]) of the field g (+ Dirichlet values dcache) at qpt_coords(), or at the
        FAST points of degree rule_deg (uniform spaces)"""
        if rule_deg > 0:
            nq = self.nelem * (rule_deg + 1) ** 3
        else:
            nq, _ = self.num_qpts()
        u, du, jw = np.zeros(nq * self.bs), np.zeros(nq * self.bs * 3), np.zeros(nq)
        dc = None if dcache is None else np.ascontiguousarray(dcache, dtype=np.float64)
        if lib().or_fs_eval_points(self.h, rule_deg, np.ascontiguousarray(g, dtype=np.float64), None if dc is None else dc.ctypes.data,
                                   u.ctypes.data, du.ctypes.data, jw.ctypes.data):
            raise RuntimeError(lib().or_last_error().decode())
        return u.reshape(nq, self.bs), du.reshape(nq, self.bs, 3), jw

    def apply(self, g, kind=0, qdata=None, param=None, nthreads=1):
        y = np.zeros(self.n * self.bs)
        qd = None if qdata is None else np.ascontiguousarray(qdata, dtype=np.float64)
        pa = None if param is None else np.ascontiguousarray(param, dtype=np.float64)
        rc = lib().or_operator_apply(self.h, kind, None if qd is None else qd.ctypes.data,
                                     None if pa is None else pa.ctypes.data,
                                     np.ascontiguousarray(g, dtype=np.float64), y, nthreads)
        if rc:
            raise RuntimeError(lib().or_last_error().decode())
        return y

    def elast_state(self, g):
        nq, _ = self.num_qpts()
        F = np.zeros(nq * 9)
        rc = lib().or_elast_state(self.h, np.ascontiguousarray(g, dtype=np.float64), F)
        if rc:
            raise RuntimeError(lib().or_last_error().decode())
        return F

    def plap_stash(self, g, p, eps, nthreads=1):
        nq, _ = self.num_qpts()
        st = np.zeros(nq * 4)
        rc = lib().or_plap_stash_mt(self.h, p, eps, np.ascontiguousarray(g, dtype=np.float64), st, nthreads)
        if rc:
            raise RuntimeError(lib().or_last_error().decode())
        return st

    def q1_assemble(self, kind=0, param=None, grf=None, quirk=1, state=None, state_dcache=None):
        """Q1-embedded matrix; kind 1 (p-Laplacian Jacobian) takes param = (p, eps) and the state g (whose Dirichlet
        values are state_dcache, None = 0)."""
        nrows = self.n * self.bs
        rp = np.zeros(nrows + 1, np.int32)
        colp = ctypes.POINTER(ctypes.c_int32)()
        valp = ctypes.POINTER(ctypes.c_double)()
        pa = None if param is None else np.ascontiguousarray(param, dtype=np.float64)
        gr = None if grf is None else np.ascontiguousarray(grf, dtype=np.float64)
        if kind == 1 and state_dcache is not None:
            nnz = lib().or_q1_assemble_plap_dir(self.h, float(pa[0]), float(pa[1]), np.ascontiguousarray(state, np.float64),
                                                np.ascontiguousarray(state_dcache, np.float64), quirk, rp,
                                                ctypes.byref(colp), ctypes.byref(valp))
        elif kind == 1:
            nnz = lib().or_q1_assemble_plap(self.h, float(pa[0]), float(pa[1]), np.ascontiguousarray(state, np.float64),
                                            quirk, rp, ctypes.byref(colp), ctypes.byref(valp))
        else:
            nnz = lib().or_q1_assemble(self.h, kind, None if pa is None else pa.ctypes.data,
                                       None if gr is None else gr.ctypes.data, quirk, rp,
                                       ctypes.byref(colp), ctypes.byref(valp))
        if nnz < 0:
            raise RuntimeError(lib().or_last_error().decode())
        col = np.ctypeslib.as_array(colp, shape=(max(nnz, 1),))[:nnz].copy()
        val = np.ctypeslib.as_array(valp, shape=(max(nnz, 1),))[:nnz].copy()
        lib().or_free(ctypes.cast(colp, ctypes.c_void_p))
        lib().or_free(ctypes.cast(valp, ctypes.c_void_p))
        return rp, col, val

    def facets(self, weak_mask):
        """(element, side, point offsets) of the faces of the weak sets"""
        nf = ctypes.c_int64()
        lib().or_facet_count(self.h, weak_mask, ctypes.byref(nf), None, None, None)
        fel, fside, qoff = (np.zeros(nf.value + 1, np.int32) for _ in range(3))
        lib().or_facet_count(self.h, weak_mask, ctypes.byref(nf), fel.ctypes.data, fside.ctypes.data, qoff.ctypes.data)
        return fel[:nf.value], fside[:nf.value], qoff

    def facet_points(self, weak_mask, g=None):
        """jw [nq], x [nq,3], normal [nq,3], u [nq,bs] at the facet points"""
        nq = lib().or_facet_count(self.h, weak_mask, None, None, None, None)
        jw, x, nrm, u = np.zeros(nq), np.zeros(3 * nq), np.zeros(3 * nq), np.zeros(nq * self.bs)
        gg = None if g is None else np.ascontiguousarray(g, np.float64)
        if lib().or_facet_points(self.h, weak_mask, None if gg is None else gg.ctypes.data, jw, x, nrm, u):
            raise RuntimeError(lib().or_last_error().decode())
        return jw, x.reshape(nq, 3), nrm.reshape(nq, 3), u.reshape(nq, self.bs)

    def facet_commit(self, weak_mask, v, y=None, add=False):
        out = np.zeros(self.n * self.bs) if y is None else np.array(y, dtype=np.float64)
        if lib().or_facet_commit(self.h, weak_mask, np.ascontiguousarray(v, np.float64).ravel(), out, 1 if add else 0):
            raise RuntimeError(lib().or_last_error().decode())
        return out

    def cg_solve(self, b, csr, kind=0, qdata=None, param=None, cheb_degree=3, rtol=1e-8, maxit=500, nthreads=1):
        rp, col, val = csr
        x = np.zeros(self.n * self.bs)
        rn = ctypes.c_double()
        qd = None if qdata is None else np.ascontiguousarray(qdata, dtype=np.float64)
        pa = None if param is None else np.ascontiguousarray(param, dtype=np.float64)
        its = lib().or_cg_solve(self.h, kind, None if qd is None else qd.ctypes.data,
                                None if pa is None else pa.ctypes.data, rp, col, val, cheb_degree,
                                np.ascontiguousarray(b, dtype=np.float64), x, rtol, maxit, ctypes.byref(rn), nthreads)
        return x, its, rn.value


def facet_rule(side, order, method=0):
    """nodes [n][3] and weights [n] of the facet rule on one hex side"""
    nodes, w = np.zeros(3 * 4096), np.zeros(4096)
    n = lib().or_facet_rule(side, method, order, nodes, w)
    if n < 0:
        raise RuntimeError(lib().or_last_error().decode())
    return nodes[:3 * n].reshape(n, 3), w[:n]


def stokes_apply(fu, fp, mode, rheo=(1.0, 1.0, 2.0, 0.0), xu=None, xp=None, state=None, state_dir=None):
    """(yu, yp) of the Stokes block apply: mode 0 A, 1 Bt, 2 B, 3 coupled (Jacobian at the velocity state, whose
    Dirichlet values are state_dir [nc - n, 3], None = 0), 4 the nonlinear function at xu, xp"""
    yu, yp = np.zeros(fu.n * 3), np.zeros(fp.n)
    if state_dir is None:
        keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (state, xu, xp)]
        addr = [None if a is None else a.ctypes.data for a in keep]
        rc = lib().or_stokes_apply(fu.h, fp.h, mode, np.asarray(rheo, np.float64), *addr, yu.ctypes.data, yp.ctypes.data)
    else:
        keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (state, state_dir, xu, xp)]
        addr = [None if a is None else a.ctypes.data for a in keep]
        rc = lib().or_stokes_apply_state(fu.h, fp.h, mode, np.asarray(rheo, np.float64), *addr, yu.ctypes.data,
                                         yp.ctypes.data)
    if rc:
        raise RuntimeError(lib().or_last_error().decode())
    return yu, yp


def stokes_function(fu, fp, rheo, xu, xp, udir=None, fq=None, fpq=None):
    """(yu, yp) of StokesFunction: Dirichlet velocity values udir [nc - n, 3], forcing fq [nq, 3] and fpq [nq] at
    fu.qpt_coords() (None = 0)"""
    yu, yp = np.zeros(fu.n * 3), np.zeros(fp.n)
    keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (xu, udir, xp, fq, fpq)]
    addr = [None if a is None else a.ctypes.data for a in keep]
    if lib().or_stokes_function(fu.h, fp.h, np.asarray(rheo, np.float64), *addr, yu.ctypes.data, yp.ctypes.data):
        raise RuntimeError(lib().or_last_error().decode())
    return yu, yp


def grf_make(nf, var, ell, seed):
    g = np.zeros(3 + 4 * nf)
    lib().or_grf_make(nf, var, ell, seed, g)
    return g


def grf_eval(grf, x):
    return lib().or_grf_eval(np.ascontiguousarray(grf, dtype=np.float64), np.ascontiguousarray(x, dtype=np.float64))


def csr_mult(csr, x):
    rp, col, val = csr
    y = np.zeros(len(rp) - 1)
    lib().or_csr_mult(len(rp) - 1, rp, col, val, np.ascontiguousarray(x, dtype=np.float64), y)
    return y
