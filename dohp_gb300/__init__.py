"""dohp_gb300: GB300-native matrix-free hp-FEM operator path with dohp's C API.

This module is a thin ctypes binding of the C ABI declared in include/dohp_gb300.h (the product is the
CUDA library libdohp_gb300.so built in-tree by dohp_gb300/build.py). Vectors passed to the library are
CUDA device pointers; the helpers accept torch tensors (torch is used only for device memory and
streams). Importing this module never falls back to a CPU implementation: if the library is missing the
import of `lib()` raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libdohp_gb300.so")

dAPPLY_INTERP, dAPPLY_INTERP_TRANSPOSE, dAPPLY_GRAD, dAPPLY_GRAD_TRANSPOSE = 40001, 40002, 40003, 40004
INSERT_VALUES, ADD_VALUES = 1, 2
dFS_HOMOGENEOUS, dFS_INHOMOGENEOUS = 0, 1
FAST, SPARSE, SELF = 0, 1, 2
dFSBSTATUS_DIRICHLET, dFSBSTATUS_WEAK = 1 << 16, 1 << 17
dOP_DIFFUSION, dOP_PLAPLACE_JACOBIAN, dOP_ELASTICITY = 0, 1, 2
dPREC_FP64, dPREC_FP32, dPREC_BF16, dPREC_FF = 0, 1, 2, 3
dKSP_CG, dKSP_FGMRES = 0, 1
dPC_NONE, dPC_JACOBI, dPC_CHEBYSHEV_Q1, dPC_MG_Q1 = 0, 1, 2, 3

_lib = None
_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_dbl = ctypes.c_double


class DohpError(RuntimeError):
    pass


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise DohpError("dohp_gb300 CUDA library not built: run `python dohp_gb300/build.py` (missing %s)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        L.dGetLastError.restype = ctypes.c_char_p
        _lib = L
    return _lib


def chk(rc):
    if rc:
        raise DohpError(lib().dGetLastError().decode())


def ptr(t):
    """Device (or host) address of a torch tensor or numpy array; None -> NULL."""
    if t is None:
        return None
    if isinstance(t, np.ndarray):
        return _vp(t.ctypes.data)
    return _vp(t.data_ptr())


def exported_symbols():
    """Names declared in include/dohp_gb300.h (for the ABI completeness test)."""
    import re
    hdr = open(os.path.join(HERE, "..", "include", "dohp_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:dErr|const char \*)\s*(\w+)\s*\(", hdr, re.M)))


class Jacobi:
    def __init__(self):
        self.h = _vp()
        chk(lib().dJacobiCreate(ctypes.byref(self.h)))

    def efs(self, degree, method=FAST, rule_order=None):
        degree = np.asarray(degree if np.ndim(degree) else [degree] * 3, dtype=np.int32)
        rule_order = np.asarray(rule_order if rule_order is not None else 2 * degree, dtype=np.int32)
        h = _vp()
        chk(lib().dJacobiGetEFSTensor(self.h, ptr(degree), ctypes.c_int(method), ptr(rule_order), ctypes.byref(h)))
        return EFS(h, self)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dJacobiDestroy(ctypes.byref(self.h))


class EFS:
    def __init__(self, h, jac):
        self.h, self._jac = h, jac
        P = np.zeros(3, np.int32); Q = np.zeros(3, np.int32)
        chk(lib().dEFSGetTensorTables(h, ptr(P), ptr(Q), None, None, None))
        self.P, self.Q = P.tolist(), Q.tolist()
        nodes = np.zeros(P.sum()); pts = np.zeros(Q.sum()); wts = np.zeros(Q.sum())
        chk(lib().dEFSGetTensorTables(h, ptr(P), ptr(Q), ptr(nodes), ptr(pts), ptr(wts)))
        self.nodes, self.points, self.weights = nodes, pts, wts

    def apply(self, nelem, jinv, D, x, y, amode, imode=INSERT_VALUES, stream=None):
        chk(lib().dEFSApplyBatched(self.h, _i32(nelem), ptr(jinv), _i32(D), ptr(x), ptr(y), ctypes.c_int(amode),
                                   ctypes.c_int(imode), _vp(stream)))


class Mesh:
    """A hexahedral mesh given by its entities (dMeshCreateFromConnectivity): vertex coordinates [nv][3], edges
    [ne][2], quadrilaterals [nf][4] and hexahedra [nr][8] (ITAPS vertex order), each in creation order, as a dohp
    caller builds one through iMesh. It has no boundary sets."""

    def __init__(self, vtx, econn, fconn, hconn):
        vtx = np.ascontiguousarray(vtx, np.float64).reshape(-1, 3)
        conn = [np.ascontiguousarray(c, np.int32).ravel() for c in (econn, fconn, hconn)]
        self.h = _vp()
        chk(lib().dMeshCreateFromConnectivity(_i32(len(vtx)), ptr(vtx), _i32(len(conn[0]) // 2), ptr(conn[0]),
                                              _i32(len(conn[1]) // 4), ptr(conn[1]), _i32(len(conn[2]) // 8), ptr(conn[2]),
                                              ctypes.byref(self.h)))

    def adjacency(self):
        """dMeshGetAdjacency: toff [5], adjoff [nents+1], adjind, adjperm (copies)"""
        toff = np.zeros(5, np.int32)
        ao, ai, ap = [ctypes.POINTER(ctypes.c_int32)() for _ in range(3)]
        chk(lib().dMeshGetAdjacency(self.h, ptr(toff), ctypes.byref(ao), ctypes.byref(ai), ctypes.byref(ap)))
        adjoff = np.ctypeslib.as_array(ao, (int(toff[4]) + 1,)).copy()
        na = int(adjoff[-1])
        return toff, adjoff, np.ctypeslib.as_array(ai, (na,)).copy(), np.ctypeslib.as_array(ap, (na,)).copy()

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dMeshDestroy(ctypes.byref(self.h))


class FS:
    """dFS on a seeded perturbed block mesh (dMeshGenerateBlock + dFSBuildSpace), or on a given Mesh."""

    def __init__(self, npoints, degree=4, box=(0, 1, 0, 1, 0, 1), perturb=0.1, seed=1, bs=1,
                 dirichlet=(100, 200, 300), elem_degree=None, stream=None, weak=(), mesh_of=None, mesh=None):
        """mesh_of: another FS whose mesh this space shares (a second field on the same mesh, e.g. the pressure
        of a Stokes pair); mesh: a Mesh from connectivity (no boundary sets: pass dirichlet=()); npoints, box,
        perturb and seed are then ignored"""
        L = lib()
        self.mesh = _vp()
        self._mesh_owner = mesh_of if mesh is None else mesh
        if mesh is not None:
            self.mesh = mesh.h
        elif mesh_of is not None:
            self.mesh = mesh_of.mesh
        else:
            chk(L.dMeshCreateBlock(ptr(np.asarray(npoints, np.int32)), ptr(np.asarray(box, np.float64)), _dbl(perturb),
                                   ctypes.c_uint64(seed), ctypes.byref(self.mesh)))
        self.jac = Jacobi()
        self.h = _vp()
        chk(L.dFSCreate(self.mesh, self.jac.h, ctypes.byref(self.h)))
        ed = None if elem_degree is None else np.ascontiguousarray(elem_degree, np.int32)
        chk(L.dFSSetDegree(self.h, _i32(degree), ptr(ed)))
        chk(L.dFSSetBlockSize(self.h, _i32(bs)))
        for s in set(dirichlet) | set(weak):
            st = (dFSBSTATUS_DIRICHLET if s in dirichlet else 0) | (dFSBSTATUS_WEAK if s in weak else 0)
            chk(L.dFSRegisterBoundary(self.h, _i32(s), ctypes.c_int(st)))
        if stream is not None:
            chk(L.dFSSetStream(self.h, _vp(stream)))
        chk(L.dFSSetUp(self.h))
        n, nc, nexp, b, ne = _i32(), _i32(), _i32(), _i32(), _i32()
        chk(L.dFSGetSizes(self.h, ctypes.byref(n), ctypes.byref(nc), ctypes.byref(nexp), ctypes.byref(b), ctypes.byref(ne)))
        self.n, self.nc, self.nexp, self.bs, self.nelem = n.value, nc.value, nexp.value, b.value, ne.value
        nq = _i64()
        chk(L.dFSGetNumQuadraturePoints(self.h, ctypes.byref(nq)))
        self.nq = nq.value

    def __del__(self):
        if _lib is None:
            return
        if getattr(self, "h", None):
            _lib.dFSDestroy(ctypes.byref(self.h))
        if getattr(self, "mesh", None) and getattr(self, "_mesh_owner", None) is None:
            _lib.dMeshDestroy(ctypes.byref(self.mesh))

    def set_stream(self, stream):
        chk(lib().dFSSetStream(self.h, _vp(stream)))

    def emap(self):
        em = np.zeros(self.nexp, np.int32); xs = np.zeros(self.nelem + 1, np.int32)
        chk(lib().dFSGetExpandedMap(self.h, ptr(em), ptr(xs)))
        return em, xs

    def elem_degree(self):
        d = np.zeros(3 * self.nelem, np.int32)
        chk(lib().dFSGetElementDegrees(self.h, ptr(d)))
        return d.reshape(-1, 3)

    def global_to_expanded(self, g, x, inhomogeneous=False, add=False):
        chk(lib().dFSGlobalToExpanded(self.h, ptr(g), ptr(x), ctypes.c_int(1 if inhomogeneous else 0),
                                      ctypes.c_int(ADD_VALUES if add else INSERT_VALUES)))

    def expanded_to_global(self, x, g, add=False):
        chk(lib().dFSExpandedToGlobal(self.h, ptr(x), ptr(g), ctypes.c_int(0), ctypes.c_int(ADD_VALUES if add else INSERT_VALUES)))

    def dirichlet_commit(self, closure):
        chk(lib().dFSInhomogeneousDirichletCommit(self.h, ptr(closure)))

    def qpt_coords(self, xq):
        chk(lib().dFSGetQuadratureCoordinates(self.h, ptr(xq)))

    def nodal_coordinates(self, expanded=True):
        """dFSGetNodalCoordinatesExpanded [nexp][3] / dFSGetNodalCoordinatesGlobal [nc][3], host arrays"""
        out = np.zeros(((self.nexp if expanded else self.nc), 3))
        f = lib().dFSGetNodalCoordinatesExpanded if expanded else lib().dFSGetNodalCoordinatesGlobal
        chk(f(self.h, ptr(out), ctypes.c_int(0)))
        return out

    def lognormal(self, grf, kq):
        chk(lib().dFSEvaluateLognormal(self.h, ptr(np.ascontiguousarray(grf, np.float64)), ptr(kq)))

    def operator(self, kind=dOP_DIFFUSION, param=None):
        return Operator(self, kind, param)

    def matrix(self):
        return Mat(self)


class Operator:
    def __init__(self, fs, kind=dOP_DIFFUSION, param=None):
        self.fs = fs
        self.h = _vp()
        pa = None if param is None else np.asarray(param, np.float64)
        chk(lib().dFSCreateOperator(fs.h, ctypes.c_int(kind), ptr(pa), ctypes.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dOperatorDestroy(ctypes.byref(self.h))

    def set_qdata(self, q):
        chk(lib().dOperatorSetQuadratureData(self.h, ptr(q)))

    def set_precision(self, prec):
        chk(lib().dOperatorSetPrecision(self.h, ctypes.c_int(prec)))

    def mult(self, x, y):
        chk(lib().dOperatorMult(self.h, ptr(x), ptr(y)))

    def mult_host(self, x, y):
        chk(lib().dOperatorMultHost(self.h, ptr(x), ptr(y)))

    def plap_stash(self, g, p, eps):
        """dOperatorComputePLaplaceStash: the Jacobian at state g (device vector)."""
        chk(lib().dOperatorComputePLaplaceStash(self.h, ptr(g), _dbl(p), _dbl(eps)))

    def plap_function(self, g, p, eps, y):
        """dOperatorPLaplaceFunction: y = N(g) (no forcing); the stash of g stays for the Jacobian."""
        chk(lib().dOperatorPLaplaceFunction(self.h, ptr(g), _dbl(p), _dbl(eps), ptr(y)))

    def elasticity_state(self, g):
        """dOperatorElasticityState: St. Venant-Kirchhoff Jacobian at g from now on (None: linear)"""
        chk(lib().dOperatorElasticityState(self.h, ptr(g)))

    def elasticity_function(self, g, y):
        chk(lib().dOperatorElasticityFunction(self.h, ptr(g), ptr(y)))

    def get_qdata(self, out):
        chk(lib().dOperatorGetQuadratureData(self.h, ptr(out)))


class Mat:
    def __init__(self, fs):
        self.fs = fs
        self.h = _vp()
        chk(lib().dFSCreateMatrix(fs.h, ctypes.byref(self.h)))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dMatDestroy(ctypes.byref(self.h))

    def assemble(self, kind=dOP_DIFFUSION, param=None, grf=None, quirk=1):
        pa = None if param is None else np.asarray(param, np.float64)
        g = None if grf is None else np.ascontiguousarray(grf, np.float64)
        chk(lib().dFSAssembleQ1(self.fs.h, self.h, ctypes.c_int(kind), ptr(pa), ptr(g), ctypes.c_int(quirk)))

    def assemble_plap(self, g, p, eps, quirk=1):
        chk(lib().dFSAssembleQ1PLaplace(self.fs.h, self.h, ptr(g), _dbl(p), _dbl(eps), ctypes.c_int(quirk)))

    def csr_host(self):
        nr, nnz = _i32(), _i64()
        chk(lib().dMatGetCSR(self.h, ctypes.byref(nr), ctypes.byref(nnz), None, None, None))
        rp = np.zeros(nr.value + 1, np.int32); col = np.zeros(nnz.value, np.int32); val = np.zeros(nnz.value)
        chk(lib().dMatGetCSRHost(self.h, ptr(rp), ptr(col), ptr(val)))
        return rp, col, val

    def mult(self, x, y):
        chk(lib().dMatMult(self.h, ptr(x), ptr(y)))

    def set_values_expanded(self, idxm, idxn, v, imode=ADD_VALUES):
        """dFSMatSetValuesBlockedExpanded: a block of values in expanded indices (host arrays)"""
        im, jn = np.ascontiguousarray(idxm, np.int32), np.ascontiguousarray(idxn, np.int32)
        vv = np.ascontiguousarray(v, np.float64)
        chk(lib().dFSMatSetValuesBlockedExpanded(self.fs.h, self.h, _i32(len(im)), ptr(im), _i32(len(jn)), ptr(jn), ptr(vv),
                                                 ctypes.c_int(imode)))


class KSP:
    def __init__(self, op, pmat=None, ksp_type=dKSP_CG, pc=dPC_CHEBYSHEV_Q1, cheb_degree=3, inner_prec=dPREC_FP64,
                 restart=30):
        self.h = _vp()
        self.op, self.pmat = op, pmat
        chk(lib().dKSPCreate(op.h, None if pmat is None else pmat.h, ctypes.c_int(ksp_type), ctypes.c_int(pc),
                             ctypes.byref(self.h)))
        chk(lib().dKSPSetOptions(self.h, _i32(cheb_degree), ctypes.c_int(inner_prec), _i32(restart)))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dKSPDestroy(ctypes.byref(self.h))

    def set_operators(self, op=None, pmat=None):
        chk(lib().dKSPSetOperators(self.h, None if op is None else op.h, None if pmat is None else pmat.h))
        if op is not None:
            self.op = op
        if pmat is not None:
            self.pmat = pmat

    def solve(self, b, x, rtol=1e-8, maxit=1000):
        its, rn = _i32(), _dbl()
        chk(lib().dKSPSolve(self.h, ptr(b), ptr(x), _dbl(rtol), _i32(maxit), ctypes.byref(its), ctypes.byref(rn)))
        return its.value, rn.value


def grf_create(nf, var, ell, seed):
    g = np.zeros(3 + 4 * nf)
    chk(lib().dGRFCreate(_i32(nf), _dbl(var), _dbl(ell), ctypes.c_uint64(seed), ptr(g)))
    return g


def _op_mult_expanded(self, x, yexp):
    chk(lib().dOperatorMultExpanded(self.h, ptr(x), ptr(yexp)))


dLAUNCH_DEFAULT, dLAUNCH_PER_ORDER, dLAUNCH_PERSISTENT, dLAUNCH_GRAPH = 0, 1, 2, 3


def _op_set_launch(self, mode):
    chk(lib().dOperatorSetLaunchMode(self.h, ctypes.c_int(mode)))


def _op_autotune(self, cache_path=None):
    chk(lib().dOperatorAutotune(self.h, None if cache_path is None else ctypes.c_char_p(cache_path.encode())))


def _op_tiles(self):
    nb = _i32()
    chk(lib().dOperatorGetTiles(self.h, ctypes.byref(nb), None, None, None))
    o = np.zeros(max(nb.value, 1), np.int32); c = np.zeros_like(o); t = np.zeros_like(o)
    chk(lib().dOperatorGetTiles(self.h, ctypes.byref(nb), ptr(o), ptr(c), ptr(t)))
    return [(int(o[i]), int(c[i]), int(t[i])) for i in range(nb.value)]


Operator.mult_expanded = _op_mult_expanded
Operator.set_launch = _op_set_launch
Operator.autotune = _op_autotune
Operator.tiles = _op_tiles


class _DeviceArray:
    """Exposes a library-owned device array to torch through __cuda_array_interface__ (no copy)."""

    def __init__(self, addr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8", "data": (addr, False),
                                         "version": 3, "strides": None}


def _np(t):
    """pointer argument of a variadic call: the address, or an explicit NULL pointer"""
    q = ptr(t)
    return q if q is not None else _vp(0)


class RulesetIterator:
    """dRulesetIterator over all elements at once (the batched device form of dohp's element loop): link 0 is the
    coordinate space, link 1 the space fs, links 2.. the spaces given to add_fs (same mesh). get() returns torch views
    of the library's quadrature arrays for link 1: jw[nq], x[nq,3], dx[nq,3,3], u[nq,bs], du[nq,bs,3], v[nq,bs],
    dv[nq,bs,3], and under "fields" the (u, du, v, dv) views of every field link. Only v and dv are meant to be
    written (torch has no read-only device tensors). The test vectors of Start are the wrapper's own global
    buffers; finish(y) restricts into them and copies (or adds) link 1's into y."""

    def __init__(self, fs, method=FAST):
        self.fs = fs
        self.fields = [fs]
        self.h = _vp()
        self._y = []
        chk(lib().dRulesetIteratorCreate(fs.h, ctypes.c_int(method), ctypes.byref(self.h)))

    def __del__(self):
        if _lib is not None and getattr(self, "h", None):
            _lib.dRulesetIteratorDestroy(ctypes.byref(self.h))

    def add_fs(self, fs):
        chk(lib().dRulesetIteratorAddFS(self.h, fs.h))
        self.fields.append(fs)

    def add_stash(self, elembytes, nodebytes):
        chk(lib().dRulesetIteratorAddStash(self.h, _i32(elembytes), _i32(nodebytes)))

    def stash(self):
        """device addresses of the element and point stashes (0 when absent)"""
        e, n = _vp(), _vp()
        chk(lib().dRulesetIteratorGetStash(self.h, ctypes.byref(e), ctypes.byref(n)))
        return e.value or 0, n.value or 0

    def start(self, g=None, hmode=dFS_HOMOGENEOUS, *more):
        """g: link 1's trial vector; more: (trial vector, mode) pairs for links 2.."""
        import torch
        xs = [(g, hmode)] + [(more[i], more[i + 1]) for i in range(0, len(more), 2)]
        xs += [(None, dFS_HOMOGENEOUS)] * (len(self.fields) - len(xs))
        self._y = [torch.zeros(f.n * f.bs, dtype=torch.float64, device="cuda") for f in self.fields]
        args = [_vp(0), _vp(0)]  # link 0: the space's own coordinates, no test vector
        for (x, m), y in zip(xs, self._y):
            args.append(_np(x))
            if x is not None:
                args.append(ctypes.c_int(m))
            args += [_np(y), ctypes.c_int(dFS_HOMOGENEOUS)]
        chk(lib().dRulesetIteratorStart(self.h, *args))

    def get(self):
        import torch
        Q = _i32()
        jw = _vp()
        link0 = [_vp(), _vp()]
        per = [[_vp() for _ in range(4)] for _ in self.fields]
        args = [ctypes.byref(Q), ctypes.byref(jw), ctypes.byref(link0[0]), ctypes.byref(link0[1]), _vp(0), _vp(0)]
        for q in per:
            args += [ctypes.byref(v) for v in q]
        chk(lib().dRulesetIteratorGetPatchApplied(self.h, *args))
        n = Q.value
        view = lambda q, shape: torch.as_tensor(_DeviceArray(q.value, shape), device="cuda")
        fields = []
        for f, q in zip(self.fields, per):
            bs = f.bs
            fields.append({k: view(v, s) for k, v, s in zip(("u", "du", "v", "dv"), q, [(n, bs), (n, bs, 3), (n, bs), (n, bs, 3)])})
        out = {"jw": view(jw, (n,)), "x": view(link0[0], (n, 3)), "dx": view(link0[1], (n, 3, 3))}
        out.update(fields[0])
        out["fields"] = fields
        return out

    def _field_ptrs(self):
        """(v, dv) addresses of every field link (the arrays GetPatchApplied returned)"""
        Q, jw = _i32(), _vp()
        per = [[_vp() for _ in range(4)] for _ in self.fields]
        args = [ctypes.byref(Q), ctypes.byref(jw), _vp(0), _vp(0), _vp(0), _vp(0)]
        for q in per:
            args += [_vp(0), _vp(0), ctypes.byref(q[2]), ctypes.byref(q[3])]
        chk(lib().dRulesetIteratorGetPatchApplied(self.h, *args))
        return [(q[2], q[3]) for q in per]

    def commit(self, imode=INSERT_VALUES, use_v=True, use_dv=True, links=None):
        """integrate v / dv of link 1 (use_v, use_dv), or of the field links listed in links as (use_v, use_dv) pairs"""
        flags = links if links is not None else [(use_v, use_dv)] + [(False, False)] * (len(self.fields) - 1)
        ptrs = self._field_ptrs()
        args = [_vp(0), _vp(0)]
        for (uv, udv), (v, dv) in zip(flags, ptrs):
            args += [v if uv else _vp(0), dv if udv else _vp(0)]
        chk(lib().dRulesetIteratorCommitPatchApplied(self.h, ctypes.c_int(imode), *args))

    def finish(self, y=None, imode=INSERT_VALUES, ys=None):
        """restrict the test vectors; y receives link 1's (copied, or added with ADD_VALUES), ys those of all links"""
        chk(lib().dRulesetIteratorSetMode(self.h, ctypes.c_int(INSERT_VALUES)))
        chk(lib().dRulesetIteratorFinish(self.h))
        outs = [y] if ys is None else ys
        for out, buf in zip(outs, self._y):
            if out is None:
                continue
            if imode == ADD_VALUES:
                out.add_(buf)
            else:
                out.copy_(buf)

    def error_norms(self, exact_u=None, exact_du=None):
        """dRulesetIteratorErrorNorms: ({L1, L2, Linf} of u - exact_u, the same of |grad u - exact_du|)"""
        ue, ge = np.zeros(3), np.zeros(3)
        chk(lib().dRulesetIteratorErrorNorms(self.h, ptr(exact_u), ptr(exact_du), ptr(ue), ptr(ge)))
        return ue, ge


class FacetIterator:
    """dFacetIterator over the faces of the weak sets (FAST rules). get() returns torch views of the library's
    facet-point arrays: jw[nq] (area weight), x[nq,3], normal[nq,3], u[nq,bs], v[nq,bs] (writable, zeroed)."""

    def __init__(self, fs, method=FAST):
        self.fs = fs
        self.h = _vp()
        chk(lib().dFacetIteratorCreate(fs.h, ctypes.c_int(method), ctypes.byref(self.h)))

    def __del__(self):
        if _lib is not None and getattr(self, "h", None):
            _lib.dFacetIteratorDestroy(ctypes.byref(self.h))

    def facets(self):
        """(element, side, point offsets) as numpy arrays"""
        nf = _i64()
        p = [ctypes.POINTER(ctypes.c_int32)() for _ in range(3)]
        chk(lib().dFacetIteratorGetFacets(self.h, ctypes.byref(nf), *[ctypes.byref(q) for q in p]))
        n = nf.value
        if n == 0:
            return np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(1, np.int32)
        return tuple(np.ctypeslib.as_array(q, shape=(m,)).copy() for q, m in zip(p, (n, n, n + 1)))

    def start(self, g=None, hmode=dFS_HOMOGENEOUS):
        chk(lib().dFacetIteratorStart(self.h, ptr(g), ctypes.c_int(hmode)))

    def get(self):
        import torch
        nq = _i64()
        p = [_vp() for _ in range(5)]
        chk(lib().dFacetIteratorGetApplied(self.h, ctypes.byref(nq), *[ctypes.byref(q) for q in p]))
        n, bs = nq.value, self.fs.bs
        if n == 0:
            return {k: torch.zeros(s, dtype=torch.float64, device="cuda") for k, s in
                    zip(["jw", "x", "normal", "u", "v"], [(0,), (0, 3), (0, 3), (0, bs), (0, bs)])}
        shapes = [(n,), (n, 3), (n, 3), (n, bs), (n, bs)]
        names = ["jw", "x", "normal", "u", "v"]
        return {k: torch.as_tensor(_DeviceArray(q.value, s), device="cuda") for k, q, s in zip(names, p, shapes)}

    def commit(self, imode=ADD_VALUES):
        chk(lib().dFacetIteratorCommit(self.h, ctypes.c_int(imode)))

    def finish(self, y=None, imode=INSERT_VALUES):
        chk(lib().dFacetIteratorFinish(self.h, ptr(y), ctypes.c_int(imode)))


def facet_rule(side, order, method=FAST):
    """dFSGetFacetRule: nodes [n,3] in hex reference coordinates and weights [n]"""
    nodes, w, n = np.zeros(3 * 81), np.zeros(81), _i32()
    chk(lib().dFSGetFacetRule(_i32(side), ctypes.c_int(method), _i32(order), ctypes.byref(n), ptr(nodes), ptr(w)))
    return nodes[:3 * n.value].reshape(-1, 3), w[:n.value]


dSTOKES_MULT_A, dSTOKES_MULT_BT, dSTOKES_MULT_B, dSTOKES_MULT_COUPLED = 0, 1, 2, 3


class Stokes:
    """dStokes on a velocity space fsu (bs 3) and a pressure space fsp (bs 1) sharing its mesh
    (FS(..., mesh_of=fsu)); rheo = (B, eps, p, nu): eta = B (eps^2/2 + Du:Du/2)^((p-2)/2), Newtonian at p = 2."""

    def __init__(self, fsu, fsp, rheo=None):
        self.fsu, self.fsp = fsu, fsp
        self.h = _vp()
        r = None if rheo is None else np.asarray(rheo, np.float64)
        chk(lib().dStokesCreate(fsu.h, fsp.h, ptr(r), ctypes.byref(self.h)))

    def __del__(self):
        if _lib is not None and getattr(self, "h", None):
            _lib.dStokesDestroy(ctypes.byref(self.h))

    def mult(self, mode, xu=None, xp=None, yu=None, yp=None):
        chk(lib().dStokesMult(self.h, ctypes.c_int(mode), ptr(xu), ptr(xp), ptr(yu), ptr(yp)))

    def function(self, xu, xp, yu, yp):
        """dStokesFunction: (yu, yp) = N(xu, xp) (velocity Dirichlet values from fsu.dirichlet_commit); the state of
        the following Jacobian applies"""
        chk(lib().dStokesFunction(self.h, ptr(xu), ptr(xp), ptr(yu), ptr(yp)))

    def integrate_pressure(self, fq, yp):
        """dStokesIntegratePressure: yp = int q f, f at the velocity's quadrature points"""
        chk(lib().dStokesIntegratePressure(self.h, ptr(fq), ptr(yp)))

    def solve(self, bu, bp, xu, xp, rtol=1e-8, maxit=500):
        its, rn = _i32(), _dbl()
        chk(lib().dStokesSolve(self.h, ptr(bu), ptr(bp), ptr(xu), ptr(xp), _dbl(rtol), _i32(maxit), ctypes.byref(its),
                               ctypes.byref(rn)))
        return its.value, rn.value

    def newton(self, bu, bp, xu, xp, rtol=1e-8, atol=0.0, lin_rtol=1e-4, lin_maxit=500, max_it=30):
        """dStokesNewtonSolve: returns (steps, residual norms [steps+1], linear iterations [steps])."""
        opt = dNewtonOptions(max_it, rtol, atol, lin_rtol, lin_maxit, 0)
        its = _i32()
        fn = np.zeros(max_it + 1)
        li = np.zeros(max_it, np.int32)
        chk(lib().dStokesNewtonSolve(self.h, ptr(bu), ptr(bp), ptr(xu), ptr(xp), ctypes.byref(opt), ctypes.byref(its),
                                     ptr(fn), ptr(li)))
        k = its.value
        return k, fn[:k + 1], li[:k]


class dNewtonOptions(ctypes.Structure):
    _fields_ = [("max_it", _i32), ("rtol", _dbl), ("atol", _dbl), ("lin_rtol", _dbl), ("lin_maxit", _i32),
                ("reference_quirk", ctypes.c_int)]


def plap_newton(op, pmat, ksp, b, u, p, eps, rtol=1e-8, atol=0.0, lin_rtol=1e-3, lin_maxit=500, max_it=30, quirk=1):
    """dPLaplaceNewtonSolve: returns (steps, residual norms [steps+1], linear iterations [steps])."""
    opt = dNewtonOptions(max_it, rtol, atol, lin_rtol, lin_maxit, quirk)
    its = _i32()
    fn = np.zeros(max_it + 1)
    li = np.zeros(max_it, np.int32)
    chk(lib().dPLaplaceNewtonSolve(op.h, pmat.h, ksp.h, ptr(b), ptr(u), _dbl(p), _dbl(eps), ctypes.byref(opt),
                                   ctypes.byref(its), ptr(fn), ptr(li)))
    k = its.value
    return k, fn[:k + 1], li[:k]


LEARNED_GRID_VERTEX, LEARNED_GRID_GLL = 0, 1


class Learned:
    """dLearned: learned correction (U-Net on the vertex lattice, or on the GLL lattice of the Q1-embedded matrix
    trained on crop^3 windows) for FGMRES."""

    def __init__(self, fs, seed=0, grid=LEARNED_GRID_VERTEX, crop=0):
        self.fs = fs
        self.h = _vp()
        if grid == LEARNED_GRID_VERTEX and not crop:
            chk(lib().dLearnedCreate(fs.h, ctypes.c_uint64(seed), ctypes.byref(self.h)))
        else:
            chk(lib().dLearnedCreateOnGrid(fs.h, ctypes.c_int(grid), _i32(crop), ctypes.c_uint64(seed), ctypes.byref(self.h)))
        d = np.zeros(3, np.int32)
        npar, npairs = _i64(), _i64()
        chk(lib().dLearnedGetSizes(self.h, ptr(d), ctypes.byref(npar), ctypes.byref(npairs)))
        self.dims, self.nparam = tuple(int(v) for v in d), npar.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dLearnedDestroy(ctypes.byref(self.h))

    @property
    def npairs(self):
        npairs = _i64()
        chk(lib().dLearnedGetSizes(self.h, None, None, ctypes.byref(npairs)))
        return npairs.value

    def set_field(self, grf=None):
        g = None if grf is None else np.ascontiguousarray(grf, np.float64)
        chk(lib().dLearnedSetField(self.h, ptr(g)))

    def collect(self, ksp, b, rtol=1e-10, maxit=5000, every=1, max_pairs=100, rough_start=False):
        n = _i32()
        chk(lib().dLearnedCollectPairs(self.h, ksp.h, ptr(b), _dbl(rtol), _i32(maxit), _i32(every), _i32(max_pairs),
                                       ctypes.c_int(int(rough_start)), ctypes.byref(n)))
        return n.value

    def train(self, epochs, batch=8, lr=1e-3, seed=0):
        losses = np.zeros(epochs)
        chk(lib().dLearnedTrain(self.h, _i32(epochs), _i32(batch), _dbl(lr), ctypes.c_uint64(seed), ptr(losses)))
        return losses

    def apply(self, r, z):
        chk(lib().dLearnedApply(self.h, ptr(r), ptr(z)))

    def forward(self, x, y):
        chk(lib().dLearnedForward(self.h, _i32(x.shape[0]), ptr(x), ptr(y)))

    def loss_grad(self, x, t, grad):
        lv = _dbl()
        chk(lib().dLearnedLossGrad(self.h, _i32(x.shape[0]), ptr(x), ptr(t), ctypes.byref(lv), ptr(grad)))
        return lv.value

    def get_weights(self):
        w = np.zeros(self.nparam, np.float32)
        chk(lib().dLearnedGetWeights(self.h, ptr(w)))
        return w

    def set_weights(self, w, target_scale=0.0):
        chk(lib().dLearnedSetWeights(self.h, ptr(np.ascontiguousarray(w, np.float32)), _dbl(target_scale)))

    def save(self, path, with_moments=False):
        chk(lib().dLearnedSave(self.h, str(path).encode(), ctypes.c_int(int(with_moments))))

    def load(self, path):
        chk(lib().dLearnedLoad(self.h, str(path).encode()))

    def scale(self):
        v = _dbl()
        chk(lib().dLearnedGetScale(self.h, ctypes.byref(v)))
        return v.value

    def restrict(self, r, rc):
        chk(lib().dLearnedRestrict(self.h, ptr(r), ptr(rc)))

    def prolong(self, c, z):
        chk(lib().dLearnedProlong(self.h, ptr(c), ptr(z)))

    def stats(self):
        a, d = _i64(), _i64()
        chk(lib().dLearnedGetStats(self.h, ctypes.byref(a), ctypes.byref(d)))
        return a.value, d.value

    def layer(self, layer, x, y, dims, transpose=False):
        """one convolution layer on device FP32 arrays (forward, or its data gradient with transpose)"""
        d = np.asarray(dims, np.int32)
        chk(lib().dLearnedLayerApply(self.h, _i32(layer), _i32(int(transpose)), _i32(x.shape[0]), ptr(d), ptr(x), ptr(y)))

    def layer_weight_grad(self, layer, x, gy, grad, dims):
        """one layer's weight and bias gradient (device FP32 arrays)"""
        d = np.asarray(dims, np.int32)
        chk(lib().dLearnedLayerWeightGrad(self.h, _i32(layer), _i32(x.shape[0]), ptr(d), ptr(x), ptr(gy), ptr(grad)))

    def set_tensor_cores(self, on=True):
        chk(lib().dLearnedSetTensorCores(self.h, ctypes.c_int(int(on))))

    def pair(self, p):
        """recorded pair p: (origin, input, target), the arrays shaped as its window"""
        win, org = np.zeros(3, np.int32), np.zeros(3, np.int32)
        chk(lib().dLearnedGetPair(self.h, _i32(p), ptr(win), ptr(org), None, None))
        inp, tg = np.zeros(tuple(win), np.float32), np.zeros(tuple(win), np.float32)
        chk(lib().dLearnedGetPair(self.h, _i32(p), ptr(win), ptr(org), ptr(inp), ptr(tg)))
        return tuple(int(v) for v in org), inp, tg


def _ksp_set_learned(self, net, policy=2):
    """policy: 0 every preconditioner application, 1 first vector of each restart cycle, 2 adaptive"""
    chk(lib().dKSPSetLearnedCorrection(self.h, None if net is None else net.h))
    chk(lib().dKSPSetCorrectionPolicy(self.h, ctypes.c_int(policy)))
    self.net = net


def _ksp_stats(self):
    a, r, on = _i64(), _i64(), ctypes.c_int()
    chk(lib().dKSPGetStats(self.h, ctypes.byref(a), ctypes.byref(r), ctypes.byref(on)))
    return a.value, r.value, bool(on.value)


KSP.set_learned = _ksp_set_learned
KSP.stats = _ksp_stats
