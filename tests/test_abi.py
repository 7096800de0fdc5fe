"""CPU-side checks of the product library: it loads, exports every entry point include/dohp_gb300.h
declares, and its host-side space build (block mesh, adjacency, numbering, E map) is bit-exact with the
oracle. No GPU is touched."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    import subprocess, sys, os
    if not os.path.exists(dg.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    return dg.lib()


def test_exports_every_declared_symbol(L):
    names = dg.exported_symbols()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def host_fs(npoints, degree, box=(0, 1, 0, 1, 0, 1), perturb=0.1, seed=1, bs=1, dirichlet=(100, 200, 300), elem_degree=None):
    L = dg.lib()
    mesh = ctypes.c_void_p()
    dg.chk(L.dMeshCreateBlock(dg.ptr(np.asarray(npoints, np.int32)), dg.ptr(np.asarray(box, np.float64)),
                              ctypes.c_double(perturb), ctypes.c_uint64(seed), ctypes.byref(mesh)))
    fs = ctypes.c_void_p()
    dg.chk(L.dFSCreate(mesh, None, ctypes.byref(fs)))
    ed = None if elem_degree is None else np.ascontiguousarray(elem_degree, np.int32)
    dg.chk(L.dFSSetDegree(fs, ctypes.c_int32(degree), dg.ptr(ed)))
    dg.chk(L.dFSSetBlockSize(fs, ctypes.c_int32(bs)))
    for s in dirichlet:
        dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(s), ctypes.c_int(dg.dFSBSTATUS_DIRICHLET)))
    rc = L.dFSBuildSpace(fs)
    if rc:
        msg = L.dGetLastError().decode()
        L.dFSDestroy(ctypes.byref(fs)); L.dMeshDestroy(ctypes.byref(mesh))
        raise dg.DohpError(msg)
    sz = [ctypes.c_int32() for _ in range(5)]
    dg.chk(L.dFSGetSizes(fs, *[ctypes.byref(s) for s in sz]))
    n, nc, nexp, b, ne = [s.value for s in sz]
    em = np.zeros(nexp, np.int32); xs = np.zeros(ne + 1, np.int32)
    dg.chk(L.dFSGetExpandedMap(fs, dg.ptr(em), dg.ptr(xs)))
    L.dFSDestroy(ctypes.byref(fs)); L.dMeshDestroy(ctypes.byref(mesh))
    return dict(n=n, nc=nc, nexp=nexp, nelem=ne, emap=em, xstart=xs)


MASKS = {(100, 200, 300): 7, (100,): 1, (200, 300): 6, (): 0}


@pytest.mark.parametrize("npoints,degree", [((3, 2, 2), 2), ((4, 3, 5), 1), ((4, 4, 4), 3), ((3, 4, 3), 5), ((3, 3, 3), 8)])
@pytest.mark.parametrize("dirichlet", list(MASKS))
def test_host_space_bit_exact_with_oracle(L, npoints, degree, dirichlet):
    h = host_fs(npoints, degree, dirichlet=dirichlet)
    o = po.FS(*npoints, degree=degree, perturb=0.1, seed=1, dirichlet_mask=MASKS[dirichlet])
    assert (h["n"], h["nc"], h["nexp"], h["nelem"]) == (o.n, o.nc, o.nexp, o.nelem)
    np.testing.assert_array_equal(h["emap"], o.emap())
    np.testing.assert_array_equal(h["xstart"], o.xstart())


def test_bu0_numbering_from_product(L):
    """bu-0 golden (src/fs/tests/refout/bu-0.refout) reproduced by the product's host build."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "bu0.npz"))
    h = host_fs((3, 2, 2), 2, box=(-1, 1, -1, 1, -1, 1), perturb=0.0, dirichlet=(100,))
    closure = g["closure"]
    x = np.where(h["emap"] < h["n"], closure[np.minimum(h["emap"], h["n"] - 1)], 0.0)
    np.testing.assert_array_equal(x, g["homogeneous"])


def host_ecsr(npoints, degree, elem_degree, dirichlet=(100, 200, 300)):
    L = dg.lib()
    mesh = ctypes.c_void_p()
    dg.chk(L.dMeshCreateBlock(dg.ptr(np.asarray(npoints, np.int32)), dg.ptr(np.asarray((0, 1, 0, 1, 0, 1), np.float64)),
                              ctypes.c_double(0.1), ctypes.c_uint64(1), ctypes.byref(mesh)))
    fs = ctypes.c_void_p()
    dg.chk(L.dFSCreate(mesh, None, ctypes.byref(fs)))
    dg.chk(L.dFSSetDegree(fs, ctypes.c_int32(degree), dg.ptr(np.ascontiguousarray(elem_degree, np.int32))))
    for s in dirichlet:
        dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(s), ctypes.c_int(dg.dFSBSTATUS_DIRICHLET)))
    dg.chk(L.dFSBuildSpace(fs))
    sz = [ctypes.c_int32() for _ in range(5)]
    dg.chk(L.dFSGetSizes(fs, *[ctypes.byref(s) for s in sz]))
    nnz = ctypes.c_int64()
    dg.chk(L.dFSGetElementAssemblyMatrix(fs, ctypes.byref(nnz), None, None, None))
    p = np.zeros(sz[2].value + 1, np.int32); c = np.zeros(nnz.value, np.int32); v = np.zeros(nnz.value)
    dg.chk(L.dFSGetElementAssemblyMatrix(fs, None, dg.ptr(p), dg.ptr(c), dg.ptr(v)))
    L.dFSDestroy(ctypes.byref(fs)); L.dMeshDestroy(ctypes.byref(mesh))
    return sz[0].value, sz[1].value, p, c, v


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_hp_element_assembly_matrix_matches_oracle(L, seed):
    """per-element orders 2..8 (config-2 style): interpolation-constrained E, sparsity bit-exact with the
    oracle's extension, weights within 1e-14."""
    npoints = (4, 4, 3)
    ed = np.random.default_rng(seed).integers(2, 9, size=3 * 3 * 2).astype(np.int32)
    n, nc, p, c, v = host_ecsr(npoints, 4, ed)
    o = po.FS(*npoints, degree=4, perturb=0.1, seed=1, elem_degree=ed)
    op_, oc, ov = o.ecsr()
    assert (n, nc) == (o.n, o.nc)
    np.testing.assert_array_equal(p, op_)
    np.testing.assert_array_equal(c, oc)
    np.testing.assert_allclose(v, ov, rtol=0, atol=1e-14)


def test_grf_parameters_match_oracle(L):
    g = dg.grf_create(64, 2.0, 0.1, 42)
    o = po.grf_make(64, 2.0, 0.1, 42)
    np.testing.assert_array_equal(g, o)


def test_errors_are_reported_not_aborted(L):
    mesh = ctypes.c_void_p()
    rc = L.dMeshCreateBlock(dg.ptr(np.asarray([1, 2, 2], np.int32)), dg.ptr(np.zeros(6)), ctypes.c_double(0),
                            ctypes.c_uint64(0), ctypes.byref(mesh))
    assert rc != 0 and b"vertices" in L.dGetLastError()


def test_facet_rules_host_side_match_oracle(L):
    """dFSGetFacetRule is host code (tensorquad.c:309-355 restated): same nodes and weights as the oracle"""
    for side in range(6):
        for order in range(0, 17, 2):
            n, w = dg.facet_rule(side, order)
            no, wo = po.facet_rule(side, order)
            np.testing.assert_allclose(n, no, rtol=0, atol=1e-15)
            np.testing.assert_allclose(w, wo, rtol=1e-15, atol=0)
    with pytest.raises(dg.DohpError):
        dg.facet_rule(6, 4)


def test_boundary_status_values(L):
    """the reference's dFSBStatus values (include/dohpfs.h:41-47): DIRICHLET and WEAK above the 16-bit count"""
    assert dg.dFSBSTATUS_DIRICHLET == 1 << 16 and dg.dFSBSTATUS_WEAK == 1 << 17
    mesh, fs = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dMeshCreateBlock(dg.ptr(np.asarray((3, 3, 3), np.int32)), dg.ptr(np.asarray((0, 1, 0, 1, 0, 1), np.float64)),
                              ctypes.c_double(0.1), ctypes.c_uint64(1), ctypes.byref(mesh)))
    dg.chk(L.dFSCreate(mesh, None, ctypes.byref(fs)))
    dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(200), ctypes.c_int(dg.dFSBSTATUS_WEAK | dg.dFSBSTATUS_DIRICHLET)))
    with pytest.raises(dg.DohpError):
        dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(400), ctypes.c_int(dg.dFSBSTATUS_WEAK)))
    with pytest.raises(dg.DohpError):
        dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(100), ctypes.c_int(1 << 20)))
    L.dFSDestroy(ctypes.byref(fs))
    L.dMeshDestroy(ctypes.byref(mesh))


def test_null_handles_are_errors_not_crashes(L):
    """every entry point that takes an object handle returns a nonzero dErr with a message for a NULL handle (and
    NULL or zero everywhere else) instead of dereferencing it: the reference's error convention (dCHK / dERROR,
    include/dohp.h:43-44; invalid input returns an error, never aborts). Runs without a GPU: each check comes
    before any device call."""
    import re
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "dohp_gb300.h")).read(), flags=re.S)
    handles = set(re.findall(r"typedef struct _p_\w+ \*(d\w+);", src))
    checked = []
    for m in re.finditer(r"dErr (d\w+)\(([^;]*?)\);", src, flags=re.S):
        name, params = m.group(1), [a.strip() for a in " ".join(m.group(2).split()).split(",") if a.strip()]
        if not params or name.endswith("Destroy"):
            continue
        first = params[0]
        if first.replace("const", "").split()[0] not in handles or "*" in first:
            continue
        rc = getattr(L, name)(*([None] * len(params)))
        assert rc != 0 and L.dGetLastError(), name
        checked.append(name)
    assert len(checked) > 80


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """without the built CUDA library the package raises instead of falling back to any CPU path"""
    monkeypatch.setattr(dg, "_lib", None)
    monkeypatch.setattr(dg, "LIB_PATH", str(tmp_path / "absent.so"))
    with pytest.raises(dg.DohpError, match="not built"):
        dg.lib()
    with pytest.raises(dg.DohpError):
        dg.FS((3, 3, 3), degree=2)


def test_refuses_spaces_beyond_32_bit_indices():
    """1e6 degree-8 elements with 3 components: 2.19e9 expanded values, refused before any allocation of that size"""
    with pytest.raises(dg.DohpError, match="32-bit"):
        host_fs((101, 101, 101), 8, bs=3)
