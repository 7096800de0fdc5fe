"""Meshes given by their entities (dMeshCreateFromConnectivity) through the product's C ABI on the CPU (no GPU needed):
the hand-built MOAB meshes of the reference's fs tests, pinned to what the reference verifies or prints about them:
ex1.c's hand-verified adjacency tables (src/fs/tests/ex1.c:106-138), the closure numbering, Q1 coordinates and nodal
coordinates of cunit-identity-0 / cunit-affine-0, the sub-element mesh and closure coordinates of fsex4-submesh-p1 /
-p2, and the space sizes of the fs-mf-projection targets (mesh data and printed numbers extracted into tests/golden)."""
import ctypes
import os

import numpy as np
import pytest

import dohp_gb300 as dg
import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))


def gold(name):
    return np.load(os.path.join(HERE, "golden", name + ".npz"))


@pytest.fixture(scope="module")
def L():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    return dg.lib()


def mesh_of(prefix, vtx=None):
    g = gold("hex_meshes")
    v = g[prefix + ("vtx_base" if prefix == "cunit_" else "vtx")] if vtx is None else vtx
    return dg.Mesh(v, g[prefix + "econn"], g[prefix + "fconn"], g[prefix + "rconn"])


class HostFS:
    """a dFS built on the host only (dFSBuildSpace, no device upload)"""

    def __init__(self, L, mesh, degree, bs=1):
        self.L, self._mesh = L, mesh
        self.h = ctypes.c_void_p()
        dg.chk(L.dFSCreate(mesh.h, None, ctypes.byref(self.h)))
        dg.chk(L.dFSSetDegree(self.h, ctypes.c_int32(degree), None))
        dg.chk(L.dFSSetBlockSize(self.h, ctypes.c_int32(bs)))
        dg.chk(L.dFSBuildSpace(self.h))
        sz = [ctypes.c_int32() for _ in range(5)]
        dg.chk(L.dFSGetSizes(self.h, *[ctypes.byref(s) for s in sz]))
        self.n, self.nc, self.nexp, self.bs, self.nelem = [s.value for s in sz]

    def emap(self):
        em, xs = np.zeros(self.nexp, np.int32), np.zeros(self.nelem + 1, np.int32)
        dg.chk(self.L.dFSGetExpandedMap(self.h, dg.ptr(em), dg.ptr(xs)))
        return em, xs

    def nodal(self, expanded=True):
        out = np.zeros(((self.nexp if expanded else self.nc), 3))
        f = self.L.dFSGetNodalCoordinatesExpanded if expanded else self.L.dFSGetNodalCoordinatesGlobal
        dg.chk(f(self.h, dg.ptr(out), ctypes.c_int(0)))
        return out

    def submesh(self):
        ns, nv, nc = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        dg.chk(self.L.dFSGetSubElementMeshSize(self.h, ctypes.byref(ns), ctypes.byref(nv), ctypes.byref(nc)))
        topo, off, ind = np.zeros(ns.value, np.int32), np.zeros(ns.value + 1, np.int32), np.zeros(nc.value, np.int32)
        dg.chk(self.L.dFSGetSubElementMesh(self.h, ns, nc, dg.ptr(topo), dg.ptr(off), dg.ptr(ind)))
        return nv.value, topo, off, ind

    def __del__(self):
        self.L.dFSDestroy(ctypes.byref(self.h))


@pytest.mark.parametrize("vtx", ["ex1_vtx_parametric", "ex1_vtx_affine"])
def test_ex1_adjacency_as_verified_by_the_reference(L, vtx):
    """verifyAdjacencies (ex1.c:106-138): toff, adjoff, adjind and adjperm of the two-hex mesh, entry by entry"""
    g = gold("hex_meshes")
    m = dg.Mesh(g[vtx], g["ex1_econn"], g["ex1_fconn"], g["ex1_rconn"])
    toff, adjoff, adjind, adjperm = m.adjacency()
    np.testing.assert_array_equal(toff, g["ex1_toff"])
    np.testing.assert_array_equal(adjoff, g["ex1_adjoff"])
    np.testing.assert_array_equal(adjind, g["ex1_adjind"])
    np.testing.assert_array_equal(adjperm, g["ex1_adjperm"])


def test_cunit_identity_closure_and_coordinates(L):
    """cunit-identity-0 (src/fs/tests/cunit.c, degree 2, no boundary sets, natural ordering): the expanded vector of
    closure indices + 1000 (-expanded_view), the Q1 coordinate vector (-cexp_view: the degree-1 space's nodes) and
    the coordinates of the expanded nodes (-nce_view); re-expanding the global nodal coordinates gives the expanded
    ones (-nce_compare)"""
    g = gold("cunit_identity_0")
    m = mesh_of("cunit_")
    fs = HostFS(L, m, 2)
    assert (fs.n, fs.nc, fs.nexp, fs.nelem) == (45, 45, 54, 2)
    em, xs = fs.emap()
    np.testing.assert_array_equal(xs, [0, 27, 54])
    np.testing.assert_array_equal(1000 + em, g["expanded"])
    np.testing.assert_allclose(HostFS(L, m, 1).nodal(), g["cexp"], rtol=0, atol=1e-15)
    nce = fs.nodal()
    np.testing.assert_allclose(nce, g["nce"], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(fs.nodal(expanded=False)[em], nce)


def test_cunit_affine_nodal_coordinates(L):
    """cunit-affine-0: the same mesh with its vertices mapped by x -> A x + b (cunit.c:100-102), nodal coordinates
    to the printed 6 significant digits"""
    g, hm = gold("cunit_affine_0"), gold("hex_meshes")
    v = hm["cunit_vtx_base"].reshape(-1, 3) @ hm["cunit_affine_A"].T + hm["cunit_affine_b"]
    fs = HostFS(L, mesh_of("cunit_", vtx=v), 2)
    nce = fs.nodal()
    np.testing.assert_allclose(nce, g["nce"], rtol=5e-6, atol=0)
    em, _ = fs.emap()
    np.testing.assert_allclose(fs.nodal(expanded=False)[em], nce, rtol=1e-14, atol=1e-13)


@pytest.mark.parametrize("degree,name", [(1, "fsex4_submesh_p1"), (2, "fsex4_submesh_p2")])
def test_fsex4_submesh(L, degree, name):
    """fsex4-submesh-p1 / -p2 (src/fs/tests/fsex4.c: three hexahedra around a shared edge): sub-element offsets and
    connectivity (dFSGetSubElementMesh) and the closure nodes' coordinates (dFSGetNodalCoordinatesGlobal)"""
    g = gold(name)
    fs = HostFS(L, mesh_of("fsex4_"), degree)
    nverts, topo, off, ind = fs.submesh()
    assert nverts == fs.nc == [14, 57][degree - 1]
    assert np.all(topo == 7)
    np.testing.assert_array_equal(off, g["off"])
    np.testing.assert_array_equal(ind, g["conn"])
    np.testing.assert_allclose(fs.nodal(expanded=False).ravel(), g["coords"], rtol=5e-6, atol=1e-12)


@pytest.mark.parametrize("name,degree", [("fs_mf_projection_v1", 5), ("fs_mf_op_proj_1", 6)])
def test_ex1_space_sizes(L, name, degree):
    """ex1.c's useFS line "expanded size, global size" on its two-hex parametric mesh at the targets' degrees
    (fs-mf-op-proj-0 uses degree 9, above the largest degree built here, 8: refused)"""
    g, hm = gold(name), gold("hex_meshes")
    m = dg.Mesh(hm["ex1_vtx_parametric"], hm["ex1_econn"], hm["ex1_fconn"], hm["ex1_rconn"])
    fs = HostFS(L, m, degree)
    assert [fs.nexp, fs.n] == list(g["sizes"])
    with pytest.raises(dg.DohpError, match="degree 9 out of range"):
        HostFS(L, m, 9)


def test_connectivity_errors(L):
    hm = gold("hex_meshes")
    v, e, f, r = (hm["cunit_" + k] for k in ("vtx_base", "econn", "fconn", "rconn"))
    with pytest.raises(dg.DohpError, match="no face on side"):
        dg.Mesh(v, e, f[:-4], r)
    with pytest.raises(dg.DohpError, match="no edge on side"):
        dg.Mesh(v, e[:-2], f, r)
    bad = r.copy()
    bad[3] = 99
    with pytest.raises(dg.DohpError, match="out of range"):
        dg.Mesh(v, e, f, bad)
    with pytest.raises(dg.DohpError, match="repeats"):
        dg.Mesh(v, np.concatenate([e, e[:2]]), f, r)
    # no boundary sets on such a mesh; the block-lattice parts refuse it
    m = mesh_of("cunit_")
    h = ctypes.c_void_p()
    dg.chk(L.dFSCreate(m.h, None, ctypes.byref(h)))
    dg.chk(L.dFSSetDegree(h, ctypes.c_int32(2), None))
    dg.chk(L.dFSRegisterBoundary(h, ctypes.c_int32(100), ctypes.c_int(dg.dFSBSTATUS_DIRICHLET)))
    assert L.dFSBuildSpace(h) != 0
    assert b"a mesh from connectivity has none" in L.dGetLastError()
    L.dFSDestroy(ctypes.byref(h))


@pytest.mark.parametrize("degree,name", [(1, "fsex4_submesh_p1_read"), (2, "fsex4_submesh_p2")])
def test_fsex4_read_back(L, tmp_path, degree, name):
    """fsex4-submesh-p1-read / -p2-read: the space and its vector 0.1 i (FSEx4FillVec, fsex4.c:85-97) written to a
    DHM file at time 0.1 and read back (dFSLoadDHM rebuilds the mesh from the entities written): one step at time
    0.1, the same sub-element mesh and closure coordinates, and the vector"""
    g = gold(name)
    fs = HostFS(L, mesh_of("fsex4_"), degree)
    x = 0.1 * np.arange(fs.nc)
    path = str(tmp_path / "fsex4.dhm").encode()
    v = ctypes.c_void_p()
    dg.chk(L.dViewerDHMOpen(path, ctypes.c_int(1), ctypes.byref(v)))
    dg.chk(L.dViewerDHMSetTime(v, ctypes.c_double(0.1)))
    dg.chk(L.dFSViewDHM(fs.h, b"dFS_0", v))
    dg.chk(L.dVecViewDHM(fs.h, b"Vec_global_0", dg.ptr(x), ctypes.c_int(0), v))
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    dg.chk(L.dViewerDHMOpen(path, ctypes.c_int(0), ctypes.byref(v)))
    ns = ctypes.c_int32()
    dg.chk(L.dViewerDHMGetSteps(v, ctypes.byref(ns), None))
    times = np.zeros(ns.value)
    dg.chk(L.dViewerDHMGetSteps(v, ctypes.byref(ns), dg.ptr(times)))
    np.testing.assert_array_equal(times, g["time"])
    mesh2, h2 = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSLoadDHM(v, b"dFS_0", None, ctypes.byref(mesh2), ctypes.byref(h2)))
    back = HostFS.__new__(HostFS)
    back.L, back._mesh, back.h = L, None, h2
    sz = [ctypes.c_int32() for _ in range(5)]
    dg.chk(L.dFSGetSizes(h2, *[ctypes.byref(s) for s in sz]))
    back.n, back.nc, back.nexp, back.bs, back.nelem = [s.value for s in sz]
    nverts, topo, off, ind = back.submesh()
    np.testing.assert_array_equal(off, g["off_read"])
    np.testing.assert_array_equal(ind, g["conn_read"])
    np.testing.assert_allclose(back.nodal(expanded=False).ravel(), g["coords_read"], rtol=5e-6, atol=1e-12)
    got = np.zeros(back.nc)
    dg.chk(L.dVecLoadDHM(v, b"Vec_global_0", h2, dg.ptr(got), ctypes.c_int(0)))
    np.testing.assert_array_equal(got, x)
    if "loaded" in g:
        np.testing.assert_allclose(got, g["loaded"], rtol=1e-12, atol=1e-15)
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    del back
    L.dMeshDestroy(ctypes.byref(mesh2))


def product_ecsr(L, mesh, degree, elem_degree=None):
    h = ctypes.c_void_p()
    dg.chk(L.dFSCreate(mesh.h, None, ctypes.byref(h)))
    ed = None if elem_degree is None else np.ascontiguousarray(elem_degree, np.int32)
    dg.chk(L.dFSSetDegree(h, ctypes.c_int32(degree), dg.ptr(ed)))
    dg.chk(L.dFSBuildSpace(h))
    sz = [ctypes.c_int32() for _ in range(5)]
    dg.chk(L.dFSGetSizes(h, *[ctypes.byref(s) for s in sz]))
    nnz = ctypes.c_int64()
    dg.chk(L.dFSGetElementAssemblyMatrix(h, ctypes.byref(nnz), None, None, None))
    p, c, v = np.zeros(sz[2].value + 1, np.int32), np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    dg.chk(L.dFSGetElementAssemblyMatrix(h, None, dg.ptr(p), dg.ptr(c), dg.ptr(v)))
    L.dFSDestroy(ctypes.byref(h))
    return sz[0].value, sz[1].value, p, c, v


@pytest.mark.parametrize("prefix,vtx", [("ex1_", "ex1_vtx_parametric"), ("fsex4_", "fsex4_vtx"), ("cunit_", "cunit_vtx_base")])
def test_element_assembly_matches_the_oracle_at_every_degree(L, prefix, vtx):
    """E on the hand-built meshes against the oracle's restatement (its own adjacency search, or_fs_create_conn), at
    every degree 1..8 and with per-element degrees (interpolation-constrained rows across the shared edge and faces):
    sparsity and map bit-exact, weights to 1e-14"""
    hm = gold("hex_meshes")
    conn = (hm[vtx], hm[prefix + "econn"], hm[prefix + "fconn"], hm[prefix + "rconn"])
    mesh = dg.Mesh(*conn)
    nr = len(conn[3]) // 8
    cases = [(p, None) for p in range(1, 9)]
    cases += [(8, np.random.default_rng(s).integers(1, 9, size=nr).astype(np.int32)) for s in range(6)]
    for degree, ed in cases:
        n, nc, p, c, v = product_ecsr(L, mesh, degree, ed)
        o = po.FS(0, 0, 0, degree=degree, elem_degree=ed, conn=conn)
        op_, oc, ov = o.ecsr()
        assert (n, nc) == (o.n, o.nc), (degree, ed)
        np.testing.assert_array_equal(p, op_)
        np.testing.assert_array_equal(c, oc)
        np.testing.assert_allclose(v, ov, rtol=0, atol=1e-14)


def test_oracle_adjacency_and_closure_on_the_reference_meshes():
    """the oracle's own adjacency search reproduces ex1.c's hand-verified tables, and its closure numbering the
    cunit-identity-0 expanded vector"""
    hm = gold("hex_meshes")
    o = po.FS(0, 0, 0, degree=2, conn=(hm["ex1_vtx_parametric"], hm["ex1_econn"], hm["ex1_fconn"], hm["ex1_rconn"]))
    ao, ai, ap = o.adjacency()
    np.testing.assert_array_equal(ao, hm["ex1_adjoff"])
    np.testing.assert_array_equal(ai, hm["ex1_adjind"])
    np.testing.assert_array_equal(ap, hm["ex1_adjperm"])
    o = po.FS(0, 0, 0, degree=2, conn=(hm["cunit_vtx_base"], hm["cunit_econn"], hm["cunit_fconn"], hm["cunit_rconn"]))
    np.testing.assert_array_equal(1000 + o.emap(), gold("cunit_identity_0")["expanded"])
