"""DHM files (src/viewer/dhm.c, src/fs/impls/cont/contviewdhm.c) on the CPU: the lookup3 checksum against Bob Jenkins'
published test values, the group layout of a written file walked by an independent reader of the HDF5 format written
here (superblock, object headers and their checksums, link messages), and the round trip of spaces and vectors through
the library's own reader: time steps, closure vectors bit for bit, and the space rebuilt from the file with the same
element-to-node map."""
import ctypes
import os
import struct

import numpy as np
import pytest

import dohp_gb300 as dg


@pytest.fixture(scope="module")
def L():
    import subprocess, sys
    subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    L = dg.lib()
    L.dHDF5Checksum.restype = ctypes.c_uint32
    L.dHDF5Checksum.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32]
    return L


def test_lookup3_published_values(L):
    # lookup3.c (Bob Jenkins, 2006), driver5
    assert L.dHDF5Checksum(b"", 0, 0) == 0xDEADBEEF
    assert L.dHDF5Checksum(b"", 0, 0xDEADBEEF) == 0xBD5B7DDE
    s = b"Four score and seven years ago"
    assert L.dHDF5Checksum(s, len(s), 0) == 0x17770551
    assert L.dHDF5Checksum(s, len(s), 1) == 0xCD628161


def lookup3(data, init=0):
    """the same hash in Python (independent restatement, for checking the file's checksums)"""
    M = 0xFFFFFFFF
    rot = lambda x, k: ((x << k) | (x >> (32 - k))) & M
    a = b = c = (0xDEADBEEF + len(data) + init) & M
    k, n = bytes(data), len(data)
    w = lambda i: k[i] | (k[i + 1] << 8) | (k[i + 2] << 16) | (k[i + 3] << 24)
    while n > 12:
        a, b, c = (a + w(0)) & M, (b + w(4)) & M, (c + w(8)) & M
        a = (a - c) & M; a ^= rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= rot(b, 4); b = (b + a) & M
        k, n = k[12:], n - 12
    if n == 0:
        return c
    k = k + bytes(12 - n)  # the last block, zero padded (hashlittle adds only the bytes present)
    a, b, c = (a + w(0)) & M, (b + w(4)) & M, (c + w(8)) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


def walk(buf):
    """groups and datasets of a version-2-superblock HDF5 file: {path: kind}; every checksum verified"""
    assert buf[:8] == b"\x89HDF\r\n\x1a\n" and buf[8] == 2
    assert struct.unpack_from("<I", buf, 44)[0] == lookup3(buf[:44])
    eof, root = struct.unpack_from("<QQ", buf, 28)
    assert eof == len(buf)
    out = {}

    def obj(addr, path):
        assert buf[addr:addr + 4] == b"OHDR" and buf[addr + 4] == 2
        flags = buf[addr + 5]
        csz = 1 << (flags & 3)
        chunk = int.from_bytes(buf[addr + 6:addr + 6 + csz], "little")
        m0 = addr + 6 + csz
        end = m0 + chunk
        assert struct.unpack_from("<I", buf, end)[0] == lookup3(buf[addr:end])
        kinds, links = set(), []
        p = m0
        while p + 4 <= end:
            mtype, msize = buf[p], struct.unpack_from("<H", buf, p + 1)[0]
            body = p + 4
            kinds.add(mtype)
            if mtype == 0x06:
                nlen = buf[body + 2]
                name = buf[body + 3:body + 3 + nlen].decode()
                links.append((name, struct.unpack_from("<Q", buf, body + 3 + nlen)[0]))
            p = body + msize
        out[path or "/"] = "dataset" if 0x08 in kinds else "group" if 0x02 in kinds else "type"
        for name, a in links:
            obj(a, path + "/" + name)

    obj(root, "")
    return out


def build_fs(L, npts, degree, bs, dirichlet=(100, 200, 300), elem_degree=None):
    mesh, fs, jac = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dJacobiCreate(ctypes.byref(jac)))
    dg.chk(L.dMeshCreateBlock(dg.ptr(np.asarray(npts, np.int32)), dg.ptr(np.array([0, 1, 0, 1, 0, 1.0])), ctypes.c_double(0.1),
                              ctypes.c_uint64(3), ctypes.byref(mesh)))
    dg.chk(L.dFSCreate(mesh, jac, ctypes.byref(fs)))
    ed = None if elem_degree is None else np.ascontiguousarray(elem_degree, np.int32)
    dg.chk(L.dFSSetDegree(fs, ctypes.c_int32(degree), dg.ptr(ed)))
    dg.chk(L.dFSSetBlockSize(fs, ctypes.c_int32(bs)))
    for sid in dirichlet:
        dg.chk(L.dFSRegisterBoundary(fs, ctypes.c_int32(sid), ctypes.c_int(dg.dFSBSTATUS_DIRICHLET)))
    dg.chk(L.dFSBuildSpace(fs))
    return mesh, fs, jac


def sizes(L, fs):
    s = [ctypes.c_int32() for _ in range(5)]
    dg.chk(L.dFSGetSizes(fs, *[ctypes.byref(x) for x in s]))
    return [x.value for x in s]


def emap(L, fs):
    n, nc, nexp, bs, ne = sizes(L, fs)
    em, xs = np.zeros(nexp, np.int32), np.zeros(ne + 1, np.int32)
    dg.chk(L.dFSGetExpandedMap(fs, dg.ptr(em), dg.ptr(xs)))
    return em, xs


def test_write_walk_and_read_back(L, tmp_path):
    path = str(tmp_path / "out.dhm")
    ed = np.random.default_rng(1).integers(2, 5, size=27).astype(np.int32)
    mesh, fs, jac = build_fs(L, (4, 4, 4), 3, 3, elem_degree=ed)
    mesh2, fs2, _ = build_fs(L, (5, 4, 3), 2, 1, dirichlet=(100,))
    n, nc, nexp, bs, ne = sizes(L, fs)
    rng = np.random.default_rng(7)
    u = [rng.standard_normal(nc * bs) for _ in range(2)]
    p = rng.standard_normal(sizes(L, fs2)[1])
    v = ctypes.c_void_p()
    dg.chk(L.dViewerDHMOpen(path.encode(), ctypes.c_int(1), ctypes.byref(v)))
    dg.chk(L.dViewerDHMSetTimeUnits(v, b"s", ctypes.c_double(1.0)))
    dg.chk(L.dFSViewDHM(fs, b"velocity", v))
    dg.chk(L.dFSViewDHM(fs2, b"pressure", v))
    for k, t in enumerate((0.5, 1.25)):
        dg.chk(L.dViewerDHMSetTime(v, ctypes.c_double(t)))
        dg.chk(L.dVecViewDHM(fs, b"u", dg.ptr(u[k]), ctypes.c_int(0), v))
    dg.chk(L.dVecViewDHM(fs2, b"p", dg.ptr(p), ctypes.c_int(0), v))
    assert L.dVecViewDHM(fs2, b"p", dg.ptr(p), ctypes.c_int(0), v) != 0  # one vector per name and step
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    # layout, through an independent reader of the format (every checksum checked)
    tree = walk(open(path, "rb").read())
    for g in ("/dohp", "/dohp/mesh", "/dohp/fs", "/dohp/step", "/dohp/type", "/dohp/step/000", "/dohp/step/001", "/dohp/mesh/mesh0/000",
              "/dohp/mesh/mesh1/000"):
        assert tree[g] == "group", g
    for d in ("/dohp/fs/velocity", "/dohp/fs/pressure", "/dohp/step/000/u", "/dohp/step/001/u", "/dohp/step/001/p",
              "/dohp/mesh/mesh0/000/vertices", "/dohp/mesh/mesh0/000/hexes", "/dohp/mesh/mesh0/000/velocity_degree"):
        assert tree[d] == "dataset", d
    for t in ("Units_type", "Time_type", "BoundingBox_type", "FS_type", "Vec_type"):
        assert tree["/dohp/type/" + t] == "type"
    # read back through the library
    dg.chk(L.dViewerDHMOpen(path.encode(), ctypes.c_int(0), ctypes.byref(v)))
    ns = ctypes.c_int32()
    dg.chk(L.dViewerDHMGetSteps(v, ctypes.byref(ns), None))
    times = np.zeros(ns.value)
    dg.chk(L.dViewerDHMGetSteps(v, ctypes.byref(ns), dg.ptr(times)))
    np.testing.assert_array_equal(times, [0.5, 1.25])
    mesh3, fs3 = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSLoadDHM(v, b"velocity", jac, ctypes.byref(mesh3), ctypes.byref(fs3)))
    assert sizes(L, fs3) == sizes(L, fs)
    for a, b in zip(emap(L, fs3), emap(L, fs)):
        np.testing.assert_array_equal(a, b)
    for k in range(2):
        dg.chk(L.dViewerDHMSetTimeStep(v, ctypes.c_int32(k)))
        t = ctypes.c_double()
        dg.chk(L.dViewerDHMGetTime(v, ctypes.byref(t)))
        assert t.value == (0.5, 1.25)[k]
        got = np.zeros(nc * bs)
        dg.chk(L.dVecLoadDHM(v, b"u", fs3, dg.ptr(got), ctypes.c_int(0)))
        np.testing.assert_array_equal(got, u[k])
    assert L.dVecLoadDHM(v, b"p", fs3, dg.ptr(np.zeros(nc * bs)), ctypes.c_int(0)) != 0  # p is in step 1 only, and on the other space
    mesh4, fs4 = ctypes.c_void_p(), ctypes.c_void_p()
    dg.chk(L.dFSLoadDHM(v, b"pressure", jac, ctypes.byref(mesh4), ctypes.byref(fs4)))
    got = np.zeros(sizes(L, fs4)[1])
    dg.chk(L.dVecLoadDHM(v, b"p", fs4, dg.ptr(got), ctypes.c_int(0)))
    np.testing.assert_array_equal(got, p)
    assert L.dViewerDHMSetTimeStep(v, ctypes.c_int32(2)) != 0
    assert L.dFSLoadDHM(v, b"nothere", jac, ctypes.byref(mesh4), ctypes.byref(fs4)) != 0
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    for f in (fs, fs2, fs3):
        L.dFSDestroy(ctypes.byref(f))
    for m in (mesh, mesh2, mesh3):
        L.dMeshDestroy(ctypes.byref(m))


def test_not_an_hdf5_file(L, tmp_path):
    bad = tmp_path / "bad.dhm"
    bad.write_bytes(b"not hdf5" * 10)
    v = ctypes.c_void_p()
    assert L.dViewerDHMOpen(str(bad).encode(), ctypes.c_int(0), ctypes.byref(v)) != 0
    assert b"not an HDF5 file" in L.dGetLastError()


def test_damaged_files_are_refused(L, tmp_path):
    """a flipped byte in the superblock or in an object header fails its checksum, a truncated file is refused; no
    damaged file is read as data"""
    path = tmp_path / "ok.dhm"
    mesh, fs, jac = build_fs(L, (3, 3, 3), 2, 1)
    u = np.random.default_rng(3).standard_normal(sizes(L, fs)[1])
    v = ctypes.c_void_p()
    dg.chk(L.dViewerDHMOpen(str(path).encode(), ctypes.c_int(1), ctypes.byref(v)))
    dg.chk(L.dFSViewDHM(fs, b"f", v))
    dg.chk(L.dViewerDHMSetTime(v, ctypes.c_double(0.0)))
    dg.chk(L.dVecViewDHM(fs, b"u", dg.ptr(u), ctypes.c_int(0), v))
    dg.chk(L.dViewerDestroy(ctypes.byref(v)))
    raw = bytearray(path.read_bytes())

    def refused(data, what):
        bad = tmp_path / "bad.dhm"
        bad.write_bytes(bytes(data))
        w = ctypes.c_void_p()
        if L.dViewerDHMOpen(str(bad).encode(), ctypes.c_int(0), ctypes.byref(w)) != 0:
            assert what.encode() in L.dGetLastError(), L.dGetLastError()
            return
        m2, f2 = ctypes.c_void_p(), ctypes.c_void_p()
        rc = L.dFSLoadDHM(w, b"f", jac, ctypes.byref(m2), ctypes.byref(f2))
        L.dViewerDestroy(ctypes.byref(w))
        assert rc != 0 and what.encode() in L.dGetLastError(), L.dGetLastError()

    sb = bytearray(raw)
    sb[20] ^= 0xFF  # inside the superblock's addresses
    refused(sb, "superblock checksum")
    heads = [i for i in range(len(raw) - 4) if raw[i:i + 4] == b"OHDR"]
    assert len(heads) > 5
    for h in heads[:3]:
        oh = bytearray(raw)
        oh[h + 12] ^= 0x55  # inside the header's messages
        refused(oh, "checksum")
    refused(raw[:len(raw) // 2], "")
    L.dFSDestroy(ctypes.byref(fs))
    L.dMeshDestroy(ctypes.byref(mesh))
