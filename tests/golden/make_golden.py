"""Extract golden vectors from the dohp reference's own test outputs (refout files) into small
fixtures under tests/golden/. Run in a checkout where the dohp source tree is available:

    python tests/golden/make_golden.py /path/to/dohp

The refout files are read as text (they are the reference's expected stdout for its CTest
targets, see src/*/tests/CMakeLists.txt). Only numbers are extracted; large matrices are
subsampled to keep the fixtures small. Nothing at test time reads the reference tree.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = re.compile(r"[-+]?\d+\.\d+(?:e[-+]?\d+)?|[-+]?\d+(?:e[-+]?\d+)?")


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read().splitlines()


def explicit_bases(root, name, full_elems=(0, 1), head_rows=16):
    """jacobi-3-tensor-{gauss,lobatto}: interp (Q,P), grad (Q,3P), mass (P,P) per element."""
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    out = {}
    elem = -1
    i = 0
    while i < len(lines):
        m = re.match(r"(Interpolation|Gradient|Mass) matrix of size \((\d+),(\d+)(\*3)?\)", lines[i])
        if not m:
            i += 1
            continue
        kind, rows, cols = m.group(1), int(m.group(2)), int(m.group(3)) * (3 if m.group(4) else 1)
        if kind == "Interpolation":
            elem += 1
        mat = np.array([[float(v) for v in lines[i + 1 + r].split()] for r in range(rows)])
        assert mat.shape == (rows, cols)
        if elem in full_elems or kind == "Mass":
            out[f"e{elem}_{kind.lower()}"] = mat
        else:
            out[f"e{elem}_{kind.lower()}_head"] = mat[:head_rows]
        i += 1 + rows
    return out


def modal_values(root, name):
    """jacobi-2-modal-*: per element (modal orders 0..3) the values of the modes (weights 2, 3, 5, 7, ... as
    ex2.c sets them) at the rule points, and the modes after the mass matrix (INTERP_TRANSPOSE of the weighted
    values)."""
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    out, elem, cur = {}, -1, None
    for ln in lines:
        if ln.startswith("Values of"):
            elem += 1
            cur = out.setdefault(f"e{elem}_values", [])
        elif ln.startswith("Modal values after"):
            cur = out.setdefault(f"e{elem}_mass_applied", [])
        else:
            cur.extend(float(v) for v in ln.split(":", 1)[1].split())
    return {k: np.array(v) for k, v in out.items()}


def c_arrays(root, rel, names):
    """integer / real array initialisers {..} of the named C arrays in a reference source file (test input data)"""
    src = "\n".join(read(root, rel))
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name in names:
        m = re.search(r"\b" + re.escape(name) + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\}\s*[;,]", src, re.S)
        assert m, (rel, name)
        out[name] = np.array([float(v) for v in NUM.findall(m.group(1))])
    return out


def hex_meshes(root):
    """The hand-built MOAB meshes of the fs tests (vertices, edges, faces, hexahedra in creation order) and the
    adjacency ex1.c verifies by hand (verifyAdjacencies, src/fs/tests/ex1.c:106-138); the affine deformation of
    cunit.c"""
    a = c_arrays(root, "src/fs/tests/ex1.c", ["vtx_affine", "vtx_parametric", "rconn", "fconn", "econn", "toff", "adjoff",
                                              "adjind", "adjperm"])
    out = {"ex1_" + k: v for k, v in a.items()}
    b = c_arrays(root, "src/fs/tests/cunit.c", ["vtx_base", "rconn", "fconn", "econn"])
    out.update({"cunit_" + k: v for k, v in b.items()})
    src = "\n".join(read(root, "src/fs/tests/cunit.c"))
    m = re.search(r"tmpctx\s*=\s*\{\.A\s*=\s*\{(.*?)\}\s*,\s*\.b\s*=\s*\{(.*?)\}\s*\}", src, re.S)
    out["cunit_affine_A"] = np.array([float(v) for v in NUM.findall(m.group(1))]).reshape(3, 3)
    out["cunit_affine_b"] = np.array([float(v) for v in NUM.findall(m.group(2))])
    c = c_arrays(root, "src/fs/tests/fsex4.c", ["vtx", "econn", "fconn", "rconn"])
    out.update({"fsex4_" + k: v for k, v in c.items()})
    return out


def cunit(root, name):
    """cunit-*: the expanded vector of closure indices + 1000, the expanded (Q1) coordinates and the coordinates of the
    expanded nodes (degree 2 on the two-hex mesh)"""
    lines = read(root, f"src/fs/tests/refout/{name}.refout")
    out, key = {}, None
    for ln in lines:
        if ln.startswith("Expanded vector"):
            key = "expanded"
        elif ln.startswith("Expanded coordinate vector"):
            key = "cexp"
        elif ln.startswith("Nodal coordinates in expanded space"):
            key = "nce"
        elif ln.startswith("Comparison of"):
            key = None
        elif key == "expanded" and re.fullmatch(r"\s*\d+(\.\d+)?\s*", ln):
            out.setdefault(key, []).append(float(ln))
        elif key in ("cexp", "nce") and ln.startswith("[0]"):
            out.setdefault(key, []).append([float(v) for v in ln.split(":", 1)[1].split()])
    return {k: np.array(v) for k, v in out.items()}


def submesh(root, name):
    """fsex4-submesh-*: sub-element offsets and connectivity, closure node coordinates; with -read_back the same
    printed again from the space read back from the DHM file (suffix _read), the file's step time and, with
    -read_back_vec, the vector read back"""
    lines = read(root, f"src/fs/tests/refout/{name}.refout")
    out, key, sfx = {}, None, ""
    for ln in lines:
        m = re.match(r"\[0\] step 0\s+time (\S+)", ln)
        if m:
            out["time"] = [float(m.group(1))]
        if ln.startswith("Offsets for"):
            sfx = "_read" if "off" in out else ""
            key = "off"
        elif ln.startswith("Connectivity"):
            key = "conn"
        elif ln.startswith("Coordinates"):
            key = "coords"
        elif ln.startswith("Loaded vector"):
            key, sfx = "loaded", ""
        elif ln.startswith("[0]"):
            key = None
        elif key in ("off", "conn") and re.match(r"\s*\d+:", ln):
            out.setdefault(key + sfx, []).extend(int(v) for v in ln.split(":", 1)[1].split())
        elif key in ("coords", "loaded") and re.fullmatch(r"\s*-?[\d.e+-]+\s*", ln):
            out.setdefault(key + sfx, []).append(float(ln))
    return {k: np.array(v) for k, v in out.items()}


def projection(root, name):
    """fs-mf-projection-* / fs-mf-op-proj-*: sizes, the sums of ex1.c's useFS, the SNES function norms and the
    projection residual norms"""
    lines = read(root, f"src/fs/tests/refout/{name}.refout")
    out = {"snes": []}
    for ln in lines:
        m = re.match(r"expanded size (\d+), global size (\d+)", ln)
        if m:
            out["sizes"] = [int(m.group(1)), int(m.group(2))]
        m = re.match(r"\|x\| = (\S+), \|g\| = (\S+), \|y\| = (\S+)", ln)
        if m:
            out["sums"] = [float(m.group(k)) for k in (1, 2, 3)]
        m = re.match(r"\s*\d+ SNES Function norm (< 1.e-11|\S+)", ln)
        if m:
            out["snes"].append(0.0 if m.group(1).startswith("<") else float(m.group(1)))
        m = re.match(r"(Algebraic|Pointwise|Gradient) .*\|x\|_1 (\S+)\s+\|x\|_2 (\S+)\s+\|x\|_inf (\S+)", ln)
        if m:
            out[m.group(1).lower()] = [float(m.group(k)) for k in (2, 3, 4)]
    return {k: np.array(v) for k, v in out.items()}


def sparse_bases(root, name, max_patches=4):
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    tabs = {}
    for ln in lines:
        m = re.match(r"elem (\d+):? +(?:patch (\d+) +)?(qidx\(patch,q\)|bidx\(patch,b\)|interp|deriv)\[ *(\d+)\]\[ *\d+: *\d+\]\s+(.*)", ln)
        if not m:
            continue
        e, patch, what, row, rest = int(m.group(1)), m.group(2), m.group(3), int(m.group(4)), m.group(5)
        vals = [float(v) for v in rest.split()]
        key = (e, what.split("(")[0], None if patch is None else int(patch))
        tabs.setdefault(key, {})[row] = vals
    out = {}
    for (e, what, patch), rows in tabs.items():
        if patch is not None and patch >= max_patches:
            continue
        arr = np.array([rows[r] for r in sorted(rows)])
        if what in ("qidx", "bidx"):
            out[f"e{e}_{what}"] = arr.astype(np.int32)
        else:
            out[f"e{e}_p{patch}_{what}"] = arr
    return out


def patches(root, name):
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    out = {}
    elem = -1
    for ln in lines:
        m = re.match(r"Element (\d+): npatches (\d+)\s+patchsize (\d+)", ln)
        if m:
            elem = int(m.group(1))
            out[f"e{elem}_shape"] = np.array([int(m.group(2)), int(m.group(3))], dtype=np.int32)
            continue
        m = re.match(r"\s+(indices|weights)\[ *(\d+)\]\[ *\d+: *\d+\]\s+(.*)", ln)
        if m:
            key = f"e{elem}_{m.group(1)}"
            vals = [float(v) for v in m.group(3).split()]
            out.setdefault(key, []).append(vals)
    return {k: (np.array(v, dtype=np.int32 if "indices" in k else np.float64) if isinstance(v, list) else v)
            for k, v in out.items()}


def interp_errors(root, name):
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    rows = []
    for ln in lines:
        m = re.match(r"L2 error for element +(\d+) \( *(\d+), *\d+, *\d+\) with rule \( *(\d+), *\d+, *\d+\) interp +(\S+), derivative +(\S+)", ln)
        if m:
            rows.append([int(m.group(1)), int(m.group(2)), int(m.group(3)), float(m.group(4)), float(m.group(5))])
    return {"rows": np.array(rows)}


def vec_after(lines, header):
    i = lines.index(header)
    vals = []
    for ln in lines[i + 1:]:
        s = ln.strip()
        if not s or s.startswith("Vector Object") or s.startswith("type:") or s.startswith("Process"):
            if vals and (s.startswith("Vector Object") is False and not s.startswith("type") and not s.startswith("Process")):
                break
            continue
        if re.match(r"^[A-Za-z]", s):
            break
        vals.append(float(s))
    return np.array(vals)


def bu0(root):
    lines = read(root, "src/fs/tests/refout/bu-0.refout")
    return {
        "closure": vec_after(lines, "Global closure vector, should be a sequence starting with 1000"),
        "homogeneous": vec_after(lines, "Expanded vector projected into homogeneous space"),
        "inhomogeneous": vec_after(lines, "Expanded vector projected into inhomogeneous space"),
        "coords": vec_after(lines, "Global coordinate vector (3 dofs per closure node)"),
    }


def sparse_efs(root, name="jacobi-3-tensor-sparse-gauss"):
    """jacobi-3-tensor-sparse-gauss (src/jacobi/tests/CMakeLists.txt:13, -just_view): per element basis size P, the
    first direction's SPARSE rule (points, weights) and the basis at it (interp, deriv rows, nodes)."""
    lines = read(root, f"src/jacobi/tests/refout/{name}.refout")
    out = {}
    i = 0
    rule = None
    while i < len(lines):
        ln = lines[i]
        m = re.match(r"\s*TensorRule with (\d+) nodes", ln)
        if m and rule is None:
            q = [float(v) for v in lines[i + 1].split("]")[-1].split()]
            w = [float(v) for v in lines[i + 2].split("]")[-1].split()]
            rule = (q, w)
        m = re.match(r"TensorBasis with rule=(\d+) basis=(\d+)", ln)
        if m:
            Q, P = int(m.group(1)), int(m.group(2))
            if f"P{P}_interp" not in out:
                rows = lambda k: np.array([[float(v) for v in lines[k + r].split("]")[-1].split()] for r in range(Q)])
                out[f"P{P}_q"], out[f"P{P}_w"] = np.array(rule[0]), np.array(rule[1])
                out[f"P{P}_interp"] = rows(i + 1)
                out[f"P{P}_deriv"] = rows(i + 1 + Q)
                out[f"P{P}_node"] = np.array([float(v) for v in lines[i + 1 + 2 * Q].split("]")[-1].split()])
            i += 1 + 2 * Q
            continue
        if ln.startswith("dEFS type"):
            rule = None
        i += 1
    return out


def solver_log(root, name):
    """stokes-q3q2-{scr,fgmres}, ellip-e0-*, elast-e0-b3-g01 (src/fs/tests/CMakeLists.txt:49-70, manufactured
    solutions on the default 4^3 block of [-1,1]^3): residual norms at the nodal interpolant of the exact solution
    (Stokes only), the first SNES function norm (at zero with the exact Dirichlet values), and the norm triples
    printed after the solve (stokes.c:1128-1133, 1161-1169; ellip.c:750-757; elast.c:539-546)."""
    lines = read(root, f"src/fs/tests/refout/{name}.refout")
    out = {}
    ksp, first_done = [], False
    for ln in lines:
        m = re.match(r"\s*(\d+) KSP Residual norm ([-+0-9.e]+)", ln)
        if m and not first_done:  # the first linear solve's history, up to 20 norms
            if int(m.group(1)) == len(ksp) and len(ksp) < 20:
                ksp.append(float(m.group(2)))
            else:
                first_done = True
        m = re.match(r"Norm of discrete (linear )?residual (?:for|at) exact solution (\S+)", ln)
        if m:
            out["linear_residual_exact" if m.group(1) else "residual_exact"] = np.array([float(m.group(2))])
        m = re.match(r"\s*0 SNES Function norm (\S+)", ln)
        if m and "fnorm0" not in out:
            out["fnorm0"] = np.array([float(m.group(1))])
        m = re.match(r"(Algebraic|Interpolation) residual\s+\|x\|_1 (\S+)\s+\|x\|_2 (\S+)\s+\|x\|_inf (\S+)", ln)
        m = m or re.match(r"Pointwise (velocity|solution|gradient|pressure) error\s+\|x\|_1 (\S+)\s+\|x\|_2 (\S+)\s+\|x\|_inf (\S+)", ln)
        if m:
            out[m.group(1).lower()] = np.array([float(m.group(k)) for k in (2, 3, 4)])
    if ksp:
        out["ksp_first_solve"] = np.array(ksp)
    return out


def main(root):
    fixtures = {
        "jacobi3_gauss": explicit_bases(root, "jacobi-3-tensor-gauss"),
        "jacobi3_lobatto": explicit_bases(root, "jacobi-3-tensor-lobatto"),
        "jacobi3_modal_gauss": explicit_bases(root, "jacobi-3-modal-gauss", full_elems=(0, 1, 2, 3), head_rows=64),
        "jacobi2_modal_fast_gauss": modal_values(root, "jacobi-2-modal-fast-gauss"),
        "jacobi2_modal_fast_lobatto": modal_values(root, "jacobi-2-modal-fast-lobatto"),
        "jacobi2_modal_sparse_gauss": modal_values(root, "jacobi-2-modal-sparse-gauss"),
        "hex_meshes": hex_meshes(root),
        "cunit_identity_0": cunit(root, "cunit-identity-0"),
        "cunit_affine_0": cunit(root, "cunit-affine-0"),
        "fsex4_submesh_p1": submesh(root, "fsex4-submesh-p1"),
        "fsex4_submesh_p1_read": submesh(root, "fsex4-submesh-p1-read"),
        "fsex4_submesh_p2": submesh(root, "fsex4-submesh-p2-read"),
        "fs_mf_projection_v1": projection(root, "fs-mf-projection-v1"),
        "fs_mf_projection_v3": projection(root, "fs-mf-projection-v3"),
        "fs_mf_projection_v3_sparse": projection(root, "fs-mf-projection-v3-sparse"),
        "fs_mf_op_proj_0": projection(root, "fs-mf-op-proj-0"),
        "fs_mf_op_proj_1": projection(root, "fs-mf-op-proj-1"),
        "jacobi3_sparsex_r4": sparse_bases(root, "jacobi-3-tensor-sparsex-r4"),
        "jacobi3_sparsex_r6": sparse_bases(root, "jacobi-3-tensor-sparsex-r6"),
        "jacobi4_fast": patches(root, "jacobi-4-tensor-fast"),
        "jacobi4_sparse": patches(root, "jacobi-4-tensor-sparse"),
        "jacobi1_gauss": interp_errors(root, "jacobi-1"),
        "jacobi1_lobatto": interp_errors(root, "jacobi-1-lobatto"),
        "bu0": bu0(root),
        "stokes_q3q2_scr": solver_log(root, "stokes-q3q2-scr"),
        "stokes_q3q2_fgmres": solver_log(root, "stokes-q3q2-fgmres"),
        "jacobi3_sparse_efs": sparse_efs(root),
        "ellip_e0_b1_p16": solver_log(root, "ellip-e0-b1-p16"),
        "ellip_e0_b3_p16": solver_log(root, "ellip-e0-b3-p16"),
        "ellip_e0_b3_p14": solver_log(root, "ellip-e0-b3-p14-sse"),
        "ellip_e0_b3_p17_lam1": solver_log(root, "ellip-e0-b3-p17-lam1-sse"),
        "elast_e0_b3_g01": solver_log(root, "elast-e0-b3-g01"),
        "ellip_morph": solver_log(root, "ellip-morph"),
        "ellip_morph_qfast": solver_log(root, "ellip-morph-qfast"),
    }
    meta = {}
    for name, arrs in fixtures.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrs)
        meta[name] = sorted(arrs)
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrote", len(fixtures), "fixtures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path to the dohp source tree>")
    main(sys.argv[1])
