"""The C ABI from plain C (no Python, no PyTorch): tests/capi/poisson_cg.c builds the Poisson problem on an 8^3 mesh,
assembles the Q1-embedded matrix, solves with CG + Chebyshev-Jacobi and checks the true residual with the operator.
On the CPU the program is compiled and linked as C99 against include/dohp_gb300.h and the library (the header is
valid C and every entry point it calls is exported); on the GPU it runs. tests/capi/jacobi_explicit.c follows the
reference's explicit-basis program (src/jacobi/tests/ex3.c) through the host-side jacobi entry points; it runs on the
CPU and its printed matrices are those of the jacobi-3-tensor-gauss / -lobatto / jacobi-3-modal-gauss refouts."""
import os
import re
import shutil
import subprocess
import sys

import numpy as np
import pytest

import dohp_gb300 as dg

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def compile_program(out, source="poisson_cg.c"):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    if not os.path.exists(dg.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    libdir = os.path.dirname(dg.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include"),
           os.path.join(HERE, "capi", source), "-o", str(out), "-L" + libdir, "-ldohp_gb300",
           "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-lm", "-Wl,-rpath," + libdir + ":" + os.path.join(CUDA, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_compiles_and_links_as_c(tmp_path):
    compile_program(tmp_path / "poisson_cg")


@pytest.mark.gpu
def test_runs_from_plain_c(tmp_path):
    exe = tmp_path / "poisson_cg"
    compile_program(exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(kv.split("=") for kv in r.stdout.split())
    assert int(fields["n"]) == 29791 and 40 <= int(fields["its"]) <= 120
    assert float(fields["true"]) <= 1.01e-8


def parse_explicit(text):
    """the matrices of ex3.c's output ("<kind> matrix of size (Q,P[*3])" then the rows), per element"""
    out, elem, lines, i = {}, -1, text.splitlines(), 0
    while i < len(lines):
        m = re.match(r"(Interpolation|Gradient|Mass) matrix of size \((\d+),(\d+)(\*3)?\)", lines[i])
        if not m:
            i += 1
            continue
        kind, rows = m.group(1).lower(), int(m.group(2))
        elem += kind == "interpolation"
        out[f"e{elem}_{kind}"] = np.array([[float(v) for v in lines[i + 1 + r].split()] for r in range(rows)])
        i += 1 + rows
    return out


@pytest.mark.parametrize("args,name", [(("tensor", "gauss", "8"), "jacobi3_gauss"), (("tensor", "lobatto", "6"), "jacobi3_lobatto"),
                                       (("modal", "gauss", "6"), "jacobi3_modal_gauss")])
def test_reference_explicit_program_from_c(tmp_path, args, name):
    exe = tmp_path / "jacobi_explicit"
    compile_program(exe, "jacobi_explicit.c")
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = parse_explicit(r.stdout)
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    for key in g.files:  # full matrices, or the first rows where the fixture keeps only those
        base = key.replace("_head", "")
        ref = g[key]
        np.testing.assert_allclose(got[base][:len(ref)], ref, rtol=0, atol=1.5e-6, err_msg=key)
