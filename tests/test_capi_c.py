"""The C ABI from plain C (no Python, no PyTorch): tests/capi/poisson_cg.c builds the Poisson problem on an 8^3 mesh,
assembles the Q1-embedded matrix, solves with CG + Chebyshev-Jacobi and checks the true residual with the operator.
On the CPU the program is compiled and linked as C99 against include/dohp_gb300.h and the library (the header is
valid C and every entry point it calls is exported); on the GPU it runs."""
import os
import shutil
import subprocess
import sys

import pytest

import dohp_gb300 as dg

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def compile_program(out):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    if not os.path.exists(dg.LIB_PATH):
        subprocess.run([sys.executable, os.path.join(os.path.dirname(dg.__file__), "build.py")], check=True)
    libdir = os.path.dirname(dg.LIB_PATH)
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA, "include"),
           os.path.join(HERE, "capi", "poisson_cg.c"), "-o", str(out), "-L" + libdir, "-ldohp_gb300",
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
