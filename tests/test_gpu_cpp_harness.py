"""A C++ caller written against the reference's host API (via the drop-in
shim include/apsep.cuh) builds with nvcc, links libapsep.so, and passes the
reference harnesses' correctness checks."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "tests", "cpp", "_build")


def build_harness():
    from apsep_gb300 import build
    lib = build.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "apsep_main")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    oracle_o = os.path.join(OUT, "apsep_oracle.o")
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-c", os.path.join(ROOT, "oracle", "apsep_oracle.c"),
                           "-o", oracle_o])
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "apsep_main.cu"),
                           oracle_o, "-L", os.path.dirname(lib), "-lapsep",
                           "-Xlinker", "-rpath=" + os.path.dirname(lib), "-o", exe])
    return exe


def test_harness_compiles_against_shim():
    """Compilation alone needs no GPU."""
    exe = build_harness()
    assert os.path.isfile(exe)


@pytest.mark.gpu
def test_harness_correctness_on_gpu():
    exe = build_harness()
    r = subprocess.run([exe, "--quick"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "ALL PASSED" in r.stdout
