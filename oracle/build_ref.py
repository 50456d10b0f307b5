"""Recipe: compile the reference's own oracles into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  Compiles oracle/ref_cpu_wrap.cu, which #includes
the reference's src/main.cu (cpuApsep, main.cu:102-113) and
src/bench_spt_le.cu (cpuPSE, bench_spt_le.cu:24-35) from where they lie in the
reference checkout, into oracle/_ref/libapsep_ref_cpu.so; and
oracle/ref_spt_wrap.cu, which instantiates the reference's own GPU kernel
apsepKernelSPT (src/apsep.cuh:2634) for int32 keys, into device code only,
oracle/_ref/apsep_ref_spt.ptx (compute_103a; loaded by the GPU tests through
the driver API, so it needs no host code of this machine's architecture).
Nothing is copied out of the reference; both outputs are git-ignored.

The reference tree is looked up in $APSEP_REFERENCE_DIR, else in a directory
named `reference` beside this repository's root.  When it is absent (e.g. on
a machine that only has this repository) build() returns None and the callers
fall back to the oracle restatement, saying so.

Flags: -std=c++17 (the reference Makefile's -std=c++14 no longer compiles
against CUDA 13's cooperative-groups headers), and -DmemoryClockRate=... to
map the one removed cudaDeviceProp field main.cu reads (main.cu:387) onto an
existing int field; that statement is in main(), which is renamed and never
run.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libapsep_ref_cpu.so")
SPT_PTX = os.path.join(OUT_DIR, "apsep_ref_spt.ptx")


REPO_ROOT = os.path.dirname(HERE)


def reference_dir() -> str | None:
    d = os.environ.get("APSEP_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO_ROOT), "reference")
    src = os.path.join(d, "src")
    if os.path.isfile(os.path.join(src, "main.cu")) and os.path.isfile(
            os.path.join(src, "bench_spt_le.cu")):
        return d
    return None


def build_spt_ptx(force: bool = False, verbose: bool = False) -> str | None:
    """Build (if needed) and return the path of the reference kernel's PTX."""
    ref = reference_dir()
    if ref is None:
        return SPT_PTX if os.path.isfile(SPT_PTX) else None
    src = os.path.join(HERE, "ref_spt_wrap.cu")
    deps = [src, os.path.join(ref, "src", "apsep.cuh")]
    if (not force and os.path.isfile(SPT_PTX)
            and all(os.path.getmtime(SPT_PTX) >= os.path.getmtime(d) for d in deps)):
        return SPT_PTX
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [nvcc, "-std=c++17", "-ptx", "-arch=compute_103a", "-I", os.path.join(ref, "src"),
           "-o", SPT_PTX, src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return None
    return SPT_PTX


def build(force: bool = False, verbose: bool = False) -> str | None:
    """Build (if needed) the reference's oracles; return the path of the CPU
    library (the kernel's PTX: build_spt_ptx / SPT_PTX)."""
    build_spt_ptx(force, verbose)
    ref = reference_dir()
    if ref is None:
        return LIB if os.path.isfile(LIB) and _loads(LIB) else None
    src = os.path.join(HERE, "ref_cpu_wrap.cu")
    deps = [src, os.path.join(ref, "src", "main.cu"),
            os.path.join(ref, "src", "bench_spt_le.cu"),
            os.path.join(ref, "src", "apsep.cuh")]
    if (not force and os.path.isfile(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)
            and _loads(LIB)):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = [nvcc, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC",
           "-gencode", "arch=compute_103a,code=sm_103a",
           "-DmemoryClockRate=memoryBusWidth",
           "-I", os.path.join(ref, "src"), "-o", LIB, src, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return None
    return LIB if _loads(LIB) else None


def _loads(path: str) -> bool:
    import ctypes
    try:
        ctypes.CDLL(path)
        return True
    except OSError:
        return False


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference CPU oracle not built (reference tree absent or build failed)")
    sys.exit(0 if p else 1)
