"""Builds the in-tree CUDA library ``nosh_gb300/libnosh_gb300.so`` for sm_103a.

Every translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo`` and linked into one
shared library exposing the C ABI declared in ``include/nosh_gb300.h``.
Host code is portable (no architecture-specific flags), so the same recipe
builds on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnosh_gb300.so")
SOURCES = ["mesh.cu", "ops.cu", "amg.cu", "solver.cu", "continuation.cu", "mpnn.cu", "capi.cu", "eig.cu",
           "minres_sys.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def flags():
    return [
        "-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
        "-Xcompiler", "-Wall", "--expt-relaxed-constexpr",
        "-I", os.path.join(ROOT, "include"), "-I", CSRC,
    ]


def _needs(obj, deps):
    return not os.path.exists(obj) or any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "nosh_gb300.h"))
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _needs(o, [s, *headers]):
            jobs.append((s, o))
    nv = nvcc()

    def run(job):
        s, o = job
        cmd = [nv, *flags(), "-c", s, "-o", o]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or _needs(LIB, objs):
        cmd = [nv, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


CPP_TESTS = {"test_reference_api": os.path.join(ROOT, "tests", "cpp", "test_reference_api.cpp"),
             "test_stepper": os.path.join(ROOT, "tests", "cpp", "test_stepper.cpp"),
             "test_io": os.path.join(ROOT, "tests", "cpp", "test_io.cpp"),
             "test_eig": os.path.join(ROOT, "tests", "cpp", "test_eig.cpp")}


def build_cpp_tests(force: bool = False) -> dict:
    """Compile the C++ programs that exercise include/nosh_gb300.hpp against
    the library (g++, linked with an rpath to the in-tree library)."""
    out = {}
    cxx = shutil.which("g++") or "g++"
    for name, src in CPP_TESTS.items():
        exe = os.path.join(BUILD, name)
        deps = [src, LIB, os.path.join(ROOT, "include", "nosh_gb300.h"), os.path.join(ROOT, "include", "nosh_gb300.hpp")]
        if force or _needs(exe, deps):
            cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), src, "-L", PKG,
                   "-lnosh_gb300", "-Wl,-rpath," + PKG, "-o", exe]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"g++ failed on {name}:\n{r.stderr}")
        out[name] = exe
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
    print(build_cpp_tests(force="--force" in sys.argv))
