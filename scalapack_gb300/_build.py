"""Build libsl1x1gpu.so in-tree (scalapack_gb300/_lib/) with nvcc for sm_103a.

Each translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and the objects are
linked into one shared library with the CUDA runtime linked statically, so the
library has no run-time dependency beyond the NVIDIA driver.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libsl1x1gpu.so"
ILP64_NAME = "libsl1x1gpu_ilp64.so"  # the same entry points with 8-byte INTEGERs
SOURCES = ["api.cpp", "expert_api.cpp", "redist.cpp", "prof.cpp", "dgemm_f64.cu", "lu_f64.cu", "noalloc.cu", "mixed_gemm.cu", "ozgemm_f64.cu", "mixed.cu", "batched.cu", "aux.cu", "refine.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the sl1x1 CUDA library cannot be built")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def ilp64_path() -> str:
    return os.path.join(LIBDIR, ILP64_NAME)


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "sl1x1.h"))
    procs = []
    objs = []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [sp] + headers):
            continue
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-Wall", "-c", sp, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s} ---\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    so = lib_path()
    if force or _stale(so, objs):
        # -Bsymbolic: the library's calls to its own entry points stay inside it
        # even when the ILP64 library's same-named symbols come first
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-Xlinker", "-Bsymbolic", "-o", so, *objs,
               "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    # the ILP64 (8-byte INTEGER) entry points: host code that loads this library
    src64 = os.path.join(CSRC, "ilp64.cpp")
    so64 = ilp64_path()
    hdr64 = os.path.join(os.path.dirname(HERE), "include", "sl1x1_ilp64.h")
    if force or _stale(so64, [src64, hdr64]):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-fPIC", "-shared", "-o", so64, src64, "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("ILP64 build failed:\n" + r.stdout.decode(errors="replace"))
    return so


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
