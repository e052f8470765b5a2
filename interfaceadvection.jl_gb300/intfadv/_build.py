"""Build libintfadv_gb300.so in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` compiles to an object in parallel; objects link into the
shared library next to this package.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # interfaceadvection.jl_gb300/
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "build")
LIBPATH = os.path.join(PKG_ROOT, "libintfadv_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libintfadv_gb300")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(os.path.dirname(PKG_ROOT), "include", "intfadv.h"))
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA source and link the library; returns its path."""
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= _deps_mtime():
        return LIBPATH
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *FLAGS, *ARCH, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIBPATH)
    return LIBPATH
