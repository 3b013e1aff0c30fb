"""Build libreaxgpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into a shared
library next to this file.  No CMake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libreaxgpu.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["ffield.cpp", "tables.cpp", "lists.cu", "bonded.cu", "nonbonded.cu", "qeq.cu",
           "nve.cu", "peak.cu", "noalloc.cu", "reaxgpu.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path, os.path.join(CSRC, "rg_internal.h"),
            os.path.join(HERE, "..", "include", "reaxgpu.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(p) for p in deps):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", *ARCH, *extra]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-c", path, "-o", obj, "-O2", "-std=c++17",
               "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("RG_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if os.path.exists(OUT) and not force and \
            all(os.path.getmtime(OUT) >= os.path.getmtime(o) for o in objs):
        return OUT
    cmd = [nvcc(), "-shared", "-o", OUT, *objs, *ARCH, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return OUT


HOST = os.path.join(HERE, "host")
REAX_MD = os.path.join(HERE, "reax_md")


def build_host(force: bool = False) -> str:
    """The C++ host styles (host/reax_styles.*) and the reax_md deck driver,
    linked against libreaxgpu.so (g++, rpath to this directory)."""
    lib = build()
    srcs = [os.path.join(HOST, f) for f in ("reax_styles.cpp", "reax_md.cpp")]
    deps = srcs + [os.path.join(HOST, "reax_styles.h"), lib,
                   os.path.join(HERE, "..", "include", "reaxgpu.h")]
    if not force and os.path.exists(REAX_MD) and \
            all(os.path.getmtime(REAX_MD) >= os.path.getmtime(d) for d in deps):
        return REAX_MD
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-o", REAX_MD, *srcs,
           "-I", os.path.join(HERE, "..", "include"), "-L", HERE, "-lreaxgpu",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return REAX_MD


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
    print(build_host(force="--force" in sys.argv))
