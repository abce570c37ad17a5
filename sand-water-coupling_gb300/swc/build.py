"""Builds libswc_gb300.so (the C-ABI library) from csrc/ with nvcc for sm_103a.

Each translation unit is compiled in parallel to an object file, then linked
into one shared library with no dependency on PyTorch.  Rebuilds only when a
source or header is newer than the library.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_PATH = os.path.join(PKG_ROOT, "swc", "libswc_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++20", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", os.path.join(REPO_ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = _sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(REPO_ROOT, "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nv = nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        cmd = [nv] + ARCH + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB_PATH + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


EXAMPLES_DIR = os.path.join(PKG_ROOT, "examples")
EXAMPLES_BIN = os.path.join(BUILD_DIR, "examples")


def build_examples(force: bool = False) -> list:
    """C++ callers of include/swc/DualParticleSphLiquid.hpp, linked against the library."""
    lib = build()
    os.makedirs(EXAMPLES_BIN, exist_ok=True)
    out = []
    for src in sorted(glob.glob(os.path.join(EXAMPLES_DIR, "*.cpp"))):
        exe = os.path.join(EXAMPLES_BIN, os.path.splitext(os.path.basename(src))[0])
        if force or not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(src),
                                                                            os.path.getmtime(lib)):
            cmd = [os.environ.get("CXX", "g++"), "-std=c++20", "-O2", "-I", os.path.join(REPO_ROOT, "include"), src,
                   "-L", os.path.dirname(lib), "-lswc_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", exe]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"example build failed: {os.path.basename(src)}\n{r.stderr[-3000:]}")
        out.append(exe)
    return out


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
