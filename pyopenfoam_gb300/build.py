"""Compile libgbfoam.so (the sm_103a kernels and the C ABI) in-tree.

nvcc compiles every translation unit of ``csrc/`` for sm_103a in parallel and
links one shared library against the shared CUDA runtime, so that the
process's single libcudart instance (the one torch loads) owns all streams.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
CSRC = os.path.join(_PKG, "csrc")
INCLUDE = os.path.join(_ROOT, "include")
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgbfoam.so")

SOURCES = [
    "capi.cu",
    "topology.cpp",
    "amul.cu",
    "precond.cu",
    "pcg.cu",
    "pbicgstab.cu",
    "mixed.cu",
    "mixed_bicg.cu",
    "assemble.cu",
    "batched.cu",
    "geometry.cu",
    "pressure.cu",
    "smooth.cu",
    "gamg.cu",
    "selftest.cu",
    "hostcopy.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libgbfoam needs the CUDA toolkit to build")


def _cuda_lib_dir(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, h) for h in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    return hs


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Build (if stale) and return the path of libgbfoam.so."""
    nvcc = _nvcc()
    objdir = os.path.join(BUILD_DIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    headers = _headers()
    common = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC, "-Xcompiler", "-fPIC"]

    def compile_one(src: str) -> str:
        path = os.path.join(CSRC, src)
        obj = os.path.join(objdir, src + ".o")
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc] + ARCH + common + ["-lineinfo", "-c", path, "-o", obj + ".tmp"]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-O3"]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
            os.replace(obj + ".tmp", obj)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))

    if force or _stale(LIB_PATH, objs):
        libdir = _cuda_lib_dir(nvcc)
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
            "-Xlinker", f"-rpath={libdir}"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libgbfoam.so failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
