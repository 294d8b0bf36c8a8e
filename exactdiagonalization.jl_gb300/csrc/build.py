"""Build recipe of libedgpu.so (sm_103a).

Each translation unit is compiled by nvcc in parallel into ../_build/, then linked (with the static
CUDA runtime) into ../edgpu/libedgpu.so, next to the Python package that loads it.  Objects are
rebuilt only when a source or a header is newer.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "edgpu", "libedgpu.so")
SOURCES = ["api.cpp", "enumerate.cu", "hx32.cu", "hx64.cu", "hxbond.cu", "hxtable.cu", "linalg.cu", "noalloc.cu", "hxslab.cu"]
HEADERS = ["edgpu_internal.h", "edgpu_device.cuh", "hx_kernel.cuh", "hx_rows.cuh", "hx_bond.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _newest_dep() -> float:
    deps = [os.path.join(HERE, h) for h in HEADERS] + [os.path.join(ROOT, "include", "edgpu.h")]
    return max(os.path.getmtime(d) for d in deps)


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    s = os.path.join(HERE, src)
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(s), _newest_dep()):
        return obj
    cmd = [nvcc()] + ARCH + FLAGS + ["-c", s, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), SOURCES))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
