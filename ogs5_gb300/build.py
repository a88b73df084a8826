"""Builds libogs_gpu.so in-tree for sm_103a.

Each .cu file under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3``; the objects
are linked into ``ogs5_gb300/_build/libogs_gpu.so`` with the static CUDA
runtime.  Rebuilds only what changed (mtime of sources and headers).
``build(debug=True)`` makes the bounds-checked variant (-DOGS_BOUNDS_CHECK)
in ``ogs5_gb300/_build/debug/libogs_gpu_debug.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libogs_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-Xptxas", "-v",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
            + glob.glob(os.path.join(CSRC, "**", "*.h"), recursive=True)
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


DEBUG_BUILD = os.path.join(BUILD, "debug")
DEBUG_LIB = os.path.join(DEBUG_BUILD, "libogs_gpu_debug.so")


def _compile(src: str, debug: bool = False) -> tuple[str, str]:
    out_dir = DEBUG_BUILD if debug else BUILD
    obj = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0] + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj, ""
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *(["-DOGS_BOUNDS_CHECK"] if debug else []), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    with open(obj + ".log", "w") as f:
        f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-4000:]}")
    return obj, r.stderr


def build(verbose: bool = False, debug: bool = False) -> str:
    """Compiles and links; returns the path of the library (the bounds-checked
    variant with debug)."""
    out_dir, lib = (DEBUG_BUILD, DEBUG_LIB) if debug else (BUILD, LIB)
    os.makedirs(out_dir, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(16, len(srcs))) as ex:
        objs = [o for o, _ in ex.map(lambda f: _compile(f, debug), srcs)]
    if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", lib + ".tmp", *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
        os.replace(lib + ".tmp", lib)
    if verbose:
        print(lib)
    return lib


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
