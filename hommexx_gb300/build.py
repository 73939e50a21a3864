"""Builds libhxgpu.so in place (hommexx_gb300/libhxgpu.so) with nvcc for sm_103a.

The translation units compile in parallel; the library links only the CUDA
runtime.  ``HX_NVCC`` overrides the compiler path and ``HX_ARCH`` the -gencode
argument (default ``arch=compute_103a,code=sm_103a``).

``build(bounds_check=True)`` (or ``HX_BOUNDS_CHECK=1`` in the environment) builds the
debug variant hommexx_gb300/libhxgpu_bc.so instead, compiled with -DHX_BOUNDS_CHECK:
device index checks on the DSS table sources, the remap's source-cell search and the
tracer slab offsets, which record a violation in the session's flag word (reported as
HX_ERR_CUDA) and skip the access.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libhxgpu.so")
BUILD_BC = os.path.join(HERE, "_build_bc")
LIB_BC = os.path.join(HERE, "libhxgpu_bc.so")
SOURCES = ["hx_kernels.cu", "hx_adjoint.cu", "hx_tangent.cu", "hx_abi.cu", "hx_noalloc.cu", "hx_mesh.cu", "hx_peak.cu"]


def nvcc() -> str:
    cand = os.environ.get("HX_NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def flags():
    arch = os.environ.get("HX_ARCH", "arch=compute_103a,code=sm_103a")
    return ["-gencode", arch, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]


def _compile(src: str, bounds_check: bool = False) -> str:
    obj = os.path.join(BUILD_BC if bounds_check else BUILD, os.path.splitext(src)[0] + ".o")
    extra = ["-DHX_BOUNDS_CHECK"] if bounds_check else []
    cmd = [nvcc(), *flags(), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "hxgpu.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, bounds_check: bool | None = None) -> str:
    if bounds_check is None:
        bounds_check = os.environ.get("HX_BOUNDS_CHECK", "0") not in ("", "0")
    lib, bdir = (LIB_BC, BUILD_BC) if bounds_check else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    os.makedirs(bdir, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(lambda src: _compile(src, bounds_check), SOURCES))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *flags(), "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, bounds_check=True if "--bounds-check" in sys.argv else None))
