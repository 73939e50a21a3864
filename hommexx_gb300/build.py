"""Builds libhxgpu.so in place (hommexx_gb300/libhxgpu.so) with nvcc for sm_103a.

The translation units compile in parallel; the library links only the CUDA
runtime.  ``HX_NVCC`` overrides the compiler path and ``HX_ARCH`` the -gencode
argument (default ``arch=compute_103a,code=sm_103a``).
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
SOURCES = ["hx_kernels.cu", "hx_adjoint.cu", "hx_tangent.cu", "hx_abi.cu", "hx_noalloc.cu", "hx_mesh.cu", "hx_peak.cu"]


def nvcc() -> str:
    cand = os.environ.get("HX_NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def flags():
    arch = os.environ.get("HX_ARCH", "arch=compute_103a,code=sm_103a")
    return ["-gencode", arch, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *flags(), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "hxgpu.h"))
    deps.append(__file__)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *flags(), "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
