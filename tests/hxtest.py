"""Shared helpers for the tests: build/load the CUDA library and the CPU oracle, set up
identical seeded inputs on both, compare fields.

The oracle (oracle/liboracle.so) is only ever the checker here.
"""
from __future__ import annotations

import os
import subprocess
import sys
from functools import lru_cache

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from hommexx_gb300 import abi, mesh as M, state as S  # noqa: E402

ORACLE_SO = os.path.join(ROOT, "oracle", "liboracle.so")

FIELDS_DYN = ("v", "T", "dp3d")


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ORACLE_SO


def build_gpu_lib() -> str:
    from hommexx_gb300 import build as B
    return B.build()


@lru_cache(maxsize=None)
def mesh(ne: int):
    return M.build_mesh(ne)


@lru_cache(maxsize=None)
def hvc():
    return S.hybrid_coordinate()


@lru_cache(maxsize=None)
def state(ne: int, Q: int):
    return S.initial_state(mesh(ne), Q, hvc())


_LIBS = {}


def lib(path: str) -> abi.HxLibrary:
    if path not in _LIBS:
        _LIBS[path] = abi.HxLibrary(path)
    return _LIBS[path]


def setup(path: str, ne: int = 4, Q: int = 4, precision: int = 0, diagnostics: bool = False,
          **kw) -> abi.HxLibrary:
    """(Re)initialise the library at ``path`` with the seeded state; with ``diagnostics``
    the host arrays of init_diagnostics_c are set up too (``L.diag``)."""
    L = lib(path)
    if L.nelem:
        L.finalize()
    p = abi.SimParams(qsize=Q, **kw)
    L.init(mesh(ne), hvc(), p, state(ne, Q), precision=precision, diagnostics=diagnostics)
    return L


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| (field-normwise relative error)."""
    den = float(np.max(np.abs(b)))
    if den == 0.0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b))) / den


def compare(ga: abi.HxLibrary, oa: abi.HxLibrary, names, tl=0):
    out = {}
    for n in names:
        out[n] = rel_err(ga.get(n, tl), oa.get(n, tl))
    return out
