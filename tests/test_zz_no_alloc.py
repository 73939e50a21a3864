"""hx_dss_noalloc: the DSS entry point for callers that cannot allocate device memory
when they call it (a host model that reserves its whole GPU memory budget at start-up,
code where cudaMalloc is not allowed).  Its scratch is a fixed __device__ array inside
the library, so it must give exactly what the allocating entry point (hx_run_dss) gives.

This file is collected last, so a run that stops at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

import hxtest as H

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_noalloc_dss_matches_allocating_dss_twice(gpu_path):
    torch = pytest.importorskip("torch")
    L = H.setup(gpu_path, 4, 2)
    E = L.nelem
    rng = np.random.default_rng(2024)
    for call in range(2):          # two calls in a row: the shared scratch is reused
        for rsmp in (1, 0):
            f = rng.standard_normal((E, 72, 4, 4))
            L.set("T", 0, f)
            L.call("hx_run_dss", b"T", 0, rsmp)
            ref = L.get("T", 0)
            d_in = _dev(torch, f)
            d_out = torch.empty_like(d_in)
            torch.cuda.synchronize()
            rc = L.lib.hx_dss_noalloc(ctypes.c_void_p(d_in.data_ptr()),
                                      ctypes.c_void_p(d_out.data_ptr()), E, rsmp)
            assert rc == 0
            assert L.lib.hx_synchronize() == 0
            got = d_out.cpu().numpy()
            assert np.array_equal(got, ref), (call, rsmp, float(np.max(np.abs(got - ref))))
            # in place (output aliases input)
            rc = L.lib.hx_dss_noalloc(ctypes.c_void_p(d_in.data_ptr()),
                                      ctypes.c_void_p(d_in.data_ptr()), E, rsmp)
            assert rc == 0 and L.lib.hx_synchronize() == 0
            assert np.array_equal(d_in.cpu().numpy(), ref)


def test_noalloc_rejects_sizes(gpu_path):
    torch = pytest.importorskip("torch")
    L = H.setup(gpu_path, 4, 2)
    d = torch.zeros((L.nelem, 72, 16), dtype=torch.float64, device="cuda")
    # element count that does not match the session
    assert L.lib.hx_dss_noalloc(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                L.nelem + 1, 0) == 13
    # a mesh larger than the fixed scratch (ne=10: 600 elements > 455)
    L = H.setup(gpu_path, 10, 1)
    big = torch.zeros((L.nelem, 72, 16), dtype=torch.float64, device="cuda")
    assert L.lib.hx_dss_noalloc(ctypes.c_void_p(big.data_ptr()), ctypes.c_void_p(big.data_ptr()),
                                L.nelem, 1) == 13
