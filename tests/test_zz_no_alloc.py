"""hx_dss_noalloc: the DSS entry point for callers that cannot allocate device memory
when they call it (a host model that reserves its whole GPU memory budget at start-up,
code where cudaMalloc is not allowed).  Its scratch is a fixed __device__ array inside
the library, so it must give exactly what the allocating entry point (hx_run_dss) gives.

This file is collected last, so a run that stops at the first failure has already run
every other test.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

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


_FRESH = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    import hxtest as H
    L = H.setup(sys.argv[2], 4, 2)
    E = L.nelem
    f = np.random.default_rng(7).standard_normal((E, 72, 4, 4))
    L.set("T", 0, f)
    L.call("hx_run_dss", b"T", 0, 1)
    ref = L.get("T", 0)
    d_in = torch.tensor(f, dtype=torch.float64, device="cuda")
    d_out = torch.empty_like(d_in)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert L.lib.hx_dss_noalloc(ctypes.c_void_p(d_in.data_ptr()), ctypes.c_void_p(d_out.data_ptr()), E, 1) == 0
        assert L.lib.hx_synchronize() == 0
    free1 = torch.cuda.mem_get_info()[0]
    assert np.array_equal(d_out.cpu().numpy(), ref)
    print("FREE", free0, free1)
""")


def test_noalloc_allocates_nothing_in_a_fresh_process(gpu_path):
    """The property the entry point exists for: in a new process, after session set-up
    and before the first call, free device memory is recorded; two calls and a
    synchronisation later it is unchanged (the fixed scratch became resident during
    init_boundary_exchanges_c, not at the first call)."""
    pytest.importorskip("torch")
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-c", _FRESH, here, gpu_path], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [x for x in r.stdout.splitlines() if x.startswith("FREE")][-1].split()
    assert int(line[1]) == int(line[2]), line
