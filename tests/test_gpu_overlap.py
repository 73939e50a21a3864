"""Copies that overlap the step (hx_set_async_copies, hx_stream_results): the state each
interval hands back is bit-identical to the plain init / run / push sequence, with the
host buffers page-locked as the benchmark uses them, with Qdp read early (moist
dynamics, diagnostics) and late (tracer advection), and a push to other buffers still
copies."""
import ctypes

import numpy as np
import pytest

import hxtest as H

pytestmark = pytest.mark.gpu
DT = 300.0


def _pin(L, arrays, on=True):
    for a in arrays:
        f = L.lib.hx_host_register if on else L.lib.hx_host_unregister
        if on:
            assert f(ctypes.c_void_p(a.ctypes.data), ctypes.c_size_t(a.nbytes)) == 0
        else:
            f(ctypes.c_void_p(a.ctypes.data))


@pytest.mark.parametrize("kw", [dict(rsplit=3), dict(rsplit=1, moisture=True),
                                dict(rsplit=2, disable_diagnostics=False, state_frequency=1)])
def test_overlapped_copies_match_plain(gpu_path, kw):
    diag = not kw.get("disable_diagnostics", True)
    st = H.state(4, 4)
    host_in = {k: np.ascontiguousarray(st[k]).copy() for k in ("v", "T", "dp3d", "Qdp", "ps_v")}
    # plain sequence
    L = H.setup(gpu_path, 4, 4, diagnostics=diag, **kw)
    want = []
    for _ in range(3):
        L.set_state(host_in)
        L.run_subcycle(DT)
        want.append({k: v.copy() for k, v in L.push_results().items()})
    # overlapped sequence into page-locked buffers
    L = H.setup(gpu_path, 4, 4, diagnostics=diag, **kw)
    res = L.push_results()
    for a in res.values():
        a.fill(np.nan)
    _pin(L, list(host_in.values()) + list(res.values()))
    try:
        L.set_async_copies(True)
        L.stream_results(res)
        for i in range(3):
            L.set_state(host_in)
            L.run_subcycle(DT)
            got = L.push_results(res)          # same pointers: returns at once
            for k in want[i]:
                assert np.array_equal(got[k], want[i][k]), (i, k)
        other = L.push_results()                # other buffers: a real copy
        for k in want[-1]:
            assert np.array_equal(other[k], want[-1][k]), k
        L.stream_results(None)
        L.set_async_copies(False)
    finally:
        _pin(L, list(host_in.values()) + list(res.values()), on=False)
