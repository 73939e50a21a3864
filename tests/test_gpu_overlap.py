"""Copies that overlap the step (hx_set_async_copies, hx_stream_results): the state each
interval hands back is bit-identical to the plain init / run / push sequence, with the
host buffers page-locked as the benchmark uses them, with Qdp read early (moist
dynamics, diagnostics) and late (tracer advection), and a push to other buffers still
copies.  The results stream out in pieces: dynamics levels n0 and nm1 during the
interval's last dynamics step, the tracer level the last tracer step only reads before
that step, and the rest from an element-chunked final remap (several chunks from ne8
up, one at ne4); qsplit 2, rsplit 0, no tracers and the mixed form move those points."""
import ctypes

import numpy as np
import pytest

import hxtest as H

pytestmark = pytest.mark.gpu
DT = 300.0


def _pin(L, arrays, on=True):
    for a in arrays:
        if a.nbytes == 0:
            continue
        f = L.lib.hx_host_register if on else L.lib.hx_host_unregister
        if on:
            assert f(ctypes.c_void_p(a.ctypes.data), ctypes.c_size_t(a.nbytes)) == 0
        else:
            f(ctypes.c_void_p(a.ctypes.data))


CASES = [
    dict(rsplit=3),
    dict(rsplit=1, moisture=True),
    dict(rsplit=2, disable_diagnostics=False, state_frequency=1),
    dict(ne=8, rsplit=3),
    dict(ne=16, rsplit=3, precision=1),
    dict(ne=8, rsplit=2, qsplit=2),
    dict(ne=8, rsplit=0),
    dict(ne=8, Q=0, rsplit=3),
]


@pytest.mark.parametrize("kw", CASES, ids=lambda kw: "-".join(f"{k}{v}" for k, v in kw.items()))
def test_overlapped_copies_match_plain(gpu_path, kw):
    kw = dict(kw)
    ne, Q, prec = kw.pop("ne", 4), kw.pop("Q", 4), kw.pop("precision", 0)
    diag = not kw.get("disable_diagnostics", True)
    st = H.state(ne, Q)
    host_in = {k: np.ascontiguousarray(st[k]).copy() for k in ("v", "T", "dp3d", "Qdp", "ps_v")}
    # plain sequence
    L = H.setup(gpu_path, ne, Q, precision=prec, diagnostics=diag, **kw)
    want = []
    for _ in range(3):
        L.set_state(host_in)
        L.run_subcycle(DT)
        want.append({k: v.copy() for k, v in L.push_results().items()})
    # overlapped sequence into page-locked buffers
    L = H.setup(gpu_path, ne, Q, precision=prec, diagnostics=diag, **kw)
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


def test_async_state_visible_to_other_calls(gpu_path):
    """With the time levels nm1 and np1 and Qdp still streaming in after
    init_elements_states_c, any other call of the library sees the whole new state."""
    L = H.setup(gpu_path, 4, 4, rsplit=3)
    st = H.state(4, 4)
    host_in = {k: np.ascontiguousarray(st[k]).copy() for k in ("v", "T", "dp3d", "Qdp", "ps_v")}
    for k in ("T", "dp3d"):
        host_in[k] += 1.0
    host_in["v"] *= 1.5
    host_in["Qdp"] *= 0.5
    _pin(L, list(host_in.values()))
    try:
        L.set_async_copies(True)
        L.set_state(host_in)
        for tl in range(3):
            for k in ("v", "T", "dp3d"):
                assert np.array_equal(L.get(k, tl), host_in[k][:, tl]), (k, tl)
        L.set_state(host_in)
        r = L.push_results()
        for k in ("v", "T", "dp3d", "Qdp", "ps_v"):
            assert np.array_equal(r[k], host_in[k]), k
        L.set_async_copies(False)
    finally:
        _pin(L, list(host_in.values()), on=False)


@pytest.mark.parametrize("kw", [dict(rsplit=3), dict(ne=8, rsplit=3, precision=1)],
                         ids=lambda kw: "-".join(f"{k}{v}" for k, v in kw.items()))
def test_overlapped_copies_in_place(gpu_path, kw):
    """The coupled driver's pattern: the same state arrays are the source of
    init_elements_states_c and the destination of cxx_push_results_to_f90, so each
    interval starts from the previous one's result while the copies overlap the step.
    Three intervals match the plain sequence run the same way, bit for bit."""
    kw = dict(kw)
    ne, Q, prec = kw.pop("ne", 4), kw.pop("Q", 4), kw.pop("precision", 0)
    keys = ("v", "T", "dp3d", "Qdp", "ps_v")
    st = H.state(ne, Q)
    # plain sequence, in place
    L = H.setup(gpu_path, ne, Q, precision=prec, **kw)
    host = {k: np.ascontiguousarray(st[k]).copy() for k in keys}
    want = []
    for _ in range(3):
        L.set_state(host)
        L.run_subcycle(DT)
        r = L.push_results()
        for k in keys:
            host[k][...] = r[k]
        want.append({k: v.copy() for k, v in r.items()})
    # overlapped sequence, in place, page-locked
    L = H.setup(gpu_path, ne, Q, precision=prec, **kw)
    host = {k: np.ascontiguousarray(st[k]).copy() for k in keys}
    r0 = L.push_results()
    res = {k: host[k] if k in host else np.full_like(v, np.nan) for k, v in r0.items()}
    _pin(L, list(res.values()))
    try:
        L.set_async_copies(True)
        L.stream_results(res)
        for i in range(3):
            L.set_state(host)
            L.run_subcycle(DT)
            got = L.push_results(res)
            for k in want[i]:
                assert np.array_equal(got[k], want[i][k]), (i, k)
        L.stream_results(None)
        L.set_async_copies(False)
    finally:
        _pin(L, list(res.values()), on=False)
