"""Energy and tracer mass diagnostics of the oracle (src/share/cxx/Diagnostics.cpp and
the compute_diagnostics gate of src/share/cxx/prim_driver.cpp:49-58, 60-87, 140-144),
held to a numpy restatement computed from the state that cxx_push_results_to_f90 hands
back, and to global tracer mass conservation.

Slots of the init_diagnostics_c arrays: prim_diag_scalars writes Qvar/Qmass slots 3
(before forcing), 0 (after forcing) and 1 (after the remap), prim_energy_halftimes writes
IEner/KEner/PEner slots 2, 0 and 1; Qvar/Qmass slot 2 and energy slot 3 stay untouched.
"""
import numpy as np
import pytest

import hxtest as H

DT = 300.0
CP, CPV = 1005.0, 1870.0
NE, Q = 2, 3


def _energies(st, hv, phis, tl, tq, cpstar):
    """Column energies of Diagnostics.cpp:86-185 at dynamics level tl, tracer level tq."""
    ps = st["ps_v"][:, tl]
    dA, dB = np.diff(hv.hyai), np.diff(hv.hybi)
    dp = dA[None, :, None, None] * hv.ps0 + dB[None, :, None, None] * ps[:, None]
    T = st["T"][:, tl]
    u, v = st["v"][:, tl, :, 0], st["v"][:, tl, :, 1]
    cps = CP * (1.0 + (CPV / CP - 1.0) * st["Qdp"][:, tq, 0] / dp) if cpstar else np.full_like(dp, CP)
    return dict(IEner=np.sum(cps * T * dp, axis=1), IEner_wet=np.sum((cps - CP) * T * dp, axis=1),
                KEner=np.sum((u * u + v * v) * 0.5 * dp, axis=1),
                PEner=np.sum(phis[:, None] * dp, axis=1))


def _rel(a, b):
    return H.rel_err(a, b)


@pytest.mark.parametrize("cpstar", [False, True])
def test_diagnostics_match_restatement(oracle_path, cpstar):
    L = H.setup(oracle_path, NE, Q, rsplit=3, disable_diagnostics=False, state_frequency=1,
                use_cpstar=cpstar, diagnostics=True)
    st0 = H.state(NE, Q)
    hv, m = H.hvc(), H.mesh(NE)
    L.run_subcycle(DT)
    d = L.diag
    r = L.push_results()
    n0 = L.tl[1]
    nstep = L.tl[3]
    tq = 1 if ((nstep - 1) // 1) % 2 == 0 else 0  # np1_qdp of the remap
    # before the step: the initial state at n0 = 1, n0_qdp = 0
    e0 = _energies(st0, hv, m.phis, 1, 0, cpstar)
    for k in ("IEner", "KEner", "PEner"):
        for slot in (2, 0):
            assert _rel(d[k][:, slot], e0[k]) < 1e-13, (k, slot)
        assert np.isnan(d[k][:, 3]).all(), k
    # after the remap: the pushed state at the new n0
    e1 = _energies(r, hv, m.phis, n0, tq, cpstar)
    for k in ("IEner", "KEner", "PEner"):
        assert _rel(d[k][:, 1], e1[k]) < 1e-13, k
    if cpstar:
        assert _rel(d["IEner_wet"], e1["IEner_wet"]) < 1e-12
        assert np.max(np.abs(d["IEner_wet"])) > 0
    else:
        assert np.array_equal(d["IEner_wet"], np.zeros_like(d["IEner_wet"]))
    # tracers: Q starts at zero (update_q has not run), so Qvar is 0 before the step
    assert np.array_equal(d["Q"], r["Q"])
    qm0 = np.sum(st0["Qdp"][:, 0], axis=2)  # (E,Q,4,4)
    for slot in (3, 0):
        assert np.array_equal(d["Qvar"][:, slot], np.zeros_like(qm0))
        assert _rel(d["Qmass"][:, slot], qm0) < 1e-14
    qm1 = np.sum(r["Qdp"][:, tq], axis=2)
    assert _rel(d["Qmass"][:, 1], qm1) < 1e-14
    assert _rel(d["Qvar"][:, 1], np.sum(r["Qdp"][:, tq] * r["Q"], axis=2)) < 1e-14
    assert np.array_equal(d["Q1mass"], d["Qmass"][:, 1])
    assert np.isnan(d["Qvar"][:, 2]).all() and np.isnan(d["Qmass"][:, 2]).all()
    # the interval conserves global tracer mass
    w = m.spheremp[:, None]
    for q in range(Q):
        a = np.sum(w[:, 0] * d["Qmass"][:, 0, q])
        b = np.sum(w[:, 0] * d["Qmass"][:, 1, q])
        assert abs(a - b) <= 1e-13 * abs(a)


@pytest.mark.parametrize("kw,last,expect", [
    (dict(disable_diagnostics=True, state_frequency=1), 1 << 30, [False, False]),
    (dict(disable_diagnostics=False, state_frequency=2), 1 << 30, [False, True]),
    (dict(disable_diagnostics=False, state_frequency=1000), 1, [True, True]),
    (dict(disable_diagnostics=False, state_frequency=1000), 1 << 30, [False, False]),
])
def test_diagnostics_gate(oracle_path, kw, last, expect):
    """compute_diagnostics (prim_driver.cpp:49-58): nstep_end % state_frequency == 0, or
    the last time step reached, unless disable_diagnostics."""
    L = H.setup(oracle_path, NE, Q, rsplit=1, diagnostics=True, **kw)
    for want in expect:
        for a in L.diag.values():
            a.fill(np.nan)
        L.run_subcycle(DT, last_step=last)
        got = not np.isnan(L.diag["KEner"][:, 1]).any()
        assert got == want
        assert np.isnan(L.diag["Q"]).all() != want
