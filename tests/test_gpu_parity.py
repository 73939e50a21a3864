"""Parity of the CUDA library (libhxgpu.so) with the CPU oracle, phase by phase and for
whole remap intervals, through the C ABI, on the same seeded inputs.

FP64 plain form: every field within 1e-12 relative (max |gpu - oracle| / max |oracle|),
the parity bar of the FP64 step.  The DSS sums in the reference's fixed
order in double, so it is compared bit for bit.
"""
import numpy as np
import pytest

import hxtest as H

pytestmark = pytest.mark.gpu

TOL = 1e-12
DT = 300.0


@pytest.fixture
def pair(gpu_path, oracle_path):
    def make(ne=4, Q=4, precision=0, **kw):
        kw.setdefault("nu", 1e16)
        g = H.setup(gpu_path, ne, Q, precision=precision, **kw)
        o = H.setup(oracle_path, ne, Q, **kw)
        return g, o
    return make


def _assert_close(errs, tol=TOL):
    bad = {k: v for k, v in errs.items() if not (v <= tol)}
    assert not bad, f"relative errors above {tol}: {bad} (all: {errs})"


@pytest.mark.parametrize("name,rsmp", [("T", 1), ("dp3d", 0), ("v", 1)])
def test_dss_bitwise(pair, name, rsmp):
    g, o = pair()
    rng = np.random.default_rng(11)
    f = rng.standard_normal(g.field_shape(name))
    for L in (g, o):
        L.set(name, 1, f)
        L.call("hx_run_dss", name.encode(), 1, rsmp)
    a, b = g.get(name, 1), o.get(name, 1)
    assert np.array_equal(a, b), f"max diff {np.max(np.abs(a - b))}"


def test_dss_of_constant_is_multiplicity(pair):
    g, _ = pair()
    m = H.mesh(4)
    ones = np.ones(g.field_shape("T"))
    g.set("T", 0, ones)
    g.call("hx_run_dss", b"T", 0, 0)
    out = g.get("T", 0)
    # multiplicity of each GLL point: 1 interior, 2 edge, 3 or 4 at element corners
    mult = np.ones((m.nelem, 16))
    groups = H.M.dss_point_sources(m)
    for pts in groups.values():
        for (e, i, j) in pts:
            mult[e, 4 * i + j] = len(pts)
    assert np.array_equal(out, np.broadcast_to(mult.reshape(m.nelem, 1, 4, 4), out.shape))


def test_caar_stage(pair):
    g, o = pair()
    for L in (g, o):
        L.call("hx_run_caar_stage", 0, 1, 2, DT / 5.0, 0.25)
    errs = H.compare(g, o, ("v", "T", "dp3d"), tl=2)
    errs.update(H.compare(g, o, ("vn0", "omega_p", "phi")))
    _assert_close(errs)


def test_caar_stage_vertically_eulerian(pair):
    """rsplit = 0: eta_dot_dpdn from the div(v dp) scan, vertical advection of T and v,
    eta_dot_dpdn accumulation (CaarFunctorImpl.hpp:137-143, 236-300, 496-597)."""
    g, o = pair(rsplit=0)
    for L in (g, o):
        L.call("hx_run_caar_stage", 0, 1, 2, DT / 5.0, 0.25)
    errs = H.compare(g, o, ("v", "T", "dp3d"), tl=2)
    errs.update(H.compare(g, o, ("vn0", "omega_p", "phi", "eta_dot_dpdn")))
    _assert_close(errs)


def test_caar_stage_in_place(pair):
    """n0 == np1 (stages 3-5 of the RK5 scheme read and write the same level)."""
    g, o = pair()
    for L in (g, o):
        L.call("hx_run_caar_stage", 0, 1, 1, DT / 3.0, 0.0)
    _assert_close(H.compare(g, o, ("v", "T", "dp3d"), tl=1))


def test_rk5(pair):
    g, o = pair()
    for L in (g, o):
        L.call("hx_run_rk5", 0, 1, 2, -1, DT, 1.0)
    errs = {}
    for tl in range(3):
        for k, v in H.compare(g, o, ("v", "T", "dp3d"), tl=tl).items():
            errs[f"{k}[{tl}]"] = v
    errs.update(H.compare(g, o, ("vn0", "omega_p")))
    _assert_close(errs)


@pytest.mark.parametrize("nu_top", [2.5e5, 0.0])
def test_hypervis(pair, nu_top):
    g, o = pair(nu_top=nu_top)
    for L in (g, o):
        L.call("hx_run_hypervis", 2, DT, 1.0)
    errs = H.compare(g, o, ("v", "T", "dp3d"), tl=2)
    errs.update(H.compare(g, o, ("dpdiss_ave",)))
    _assert_close(errs)
    # dpdiss_biharmonic accumulates the biharmonic of dp3d, a fourth derivative whose
    # value is ~1e-4 of the rounding-level terms it is built from: its relative error
    # vs the oracle scales with that cancellation (not a prognostic field).
    _assert_close(H.compare(g, o, ("dpdiss_biharmonic",)), tol=1e-10)


@pytest.mark.parametrize("limiter", [8, 9])
def test_prim_step_with_tracers(pair, limiter):
    g, o = pair(limiter_option=limiter)
    for L in (g, o):
        L.call("hx_run_prim_step", DT)
    errs = {}
    for tl in range(3):
        for k, v in H.compare(g, o, ("v", "T", "dp3d"), tl=tl).items():
            errs[f"{k}[{tl}]"] = v
    for tl in range(2):
        errs[f"Qdp[{tl}]"] = H.rel_err(g.get("Qdp", tl), o.get("Qdp", tl))
    errs.update(H.compare(g, o, ("vn0", "omega_p", "divdp", "divdp_proj", "eta_dot_dpdn")))
    _assert_close(errs)
    _assert_close(H.compare(g, o, ("dpdiss_biharmonic",)), tol=1e-10)


@pytest.mark.parametrize("rhs,dssopt", [(0.0, 2), (1.0, 0), (2.0, 1)])
def test_euler_step_stage(pair, rhs, dssopt):
    """One euler_step stage from a realistic state (after a full prim_step)."""
    g, o = pair()
    for L in (g, o):
        L.call("hx_run_prim_step", DT)               # fills vn0, divdp, derived_dp, dpdiss
        L.call("hx_run_euler_step", 0, 1, DT / 2.0, rhs, dssopt)
    errs = {f"Qdp[{tl}]": H.rel_err(g.get("Qdp", tl), o.get("Qdp", tl)) for tl in range(2)}
    errs.update(H.compare(g, o, ("omega_p", "divdp_proj", "eta_dot_dpdn")))
    _assert_close(errs)


@pytest.mark.parametrize("remap_alg", [1, 2])
def test_remap(pair, remap_alg):
    g, o = pair(remap_alg=remap_alg)
    for L in (g, o):
        L.call("hx_run_rk5", 0, 1, 2, -1, DT, 1.0)
        L.call("hx_run_remap", 2, 0, DT)
    errs = H.compare(g, o, ("v", "T"), tl=2)
    errs["Qdp[0]"] = H.rel_err(g.get("Qdp", 0), o.get("Qdp", 0))
    errs["ps_v"] = H.rel_err(g.get("ps_v", 2), o.get("ps_v", 2))
    _assert_close(errs)


@pytest.mark.parametrize("rsplit,nsub", [(1, 1), (3, 2), (0, 2)])
def test_subcycle(pair, rsplit, nsub):
    """prim_run_subcycle_c end to end, results pushed through cxx_push_results_to_f90;
    rsplit = 0 is the vertically Eulerian step (tracers alone are remapped, from the
    thickness the accumulated eta_dot_dpdn gives)."""
    g, o = pair(rsplit=rsplit)
    for _ in range(nsub):
        tg = g.run_subcycle(DT)
        to = o.run_subcycle(DT)
        assert tg == to
    rg, ro = g.push_results(), o.push_results()
    errs = {k: H.rel_err(rg[k], ro[k]) for k in rg}
    errs.update(H.compare(g, o, ("eta_dot_dpdn",)))
    _assert_close(errs)


@pytest.mark.parametrize("ne,Q,kw", [
    (1, 1, dict(rsplit=3)),                                   # 6 elements: every corner a cube corner
    (2, 0, dict(rsplit=3)),                                   # no tracers
    (2, 7, dict(rsplit=2, qsplit=2)),                         # odd tracer count, two dynamics steps per tracer step
    (3, 3, dict(rsplit=1, hypervis_subcycle=1, nu_div=2.5e16)),  # nu_div != nu (nu_ratio)
    (2, 2, dict(rsplit=3, hypervis_subcycle=4, nu_top=0.0)),  # no sponge
])
def test_subcycle_edge_cases(pair, ne, Q, kw):
    """Two remap intervals through prim_run_subcycle_c on small, tracer-free and odd-sized
    configurations, results through cxx_push_results_to_f90."""
    g, o = pair(ne=ne, Q=Q, **kw)
    for _ in range(2):
        assert g.run_subcycle(DT) == o.run_subcycle(DT)
    rg, ro = g.push_results(), o.push_results()
    errs = {k: H.rel_err(rg[k], ro[k]) for k in rg if ro[k].size}
    _assert_close(errs)
    if Q == 0:
        assert rg["Qdp"].size == 0 and rg["Q"].size == 0


def test_subcycle_edge_mixed_ne1(pair):
    """The mixed form on the 6-element cube stays close to the FP64 oracle."""
    g, o = pair(ne=1, Q=2, precision=1, rsplit=3)
    g.run_subcycle(DT)
    o.run_subcycle(DT)
    rg, ro = g.push_results(), o.push_results()
    errs = {k: H.rel_err(rg[k], ro[k]) for k in ("T", "dp3d", "v", "Qdp", "ps_v")}
    assert errs["T"] < 1e-6 and errs["dp3d"] < 1e-5 and errs["ps_v"] < 1e-7, errs


def _forcing(ne, Q, seed):
    rng = np.random.default_rng(seed)
    E = 6 * ne * ne
    st = H.state(ne, Q)
    FM = 1e-4 * rng.standard_normal((E, 72, 2, 4, 4))
    FT = 1e-4 * rng.standard_normal((E, 72, 4, 4))
    FQ = 5e-6 * rng.standard_normal((E, Q, 72, 4, 4))
    # strong negative tracer forcing at some points so that the clipping acts
    mask = rng.random(FQ.shape) < 0.05
    FQ[mask] = -2.0 * st["Qdp"][:, 1][mask] / 900.0
    return FM, FT, FQ, st["Qdp"]


@pytest.mark.parametrize("ftype,moist", [(0, False), (0, True), (2, False)])
def test_cam_forcing(pair, ftype, moist):
    """f90_push_forcing_to_cxx / cxx_push_forcing_to_f90 around two remap intervals with
    forcing applied at their start (CamForcing.cpp: state, clipped tracer and, when
    moist, surface-pressure forcing)."""
    g, o = pair(rsplit=3, ftype=ftype, moisture=moist)
    FM, FT, FQ, Qdp = _forcing(4, 4, 7 + ftype)
    for _ in range(2):
        for L in (g, o):
            L.push_forcing(FM, FT, FQ, Qdp if _ == 0 else L.push_results()["Qdp"])
            L.run_subcycle(DT)
    rg, ro = g.push_results(), o.push_results()
    errs = {k: H.rel_err(rg[k], ro[k]) for k in rg}
    _assert_close(errs)
    fg, fo = g.pull_forcing(), o.pull_forcing()
    for k in fg:
        assert np.array_equal(fg[k], fo[k]), k
    assert np.array_equal(fg["FT"], FT)


@pytest.mark.parametrize("cpstar,ftype", [(False, -1), (True, 0)])
def test_diagnostics(pair, cpstar, ftype):
    """Energy and tracer mass diagnostics (Diagnostics.cpp) written into the
    init_diagnostics_c host arrays over two remap intervals (CAM forcing between the
    before-forcing and after-forcing slots when ftype is 0).  The slots computed before the
    first step, from identical inputs, agree bit for bit; the rest within 1e-12; the
    untouched slots stay untouched on both sides."""
    g, o = pair(rsplit=3, ftype=ftype, moisture=cpstar, use_cpstar=cpstar, disable_diagnostics=False,
                state_frequency=1, diagnostics=True)
    FM, FT, FQ, Qdp = _forcing(4, 4, 21)
    for it in range(2):
        for L in (g, o):
            if ftype == 0:
                L.push_forcing(FM, FT, FQ, Qdp if it == 0 else L.push_results()["Qdp"])
            L.run_subcycle(DT)
        if it == 0:
            for k in ("IEner", "KEner", "PEner"):
                assert np.array_equal(g.diag[k][:, 2], o.diag[k][:, 2]), k
            for k in ("Qvar", "Qmass"):
                assert np.array_equal(g.diag[k][:, 3], o.diag[k][:, 3]), k
        errs = {}
        for k in g.diag:
            a, b = g.diag[k], o.diag[k]
            assert np.array_equal(np.isnan(a), np.isnan(b)), k
            ok = ~np.isnan(b)
            errs[k] = H.rel_err(a[ok], b[ok])
        _assert_close(errs)
    assert np.isnan(g.diag["IEner"][:, 3]).all() and np.isnan(g.diag["Qvar"][:, 2]).all()


def test_diagnostics_mixed_form(pair):
    """A mixed-form session fills the init_diagnostics_c arrays like the FP64 oracle, to
    the mixed form's accuracy (diagnostics themselves are FP64 sums)."""
    g, o = pair(precision=1, rsplit=3, disable_diagnostics=False, state_frequency=1, diagnostics=True)
    g.run_subcycle(DT)
    o.run_subcycle(DT)
    for k in ("IEner", "KEner", "PEner"):
        assert np.array_equal(g.diag[k][:, 2], o.diag[k][:, 2]), k   # before the step: same inputs
        assert H.rel_err(g.diag[k][:, 1], o.diag[k][:, 1]) < 1e-6, k
    assert H.rel_err(g.diag["Qmass"][:, 1], o.diag["Qmass"][:, 1]) < 1e-5


def test_mass_conservation_gpu(pair):
    g, _ = pair(rsplit=3)
    m = H.mesh(4)
    st = H.state(4, 4)
    g.run_subcycle(DT)
    r = g.push_results()
    n0 = g.tl[1]
    ps0 = np.sum(st["ps_v"][:, 1] * m.spheremp)
    ps1 = np.sum(r["ps_v"][:, n0] * m.spheremp)
    assert abs(ps1 - ps0) / ps0 < 1e-13
    q0 = np.sum(st["Qdp"][:, 0] * m.spheremp[:, None, None])
    # tracer mass of the level holding the newest Qdp (np1_qdp of the last step)
    qa = [np.sum(r["Qdp"][:, k] * m.spheremp[:, None, None]) for k in range(2)]
    assert min(abs(x - q0) / q0 for x in qa) < 1e-12


@pytest.mark.parametrize("kw", [dict(rsplit=3), dict(rsplit=1, moisture=True), dict(rsplit=0)])
def test_mixed_precision_close(pair, kw):
    """Mixed form against the FP64 oracle after one remap interval (loose bound; the
    per-day error is reported by the benchmark): dry, moist (virtual temperature from a
    double shared array the dry mixed caar does not allocate) and vertically Eulerian."""
    g, o = pair(precision=1, **kw)
    g.run_subcycle(DT)
    o.run_subcycle(DT)
    rg, ro = g.push_results(), o.push_results()
    errs = {k: H.rel_err(rg[k], ro[k]) for k in ("T", "dp3d", "v", "Qdp", "ps_v")}
    assert errs["T"] < 1e-6 and errs["dp3d"] < 1e-6 and errs["ps_v"] < 1e-7, errs
    assert errs["v"] < 1e-5 and errs["Qdp"] < 1e-5, errs


def test_negative_thickness_reports_101(gpu_path):
    """Host-side fault injection: a negative layer thickness in the input makes the
    remap report the reference's error code 101 instead of continuing."""
    L = H.setup(gpu_path, 4, 2, rsplit=1)
    dp = L.get("dp3d", 1)
    dp[0, 40, 1, 1] = -5.0e4
    L.set("dp3d", 1, dp)
    rc = L.lib.hx_run_remap(1, 0, DT)
    assert rc == 101


def test_moist_virtual_temperature(pair):
    """moisture='moist': T_v = T (1 + (Rv/R - 1) Qdp/dp) in caar
    (CaarFunctorImpl.hpp:345-360)."""
    g, o = pair(moisture=True, rsplit=1)
    for L in (g, o):
        L.call("hx_run_prim_step", DT)
    errs = {}
    for tl in range(3):
        for k, v in H.compare(g, o, ("v", "T", "dp3d"), tl=tl).items():
            errs[f"{k}[{tl}]"] = v
    _assert_close(errs)


def test_tensor_hyperviscosity(gpu_path, oracle_path):
    """hypervis_scaling != 0: laplace_tensor and vlaplace_sphere_wk_cartesian
    (TagSecondLaplaceTensorHV, HyperviscosityFunctorImpl.hpp:105-125)."""
    from hommexx_gb300 import abi
    m = H.M.build_mesh(4, hypervis_scaling=3.2)
    st = H.state(4, 2)
    p = abi.SimParams(qsize=2, nu=3.0e-8, nu_div=3.0e-8, hypervis_scaling=3.2, rsplit=1)
    libs = []
    for path in (gpu_path, oracle_path):
        L = H.lib(path)
        if L.nelem:
            L.finalize()
        L.init(m, H.hvc(), p, st)
        L.call("hx_run_hypervis", 1, DT, 1.0)
        libs.append(L)
    g, o = libs
    _assert_close(H.compare(g, o, ("v", "T", "dp3d"), tl=1))
