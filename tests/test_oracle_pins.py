"""Pins of the CPU oracle.  The reference ships no golden vectors and cannot be built
here (Kokkos, gfortran and MPI are missing), so the oracle is held to the reference's
own property tests and to analytic identities:

* limiter 8 and CAAS (limiter 9): bounds within (1 +- 10 eps) and mass within
  1e2 eps, on the reference's feasible random problems, and equal 1-norm of the
  corrections (src/preqx/unit_tests/preqx_ut.cpp:1330-1527);
* DSS of a constant gives the point multiplicity, DSS is symmetric, mass-weighted DSS
  conserves the global integral;
* the weak Laplacian of a spherical harmonic (after DSS and the inverse mass matrix)
  approaches -l(l+1)/a^2 Y; divergence of solid-body rotation vanishes and its
  vorticity is 2 w sin(lat); the curl of a gradient and the gradient of a constant
  vanish to round-off; the weak Laplacian is symmetric and negative semi-definite;
* a remap interval conserves dry mass and tracer mass, and a constant mixing ratio
  stays constant;
* a resting atmosphere (v = 0, T and mixing ratios functions of the level only, ps
  uniform) stays at rest through a whole remap interval;
* limiters 8 and 9 keep an advected cosine bell non-negative and below its maximum;
* hyperviscosity lowers the variance of T and the kinetic energy on every level and
  keeps the layer masses;
* the PPM remap (Colella and Woodward 1984, as PpmRemap.hpp:174-689 restates it) is the
  identity when source and target grids coincide, keeps constants, and reproduces cell
  means of a profile linear in pressure exactly away from the three cells at each end of
  the column that the ghost cells reach;
* option checks return the reference's error codes.
"""
import ctypes as C
import math

import numpy as np
import pytest

import hxtest as H

EPS = np.finfo(np.float64).eps
DT = 300.0


@pytest.fixture(scope="module")
def ora(oracle_path):
    return H.lib(oracle_path)


def _lim(L, option, ptens, sph, dpm, qlim):
    dp = C.POINTER(C.c_double)
    L.lib.hx_oracle_limiter(C.c_int(option), ptens.ctypes.data_as(dp), sph.ctypes.data_as(dp),
                            dpm.ctypes.data_as(dp), qlim.ctypes.data_as(dp))


def _feasible(rng):
    """LimiterTester::init_feasible (preqx_ut.cpp:1337-1380), one level."""
    sph = rng.uniform(1.0 / 16, 2.0 / 16, 16)
    dpm = rng.uniform(0.5, 1.0, 16)
    ptens = rng.uniform(0.0, 1.0, 16)
    q = np.sort(rng.uniform(0.0, 1.0, 2))
    ptens = ptens * dpm
    m = np.sum(sph * ptens)
    lo = np.sum(sph * q[0] * dpm)
    hi = np.sum(sph * q[1] * dpm)
    dm = lo - m if m < lo else (hi - m if m > hi else 0.0)
    if dm:
        ptens = ptens + (1 + 1e2 * EPS) * dm / (16 * sph)
    m = np.sum(sph * ptens)
    assert m >= (1 - 1e1 * EPS) * lo and m <= (1 + 1e1 * EPS) * hi
    return ptens, sph, dpm, q.copy(), m


@pytest.mark.parametrize("option", [8, 9])
def test_limiter_bounds_and_mass(ora, option):
    rng = np.random.default_rng(1330 + option)
    for _ in range(400):
        ptens, sph, dpm, qlim, mass = _feasible(rng)
        _lim(ora, option, ptens, sph, dpm, qlim)
        assert (ptens >= (1 - 1e1 * EPS) * qlim[0] * dpm).all()
        assert (ptens <= (1 + 1e1 * EPS) * qlim[1] * dpm).all()
        assert abs(np.sum(sph * ptens) - mass) <= 1e2 * EPS * mass


def test_limiter_one_norm_minimal(ora):
    """Limiter 8 and CAAS both give 1-norm-minimal corrections (preqx_ut.cpp:1459-1527)."""
    rng = np.random.default_rng(1459)
    for _ in range(200):
        ptens, sph, dpm, qlim, _ = _feasible(rng)
        a, b = ptens.copy(), ptens.copy()
        qa, qb = qlim.copy(), qlim.copy()
        _lim(ora, 8, a, sph, dpm, qa)
        _lim(ora, 9, b, sph, dpm, qb)
        na = np.sum(np.abs(a - ptens) * sph)
        nb = np.sum(np.abs(b - ptens) * sph)
        assert abs(na - nb) <= 1e3 * EPS * max(nb, 1e-300)


def test_limiter_relaxes_infeasible_bounds(ora):
    """If the level's mean lies outside [qmin, qmax] the bound is moved to the mean and
    the result is the constant mean (with_limiter_shell, EulerStepFunctorImpl.hpp:727-739)."""
    sph = np.full(16, 1.0 / 16)
    dpm = np.ones(16)
    ptens = np.linspace(0.5, 1.5, 16)
    qlim = np.array([2.0, 3.0])
    _lim(ora, 8, ptens, sph, dpm, qlim)
    assert qlim[0] == pytest.approx(1.0, rel=1e-15)
    assert np.allclose(ptens, 1.0, rtol=1e-14)


def _setup(path, ne=4, Q=2, **kw):
    kw.setdefault("nu", 1e16)
    return H.setup(path, ne, Q, **kw)


def test_dss_constant_multiplicity(oracle_path):
    L = _setup(oracle_path)
    m = H.mesh(4)
    L.set("T", 0, np.ones(L.field_shape("T")))
    L.call("hx_run_dss", b"T", 0, 0)
    out = L.get("T", 0)
    mult = np.ones((m.nelem, 16))
    for pts in H.M.dss_point_sources(m).values():
        for (e, i, j) in pts:
            mult[e, 4 * i + j] = len(pts)
    assert np.array_equal(out, np.broadcast_to(mult.reshape(m.nelem, 1, 4, 4), out.shape))


def test_dss_with_rspheremp_is_projection(oracle_path):
    """DSS(spheremp f) * rspheremp is a projection: applying it twice changes nothing,
    and it preserves the spheremp-weighted global integral."""
    L = _setup(oracle_path)
    m = H.mesh(4)
    rng = np.random.default_rng(3)
    f = rng.standard_normal(L.field_shape("T"))
    sm = m.spheremp[:, None]
    L.set("T", 0, f * sm)
    L.call("hx_run_dss", b"T", 0, 1)
    g = L.get("T", 0)
    L.set("T", 0, g * sm)
    L.call("hx_run_dss", b"T", 0, 1)
    g2 = L.get("T", 0)
    assert np.abs(g2 - g).max() <= 1e-13 * np.abs(g).max()
    # the spheremp-weighted integral over all element points is unchanged
    tot_g = (g * sm).sum(axis=(0, 2, 3))
    tot_f = (f * sm).sum(axis=(0, 2, 3))
    assert np.abs(tot_g - tot_f).max() <= 1e-12 * np.abs(tot_f).max()


def _sphere_op(L, op, arr, out_shape):
    out = np.empty(out_shape)
    a = np.ascontiguousarray(arr)
    L.lib.hx_oracle_sphere_op(C.c_int(op), C.c_void_p(a.ctypes.data), C.c_void_p(out.ctypes.data))
    return out


def _lap_err(path, ne):
    L = _setup(path, ne=ne)
    m = H.mesh(ne)
    y = 0.5 * (3 * np.sin(m.lat) ** 2 - 1)                     # P_2(sin lat)
    f = np.broadcast_to(y[:, None], (m.nelem, 72, 4, 4)).copy()
    lap = _sphere_op(L, 0, f, f.shape)
    L.set("T", 0, lap)
    L.call("hx_run_dss", b"T", 0, 1)
    lap = L.get("T", 0)
    exact = -6.0 / 6.376e6 ** 2 * f
    return float(np.sqrt(np.mean((lap - exact) ** 2) / np.mean(exact ** 2)))


def test_laplacian_of_spherical_harmonic(oracle_path):
    """Weak Laplacian + DSS + inverse mass matrix of Y_2^0 -> -6/a^2 Y_2^0, with the
    error falling by more than 4x per doubling of resolution (ne 4 -> 8)."""
    e4, e8 = _lap_err(oracle_path, 4), _lap_err(oracle_path, 8)
    assert e8 < 1e-3 and e4 / e8 > 4.0, (e4, e8)


def test_curl_of_gradient_vanishes(oracle_path):
    """vorticity_sphere(gradient_sphere(f)) = 0 point by point: on each element the two
    GLL derivative matrices act along different directions and commute, and the metric
    (D after Dinv) cancels, so only round-off remains; the gradient of a constant is 0."""
    ne = 4
    L = _setup(oracle_path, ne=ne)
    m = H.mesh(ne)
    rng = np.random.default_rng(13)
    lev = rng.standard_normal((72, 1))
    y = np.sin(m.lat) * np.cos(2 * m.lon) + 0.3 * np.cos(m.lat) ** 2   # smooth, (E,4,4)
    f = (1.0 + 0.1 * lev[None, :, :, None]) * y[:, None]
    g = _sphere_op(L, 3, f, (m.nelem, 72, 2, 4, 4))
    curl = _sphere_op(L, 2, g, (m.nelem, 72, 4, 4))
    a = 6.376e6
    gscale = np.abs(g).max()
    assert gscale > 1e-8
    assert np.abs(curl).max() <= 1e-12 * gscale / a, np.abs(curl).max()
    g0 = _sphere_op(L, 3, np.full((m.nelem, 72, 4, 4), 287.0), (m.nelem, 72, 2, 4, 4))
    assert np.abs(g0).max() <= 1e-12 * 287.0 / a


def test_weak_laplacian_symmetric_negative(oracle_path):
    """laplace_simple is the weak form -sum_q (grad phi_p . grad f) w_q: summed against a
    second field it is symmetric, <g, L f> = <f, L g>, and <f, L f> <= 0 (the element
    sums need no mass weights: the weak form carries them)."""
    ne = 4
    L = _setup(oracle_path, ne=ne)
    m = H.mesh(ne)
    rng = np.random.default_rng(17)
    f = rng.standard_normal((m.nelem, 72, 4, 4))
    g = rng.standard_normal((m.nelem, 72, 4, 4))
    Lf = _sphere_op(L, 0, f, f.shape)
    Lg = _sphere_op(L, 0, g, g.shape)
    a, b = np.sum(g * Lf, axis=(0, 2, 3)), np.sum(f * Lg, axis=(0, 2, 3))  # per level
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    assert (np.sum(f * Lf, axis=(0, 2, 3)) < 0).all()


def test_solid_body_rotation(oracle_path):
    ne = 8
    L = _setup(oracle_path, ne=ne)
    m = H.mesh(ne)
    u0 = 20.0
    u = u0 * np.cos(m.lat)
    vel = np.zeros((m.nelem, 72, 2, 4, 4))
    vel[:, :, 0] = u[:, None]
    div = _sphere_op(L, 1, vel, (m.nelem, 72, 4, 4))
    vort = _sphere_op(L, 2, vel, (m.nelem, 72, 4, 4))
    a = 6.376e6
    scale = u0 / a
    # discretisation error only (sign or orientation mistakes give O(1) errors)
    assert np.abs(div).max() < 1e-2 * scale
    exact = 2 * u0 / a * np.sin(m.lat)
    assert np.abs(vort - exact[:, None]).max() < 1e-2 * scale


@pytest.mark.parametrize("rsplit", [0, 1, 3])
def test_subcycle_conserves_mass(oracle_path, rsplit):
    L = _setup(oracle_path, ne=4, Q=3, rsplit=rsplit)
    m = H.mesh(4)
    st = H.state(4, 3)
    L.run_subcycle(DT)
    r = L.push_results()
    n0 = L.tl[1]
    ps0 = np.sum(st["ps_v"][:, 1] * m.spheremp)
    ps1 = np.sum(r["ps_v"][:, n0] * m.spheremp)
    assert abs(ps1 / ps0 - 1) < 1e-14
    q0 = np.sum(st["Qdp"][:, 0] * m.spheremp[:, None, None], axis=(0, 2, 3, 4))
    newest = [np.sum(r["Qdp"][:, k] * m.spheremp[:, None, None], axis=(0, 2, 3, 4)) for k in range(2)]
    assert min(np.abs(x / q0 - 1).max() for x in newest) < 1e-13


def test_constant_mixing_ratio_survives_remap(oracle_path):
    """q = const stays close to const through advection, limiter and remap.  It is not
    exact in the reference algorithm: the dynamics' dp3d carries the nu_top sponge and
    the nu_p hyperviscosity, which the tracer mass flux reproduces only approximately,
    so the bound is the size of that inconsistency, largest at the model top."""
    ne, Q = 4, 1
    m = H.mesh(ne)
    st = {k: v.copy() for k, v in H.state(ne, Q).items()}
    st["Qdp"][:] = 0.003 * st["dp3d"][:, 1][:, None, None]
    L = H.lib(oracle_path)
    if L.nelem:
        L.finalize()
    from hommexx_gb300 import abi
    L.init(m, H.hvc(), abi.SimParams(qsize=Q, nu=1e16, rsplit=3), st)
    L.run_subcycle(DT)
    r = L.push_results()
    dev = np.abs(r["Q"] / 0.003 - 1)
    assert dev.max() < 1e-3
    assert dev[:, :, 36:].max() < 1e-5     # lower half of the column


@pytest.mark.parametrize("field,value,code", [
    ("limiter_option", 4, 11), ("remap_alg", 3, 11), ("time_step_type", 1, 11),
    ("hypervis_order", 1, 11), ("ftype", 1, 11),
])
def test_option_checks(oracle_path, gpu_lib_cpu, field, value, code):
    """cxx_f90_interface.cpp:43-52 option checks; the same codes from both libraries."""
    from hommexx_gb300 import abi
    for path in (oracle_path, gpu_lib_cpu):
        L = H.lib(path)
        L.lib.hx_set_abort_on_error(0)
        p = abi.SimParams(qsize=2, nu=1e16, **{field: value}).resolved()
        L.lib.init_simulation_params_c(*[abi._i(x) if isinstance(x, (bool, int)) and not isinstance(x, bool)
                                         else (abi._b(x) if isinstance(x, bool) else abi._d(x))
                                         for x in _param_list(p)])
        assert L.last_error()[0] == code, (path, field, L.last_error())


def _param_list(p):
    return [p.remap_alg, p.limiter_option, p.rsplit, p.qsplit, p.time_step_type, p.energy_fixer,
            p.qsize, p.state_frequency, float(p.nu), float(p.nu_p), float(p.nu_q), float(p.nu_s),
            float(p.nu_div), float(p.nu_top), p.hypervis_order, p.hypervis_subcycle,
            float(p.hypervis_scaling), p.ftype, bool(p.prescribed_wind), bool(p.moisture),
            bool(p.disable_diagnostics), bool(p.use_cpstar), bool(p.use_semi_lagrangian_transport)]


def _target_dp(ps):
    """Hybrid thickness for surface pressure ps (E,4,4) -> (E,72,4,4)."""
    hv = H.hvc()
    da, db = np.diff(hv.hyai), np.diff(hv.hybi)
    return da[None, :, None, None] * hv.ps0 + db[None, :, None, None] * ps[:, None]


def _remap_case(oracle_path, alg, src_dp, v, T):
    """Sets level 1 (v, T, dp3d) and runs the PPM remap of that level alone."""
    L = _setup(oracle_path, ne=2, Q=1, rsplit=1, remap_alg=alg)
    L.set("dp3d", 1, src_dp)
    L.set("v", 1, v)
    L.set("T", 1, T)
    L.call("hx_run_remap", 1, 0, DT)
    return L.get("v", 1), L.get("T", 1), L.get("dp3d", 1)


def _columns(ne=2, seed=5):
    rng = np.random.default_rng(seed)
    E = 6 * ne * ne
    ps = 1.0e5 + 800.0 * rng.standard_normal((E, 4, 4))
    return rng, ps, _target_dp(ps)


@pytest.mark.parametrize("alg", [1, 2])
def test_remap_identity_on_coinciding_grids(oracle_path, alg):
    """Source thickness = the target's: every cell is integrated over itself."""
    rng, ps, tgt = _columns()
    v = 20.0 * rng.standard_normal(tgt.shape[:2] + (2, 4, 4))
    T = 250.0 + 30.0 * rng.standard_normal(tgt.shape)
    v1, T1, dp1 = _remap_case(oracle_path, alg, tgt, v, T)
    assert np.abs(v1 - v).max() <= 1e-12 * np.abs(v).max()
    assert np.abs(T1 - T).max() <= 1e-12 * np.abs(T).max()
    assert np.abs(dp1 - tgt).max() <= 1e-12 * tgt.max()


@pytest.mark.parametrize("alg", [1, 2])
def test_remap_keeps_constants_and_linear_profiles(oracle_path, alg):
    """A perturbed source grid with the target's column mass: a constant stays constant
    everywhere; cell means of a + b p stay exact in the interior (the edge values are the
    cubic interpolant of the cumulative mass, exact for linear data, and the limiters
    leave monotone linear data alone).  The mirrored ghost cells make the slopes of source
    cells 0-1 and 70-71 inexact, which reaches target cells 0-2 and 69-71."""
    rng, ps, tgt = _columns(seed=6)
    k = np.arange(72)[None, :, None, None]
    pert = 1.0 + 0.15 * np.sin(0.7 * k + rng.uniform(0, 6.3, (tgt.shape[0], 1, 4, 4)))
    src = tgt * pert
    src *= tgt.sum(axis=1, keepdims=True) / src.sum(axis=1, keepdims=True)
    hv = H.hvc()
    ptop = hv.hyai[0] * hv.ps0

    def means(dp, a, b):  # cell means of a + b p over the cells of thickness dp
        pi = ptop + np.concatenate([np.zeros_like(dp[:, :1]), np.cumsum(dp, axis=1)], axis=1)
        return a + b * 0.5 * (pi[:, :-1] + pi[:, 1:])

    v = np.empty(src.shape[:2] + (2, 4, 4))
    v[:, :, 0] = 7.5                                   # constant
    v[:, :, 1] = means(src, 3.0, 2.0e-4)               # linear in p
    T = means(src, 200.0, 1.0e-3)
    v1, T1, _ = _remap_case(oracle_path, alg, src, v, T)
    assert np.abs(v1[:, :, 0] - 7.5).max() <= 1e-13 * 7.5
    inner = slice(3, 69)
    want_v, want_T = means(tgt, 3.0, 2.0e-4), means(tgt, 200.0, 1.0e-3)
    assert np.abs(v1[:, inner, 1] - want_v[:, inner]).max() <= 1e-12 * np.abs(want_v).max()
    assert np.abs(T1[:, inner] - want_T[:, inner]).max() <= 1e-12 * np.abs(want_T).max()


def resting_deviation(path, precision=0):
    """Largest departures from rest after one remap interval: v (m/s), and the relative
    changes of T, dp3d, ps_v and the mixing ratios."""
    ne, Q = 4, 2
    m = H.mesh(ne)
    st = {k: v.copy() for k, v in H.state(ne, Q).items()}
    E = m.nelem
    ps = np.full((E, 4, 4), 98000.0)
    dp = _target_dp(ps)
    Tl = 300.0 - 60.0 * np.linspace(1.0, 0.0, 72)
    for tl in range(3):
        st["v"][:, tl] = 0.0
        st["T"][:, tl] = Tl[None, :, None, None]
        st["dp3d"][:, tl] = dp
        st["ps_v"][:, tl] = ps
    for tq in range(2):
        for q in range(Q):
            st["Qdp"][:, tq, q] = (0.002 + 0.001 * q) * dp
    from hommexx_gb300 import abi
    L = H.lib(path)
    if L.nelem:
        L.finalize()
    L.init(m, H.hvc(), abi.SimParams(qsize=Q, nu=1e16, rsplit=3), st, precision=precision)
    L.run_subcycle(DT)
    r = L.push_results()
    n0 = L.tl[1]
    return dict(v=np.abs(r["v"][:, n0]).max(),
                T=np.abs(r["T"][:, n0] - Tl[None, :, None, None]).max() / 300.0,
                dp=np.abs(r["dp3d"][:, n0] - dp).max() / dp.max(),
                ps=np.abs(r["ps_v"][:, n0] - ps).max() / 98000.0,
                Q=max(np.abs(r["Q"][:, q] - (0.002 + 0.001 * q)).max() for q in range(Q)))


def test_resting_atmosphere_stays_at_rest(oracle_path):
    """v = 0, T and Qdp/dp functions of the level only, ps uniform: every horizontal
    gradient vanishes, so a whole remap interval (RK5 Caar stages, hyperviscosity,
    tracer advection with limiter, remap) leaves the state where it was."""
    d = resting_deviation(oracle_path)
    assert d["v"] < 1e-10, d     # m/s (8e-13 seen)
    assert d["T"] < 1e-12 and d["dp"] < 1e-13 and d["ps"] < 1e-13 and d["Q"] < 1e-14, d


def bell_extremes(path, limiter):
    """(min Q, max Q, max of the initial bell) after three remap intervals."""
    from hommexx_gb300 import abi
    ne = 4
    m = H.mesh(ne)
    st = {k: v.copy() for k, v in H.state(ne, 1).items()}
    d = np.arccos(np.clip(np.sin(0.3) * np.sin(m.lat) + np.cos(0.3) * np.cos(m.lat) * np.cos(m.lon - 1.0),
                          -1.0, 1.0))
    bell = np.where(d < 0.5, 0.5 * (1.0 + np.cos(np.pi * d / 0.5)), 0.0) * 1e-3
    for tq in range(2):
        st["Qdp"][:, tq, 0] = bell[:, None] * st["dp3d"][:, 1]
    L = H.lib(path)
    if L.nelem:
        L.finalize()
    L.init(m, H.hvc(), abi.SimParams(qsize=1, nu=1e16, rsplit=3, limiter_option=limiter), st)
    for _ in range(3):
        L.run_subcycle(DT)
    q = L.push_results()["Q"]
    return q.min(), q.max(), bell.max()


@pytest.mark.parametrize("limiter", [8, 9])
def test_limiters_keep_a_cosine_bell_bounded(oracle_path, limiter):
    """A cosine bell of mixing ratio (zero outside its support) advected over three remap
    intervals: the quasi-monotone limiters keep it non-negative to round-off and create
    no new maximum (EulerStepFunctorImpl.hpp:693-884 with the neighbour bounds)."""
    lo, hi, top = bell_extremes(oracle_path, limiter)
    assert lo >= -1e-20, lo          # round-off below 1e-3 mixing ratios
    assert hi <= top * (1 + 1e-12), hi


def hyperviscosity_effect(path):
    """Per level: T variance and kinetic energy before and after one hyperviscosity call,
    the largest dp3d change (relative) and the largest layer-mass change (relative)."""
    ne = 4
    L = _setup(path, ne=ne, Q=1, rsplit=1, nu=1e16, nu_top=0.0)
    w = H.mesh(ne).spheremp

    def var(T):
        mean = np.sum(T * w[:, None], axis=(0, 2, 3)) / np.sum(w)
        return np.sum((T - mean[None, :, None, None]) ** 2 * w[:, None], axis=(0, 2, 3))

    def ke(v):
        return np.sum(v ** 2 * w[:, None, None], axis=(0, 2, 3, 4))

    T0, v0, d0 = L.get("T", 2), L.get("v", 2), L.get("dp3d", 2)
    L.call("hx_run_hypervis", 2, DT, 0.0)
    T1, v1, d1 = L.get("T", 2), L.get("v", 2), L.get("dp3d", 2)
    m0, m1 = np.sum(d0 * w[:, None], axis=(0, 2, 3)), np.sum(d1 * w[:, None], axis=(0, 2, 3))
    return dict(var=(var(T0), var(T1)), ke=(ke(v0), ke(v1)),
                ddp=np.abs(d1 - d0).max() / np.abs(d0).max(), mass=np.abs(m1 / m0 - 1).max())


def test_hyperviscosity_dissipates_and_conserves_layer_mass(oracle_path):
    """One hyperviscosity call (3 subcycles of the biharmonic): per level the mass-weighted
    variance of T and the kinetic energy fall, and the layer mass sum spheremp dp3d is
    kept to round-off (the weak Laplacian and the DSS conserve global integrals)."""
    h = hyperviscosity_effect(oracle_path)
    assert (h["var"][1] < h["var"][0]).all() and (h["ke"][1] < h["ke"][0]).all()
    assert h["ddp"] > 1e-9          # it did act on dp3d
    assert h["mass"] < 1e-14
