"""Formulaic hybrid vertical coordinate and the seeded smooth initial state.

Neither is taken from the reference (its benchmark initialises the JW baroclinic test
in Fortran, ``test/reg_test/benchmarks/v1/homme-ne30-v1.nl``); both restate the
synthetic workload the GB300 benchmark uses:

* interfaces ``eta_i = 0.001 + 0.999 i / 72``; ``B = ((eta-0.2)/0.8)^2`` for
  ``eta > 0.2`` else 0; ``A = eta - B``; ``ps0 = 1e5 Pa``;
* ``ps = 1e5 + 500 S_ps``; ``dp3d = dA ps0 + dB ps`` (the same formula
  ``prim_run_subcycle_c`` uses, ``src/share/cxx/prim_driver.cpp:90-113``);
* ``u, v = 20 S`` per level; ``T = 300 - 60 (1 - p/p0) + 2 S`` per level with ``p`` at
  mid levels; ``Qdp = dp3d q`` with ``q = 0.005 (1 + S)`` per tracer and level;
* every ``S`` is an independent sum of real, fully normalised spherical harmonics of
  degree <= 6 with N(0,1) coefficients, scaled to unit maximum over the GLL points.
  Coefficients come from ``numpy.random.default_rng(seed)`` with a fixed seed per field
  family (ps 1001, u 1002, v 1003, T 1004, q 1005).

Arrays are returned in the Fortran layouts ``init_elements_states_c`` takes
(``src/share/cxx/cxx_f90_interface.cpp:235-251``), as C-ordered numpy arrays with the
index order reversed: v ``(E,3,72,2,4,4)``, T/dp3d ``(E,3,72,4,4)``,
Qdp ``(E,2,Q,72,4,4)``, ps_v ``(E,3,4,4)``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

NLEV = 72
PS0 = 1.0e5
LMAX = 6


@dataclass
class HVCoord:
    ps0: float
    hyai: np.ndarray
    hybi: np.ndarray
    hyam: np.ndarray
    hybm: np.ndarray


def hybrid_coordinate(nlev: int = NLEV) -> HVCoord:
    eta = 0.001 + 0.999 * np.arange(nlev + 1) / nlev
    b = np.where(eta > 0.2, ((eta - 0.2) / 0.8) ** 2, 0.0)
    a = eta - b
    b[-1], a[-1] = 1.0, 0.0
    am = 0.5 * (a[1:] + a[:-1])
    bm = 0.5 * (b[1:] + b[:-1])
    return HVCoord(PS0, a.copy(), b.copy(), am, bm)


def _sph_basis(lat: np.ndarray, lon: np.ndarray, lmax: int = LMAX) -> np.ndarray:
    """Real, fully normalised spherical harmonics Y_lm for l <= lmax at the points.
    Returns ``((lmax+1)^2, npts)``."""
    x = np.sin(lat).ravel()
    lonf = lon.ravel()
    sx = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    npts = x.size
    # Normalised associated Legendre P_l^m by the standard stable recursion.
    P = {}
    pmm = np.full(npts, 1.0 / math.sqrt(4.0 * math.pi))
    for m in range(lmax + 1):
        if m > 0:
            pmm = -math.sqrt((2.0 * m + 1.0) / (2.0 * m)) * sx * pmm
        P[(m, m)] = pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = math.sqrt(2.0 * m + 3.0) * x * pmm
        for l in range(m + 2, lmax + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
            b = math.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
            P[(l, m)] = a * (x * P[(l - 1, m)] - b * P[(l - 2, m)])
    rows = []
    for l in range(lmax + 1):
        rows.append(P[(l, 0)])
        for m in range(1, l + 1):
            rows.append(math.sqrt(2.0) * P[(l, m)] * np.cos(m * lonf))
            rows.append(math.sqrt(2.0) * P[(l, m)] * np.sin(m * lonf))
    return np.array(rows)


def _smooth_coefficients(basis: np.ndarray, nfields: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal((nfields, basis.shape[0]))


def _smooth_rows(coef: np.ndarray, basis: np.ndarray) -> np.ndarray:
    f = coef @ basis
    f /= np.max(np.abs(f), axis=1, keepdims=True)
    return f


def _smooth_fields(basis: np.ndarray, nfields: int, seed: int) -> np.ndarray:
    return _smooth_rows(_smooth_coefficients(basis, nfields, seed), basis)


def dynamics_direction(mesh, seed: int, hv: HVCoord | None = None, lmax: int = LMAX):
    """Seeded smooth perturbation of the dynamics state (one time level): u, v of
    1 m/s, T of 1 K and dp3d of 1 % of the layer thickness, each a random sum of
    spherical harmonics up to degree ``lmax`` per level (continuous across elements)."""
    hv = hv or hybrid_coordinate()
    E = mesh.nelem
    basis = _sph_basis(mesh.lat, mesh.lon, lmax)
    shp = (E, 4, 4)
    f = _smooth_fields(basis, 4 * NLEV, seed).reshape(4, NLEV, *shp).transpose(0, 2, 1, 3, 4)
    dp = (np.diff(hv.hyai)[None, :, None, None] * hv.ps0
          + np.diff(hv.hybi)[None, :, None, None] * PS0)
    return dict(v=np.ascontiguousarray(np.stack([f[0], f[1]], axis=2)),
                T=np.ascontiguousarray(f[2]),
                dp3d=np.ascontiguousarray(0.01 * dp * f[3]))


def initial_state(mesh, qsize: int, hv: HVCoord | None = None):
    """Seeded smooth state on ``mesh``; every time level holds the same values."""
    hv = hv or hybrid_coordinate()
    E = mesh.nelem
    basis = _sph_basis(mesh.lat, mesh.lon)
    shp = (E, 4, 4)
    s_ps = _smooth_fields(basis, 1, 1001)[0].reshape(shp)
    ps = PS0 + 500.0 * s_ps
    da = np.diff(hv.hyai)
    db = np.diff(hv.hybi)
    dp = da[None, :, None, None] * hv.ps0 + db[None, :, None, None] * ps[:, None]
    pmid = hv.hyam[None, :, None, None] * hv.ps0 + hv.hybm[None, :, None, None] * ps[:, None]
    s_u = _smooth_fields(basis, NLEV, 1002).reshape(NLEV, *shp).transpose(1, 0, 2, 3)
    s_v = _smooth_fields(basis, NLEV, 1003).reshape(NLEV, *shp).transpose(1, 0, 2, 3)
    s_t = _smooth_fields(basis, NLEV, 1004).reshape(NLEV, *shp).transpose(1, 0, 2, 3)
    T = 300.0 - 60.0 * (1.0 - pmid / hv.ps0) + 2.0 * s_t
    vel = np.stack([20.0 * s_u, 20.0 * s_v], axis=2)          # (E,72,2,4,4)
    ntl = 3
    v_all = np.ascontiguousarray(np.broadcast_to(vel[:, None], (E, ntl) + vel.shape[1:]))
    t_all = np.ascontiguousarray(np.broadcast_to(T[:, None], (E, ntl) + T.shape[1:]))
    dp_all = np.ascontiguousarray(np.broadcast_to(dp[:, None], (E, ntl) + dp.shape[1:]))
    ps_all = np.ascontiguousarray(np.broadcast_to(ps[:, None], (E, ntl, 4, 4)))
    # tracers one at a time straight into both tracer time levels (large meshes)
    qdp_all = np.empty((E, 2, qsize, NLEV, 4, 4))
    if qsize > 0:
        coef = _smooth_coefficients(basis, qsize * NLEV, 1005)
        for i in range(qsize):
            s_q = _smooth_rows(coef[i * NLEV:(i + 1) * NLEV], basis).reshape(NLEV, *shp)
            qdp = 0.005 * (1.0 + s_q.transpose(1, 0, 2, 3)) * dp   # (E,72,4,4)
            qdp_all[:, 0, i] = qdp
            qdp_all[:, 1, i] = qdp
    return dict(v=v_all, T=t_all, dp3d=dp_all, Qdp=qdp_all, ps_v=ps_all)
