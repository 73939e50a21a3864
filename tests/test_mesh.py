"""Invariants of the cubed-sphere inputs (mesh, metric, connectivity, hybrid coordinate,
seeded state): what the Fortran side guarantees the preqx step before it runs."""
import math

import numpy as np
import pytest

import hxtest as H
from hommexx_gb300 import dss_tables, mesh as M, state as S


@pytest.mark.parametrize("ne", [1, 2, 4])
def test_area_and_metric(ne):
    m = M.build_mesh(ne)
    assert m.nelem == 6 * ne * ne
    # sum of spheremp over elements (the area correction makes it 4 pi exactly)
    assert abs(m.spheremp.sum() - 4 * math.pi) < 1e-12
    # D Dinv = I (C++ index order: X[e][idim][jdim])
    I = np.einsum("ekaij,elkij->elaij", m.D, m.Dinv)
    assert np.abs(I - np.eye(2)[None, :, :, None, None]).max() < 1e-13
    det = m.D[:, 0, 0] * m.D[:, 1, 1] - m.D[:, 0, 1] * m.D[:, 1, 0]
    assert (det > 0).all(), "every element frame is right-handed"
    assert np.abs(np.abs(det) - m.metdet).max() < 1e-15
    # metinv = Dinv Dinv^T (Fortran indices) = sum_c Dinv(c,a) Dinv(c,b) here
    mi = np.einsum("ecaij,ecbij->eabij", m.Dinv, m.Dinv)
    assert np.abs(mi - m.metinv).max() <= 1e-13 * np.abs(m.metinv).max()


def test_gll_and_dvv():
    assert abs(M.GLL_W.sum() - 2.0) < 1e-15
    d = M.derivative_matrix()      # d[j][k] = L'_k(x_j)
    assert np.abs(d.sum(axis=1)).max() < 1e-14          # derivative of a constant
    assert np.abs(d @ M.GLL_X - 1.0).max() < 1e-14      # derivative of x
    assert np.abs(d @ M.GLL_X ** 3 - 3 * M.GLL_X ** 2).max() < 1e-13


@pytest.mark.parametrize("ne", [2, 4])
def test_connectivity(ne):
    m = M.build_mesh(ne)
    c = m.connections
    E = m.nelem
    for e in range(E):
        for s in range(8):
            r, rs = c[e, s]
            if r < 0:
                continue
            assert tuple(c[r, rs]) == (e, s), "connections are symmetric"
    missing = int((c[:, 4:, 0] < 0).sum())
    assert missing == 24, "one missing corner at each of the 8 cube vertices x 3 elements"
    assert (c[:, :4, 0] >= 0).all(), "every edge has a neighbour"


@pytest.mark.parametrize("ne", [2, 4])
def test_gather_table_matches_geometry(ne):
    """The reference's point/direction tables (ConnectivityHelpers.hpp) pair exactly the
    GLL points that coincide on the sphere."""
    m = M.build_mesh(ne)
    se, sp, cnt = dss_tables.build_gather_table(m.connections)
    for pts in M.dss_point_sources(m).values():
        for (e, i, j) in pts:
            p = 4 * i + j
            got = {(int(se[e, p, k]), int(sp[e, p, k]) // 4, int(sp[e, p, k]) % 4)
                   for k in range(cnt[e, p])}
            assert got == set(pts) - {(e, i, j)}


def test_rspheremp_is_inverse_assembled_mass():
    m = M.build_mesh(4)
    groups = M.dss_point_sources(m)
    for pts in groups.values():
        tot = sum(m.spheremp[e, i, j] for (e, i, j) in pts)
        for (e, i, j) in pts:
            assert abs(m.rspheremp[e, i, j] * tot - 1.0) < 1e-14


def test_hybrid_coordinate():
    hv = S.hybrid_coordinate()
    assert hv.hyai.shape == (73,) and hv.hybi.shape == (73,)
    assert hv.hybi[0] == 0.0 and hv.hyai[-1] == 0.0 and hv.hybi[-1] == 1.0
    assert (np.diff(hv.hyai + hv.hybi) > 0).all()
    eta = 0.001 + 0.999 * np.arange(73) / 72
    assert np.allclose(hv.hyai + hv.hybi, eta, atol=1e-15)


def test_seeded_state_is_deterministic_and_bounded():
    m = H.mesh(4)
    a = S.initial_state(m, 3)
    b = S.initial_state(m, 3)
    for k in a:
        assert np.array_equal(a[k], b[k])
    ps = a["ps_v"]
    assert abs(ps.max() - 1e5) <= 500 + 1e-9 and ps.min() >= 1e5 - 500 - 1e-9
    v = a["v"]
    assert np.abs(v).max() <= 20.0 + 1e-12
    q = a["Qdp"][:, 0] / a["dp3d"][:, 1][:, None]
    assert q.min() >= -1e-15 and q.max() <= 0.01 + 1e-15
    # dp3d follows the hybrid coordinate from ps
    hv = S.hybrid_coordinate()
    dp = np.diff(hv.hyai)[None, :, None, None] * 1e5 + np.diff(hv.hybi)[None, :, None, None] * ps[:, 1][:, None]
    assert np.allclose(a["dp3d"][:, 1], dp, rtol=1e-15, atol=0)
