"""Equiangular gnomonic cubed-sphere mesh, metric terms and element connectivity.

This module plays the part of the Fortran side of HOMME that builds the inputs of the
preqx step before it calls the C++ step through ``init_elements_2d_c`` and
``add_connection``.  It is input generation, not part of the timed path:

* GLL points/weights and the derivative matrix ``dvv`` follow
  ``src/share/quadrature_mod.F90`` (gausslobatto) and
  ``src/share/derivative_mod_base.F90:437-475`` (dvvinit): ``dvv(a,b) = L'_a(x_b)``.
* The metric follows ``src/share/cube_mod.F90:215-454`` (metric_atomic): ``D`` maps
  contravariant reference-element components to (east, north) components on the unit
  sphere, ``Dinv = D^-1``, ``metdet = |det D|``, ``metinv = (D^T D)^-1``, followed by
  the area correction ``alpha = 4 pi / sum(mp*metdet)`` of
  ``src/share/prim_driver_mod.F90:403-418``.
* ``mp = w_i w_j``, ``spheremp = mp*metdet``, ``rspheremp = 1/DSS(spheremp)``
  (``src/share/mass_matrix_mod.F90:98-115``); ``fcor = 2 Omega sin(lat)``
  (``src/share/cube_mod.F90:800-825``).
* Connections use the Fortran direction numbering W=1, E=2, S=3, N=4, SW=5, SE=6,
  NW=7, NE=8 that ``add_connection`` receives
  (``src/share/cxx/mpi/mpi_cxx_f90_interface.cpp:34-54``).

Array layouts are the Fortran column-major layouts that the reference's C ABI takes,
stored as C-ordered numpy arrays with the index order reversed, e.g. ``D`` is
``(nelemd, 2, 2, np, np)`` for Fortran ``D(np,np,2,2,nelemd)``.  Read with the reference
C++ index names this is ``D[ie][idim][jdim][igp][jgp]`` with ``igp`` the Fortran ``j``
(x2 direction) and ``jgp`` the Fortran ``i`` (x1 direction).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NP = 4
NLEV = 72
REARTH = 6.376e6
OMEGA = 7.292e-5

# GLL points and weights for np=4 on [-1, 1].
GLL_X = np.array([-1.0, -1.0 / math.sqrt(5.0), 1.0 / math.sqrt(5.0), 1.0])
GLL_W = np.array([1.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, 1.0 / 6.0])

# Cube faces: outward centre c, tangent a (x1 / alpha direction), tangent b
# (x2 / beta direction), with a x b = c so every element frame is right-handed.
_FACES = [
    ((1, 0, 0), (0, 1, 0), (0, 0, 1)),
    ((0, 1, 0), (-1, 0, 0), (0, 0, 1)),
    ((-1, 0, 0), (0, -1, 0), (0, 0, 1)),
    ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
    ((0, 0, -1), (0, 1, 0), (1, 0, 0)),
    ((0, 0, 1), (0, 1, 0), (-1, 0, 0)),
]

# Reference C++ connection slots (ConnectionName): S, N, W, E, SW, SE, NW, NE.
SOUTH, NORTH, WEST, EAST, SWEST, SEAST, NWEST, NEAST = range(8)
# Fortran position numbers for each C++ slot (the inverse of convert() in
# mpi_cxx_f90_interface.cpp).
F90_POS_OF_SLOT = [3, 4, 1, 2, 5, 6, 7, 8]


def legendre_np(x: float, n: int) -> float:
    """Legendre polynomial P_n(x) by the three-term recurrence."""
    p0, p1 = 1.0, x
    if n == 0:
        return p0
    for k in range(1, n):
        p0, p1 = p1, ((2 * k + 1) * x * p1 - k * p0) / (k + 1)
    return p1


def derivative_matrix() -> np.ndarray:
    """dvv in the reference C++ index order: ``dvv[j][k] = L'_k(x_j)``.

    Its flat memory equals the Fortran ``dvv(np,np)`` of dvvinit, where
    ``dvv(a,b) = L'_a(x_b)``; ``init_derivative_c`` receives this memory.
    """
    n = NP
    x = GLL_X
    leg = np.array([legendre_np(xi, n - 1) for xi in x])
    d = np.zeros((n, n))  # d[a][b] = L'_a(x_b)  (Fortran dvv(a,b))
    for a in range(n):
        for b in range(n):
            if a != b:
                d[a, b] = (1.0 / (x[b] - x[a])) * leg[b] / leg[a]
    d[n - 1, n - 1] = n * (n - 1) / 4.0
    d[0, 0] = -n * (n - 1) / 4.0
    # Fortran memory index (a + n*b) -> C++ dvv[b][a].
    return np.ascontiguousarray(d.T)


@dataclass
class Mesh:
    ne: int
    nelem: int
    dvv: np.ndarray            # (4,4) C++ order
    D: np.ndarray              # (E,2,2,4,4)
    Dinv: np.ndarray
    metinv: np.ndarray
    metdet: np.ndarray         # (E,4,4)
    mp: np.ndarray
    spheremp: np.ndarray
    rspheremp: np.ndarray
    fcor: np.ndarray
    phis: np.ndarray
    lat: np.ndarray
    lon: np.ndarray
    vec_sph2cart: np.ndarray   # (E,2,3,4,4)
    tensorvisc: np.ndarray     # (E,2,2,4,4)
    # connections[e][slot] = (remote_elem, remote_slot) or (-1, -1) when missing
    connections: np.ndarray    # (E,8,2) int
    alpha: float = 1.0
    xyz: np.ndarray = field(default=None, repr=False)  # (E,4,4,3)

    def f90_connections(self):
        """Yield the 8-int tuples ``add_connection`` receives (1-based, F90 slots)."""
        for e in range(self.nelem):
            for s in range(8):
                r, rs = self.connections[e, s]
                if r < 0:
                    continue
                yield (e + 1, e + 1, F90_POS_OF_SLOT[s], 1,
                       int(r) + 1, int(r) + 1, F90_POS_OF_SLOT[int(rs)], 1)


def _frames():
    out = []
    for c, a, b in _FACES:
        out.append((np.array(c, float), np.array(a, float), np.array(b, float)))
    return out


def build_mesh(ne: int, hypervis_scaling: float = 0.0) -> Mesh:
    """Build the equiangular cubed sphere with ``6*ne*ne`` elements of np=4."""
    nelem = 6 * ne * ne
    h = (math.pi / 2.0) / ne
    frames = _frames()
    # Element order: face-major, then x2 (row), then x1 (column).
    fidx = np.repeat(np.arange(6), ne * ne)
    ej = np.tile(np.repeat(np.arange(ne), ne), 6)
    ei = np.tile(np.arange(ne), 6 * ne)
    # alpha along x1 (Fortran i = C++ jgp), beta along x2 (Fortran j = C++ igp)
    a_lo = -math.pi / 4 + ei * h
    b_lo = -math.pi / 4 + ej * h
    s = (1.0 + GLL_X) * (h / 2.0)
    alpha = a_lo[:, None, None] + s[None, None, :]          # (E, igp(=1), jgp)
    beta = b_lo[:, None, None] + s[None, :, None]           # (E, igp, jgp(=1))
    alpha = np.broadcast_to(alpha, (nelem, NP, NP)).copy()
    beta = np.broadcast_to(beta, (nelem, NP, NP)).copy()
    # Exact zeros where the GLL point sits on a face centre line.
    alpha[np.abs(alpha) < 1e-15] = 0.0
    beta[np.abs(beta) < 1e-15] = 0.0
    ta, tb = np.tan(alpha), np.tan(beta)
    C = np.stack([frames[f][0] for f in range(6)])[fidx]   # (E,3)
    A = np.stack([frames[f][1] for f in range(6)])[fidx]
    B = np.stack([frames[f][2] for f in range(6)])[fidx]
    v = (C[:, None, None, :] + ta[..., None] * A[:, None, None, :]
         + tb[..., None] * B[:, None, None, :])              # (E,4,4,3)
    r2 = 1.0 + ta * ta + tb * tb
    r = np.sqrt(r2)
    P = v / r[..., None]
    sa2 = 1.0 + ta * ta
    sb2 = 1.0 + tb * tb
    # dP/dalpha = sec^2(alpha) (a |v|^2 - v tan(alpha)) / |v|^3, likewise for beta.
    dPa = (sa2 / (r2 * r))[..., None] * (A[:, None, None, :] * r2[..., None] - v * ta[..., None])
    dPb = (sb2 / (r2 * r))[..., None] * (B[:, None, None, :] * r2[..., None] - v * tb[..., None])
    dPx1 = dPa * (h / 2.0)
    dPx2 = dPb * (h / 2.0)
    x, y, z = P[..., 0], P[..., 1], P[..., 2]
    rho = np.hypot(x, y)
    lon = np.where(rho < 1e-14, 0.0, np.arctan2(y, x))
    lat = np.arctan2(z, rho)
    sl, cl = np.sin(lon), np.cos(lon)
    sp, cp = np.sin(lat), np.cos(lat)
    east = np.stack([-sl, cl, np.zeros_like(sl)], axis=-1)
    north = np.stack([-sp * cl, -sp * sl, cp], axis=-1)
    # Dphys[a][k]: a = physical component (east, north), k = reference direction.
    D11 = np.sum(east * dPx1, -1)
    D12 = np.sum(east * dPx2, -1)
    D21 = np.sum(north * dPx1, -1)
    D22 = np.sum(north * dPx2, -1)
    det = D11 * D22 - D12 * D21
    mp = np.broadcast_to(GLL_W[:, None] * GLL_W[None, :], (nelem, NP, NP)).copy()
    area = float(np.sum(mp * np.abs(det)))
    alpha_c = 4.0 * math.pi / area
    sq = math.sqrt(alpha_c)
    Dp = np.empty((nelem, 2, 2, NP, NP))    # Dp[e][a][k]
    Dp[:, 0, 0], Dp[:, 0, 1], Dp[:, 1, 0], Dp[:, 1, 1] = D11, D12, D21, D22
    Dinvp = np.empty_like(Dp)
    Dinvp[:, 0, 0] = D22 / det
    Dinvp[:, 0, 1] = -D12 / det
    Dinvp[:, 1, 0] = -D21 / det
    Dinvp[:, 1, 1] = D11 / det
    met = np.einsum('eakij,ealij->eklij', Dp, Dp)
    metinvp = np.empty_like(met)
    d2 = det * det
    metinvp[:, 0, 0] = met[:, 1, 1] / d2
    metinvp[:, 0, 1] = -met[:, 0, 1] / d2
    metinvp[:, 1, 0] = -met[:, 1, 0] / d2
    metinvp[:, 1, 1] = met[:, 0, 0] / d2
    Dp *= sq
    Dinvp /= sq
    metinvp /= alpha_c
    metdet = np.abs(det) * alpha_c
    # C++ order X[e][idim][jdim] = Fortran X(:,:,jdim,idim) = phys X[jdim][idim].
    D = np.ascontiguousarray(np.swapaxes(Dp, 1, 2))
    Dinv = np.ascontiguousarray(np.swapaxes(Dinvp, 1, 2))
    metinv = np.ascontiguousarray(np.swapaxes(metinvp, 1, 2))

    # Topology from shared corner/edge geometry.
    conn = _connectivity(P, nelem)
    spheremp = mp * metdet
    rsm = _dss_scalar(spheremp, conn)
    rspheremp = 1.0 / rsm
    fcor = 2.0 * OMEGA * np.sin(lat)
    vec = np.empty((nelem, 2, 3, NP, NP))
    # Fortran vec_sphere2cart(np,np,3,2): (:,:,c,1) zonal, (:,:,c,2) meridional;
    # C++ order [e][comp2][cart3].
    vec[:, 0, 0], vec[:, 0, 1], vec[:, 0, 2] = -sl, cl, 0.0
    vec[:, 1, 0], vec[:, 1, 1], vec[:, 1, 2] = -sp * cl, -sp * sl, cp
    tens = _tensor_visc(Dp, metinvp, hypervis_scaling)
    return Mesh(ne=ne, nelem=nelem, dvv=derivative_matrix(), D=D, Dinv=Dinv,
                metinv=metinv, metdet=np.ascontiguousarray(metdet), mp=mp,
                spheremp=np.ascontiguousarray(spheremp),
                rspheremp=np.ascontiguousarray(rspheremp),
                fcor=np.ascontiguousarray(fcor), phis=np.zeros((nelem, NP, NP)),
                lat=lat, lon=lon, vec_sph2cart=vec, tensorvisc=tens,
                connections=conn, alpha=alpha_c, xyz=P)


def _tensor_visc(Dp, metinvp, hypervis_scaling):
    """tensorVisc of metric_atomic (cube_mod.F90:310-440) in C++ index order."""
    E = Dp.shape[0]
    out = np.zeros((E, 2, 2, NP, NP))
    if hypervis_scaling == 0.0:
        return out
    M = np.moveaxis(metinvp, (1, 2), (-2, -1))          # (E,4,4,2,2)
    Dm = np.moveaxis(Dp, (1, 2), (-2, -1))
    tr = M[..., 0, 0] + M[..., 1, 1]
    disc = np.sqrt(4.0 * M[..., 0, 1] * M[..., 1, 0] + (M[..., 0, 0] - M[..., 1, 1]) ** 2)
    eig1 = (tr + disc) / 2.0
    eig2 = (tr - disc) / 2.0
    w, V = np.linalg.eigh(M)                              # ascending eigenvalues
    E1 = V[..., :, 1]
    E2 = np.stack([-E1[..., 1], E1[..., 0]], -1)
    DE1 = np.einsum('...ak,...k->...a', Dm, E1)
    DE2 = np.einsum('...ak,...k->...a', Dm, E2)
    lam1 = 1.0 / (eig1 ** (hypervis_scaling / 4.0)) * REARTH ** 2
    lam2 = 1.0 / (eig2 ** (hypervis_scaling / 4.0)) * REARTH ** 2
    DEL1 = (lam1 ** 2 * eig1)[..., None] * DE1
    DEL2 = (lam2 ** 2 * eig2)[..., None] * DE2
    Vt = (DEL1[..., :, None] * DE1[..., None, :] + DEL2[..., :, None] * DE2[..., None, :])
    # Vt[a][b] physical -> C++ order [e][b][a]
    out[:] = np.moveaxis(Vt, (-2, -1), (2, 1))
    return out


def _corner_keys(P):
    return np.round(P * 1e9).astype(np.int64)


# Local GLL point (igp, jgp) of each corner slot: SW, SE, NW, NE.
_CORNER_PT = {SWEST: (0, 0), SEAST: (0, 3), NWEST: (3, 0), NEAST: (3, 3)}
# Corner-slot pairs (in order along the natural edge direction) for each edge slot.
_EDGE_CORNERS = {SOUTH: (SWEST, SEAST), NORTH: (NWEST, NEAST),
                 WEST: (SWEST, NWEST), EAST: (SEAST, NEAST)}


def _connectivity(P, nelem):
    keys = _corner_keys(P)
    node_of = {}
    enodes = np.zeros((nelem, 4), dtype=np.int64)   # indexed by corner slot - 4
    for e in range(nelem):
        for cs, (ip, jp) in _CORNER_PT.items():
            k = tuple(keys[e, ip, jp])
            nid = node_of.setdefault(k, len(node_of))
            enodes[e, cs - 4] = nid
    elems_of_node = {}
    for e in range(nelem):
        for c in range(4):
            elems_of_node.setdefault(int(enodes[e, c]), []).append(e)
    edge_owner = {}
    for e in range(nelem):
        for es, (c0, c1) in _EDGE_CORNERS.items():
            pair = frozenset((int(enodes[e, c0 - 4]), int(enodes[e, c1 - 4])))
            edge_owner.setdefault(pair, []).append((e, es))
    conn = -np.ones((nelem, 8, 2), dtype=np.int64)
    for pair, owners in edge_owner.items():
        assert len(owners) == 2, "every edge is shared by exactly two elements"
        (e0, s0), (e1, s1) = owners
        conn[e0, s0] = (e1, s1)
        conn[e1, s1] = (e0, s0)
    for e in range(nelem):
        edge_nbrs = {int(conn[e, s, 0]) for s in range(4)}
        for cs in (SWEST, SEAST, NWEST, NEAST):
            nid = int(enodes[e, cs - 4])
            cands = [o for o in elems_of_node[nid] if o != e and o not in edge_nbrs]
            assert len(cands) <= 1
            if cands:
                o = cands[0]
                ocs = [c + 4 for c in range(4) if int(enodes[o, c]) == nid]
                conn[e, cs] = (o, ocs[0])
    return conn


def dss_point_sources(mesh: Mesh):
    """Geometric check table: for each (elem, igp, jgp) the set of other (elem, igp, jgp)
    at the same location.  Used by tests to validate connection-based DSS."""
    keys = _corner_keys(mesh.xyz)
    groups = {}
    E = mesh.nelem
    for e in range(E):
        for i in range(NP):
            for j in range(NP):
                groups.setdefault(tuple(keys[e, i, j]), []).append((e, i, j))
    return groups


def _dss_scalar(f, conn):
    """Plain DSS of a 2-D field using geometric point identity (for rspheremp)."""
    # Use the connection tables through the same helper the oracle restates.
    from .dss_tables import build_gather_table
    tab = build_gather_table(conn)
    E = f.shape[0]
    flat = f.reshape(E, 16)
    out = flat.copy()
    src_e, src_p, cnt = tab
    for e in range(E):
        for p in range(16):
            acc = flat[e, p]
            for k in range(cnt[e, p]):
                acc = acc + flat[src_e[e, p, k], src_p[e, p, k]]
            out[e, p] = acc
    return out.reshape(E, NP, NP)
