// hx_mesh.cu — the equiangular gnomonic cubed-sphere mesh, its metric and its element
// connectivity, generated for hx_cube_mesh.  In the reference this is the Fortran side's
// input generation (src/share/cube_mod.F90:215-454 metric_atomic, :800-825 coriolis;
// src/share/mass_matrix_mod.F90:98-115; src/share/prim_driver_mod.F90:403-418 area
// correction) before it calls init_elements_2d_c and add_connection.
//
// Geometry: face f has outward centre c, tangents a (x1 / alpha) and b (x2 / beta) with
// a x b = c; a GLL point at angles (alpha, beta) maps to P = (c + tan(alpha) a +
// tan(beta) b) / |.|.  D maps contravariant reference-element components to (east,
// north) components; Dinv = D^-1, metdet = |det D|, metinv = (D^T D)^-1, all rescaled so
// that the mesh area is 4 pi.  Elements are ordered face by face, then by row (x2),
// then by column (x1).  One thread per GLL point; the metric is elementwise work.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "hx_device.cuh"

namespace hx {
namespace {

// centre, alpha tangent, beta tangent of the six faces
__constant__ int c_faces[6][3][3] = {
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},   {{0, 1, 0}, {-1, 0, 0}, {0, 0, 1}}, {{-1, 0, 0}, {0, -1, 0}, {0, 0, 1}},
    {{0, -1, 0}, {1, 0, 0}, {0, 0, 1}},  {{0, 0, -1}, {0, 1, 0}, {1, 0, 0}}, {{0, 0, 1}, {0, 1, 0}, {-1, 0, 0}}};
const int h_faces[6][3][3] = {
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},   {{0, 1, 0}, {-1, 0, 0}, {0, 0, 1}}, {{-1, 0, 0}, {0, -1, 0}, {0, 0, 1}},
    {{0, -1, 0}, {1, 0, 0}, {0, 0, 1}},  {{0, 0, -1}, {0, 1, 0}, {1, 0, 0}}, {{0, 0, 1}, {0, 1, 0}, {-1, 0, 0}}};

struct Gll {
  double x[4], w[4];
};

// Per point: the unscaled Jacobian (D11, D12, D21, D22 = east.dP/dx1, east.dP/dx2,
// north.dP/dx1, north.dP/dx2), its determinant, lat and lon.  geo [E][7][16].
__global__ void k_cube_geometry(int ne, Gll g, double* __restrict__ geo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int E = 6 * ne * ne;
  if (i >= E * 16) return;
  const int e = i >> 4, p = i & 15, igp = p >> 2, jgp = p & 3;
  const int f = e / (ne * ne), r = e - f * ne * ne, ej = r / ne, ei = r - ej * ne;
  const double h = (M_PI / 2.0) / ne;
  double alpha = (-M_PI / 4.0 + ei * h) + (1.0 + g.x[jgp]) * (h / 2.0);
  double beta = (-M_PI / 4.0 + ej * h) + (1.0 + g.x[igp]) * (h / 2.0);
  if (fabs(alpha) < 1e-15) alpha = 0.0;
  if (fabs(beta) < 1e-15) beta = 0.0;
  const double ta = tan(alpha), tb = tan(beta);
  double C[3], A[3], B[3], v[3];
  for (int k = 0; k < 3; ++k) {
    C[k] = c_faces[f][0][k];
    A[k] = c_faces[f][1][k];
    B[k] = c_faces[f][2][k];
    v[k] = C[k] + ta * A[k] + tb * B[k];
  }
  const double r2 = 1.0 + ta * ta + tb * tb, rr = sqrt(r2);
  const double sa = (1.0 + ta * ta) / (r2 * rr) * (h / 2.0), sb = (1.0 + tb * tb) / (r2 * rr) * (h / 2.0);
  double P[3], d1[3], d2[3];
  for (int k = 0; k < 3; ++k) {
    P[k] = v[k] / rr;
    d1[k] = sa * (A[k] * r2 - v[k] * ta);  // dP/dx1
    d2[k] = sb * (B[k] * r2 - v[k] * tb);  // dP/dx2
  }
  const double rho = hypot(P[0], P[1]);
  const double lon = rho < 1e-14 ? 0.0 : atan2(P[1], P[0]);
  const double lat = atan2(P[2], rho);
  double sl, cl, sp, cp;
  sincos(lon, &sl, &cl);
  sincos(lat, &sp, &cp);
  const double east[3] = {-sl, cl, 0.0}, north[3] = {-sp * cl, -sp * sl, cp};
  double D11 = 0, D12 = 0, D21 = 0, D22 = 0;
  for (int k = 0; k < 3; ++k) {
    D11 += east[k] * d1[k];
    D12 += east[k] * d2[k];
    D21 += north[k] * d1[k];
    D22 += north[k] * d2[k];
  }
  double* o = geo + (size_t)e * 7 * 16 + p;
  o[0] = D11;
  o[16] = D12;
  o[32] = D21;
  o[48] = D22;
  o[64] = D11 * D22 - D12 * D21;
  o[80] = lat;
  o[96] = lon;
}

// The scaled metric in the layouts init_elements_2d_c takes (C index order [e][i][j]
// for Fortran X(:,:,j,i)); alpha_c = 4 pi / area.
struct MetricOut {
  double *D, *Dinv, *metinv, *metdet, *mp, *spheremp, *fcor, *vec, *tens, *lat, *lon;
};

__global__ void k_cube_metric(int E, Gll g, const double* __restrict__ geo, double alpha_c, double hvs,
                              double rearth, double omega, MetricOut o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E * 16) return;
  const int e = i >> 4, p = i & 15, igp = p >> 2, jgp = p & 3;
  const double* q = geo + (size_t)e * 7 * 16 + p;
  const double d11 = q[0], d12 = q[16], d21 = q[32], d22 = q[48], det = q[64], lat = q[80], lon = q[96];
  const double sq = sqrt(alpha_c);
  // Dp[a][k]: a = (east, north), k = reference direction
  const double Dp[2][2] = {{d11 * sq, d12 * sq}, {d21 * sq, d22 * sq}};
  const double Di[2][2] = {{d22 / det / sq, -d12 / det / sq}, {-d21 / det / sq, d11 / det / sq}};
  const double m00 = d11 * d11 + d21 * d21, m01 = d11 * d12 + d21 * d22, m11 = d12 * d12 + d22 * d22;
  const double dd = det * det;
  const double Mi[2][2] = {{m11 / dd / alpha_c, -m01 / dd / alpha_c}, {-m01 / dd / alpha_c, m00 / dd / alpha_c}};
  const size_t b4 = (size_t)e * 64 + p, b1 = (size_t)e * 16 + p;
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < 2; ++k) {
      const size_t o2 = b4 + (size_t)(k * 2 + a) * 16;  // C order [k][a] = Fortran (:,:,a,k)
      if (o.D) o.D[o2] = Dp[a][k];
      if (o.Dinv) o.Dinv[o2] = Di[a][k];
      if (o.metinv) o.metinv[o2] = Mi[a][k];
    }
  const double md = fabs(det) * alpha_c, w = g.w[igp] * g.w[jgp];
  if (o.metdet) o.metdet[b1] = md;
  if (o.mp) o.mp[b1] = w;
  if (o.spheremp) o.spheremp[b1] = w * md;
  if (o.fcor) o.fcor[b1] = 2.0 * omega * sin(lat);
  if (o.lat) o.lat[b1] = lat;
  if (o.lon) o.lon[b1] = lon;
  double sl, cl, sp, cp;
  sincos(lon, &sl, &cl);
  sincos(lat, &sp, &cp);
  if (o.vec) {
    const double vv[2][3] = {{-sl, cl, 0.0}, {-sp * cl, -sp * sl, cp}};
    for (int c = 0; c < 2; ++c)
      for (int k = 0; k < 3; ++k) o.vec[(size_t)e * 96 + (c * 3 + k) * 16 + p] = vv[c][k];
  }
  if (o.tens) {
    double V[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    if (hvs != 0.0) {
      // eigenpairs of the symmetric metinv: e1 >= e2, E1 the eigenvector of e1 (either
      // sign; the tensor below does not depend on it), E2 = E1 rotated by 90 degrees
      const double a = Mi[0][0], b = Mi[0][1], d = Mi[1][1];
      const double tr = a + d, disc = sqrt(4.0 * b * b + (a - d) * (a - d));
      const double e1 = (tr + disc) / 2.0, e2 = (tr - disc) / 2.0;
      double u0 = b, u1 = e1 - a, w0 = e1 - d, w1 = b;
      double x0, x1;
      if (u0 * u0 + u1 * u1 >= w0 * w0 + w1 * w1) { x0 = u0; x1 = u1; }
      else { x0 = w0; x1 = w1; }
      const double nrm = sqrt(x0 * x0 + x1 * x1);
      if (nrm > 0.0) { x0 /= nrm; x1 /= nrm; }
      else { x0 = 1.0; x1 = 0.0; }
      const double E1[2] = {x0, x1}, E2[2] = {-x1, x0};
      double DE1[2], DE2[2];
      for (int r = 0; r < 2; ++r) {
        DE1[r] = Dp[r][0] * E1[0] + Dp[r][1] * E1[1];
        DE2[r] = Dp[r][0] * E2[0] + Dp[r][1] * E2[1];
      }
      const double l1 = 1.0 / pow(e1, hvs / 4.0) * rearth * rearth;
      const double l2 = 1.0 / pow(e2, hvs / 4.0) * rearth * rearth;
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) V[r][c] = (l1 * l1 * e1) * DE1[r] * DE1[c] + (l2 * l2 * e2) * DE2[r] * DE2[c];
    }
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) o.tens[b4 + (size_t)(c * 2 + r) * 16] = V[r][c];  // [e][c][r] = Vt[r][c]
  }
}

}  // namespace

// Element connectivity of the cube in the session's format [E][8][2] = (remote element,
// remote slot), 0-based, slots S N W E SW SE NW NE, -1 where absent.  Element corners are
// keyed by their exact integer position on the cube lattice [-ne, ne]^3 (the corner at
// grid indices (i, j) of face f is ne c + (2i - ne) a + (2j - ne) b), so that two faces
// identify a shared corner without comparing floating-point coordinates.  Edges join the
// two elements whose corner pairs coincide; a corner slot joins the element that shares
// only that corner (none at the eight cube corners, where three elements meet).
std::vector<int> cube_connectivity(int ne) {
  const int E = 6 * ne * ne, W = 2 * ne + 1;
  auto key = [&](int f, int i, int j) {
    long long k[3];
    for (int c = 0; c < 3; ++c)
      k[c] = (long long)ne * h_faces[f][0][c] + (long long)(2 * i - ne) * h_faces[f][1][c] +
             (long long)(2 * j - ne) * h_faces[f][2][c] + ne;
    return (k[0] * W + k[1]) * W + k[2];
  };
  // corner slots 4..7 = SW, SE, NW, NE at grid offsets (di, dj)
  const int cdi[4] = {0, 1, 0, 1}, cdj[4] = {0, 0, 1, 1};
  std::unordered_map<long long, int> node_of;
  std::vector<int> enodes((size_t)E * 4);
  for (int e = 0; e < E; ++e) {
    const int f = e / (ne * ne), r = e % (ne * ne), ej = r / ne, ei = r % ne;
    for (int c = 0; c < 4; ++c) {
      const long long k = key(f, ei + cdi[c], ej + cdj[c]);
      auto it = node_of.emplace(k, (int)node_of.size()).first;
      enodes[(size_t)e * 4 + c] = it->second;
    }
  }
  std::vector<std::vector<int>> elems_of_node(node_of.size());
  for (int e = 0; e < E; ++e)
    for (int c = 0; c < 4; ++c) elems_of_node[enodes[(size_t)e * 4 + c]].push_back(e);
  // edge slots S, N, W, E and their corner-slot pairs
  const int ec[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
  std::vector<int> conn((size_t)E * 16, -1);
  std::unordered_map<long long, std::pair<int, int>> first_owner;
  for (int e = 0; e < E; ++e)
    for (int s = 0; s < 4; ++s) {
      long long a = enodes[(size_t)e * 4 + ec[s][0]], b = enodes[(size_t)e * 4 + ec[s][1]];
      if (a > b) std::swap(a, b);
      const long long k = a * (long long)node_of.size() + b;
      auto it = first_owner.find(k);
      if (it == first_owner.end()) {
        first_owner.emplace(k, std::make_pair(e, s));
      } else {
        const int e0 = it->second.first, s0 = it->second.second;
        conn[((size_t)e0 * 8 + s0) * 2] = e;
        conn[((size_t)e0 * 8 + s0) * 2 + 1] = s;
        conn[((size_t)e * 8 + s) * 2] = e0;
        conn[((size_t)e * 8 + s) * 2 + 1] = s0;
      }
    }
  for (int e = 0; e < E; ++e)
    for (int c = 0; c < 4; ++c) {
      const int nid = enodes[(size_t)e * 4 + c];
      for (int o : elems_of_node[nid]) {
        if (o == e) continue;
        bool edge_nbr = false;
        for (int s = 0; s < 4; ++s) edge_nbr |= conn[((size_t)e * 8 + s) * 2] == o;
        if (edge_nbr) continue;
        for (int oc = 0; oc < 4; ++oc)
          if (enodes[(size_t)o * 4 + oc] == nid) {
            conn[((size_t)e * 8 + 4 + c) * 2] = o;
            conn[((size_t)e * 8 + 4 + c) * 2 + 1] = 4 + oc;
          }
      }
    }
  return conn;
}

// Metric of the cube mesh into device arrays (any may be null); returns the area
// correction alpha_c.  The host sums the per-point areas in element order.
CubeMeshStatus cube_metric(int ne, double hvs, const CubeMeshDev& out, cudaStream_t s) {
  CubeMeshStatus st{};
  const int E = 6 * ne * ne;
  Gll g;
  g.x[0] = -1.0; g.x[1] = -1.0 / std::sqrt(5.0); g.x[2] = 1.0 / std::sqrt(5.0); g.x[3] = 1.0;
  g.w[0] = 1.0 / 6.0; g.w[1] = 5.0 / 6.0; g.w[2] = 5.0 / 6.0; g.w[3] = 1.0 / 6.0;
  double* geo = nullptr;
  st.err = cudaMalloc(&geo, sizeof(double) * (size_t)E * 7 * 16);
  if (st.err != cudaSuccess) return st;
  {
    KScope k("cube_geometry", s);
    k_cube_geometry<<<nblk((long long)E * 16, 128), 128, 0, s>>>(ne, g, geo);
  }
  std::vector<double> h((size_t)E * 7 * 16);
  st.err = cudaMemcpyAsync(h.data(), geo, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s);
  if (st.err == cudaSuccess) st.err = cudaStreamSynchronize(s);
  if (st.err != cudaSuccess) {
    cudaFree(geo);
    return st;
  }
  double area = 0.0;
  for (int e = 0; e < E; ++e)
    for (int p = 0; p < 16; ++p) area += g.w[p >> 2] * g.w[p & 3] * std::fabs(h[((size_t)e * 7 + 4) * 16 + p]);
  st.alpha_c = 4.0 * M_PI / area;
  MetricOut o{out.D, out.Dinv, out.metinv, out.metdet, out.mp, out.spheremp, out.fcor, out.vec,
              out.tens, out.lat, out.lon};
  {
    KScope k("cube_metric", s);
    k_cube_metric<<<nblk((long long)E * 16, 128), 128, 0, s>>>(E, g, geo, st.alpha_c, hvs, 6.376e6, 7.292e-5, o);
  }
  st.err = cudaGetLastError();
  if (st.err == cudaSuccess) st.err = cudaStreamSynchronize(s);
  cudaFree(geo);
  return st;
}

}  // namespace hx
