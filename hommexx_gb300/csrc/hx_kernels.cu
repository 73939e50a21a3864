// hx_kernels.cu — hand-written sm_103a kernels of the preqx dycore step.
//
// Thread mapping of the element kernels: one CTA per element (or per element x
// tracer), 16*LG threads; thread (p = tid % 16, lg = tid / 16) owns GLL point p on
// levels lg, lg+LG, ...  The 16 points of a level sit in one half-warp, so the 4x4
// derivative contractions of the sphere operators are register shuffles within the
// half-warp (no shared memory, no barriers).  Vertical scans go through shared memory
// ([lev][17] rows) and run as segmented warp scans in double.  DSS is a gather over a
// precomputed table (whole mesh resident, no buffers, no MPI): each output point adds
// its neighbours' values in the reference's fixed order, in double.
//
// Reference routines restated here (all under src/share/cxx/):
//   SphereOperators.hpp:291-862, CaarFunctorImpl.hpp:97-889, CaarFunctor.cpp:96-116,
//   HyperviscosityFunctorImpl.{hpp:72-257,cpp:56-112}, EulerStepFunctorImpl.hpp:118-884,
//   RemapFunctor.hpp:299-463, PpmRemap.hpp:174-689, BoundaryExchange.cpp:285-849,
//   prim_driver.cpp:90-206, prim_step.cpp:42-66, prim_advance_exp.cpp:138-156.
#include <algorithm>
#include <cstdio>

#include "hx_device.cuh"

namespace hx {

namespace {

// ======================================================================================
// Caar RK stage (CaarFunctorImpl::operator(), rsplit > 0), one CTA per element.
// Writes the pre-DSS v, T, dp3d of time level np1 to a.out; updates vn0, omega_p, phi.
// ======================================================================================
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_caar(CaarArgs<R> a) {
  constexpr int NL = NLEV / LG;
  extern __shared__ double sm[];
  // FP64 form: dp3d(n0) (later phi), T_v, div(v dp), pressure, omega integral
  // sum_{j<k} div_vdp_j, 1/p and the column sum of div(v dp) (rsplit == 0), all double.
  // Mixed form: dp3d/phi, pressure, omega integral and column sum in double; 1/p and the
  // u, v, div(v dp) of phase A in FP32 ([72][17] and [72][16] floats), so that phase C
  // neither reloads nor re-converts them and phase B sums div(v dp) from its exact FP64
  // image; T_v in double only for moist runs (dry T_v is T, read from the state).  That
  // is 48 KB instead of 73 KB: four CTAs per SM instead of three.  (The FP64 form keeps
  // its T_v array: at four CTAs per SM, with the state reread, it measured 1 % slower.)
  double *s_dp, *s_tv, *s_div, *s_p, *s_om, *s_rp, *s_tot;
  float *f_rp, *f_u, *f_w, *f_div;
  if constexpr (kF32<R>) {
    s_dp = sm;
    s_p = sm + NLEV * SROW;
    s_om = sm + 2 * NLEV * SROW;
    s_tot = sm + 3 * NLEV * SROW;
    f_rp = reinterpret_cast<float*>(s_tot + 16);
    f_u = f_rp + NLEV * SROW;
    f_w = f_u + NLEV * 16;
    f_div = f_w + NLEV * 16;
    s_tv = reinterpret_cast<double*>(f_div + NLEV * 16);  // moist only
    s_div = nullptr;
    s_rp = nullptr;
  } else {
    s_dp = sm;
    s_tv = sm + NLEV * SROW;
    s_div = sm + 2 * NLEV * SROW;
    s_p = sm + 3 * NLEV * SROW;
    s_om = sm + 4 * NLEV * SROW;
    s_rp = sm + 5 * NLEV * SROW;
    s_tot = sm + 6 * NLEV * SROW;
    f_rp = f_u = f_w = f_div = nullptr;
  }
  const bool moist = a.n0_qdp >= 0;
  const bool own_tv = !kF32<R> || moist;  // T_v kept in shared memory
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const R eta = R(a.eta_ave_w);
  const bool accum = a.eta_ave_w != 0.0;
  const size_t vN0 = ((size_t)e * NTL + a.n0) * NLEV * 32;
  const size_t sN0 = ((size_t)e * NTL + a.n0) * NLEV * 16;
  // ---- phase A: v dp, vn0, div(v dp), T_v ----
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    // hardware conversions here: after the global loads the integer-pipe form measured
    // slower (8.8 vs 8.1 ms per ne30 interval in the mixed form)
    const R u = cvt_hw<R>(a.v[vN0 + l * 32 + p]), w = cvt_hw<R>(a.v[vN0 + l * 32 + 16 + p]);
    const double td = a.T[sN0 + l * 16 + p], dd = a.dp[sN0 + l * 16 + p];
    const R d = cvt_hw<R>(dd);
    const R vd0 = u * d, vd1 = w * d;
    if (accum) {  // stages 2-4 accumulate nothing (eta_ave_w = 0)
      const size_t iv = ((size_t)e * NLEV + l) * 32 + p;
      a.vn0[iv] += dbl_hw(eta * vd0);
      a.vn0[iv + 16] += dbl_hw(eta * vd1);
    }
    const R div = divergence_sphere(t, m, vd0, vd1);
    double tv = td;
    if (a.n0_qdp >= 0) {  // moist virtual temperature, in double
      double Qt = a.qdp[((((size_t)e * QTL + a.n0_qdp) * a.qsize) * NLEV + l) * 16 + p] / dd;
      Qt *= (kRwaterVapor / kRgas - 1.0);
      Qt += 1.0;
      tv = td * Qt;
    }
    s_dp[l * SROW + p] = dd;
    if (own_tv) s_tv[l * SROW + p] = tv;
    if constexpr (kF32<R>) {
      f_u[l * 16 + p] = u;
      f_w[l * 16 + p] = w;
      f_div[l * 16 + p] = div;
    } else {
      s_div[l * SROW + p] = div;
    }
  }
  __syncthreads();
  // ---- phase B: pressure, geopotential, omega integral (double) ----
  if (tid < 128) {
    const int col = tid >> 3, seg = tid & 7, l0 = seg * 9;
    // pressure: p_k = p_{k-1} + (dp_{k-1} + dp_k)/2, p_{-1} = hyai0 ps0, dp_{-1} = 0, formed as
    // p_k = c_k + dp_k / 2 with c_k = hyai0 ps0 + sum_{j<k} dp_j
    double tot = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) tot += s_dp[(l0 + k) * SROW + col];
    double c = a.p_top + seg_excl_prefix(tot, seg);
    double r[9];
    constexpr double kHalfR = 0.5 * kRgas;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double d = s_dp[(l0 + k) * SROW + col];
      const double pr = fma(0.5, d, c);
      c += d;
      double rp;
      float rf;
      if constexpr (kF32<R>) {  // one Newton step (2^-42); the FP32 reciprocal serves phase C
        rp = rcp_newton1(pr, rf);
        f_rp[(l0 + k) * SROW + col] = rf;
      } else {  // within one ulp of 1 / p
        rp = rcp_newton(pr, rf);
        s_rp[(l0 + k) * SROW + col] = rp;
      }
      s_p[(l0 + k) * SROW + col] = pr;
      double tvk;
      if (own_tv) tvk = s_tv[(l0 + k) * SROW + col];
      else tvk = a.T[sN0 + (l0 + k) * 16 + col];
      r[k] = kHalfR * tvk * d * rp;  // R T_v dp / (2 p)
    }
    // geopotential: phi_k = phis + 2 sum_{j>k} r_j + r_k, with q = phis + 2 sum_{j>k} r_j
    // carried down the segment (the doubling is exact, on the integer pipe)
    double rt = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) rt += r[k];
    const double phis = dbl_hw(a.m.phis[(size_t)e * 16 + col]);
    double q = fma(2.0, seg_excl_suffix(rt, seg), phis);
    double* phig = a.phi + (size_t)e * NLEV * 16;
#pragma unroll
    for (int k = 8; k >= 0; --k) {
      const double ph = q + r[k];
      q += dtwice(r[k]);
      s_dp[(l0 + k) * SROW + col] = ph;  // dp no longer needed: holds phi now
      phig[(l0 + k) * 16 + col] = ph;
    }
    // omega integral: exclusive prefix of div_vdp.  The mixed form sums its FP32
    // div(v dp) in FP32 (unlike the pressure and geopotential integrals, it feeds only the
    // omega term of the FP32 tendencies) and widens the partial sums exactly on the
    // integer pipe; with rsplit = 0 the same sums give eta_dot_dpdn, whose accumulation
    // sets the tracers' source thickness, and stay in FP64.
    auto omega_fp64 = [&]() {
      double dv[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        if constexpr (kF32<R>) dv[k] = dbl(f_div[(l0 + k) * 16 + col]);
        else dv[k] = s_div[(l0 + k) * SROW + col];
      }
      double dt_ = 0.0;
#pragma unroll
      for (int k = 0; k < 9; ++k) dt_ += dv[k];
      double acc = seg_excl_prefix(dt_, seg);
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        s_om[(l0 + k) * SROW + col] = acc;
        acc = acc + dv[k];
      }
      if (seg == 7) s_tot[col] = acc;
    };
    if constexpr (kF32<R>) {
      if (a.rsplit != 0) {
        float dvf[9], tf = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          dvf[k] = f_div[(l0 + k) * 16 + col];
          tf += dvf[k];
        }
        float accf = seg_excl_prefix(tf, seg);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
          s_om[(l0 + k) * SROW + col] = dbl(accf);
          accf += dvf[k];
        }
      } else {
        omega_fp64();
      }
    } else {
      omega_fp64();
    }
  }
  __syncthreads();
  // ---- phase C: omega_p, T, v, dp3d at np1 ----
  const R dt = R(a.dt);
  const R fcor = a.m.fcor[(size_t)e * 16 + p];
  const size_t vM = ((size_t)e * NTL + a.nm1) * NLEV * 32;
  const size_t sM = ((size_t)e * NTL + a.nm1) * NLEV * 16;
  const size_t vO = ((size_t)e * NTL + a.n0orig) * NLEV * 32;
  const size_t sO = ((size_t)e * NTL + a.n0orig) * NLEV * 16;
  double* out = a.out + (size_t)e * NLEV * 64;
  const double spd = a.m.spheremp_d[(size_t)e * 16 + p];
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const double pd = s_p[l * SROW + p];
    R rp, u, w, div;
    if constexpr (kF32<R>) {
      rp = f_rp[l * SROW + p];
      u = f_u[l * 16 + p];
      w = f_w[l * 16 + p];
      div = f_div[l * 16 + p];
    } else {
      rp = s_rp[l * SROW + p];
      u = a.v[vN0 + l * 32 + p];
      w = a.v[vN0 + l * 32 + 16 + p];
      div = s_div[l * SROW + p];
    }
    // x1 and x2 derivatives of p and T; v . grad s = a0 ds/dx1 + a1 ds/dx2 with
    // (a0, a1) = (Dinv / rearth)^T v, formed once for both
    const R pr_ = rel<R>(pd);
    const R p0 = t.ddx(pr_), p1 = t.ddy(pr_);
    const double td = a.T[sN0 + l * 16 + p];
    const R tr_ = rel<R>(td);
    const R T0 = t.ddx(tr_), T1 = t.ddy(tr_);
    const R a0 = m.gr00 * u + m.gr10 * w, a1 = m.gr01 * u + m.gr11 * w;
    const R vgp = a0 * p0 + a1 * p1;
    const R omega = (vgp - (cvt<R>(s_om[l * SROW + p]) + R(0.5) * div)) * rp;
    if (accum) a.omega_p[((size_t)e * NLEV + l) * 16 + p] += dbl_hw(eta * omega);
    // time level "nm1" (RK combine of stage 5 fused here), in double
    double tm = a.T[sM + l * 16 + p], dm = a.dp[sM + l * 16 + p];
    double vm0 = a.v[vM + l * 32 + p], vm1 = a.v[vM + l * 32 + 16 + p];
    if (a.rk_combine) {
      tm = (5.0 * tm - a.T[sO + l * 16 + p]) / 4.0;
      dm = (5.0 * dm - a.dp[sO + l * 16 + p]) / 4.0;
      vm0 = (5.0 * vm0 - a.v[vO + l * 32 + p]) / 4.0;
      vm1 = (5.0 * vm1 - a.v[vO + l * 32 + 16 + p]) / 4.0;
      a.T[sM + l * 16 + p] = tm;
      a.dp[sM + l * 16 + p] = dm;
      a.v[vM + l * 32 + p] = vm0;
      a.v[vM + l * 32 + 16 + p] = vm1;
    }
    // vertically Eulerian (rsplit == 0): eta_dot_dpdn on interfaces l and l+1 from the
    // div(v dp) scan (CaarFunctorImpl.hpp:262-300), vertical advection of T and v from
    // the neighbouring levels (:496-597), accumulation (:236-248)
    R tva = R(0), vva0 = R(0), vva1 = R(0), etl = R(0), etu = R(0);
    if (a.rsplit == 0) {
      const double tot = s_tot[p];
      const double el = l == 0 ? 0.0 : c_hybi[l] * tot - s_om[l * SROW + p];
      const double eu = l + 1 == NLEV ? 0.0 : c_hybi[l + 1] * tot - s_om[(l + 1) * SROW + p];
      etl = cvt<R>(el);
      etu = cvt<R>(eu);
      const R rdp = R(0.5) * (R(1) / cvt<R>(a.dp[sN0 + l * 16 + p]));
      const R facp = rdp * etu, facm = rdp * etl;
      const double* Tc = a.T + sN0 + l * 16 + p;
      const double* vc = a.v + vN0 + l * 32 + p;
      if (l + 1 < NLEV) {
        tva += facp * (cvt<R>(Tc[16]) - cvt<R>(Tc[0]));
        vva0 += facp * (cvt<R>(vc[32]) - u);
        vva1 += facp * (cvt<R>(vc[48]) - w);
      }
      if (l > 0) {
        tva += facm * (cvt<R>(Tc[0]) - cvt<R>(Tc[-16]));
        vva0 += facm * (u - cvt<R>(vc[-32]));
        vva1 += facm * (w - cvt<R>(vc[-16]));
      }
      if (accum) a.eta_acc[((size_t)e * NLEV + l) * 16 + p] += a.eta_ave_w * el;
    }
    // temperature (compute_temperature_np1)
    R tv;
    if (own_tv) tv = cvt<R>(s_tv[l * SROW + p]);
    else tv = cvt<R>(td);
    const R vgt = a0 * T0 + a1 * T1;
    R ttens = R(kKappa) * tv * omega - vgt;
    if (a.rsplit == 0) ttens -= tva;
    // Conversions on the integer pipe here (dbl, cvt, rel): a hardware double <-> float
    // conversion takes the FP64 pipe like an FP64 add, and in phase C the integer form
    // measured faster.
    const double tnew = spd * (dbl(ttens * dt) + tm);
    // velocity (compute_velocity_np1 with compute_energy_grad): grad(KE + phi) +
    // R T_v / p grad p = (Dinv / rearth) (dE/dx + rr dp/dx) with rr = R T_v / p
    const R rr = R(kRgas) * (tv * rp);
    const R ephi = R(0.5) * (u * u + w * w) + rel<R>(s_dp[l * SROW + p]);
    const R sx = rr * p0 + t.ddx(ephi), sy = rr * p1 + t.ddy(ephi);
    R eg0 = m.gr00 * sx + m.gr01 * sy, eg1 = m.gr10 * sx + m.gr11 * sy;
    const R vort = vorticity_sphere(t, m, u, w) + fcor;
    eg0 = w * vort - eg0;
    eg1 = -(u * vort) - eg1;
    if (a.rsplit == 0) {
      eg0 -= vva0;
      eg1 -= vva1;
    }
    const double vn0_ = spd * (dbl(eg0 * dt) + vm0);
    const double vn1_ = spd * (dbl(eg1 * dt) + vm1);
    // dp3d (compute_dp3d_np1, eta_dot_dpdn = 0 for rsplit > 0)
    const double dnew = a.rsplit == 0 ? spd * (dm - dbl(((etu + div) - etl) * dt)) : spd * (dm - dbl(div * dt));
    out[l * 64 + p] = vn0_;
    out[l * 64 + 16 + p] = vn1_;
    out[l * 64 + 32 + p] = tnew;
    out[l * 64 + 48 + p] = dnew;
  }
}

// ---- DSS gathers with the contribution count as a template -------------------------
// For a thread of dss_thread_point (warps grouped by point class, so the count is
// uniform within a warp): the point's number of contributions from other elements and
// their offsets from the point's own value in a field whose elements are es doubles
// apart.
__device__ __forceinline__ int dss_offsets(const DssTable& tab, int e, int p, long long es, long long* so) {
  const int ep = e * 16 + p;
  if (!in_bounds(ep < tab.npts, tab.flag, kBoundsDssPoint)) return -1;
  int n = tab.cnt[ep];
  if (!in_bounds(n >= 0 && n <= MAXSRC, tab.flag, kBoundsDssCount)) n = 0;
#pragma unroll
  for (int k = 0; k < MAXSRC; ++k) {
    so[k] = 0;
    if (k < n) {
      int sk = tab.src[ep * MAXSRC + k];
      if (!in_bounds(sk >= 0 && sk < tab.npts, tab.flag, kBoundsDssSource)) sk = ep;
      so[k] = ((long long)(sk >> 4) - e) * es + (sk & 15) - p;
    }
  }
  return n;
}
// NF fields (16 doubles apart within a level, levels ls doubles apart) gathered on the
// nine levels lo, lo + 8, ... of point pg, in the order of dss_gather, times rs, into
// s_in[f][l][16] as R.  N is a compile-time count, so the loads of three levels are in
// flight together.
// The four fields (16 doubles apart) of one point-level gathered with a compile-time
// count of contributions, all loads in flight together, in the order of dss_gather.
template <int N>
__device__ __forceinline__ void dss_gather4_at(const double* own, const long long* so, double* g) {
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    double acc = own[f * 16];
#pragma unroll
    for (int k = 0; k < N; ++k) acc += own[so[k] + f * 16];
    g[f] = acc;
  }
}
__device__ __forceinline__ void dss_gather4(const double* own, int n, const long long* so, double* g) {
  switch (n) {
    case 0: dss_gather4_at<0>(own, so, g); break;
    case 1: dss_gather4_at<1>(own, so, g); break;
    case 2: dss_gather4_at<2>(own, so, g); break;
    case 3: dss_gather4_at<3>(own, so, g); break;
    default: g[0] = g[1] = g[2] = g[3] = 0.0; break;  // a point outside the table (index-check build)
  }
}

// DSS of the Caar output into the state of time level np1, times rspheremp
// (BoundaryExchange::exchange(rspheremp) on v, T, dp3d: CaarFunctor.cpp:114).
// Grid (E, 9), 128 threads: 8 levels per block, warps by point class.
__global__ void __launch_bounds__(128) k_dss_state(const double* __restrict__ src, double* v, double* T,
                                                   double* dp, int np1, const double* __restrict__ rsmp,
                                                   DssTable tab) {
  int lo, p;
  dss_thread_point(lo, p);
  const int e = blockIdx.x, l = blockIdx.y * 8 + lo;
  const double r = rsmp[e * 16 + p];
  long long so[MAXSRC];
  const int n = dss_offsets(tab, e, p, (long long)NLEV * 64, so);
  double g[4];
  dss_gather4(src + ((size_t)e * NLEV + l) * 64 + p, n, so, g);
  const double a0 = g[0] * r, a1 = g[1] * r, a2 = g[2] * r, a3 = g[3] * r;
  const size_t vb = (((size_t)e * NTL + np1) * NLEV + l) * 32 + p;
  const size_t sb = (((size_t)e * NTL + np1) * NLEV + l) * 16 + p;
  v[vb] = a0;
  v[vb + 16] = a1;
  T[sb] = a2;
  dp[sb] = a3;
}

template <int N, int NF, typename R>
__device__ __forceinline__ void dss_gather_levels(const double* own, const long long* so, int ls, R* s_in,
                                                  double rs, int lo, int pg) {
#pragma unroll 3
  for (int l = lo; l < NLEV; l += 8) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      double acc = own[l * ls + f * 16];
#pragma unroll
      for (int k = 0; k < N; ++k) acc += own[so[k] + l * ls + f * 16];
      s_in[(f * NLEV + l) * 16 + pg] = cvt<R>(acc * rs);
    }
  }
}
template <int NF, typename R>
__device__ __forceinline__ void dss_gather_to_smem(const double* own, int n, const long long* so, int ls, R* s_in,
                                                   double rs, int lo, int pg) {
  switch (n) {
    case 0: dss_gather_levels<0, NF>(own, so, ls, s_in, rs, lo, pg); break;
    case 1: dss_gather_levels<1, NF>(own, so, ls, s_in, rs, lo, pg); break;
    case 2: dss_gather_levels<2, NF>(own, so, ls, s_in, rs, lo, pg); break;
    case 3: dss_gather_levels<3, NF>(own, so, ls, s_in, rs, lo, pg); break;
    default:  // a point outside the table (index-check build, flagged): zeros, as dss_gather
      for (int l = lo; l < NLEV; l += 8)
        for (int f = 0; f < NF; ++f) s_in[(f * NLEV + l) * 16 + pg] = R(0);
      break;
  }
}

// ======================================================================================
// Hyperviscosity (HyperviscosityFunctorImpl): three kernels per subcycle.
// ======================================================================================
// TagFirstLaplaceHV: laplacians of the np1 state -> bufA (pre-DSS).
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_hv_lap1(HvArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const size_t vb = ((size_t)e * NTL + a.np1) * NLEV * 32;
  const size_t sb = ((size_t)e * NTL + a.np1) * NLEV * 16;
  double* out = a.bufA + (size_t)e * NLEV * 64;
  const R nr = R(a.nu_ratio1);
  LapOp<R> lap;
  lap.load(a.m, e, p);
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const R lt = lap(t, m, rel_hw<R>(a.T[sb + l * 16 + p]));
    const R ld = lap(t, m, rel_hw<R>(a.dp[sb + l * 16 + p]));
    R l0, l1;
    vlaplace_contra(t, m, nr, cvt_hw<R>(a.v[vb + l * 32 + p]), cvt_hw<R>(a.v[vb + l * 32 + 16 + p]), l0, l1);
    out[l * 64 + p] = dbl(l0);  // float -> double on the integer pipe in the mixed form
    out[l * 64 + 16 + p] = dbl(l1);
    out[l * 64 + 32 + p] = dbl(lt);
    out[l * 64 + 48 + p] = dbl(ld);
  }
}

// DSS(rspheremp) of bufA, second laplacian, TagHyperPreExchange -> bufB (pre-DSS).
// Occupancy: 6 CTAs per SM in the mixed form (80 registers), 3 in the FP64 form.
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16, kF32<R> ? 6 : 3) k_hv_lap2(HvArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  R tv[4], s2c[6];
  if (!a.consthv) {
#pragma unroll
    for (int c = 0; c < 4; ++c) tv[c] = a.m.tensorvisc[(size_t)e * 64 + c * 16 + p];
#pragma unroll
    for (int c = 0; c < 6; ++c) s2c[c] = a.m.vec_sph2cart[(size_t)e * 96 + c * 16 + p];
  }
  const size_t vb = ((size_t)e * NTL + a.np1) * NLEV * 32;
  const size_t sb = ((size_t)e * NTL + a.np1) * NLEV * 16;
  double* out = a.bufB + (size_t)e * NLEV * 64;
  const double spd = a.m.spheremp_d[(size_t)e * 16 + p];
  const double wh = a.eta_ave_w / a.hsub;  // eta_ave_w / hypervis_subcycle
  const R whr = R(wh);
  const R dt = R(a.dt);
  LapOp<R> lap;
  lap.load(a.m, e, p);
  // Mixed form: DSS(rspheremp) of the first laplacians into shared memory [4][72][16],
  // with the warps grouped by point class (dss_thread_point) so that each gather loop
  // runs one trip count per warp; every point sums in its own fixed order.  The FP64 form
  // gathers inside the level loop, where the gathers' memory latency overlaps the FP64
  // operator work of the other levels.
  extern __shared__ double hsm[];
  R* s_in = reinterpret_cast<R*>(hsm);
  const double rs = a.m.rspheremp_d[(size_t)e * 16 + p];
  if constexpr (kF32<R>) {
    static_assert(LG * 16 == 128, "dss_thread_point maps 128 threads");
    int lo, pg;
    dss_thread_point(lo, pg);
    const double rsg = a.m.rspheremp_d[(size_t)e * 16 + pg];
    long long so[MAXSRC];
    const int n = dss_offsets(a.dss, e, pg, (long long)NLEV * 64, so);
    dss_gather_to_smem<4>(a.bufA + (size_t)e * NLEV * 64 + pg, n, so, 64, s_in, rsg, lo, pg);
    __syncthreads();
  }
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    R v0, v1, t1, d1;
    if constexpr (kF32<R>) {
      v0 = s_in[(0 * NLEV + l) * 16 + p];
      v1 = s_in[(1 * NLEV + l) * 16 + p];
      t1 = s_in[(2 * NLEV + l) * 16 + p];
      d1 = s_in[(3 * NLEV + l) * 16 + p];
    } else {
      v0 = dss_gather(a.bufA, NLEV * 64, 64, e, l, p, a.dss) * rs;
      v1 = dss_gather(a.bufA + 16, NLEV * 64, 64, e, l, p, a.dss) * rs;
      t1 = dss_gather(a.bufA + 32, NLEV * 64, 64, e, l, p, a.dss) * rs;
      d1 = dss_gather(a.bufA + 48, NLEV * 64, 64, e, l, p, a.dss) * rs;
    }
    R lt, ld, l0, l1;
    if (a.consthv) {
      lt = lap(t, m, t1);
      ld = lap(t, m, d1);
      vlaplace_contra(t, m, R(a.nu_ratio2), v0, v1, l0, l1);
    } else {
      lt = laplace_tensor(t, m, tv, t1);
      ld = laplace_tensor(t, m, tv, d1);
      vlaplace_cartesian(t, m, tv, s2c, v0, v1, l0, l1);
    }
    const size_t i3 = ((size_t)e * NLEV + l) * 16 + p;
    const double dpn = a.dp[sb + l * 16 + p];
    a.dpdiss_ave[i3] += wh * dpn;
    a.dpdiss_bih[i3] += dbl(whr * ld);
    R vt0 = l0 * R(-a.nu), vt1 = l1 * R(-a.nu);
    R ttn = lt * R(-a.nu_s), dpt = ld * R(-a.nu_p);
    if (a.nu_top > 0 && __any_sync(FULL, l < 3)) {
      // nu_top sponge on the top three levels, applied to the np1 state
      const R un = cvt<R>(a.v[vb + l * 32 + p]), wn = cvt<R>(a.v[vb + l * 32 + 16 + p]);
      R lv0, lv1;
      vlaplace_contra(t, m, R(1), un, wn, lv0, lv1);
      const R ltt = lap(t, m, rel<R>(a.T[sb + l * 16 + p]));
      const R ldd = lap(t, m, rel<R>(dpn));
      if (l < 3) {
        const R sc = R((l == 0 ? 4.0 : l == 1 ? 2.0 : 1.0) * a.nu_top);
        vt0 += sc * lv0;
        vt1 += sc * lv1;
        ttn += sc * ltt;
        dpt += sc * ldd;
      }
    }
    out[l * 64 + p] = dbl(vt0);
    out[l * 64 + 16 + p] = dbl(vt1);
    out[l * 64 + 32 + p] = dbl(ttn);
    out[l * 64 + 48 + p] = dbl(dpt * dt) + dpn * spd;
  }
}

// DSS of bufB and TagUpdateStates.
// Grid (E, 9), 128 threads: 8 levels per block, warps by point class.
template <typename R>
__global__ void __launch_bounds__(128) k_hv_update(HvArgs<R> a) {
  int lo, p;
  dss_thread_point(lo, p);
  const int e = blockIdx.x, l = blockIdx.y * 8 + lo;
  const double rsd = a.m.rspheremp_d[e * 16 + p];
  const R rs = cvt<R>(rsd);
  const R dt = R(a.dt);
  long long so[MAXSRC];
  const int n = dss_offsets(a.dss, e, p, (long long)NLEV * 64, so);
  double g[4];
  dss_gather4(a.bufB + ((size_t)e * NLEV + l) * 64 + p, n, so, g);
  R vt0 = cvt<R>(g[0]);
  R vt1 = cvt<R>(g[1]);
  R tt = cvt<R>(g[2]);
  const double dpt = g[3];
  const size_t vb = (((size_t)e * NTL + a.np1) * NLEV + l) * 32 + p;
  const size_t sb = (((size_t)e * NTL + a.np1) * NLEV + l) * 16 + p;
  vt0 = dt * vt0 * rs;
  vt1 = dt * vt1 * rs;
  const double v0 = a.v[vb] + dbl(vt0), v1 = a.v[vb + 16] + dbl(vt1);
  a.v[vb] = v0;
  a.v[vb + 16] = v1;
  tt = dt * tt * rs;
  const R heating = vt0 * cvt<R>(v0) + vt1 * cvt<R>(v1);
  constexpr R rcp = R(1.0 / kCp);
  if constexpr (kF32<R>) a.T[sb] = a.T[sb] + dbl(tt - heating * rcp);
  else a.T[sb] = a.T[sb] + tt - heating * rcp;
  a.dp[sb] = dpt * rsd;
}

// ======================================================================================
// Small element-wise kernels
// ======================================================================================
__global__ void k_prim_step_init(int E, double* eta, double* vn0, double* omega_p, double* dpa,
                                 double* dpb, double* derived_dp, const double* dp, int n0,
                                 int zero_diss) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), r = idx % (NLEV * 16), l = r / 16, p = r & 15;
  eta[idx] = 0;
  omega_p[idx] = 0;
  vn0[((size_t)e * NLEV + l) * 32 + p] = 0;
  vn0[((size_t)e * NLEV + l) * 32 + 16 + p] = 0;
  if (zero_diss) {
    dpa[idx] = 0;
    dpb[idx] = 0;
  }
  derived_dp[idx] = dp[((size_t)e * NTL + n0) * NLEV * 16 + r];
}

__global__ void k_dp_from_ps(int E, double* dp, const double* ps_v, int n0, double ps0) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), r = idx % (NLEV * 16), l = r / 16, p = r & 15;
  dp[((size_t)e * NTL + n0) * NLEV * 16 + r] =
      c_ai_delta[l] * ps0 + c_bi_delta[l] * ps_v[((size_t)e * NTL + n0) * 16 + p];
}

// Grid of the per-(element, tracer) pointwise kernels: blockIdx.x = e*nq + q, blockIdx.y
// = a group of EQ_LEVELS levels, threadIdx.x = level-in-group * 16 + point.  Only
// 32-bit divisions by the tracer count (64-bit division by a runtime value is a long
// emulated sequence).
constexpr int EQ_LEVELS = 8;
constexpr int EQ_THREADS = EQ_LEVELS * 16;
__device__ __forceinline__ void eq_index(int nq, int& e, int& q, int& l, int& p) {
  const int eq = blockIdx.x;
  e = eq / nq;
  q = eq - e * nq;
  l = blockIdx.y * EQ_LEVELS + (threadIdx.x >> 4);
  p = threadIdx.x & 15;
}
// The same grid for the DSS kernels, with the warps grouped by point class.
__device__ __forceinline__ void eq_index_dss(int nq, int& e, int& q, int& l, int& p) {
  static_assert(EQ_LEVELS == 8 && EQ_THREADS == 128, "dss_thread_point covers 8 levels x 16 points");
  const int eq = blockIdx.x;
  e = eq / nq;
  q = eq - e * nq;
  int lo;
  dss_thread_point(lo, p);
  l = blockIdx.y * EQ_LEVELS + lo;
}

// update_q (prim_driver.cpp:171-206): Q = Qdp / dp, dp = dA ps0 + dB ps_v.  Grid (E, 9),
// 128 threads: one thread per (element, level, point) forms 1/dp once and divides every
// tracer by it with one corrected multiplication (div_newton, within one ulp of the IEEE
// quotient); a thickness outside (1e-30, 1e30) takes the IEEE division.
__global__ void __launch_bounds__(128) k_update_q(int Q, const double* __restrict__ qdp, double* __restrict__ Qc,
                                                  const double* __restrict__ ps_v, int np1, int np1_qdp,
                                                  double ps0) {
  const int e = blockIdx.x, l = blockIdx.y * 8 + (threadIdx.x >> 4), p = threadIdx.x & 15;
  const double dp = c_ai_delta[l] * ps0 + c_bi_delta[l] * ps_v[((size_t)e * NTL + np1) * 16 + p];
  const double* src = qdp + ((((size_t)e * QTL + np1_qdp) * Q) * NLEV + l) * 16 + p;
  double* dst = Qc + (((size_t)e * Q) * NLEV + l) * 16 + p;
  if (dp > 1e-30 && dp < 1e30) {
    float rf;
    const double r = rcp_newton(dp, rf);
    for (int q = 0; q < Q; ++q) dst[(size_t)q * NLEV * 16] = div_newton(src[(size_t)q * NLEV * 16], dp, r);
  } else {
    for (int q = 0; q < Q; ++q) dst[(size_t)q * NLEV * 16] = src[(size_t)q * NLEV * 16] / dp;
  }
}

// Tracer mass diagnostics (Diagnostics.cpp:37-84): one thread per (element, tracer, GLL
// point) sums its column of Qdp*Q and of Qdp at tracer level tq, level by level and
// without fused multiply-adds, as the reference's host loop does.  Outputs [E][Q][16].
__global__ void k_diag_scalars(int EQ, int Q, const double* __restrict__ qdp, const double* __restrict__ Qc,
                               int tq, double* __restrict__ qvar, double* __restrict__ qmass) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= EQ * 16) return;
  const int eq = i >> 4, p = i & 15, e = eq / Q, q = eq - e * Q;
  const double* a = qdp + (((size_t)e * QTL + tq) * Q + q) * NLEV * 16 + p;
  const double* b = Qc + (size_t)eq * NLEV * 16 + p;
  double sqq = 0.0, sq = 0.0;
#pragma unroll 8
  for (int l = 0; l < NLEV; ++l) {
    const double x = a[l * 16];
    sqq = __dadd_rn(sqq, __dmul_rn(x, b[l * 16]));
    sq = __dadd_rn(sq, x);
  }
  qvar[i] = sqq;
  qmass[i] = sq;
}

// Column energies (Diagnostics.cpp:86-185): one thread per (element, GLL point) at
// dynamics level t1, with dp = dA ps0 + dB ps_v and cp* = cp (1 + kq Qdp(tracer 1)/dp)
// when cpstar, else cp.  Sums in level order without fused multiply-adds.
// out: IEner, IEner_wet, KEner, PEner, each [E][16].
__global__ void k_diag_energy(int E, int Q, const double* __restrict__ T, const double* __restrict__ v,
                              const double* __restrict__ ps_v, const double* __restrict__ phis,
                              const double* __restrict__ qdp, int t1, int t1q, int cpstar, double ps0,
                              double cp, double kq, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E * 16) return;
  const int e = i >> 4, p = i & 15;
  const double ps = ps_v[((size_t)e * NTL + t1) * 16 + p], ph = phis[i];
  const double* tc = T + ((size_t)e * NTL + t1) * NLEV * 16 + p;
  const double* vc = v + ((size_t)e * NTL + t1) * NLEV * 32 + p;
  const double* qc = qdp + ((size_t)e * QTL + t1q) * Q * NLEV * 16 + p;  // tracer 1
  double ie = 0.0, iew = 0.0, ke = 0.0, pe = 0.0;
#pragma unroll 4
  for (int l = 0; l < NLEV; ++l) {
    const double dp = __dadd_rn(__dmul_rn(c_ai_delta[l], ps0), __dmul_rn(c_bi_delta[l], ps));
    double cps = cp;
    if (cpstar) cps = __dmul_rn(cp, __dadd_rn(1.0, __dmul_rn(kq, __ddiv_rn(qc[l * 16], dp))));
    const double t = tc[l * 16], u = vc[l * 32], w = vc[l * 32 + 16];
    ie = __dadd_rn(ie, __dmul_rn(__dmul_rn(cps, t), dp));
    iew = __dadd_rn(iew, __dmul_rn(__dmul_rn(__dsub_rn(cps, cp), t), dp));
    ke = __dadd_rn(ke, __dmul_rn(__dmul_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(w, w)), 0.5), dp));
    pe = __dadd_rn(pe, __dmul_rn(ph, dp));
  }
  const size_t n = (size_t)E * 16;
  out[i] = ie;
  out[n + i] = iew;
  out[2 * n + i] = ke;
  out[3 * n + i] = pe;
}

// Restart-file checksum: the sum modulo 2^64 of splitmix64(w_k + (k + 1) * golden) over
// the file's record words w_k.  Element e's segment of `words` words sits at src + e*words
// and its word j at record index k = e*rec_words + off + j.  One block per element.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) k_restart_checksum(const unsigned long long* __restrict__ src, int words,
                                                          long long rec_words, long long off,
                                                          unsigned long long* out) {
  __shared__ unsigned long long part[8];
  const int e = blockIdx.x;
  const unsigned long long* p = src + (size_t)e * words;
  const unsigned long long k0 = (unsigned long long)e * rec_words + off + 1;
  unsigned long long acc = 0;
  for (int j = threadIdx.x; j < words; j += blockDim.x) acc += splitmix64(p[j] + (k0 + j) * 0x9E3779B97F4A7C15ull);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    atomicAdd(out, t);
  }
}

// CAM forcing (CamForcing.cpp:20-170).  Layouts: ft [E][72][16], fm [E][72][2][16],
// fq [E][Q][72][16] (the Fortran layouts of the forcing arrays).
__global__ void k_state_forcing(int E, double* T, double* v, const double* ft, const double* fm, int n0,
                                double dt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), r = idx % (NLEV * 16), l = r / 16, p = r & 15;
  T[((size_t)e * NTL + n0) * NLEV * 16 + r] += dt * ft[idx];
  const size_t vb = (((size_t)e * NTL + n0) * NLEV + l) * 32 + p;
  const size_t fb = ((size_t)e * NLEV + l) * 32 + p;
  v[vb] += dt * fm[fb];
  v[vb + 16] += dt * fm[fb + 16];
}

__device__ __forceinline__ double clip_forcing(double qdp_s, double v1) {
  if (qdp_s + v1 < 0.0 && v1 < 0.0) v1 = qdp_s < 0.0 ? 0.0 : -qdp_s;
  return v1;
}

// ps_v(n0) += sum over levels of tracer 0's clipped increments (moist), one thread per
// column, levels in order; runs before the tracer forcing changes Qdp.
__global__ void k_ps_forcing(int E, int Q, const double* fq, const double* qdp, double* ps_v, int n0,
                             int n0_qdp, double dt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * 16) return;
  const int e = idx / 16, p = idx & 15;
  const double* q0 = qdp + (((size_t)e * QTL + n0_qdp) * Q) * NLEV * 16 + p;
  const double* f0 = fq + ((size_t)e * Q) * NLEV * 16 + p;
  double acc = 0.0;
  for (int l = 0; l < NLEV; ++l) acc += clip_forcing(q0[l * 16], dt * f0[l * 16]);
  ps_v[((size_t)e * NTL + n0) * 16 + p] += acc;
}

__global__ void __launch_bounds__(EQ_THREADS) k_tracer_forcing(int Q, const double* fq, double* qdp,
                                                               int n0_qdp, double dt) {
  int e, q, l, p;
  eq_index(Q, e, q, l, p);
  double& qd = qdp[((((size_t)e * QTL + n0_qdp) * Q + q) * NLEV + l) * 16 + p];
  qd += clip_forcing(qd, dt * fq[(((size_t)e * Q + q) * NLEV + l) * 16 + p]);
}

// ======================================================================================
// Tracers (EulerStepFunctorImpl)
// ======================================================================================
// PrecomputeDivDp: divdp = div(vn0), divdp_proj = divdp.
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_precompute_divdp(EulerArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const size_t iv = ((size_t)e * NLEV + l) * 32 + p;
    const R d = divergence_sphere(t, m, cvt<R>(a.vn0[iv]), cvt<R>(a.vn0[iv + 16]));
    const size_t i3 = ((size_t)e * NLEV + l) * 16 + p;
    a.divdp[i3] = dbl(d);
    a.divdp_proj[i3] = dbl(d);
  }
}

// compute_dp + compute_qmin_qmax for one element and all its tracers: the layer
// thickness dp = derived_dp - rhs_multiplier dt divdp_proj and its reciprocal are formed
// once per point and level and reused for every tracer; Q = Qdp / dp goes to qtens when
// the biharmonic needs it; per-level min/max over the 16 points (in R, exact) to
// qlim_out, combined with the previous qlim when rhs_multiplier == 1.
// Grid E, 96 threads: thread (lv = tid / 4, c = tid % 4) owns points 4c .. 4c+3 of
// levels lv, lv + 24 and lv + 48, so the min/max over a level's 16 points is three local
// steps and two shuffles among four lanes (min and max are exact: any order gives the
// same bounds).
template <typename R>
__global__ void __launch_bounds__(96) k_qminmax(EulerArgs<R> a, double* qlim_out, int store_q) {
  const int e = blockIdx.x, tid = threadIdx.x, c = tid & 3, lv = tid >> 2;
  const R rhsdt = R(a.rhs_multiplier * a.dt);
  R rdp[3][4];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const size_t i3 = ((size_t)e * NLEV + lv + 24 * r) * 16 + 4 * c;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      rdp[r][j] = recip(cvt<R>(a.derived_dp[i3 + j]) - rhsdt * cvt<R>(a.divdp_proj[i3 + j]));
  }
#pragma unroll 1
  for (int q = 0; q < a.Q; ++q) {
    const double* qsrc = a.qdp + (((size_t)e * QTL + a.n0_qdp) * a.Q + q) * NLEV * 16;
    double* qt = a.qtens + ((size_t)e * a.Q + q) * NLEV * 16;
    double* ql = qlim_out + ((size_t)e * a.Q + q) * 2 * NLEV;
    const double* qo = a.qlim + ((size_t)e * a.Q + q) * 2 * NLEV;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int l = lv + 24 * r;
      const double2* src = reinterpret_cast<const double2*>(qsrc + l * 16 + 4 * c);
      const double2 s01 = src[0], s23 = src[1];
      R v[4] = {cvt<R>(s01.x) * rdp[r][0], cvt<R>(s01.y) * rdp[r][1], cvt<R>(s23.x) * rdp[r][2],
                cvt<R>(s23.y) * rdp[r][3]};
      if (store_q) {
        double2* dst = reinterpret_cast<double2*>(qt + l * 16 + 4 * c);
        dst[0] = make_double2(dbl(v[0]), dbl(v[1]));
        dst[1] = make_double2(dbl(v[2]), dbl(v[3]));
      }
      double dmn, dmx;
      if constexpr (kF32<R>) {
        R mn = fminf(fminf(v[0], v[1]), fminf(v[2], v[3]));
        R mx = fmaxf(fmaxf(v[0], v[1]), fmaxf(v[2], v[3]));
#pragma unroll
        for (int off = 1; off <= 2; off <<= 1) {
          mn = fminf(mn, __shfl_xor_sync(FULL, mn, off, 4));
          mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, off, 4));
        }
        dmn = dbl(mn);
        dmx = dbl(mx);
      } else {  // exact min/max on the integer pipe
        const long long k0 = dkey(v[0]), k1 = dkey(v[1]), k2 = dkey(v[2]), k3 = dkey(v[3]);
        long long mn = kmin(kmin(k0, k1), kmin(k2, k3)), mx = kmax(kmax(k0, k1), kmax(k2, k3));
#pragma unroll
        for (int off = 1; off <= 2; off <<= 1) {
          mn = kmin(mn, __shfl_xor_sync(FULL, mn, off, 4));
          mx = kmax(mx, __shfl_xor_sync(FULL, mx, off, 4));
        }
        dmn = dkey_value(mn);
        dmx = dkey_value(mx);
      }
      if (c == 0) {
        if (a.rhs_multiplier == 1.0) {
          if constexpr (kF32<R>) {
            dmn = fmin(qo[l], dmn);
            dmx = fmax(qo[NLEV + l], dmx);
          } else {  // exact, on the integer pipe (one lane of four: an FP64-pipe fmin here
                    // costs a full warp instruction; 2.21 -> 2.09 ms per interval)
            dmn = dkey_value(kmin(dkey(qo[l]), dkey(dmn)));
            dmx = dkey_value(kmax(dkey(qo[NLEV + l]), dkey(dmx)));
          }
        }
        ql[l] = dmn;
        ql[NLEV + l] = dmx;
      }
    }
  }
}

// Neighbour min/max (exchange_min_max): qlim = minmax(own, all connected neighbours).
__global__ void k_minmax_nbr(int E, int Q, const double* __restrict__ pre, double* qlim,
                             const int* __restrict__ conn) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * Q * NLEV) return;
  const int l = idx % NLEV, q = (idx / NLEV) % Q, e = idx / (NLEV * Q);
  long long mn = dkey(pre[((size_t)e * Q + q) * 2 * NLEV + l]);
  long long mx = dkey(pre[((size_t)e * Q + q) * 2 * NLEV + NLEV + l]);
  for (int s = 0; s < 8; ++s) {
    const int r = conn[e * 8 + s];
    if (r < 0) continue;
    mn = kmin(mn, dkey(pre[((size_t)r * Q + q) * 2 * NLEV + l]));
    mx = kmax(mx, dkey(pre[((size_t)r * Q + q) * 2 * NLEV + NLEV + l]));
  }
  qlim[((size_t)e * Q + q) * 2 * NLEV + l] = dkey_value(mn);
  qlim[((size_t)e * Q + q) * 2 * NLEV + NLEV + l] = dkey_value(mx);
}

// BIHPre: qtens (Q) [* dpdiss_ave / dp0] -> laplace -> qscr (pre-DSS).
// The tracer-independent weight of the biharmonic's first Laplacian, dpdiss_ave / dp0,
// once per point and level (into the dpdissk scratch, which aal_setup writes later).
__global__ void k_bih_weight(int E, const double* __restrict__ dpa, double* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= E * NLEV * 16) return;
  w[i] = dpa[i] * c_rdp0[(i >> 4) % NLEV];
}

// (The mixed form converts its two inputs per point on the hardware path: this kernel's
// FP64 pipe has room, its instruction issue less.)
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_bih_pre(EulerArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int eq = blockIdx.x, e = eq / a.Q, q = eq % a.Q;
  const int tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const size_t qb = ((size_t)e * a.Q + q) * NLEV * 16;
  LapOp<R> lap;
  lap.load(a.m, e, p);
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    R s = cvt_hw<R>(a.qtens[qb + l * 16 + p]);
    if (a.nu_p > 0) s = s * cvt_hw<R>(a.dpdissk[((size_t)e * NLEV + l) * 16 + p]);  // dpdiss_ave / dp0
    a.qscr[qb + l * 16 + p] = dbl(lap(t, m, s));
  }
}

// DSS(rspheremp) of qscr, BIHPostConstHV/TensorHV laplace, rhsviss_adjustment -> qtens.
// Occupancy: 9 CTAs per SM in the mixed form, 6 in the FP64 form (at most 85 registers).
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16, kF32<R> ? 9 : 6) k_bih_post(EulerArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int eq = blockIdx.x, e = eq / a.Q, q = eq % a.Q;
  const int tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  R tv[4];
  if (!a.consthv) {
#pragma unroll
    for (int c = 0; c < 4; ++c) tv[c] = a.m.tensorvisc[(size_t)e * 64 + c * 16 + p];
  }
  const size_t qb = ((size_t)e * a.Q + q) * NLEV * 16;
  const double* fbase = a.qscr + (size_t)q * NLEV * 16;
  const R fac = R(-a.rhs_viss * a.dt * a.nu_q);
  const R cf = fac * (R(1) / m.sp);  // the factor and 1/spheremp of this point
  LapOp<R> lapo;
  if (a.consthv) lapo.load(a.m, e, p);
  // DSS(rspheremp) into shared memory [72][16] with warps grouped by point class
  __shared__ R s_in[NLEV * 16];
  {
    static_assert(LG * 16 == 128, "dss_thread_point maps 128 threads");
    int lo, pg;
    dss_thread_point(lo, pg);
    const double rsg = a.m.rspheremp_d[(size_t)e * 16 + pg];
    const long long es = (long long)a.Q * NLEV * 16;
    if constexpr (kF32<R>) {  // three levels' loads in flight (0.10 ms less per interval)
      long long so[MAXSRC];
      const int n = dss_offsets(a.dss, e, pg, es, so);
      dss_gather_to_smem<1>(fbase + (size_t)e * es + pg, n, so, 16, s_in, rsg, lo, pg);
    } else {  // one level at a time: the unrolled form spills at the FP64 form's 80 registers
#pragma unroll 1
      for (int l = lo; l < NLEV; l += 8) s_in[l * 16 + pg] = dss_gather(fbase, es, 16, e, l, pg, a.dss) * rsg;
    }
  }
  __syncthreads();
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const R s = s_in[l * 16 + p];
    const R lap = a.consthv ? lapo(t, m, s) : laplace_tensor(t, m, tv, s);
    a.qtens[qb + l * 16 + p] = dbl(cf * cvt<R>(a.dp0[l]) * lap);
  }
}

// AALSetupPhase (compute_2d_advection_step): vstar, dpdissk, f_dss * spheremp -> fscr.
template <typename R>
__global__ void k_aal_setup(EulerArgs<R> a, int E) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), l = (idx / 16) % NLEV, p = idx & 15;
  const R rhsdt = R(a.rhs_multiplier * a.dt);
  const R dpt = cvt<R>(a.derived_dp[idx]) - rhsdt * cvt<R>(a.divdp_proj[idx]);
  const size_t iv = ((size_t)e * NLEV + l) * 32 + p;
  const R rdpt = R(1) / dpt;
  a.vstar[iv] = dbl(cvt<R>(a.vn0[iv]) * rdpt);
  a.vstar[iv + 16] = dbl(cvt<R>(a.vn0[iv + 16]) * rdpt);
  R dk = dpt - R(a.dt) * cvt<R>(a.divdp[idx]);
  if (a.nu_p > 0 && a.rhs_viss != 0.0)
    dk += R(-a.rhs_viss * a.dt * a.nu_q) * cvt<R>(a.dpdiss_bih[idx]) / a.m.spheremp[e * 16 + p];
  a.dpdissk[idx] = dbl(dk);
  a.fscr[idx] = a.f_dss[idx] * a.m.spheremp_d[e * 16 + p];
}

// Is any point outside [minp, maxp]?  In FP64 on the integer pipe (exact).
template <typename R>
__device__ __forceinline__ bool any_outside(const R* x, R minp, R maxp) {
  bool out = false;
  if constexpr (kF32<R>) {
#pragma unroll
    for (int k = 0; k < 16; ++k) out |= (x[k] > maxp) | (x[k] < minp);
  } else {
    const long long kmn = dkey(minp), kmx = dkey(maxp);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const long long kx = dkey(x[k]);
      out |= (kx > kmx) | (kx < kmn);
    }
  }
  return out;
}

// The quasi-monotone limiters of with_limiter_shell (EulerStepFunctorImpl.hpp:693-884)
// on one level of 16 points, one thread, sums in point order; s1 = sum of c.  Returns
// false when the level needs no limiting (x unchanged); the bounds are relaxed to the
// level mean first, as in the reference.
template <typename R>
__device__ bool limiter_level(int option, R* x, const R* c, R s1, double& minp_io, double& maxp_io) {
  R s0 = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) s0 += x[k] * c[k];
  // The tests here and below are exact comparisons (pos, lt: on the integer pipe in FP64,
  // where a comparison on the FP64 pipe would cost a warp instruction like a multiply-add).
  if (!pos(s1)) return false;
  R minp = cvt<R>(minp_io), maxp = cvt<R>(maxp_io);
  if (lt(minp, R(0))) { minp = R(0); minp_io = 0.0; }
  if (lt(s0, minp * s1)) { minp = s0 / s1; minp_io = dbl(minp); }
  if (lt(maxp * s1, s0)) { maxp = s0 / s1; maxp_io = dbl(maxp); }
  if (!any_outside(x, minp, maxp)) return false;  // no clipping: addmass = 0
  const R mass = s0;
  if (option == 8) {
    const R tol = R(5e-14);
    for (int iter = 0; iter < 15; ++iter) {
      R addmass = 0;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const bool hi = lt(maxp, x[k]), lo = !hi && lt(x[k], minp);
        if (hi || lo) {
          const R b = hi ? maxp : minp;
          addmass += (x[k] - b) * c[k];
          x[k] = b;
        }
      }
      if (!lt(tol * fabs(mass), fabs(addmass))) break;  // |addmass| <= tol |mass|
      R wsum = 0;
      if (pos(addmass)) {
#pragma unroll
        for (int k = 0; k < 16; ++k) if (lt(x[k], maxp)) wsum += c[k];
        if (is_zero(wsum)) break;
        const R adw = addmass / wsum;
#pragma unroll
        for (int k = 0; k < 16; ++k) if (lt(x[k], maxp)) x[k] += adw;
      } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) if (lt(minp, x[k])) wsum += c[k];
        if (is_zero(wsum)) break;
        const R adw = addmass / wsum;
#pragma unroll
        for (int k = 0; k < 16; ++k) if (lt(minp, x[k])) x[k] += adw;
      }
    }
  } else {
    R addmass = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const bool hi = lt(maxp, x[k]), lo = !hi && lt(x[k], minp);
      if (hi || lo) {
        const R b = hi ? maxp : minp;
        addmass += (x[k] - b) * c[k];
        x[k] = b;
      }
    }
    if (is_zero(addmass)) return true;
    R fac = 0;
    if (pos(addmass)) {
#pragma unroll
      for (int k = 0; k < 16; ++k) fac += c[k] * (maxp - x[k]);
      if (pos(fac)) {
        fac = addmass / fac;
#pragma unroll
        for (int k = 0; k < 16; ++k) x[k] += fac * (maxp - x[k]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) fac += c[k] * (x[k] - minp);
      if (pos(fac)) {
        fac = addmass / fac;
#pragma unroll
        for (int k = 0; k < 16; ++k) x[k] += fac * (x[k] - minp);
      }
    }
  }
  return true;
}

// AALTracerPhase: qtens = Qdp - dt div(vstar Qdp) [+ qtens_biharmonic], limiter,
// spheremp -> qscr (pre-DSS).  One CTA per element loops over the tracers: vstar, the
// limiter weights c = spheremp dpdissk, 1/dpdissk and sum(c) are formed once per element
// and reused by every tracer.  The Qdp slab of the next tracer (72 x 16 contiguous
// doubles) streams into shared memory by a bulk asynchronous copy while the current
// one is limited and stored, so the tracer loop does not wait on global loads.
// Occupancy: 6 CTAs per SM in the mixed form (at most 80 registers; the kernel waits on
// memory and shared-memory latency more than it issues, so occupancy pays for a small
// spill; five CTAs with no spill measured 10 % slower), 3 in the FP64 form (168
// registers).
template <typename R> constexpr size_t aal_buf_offset() {  // bytes, 16-byte aligned
  return (NLEV * SROW * sizeof(double) + (3 * NLEV * SROW + NLEV) * sizeof(R) + 15) / 16 * 16;
}
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16, kF32<R> ? 6 : 3) k_aal_tracer(EulerArgs<R> a) {
  constexpr int NL = NLEV / LG;
  constexpr unsigned kSlab = NLEV * 16 * sizeof(double);
  constexpr unsigned kLim = 2 * NLEV * sizeof(double);
  extern __shared__ __align__(16) double tsm[];
  double* s_q = tsm;                                            // [72][17] double
  R* s_dm = reinterpret_cast<R*>(tsm + NLEV * SROW);            // dpdissk
  R* s_rdm = s_dm + NLEV * SROW;                                // 1 / dpdissk
  R* s_c = s_rdm + NLEV * SROW;                                 // spheremp * dpdissk
  R* s_c1 = s_c + NLEV * SROW;                                  // sum of c per level [72]
  double* q_buf = reinterpret_cast<double*>(reinterpret_cast<char*>(tsm) + aal_buf_offset<R>());  // [72][16]
  double* q_lim = q_buf + NLEV * 16;  // [2][2][72]: the tracer's qlim (min, max), by tracer parity
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(q_lim + 4 * NLEV);
  const int e = blockIdx.x;
  const int tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  const double* slab0 = a.qdp + ((size_t)e * QTL + a.n0_qdp) * a.Q * NLEV * 16;
  // every slab this CTA copies lies in Qdp: tracer level 0 or 1, element inside the grid
  const bool slabs_ok = in_bounds(a.n0_qdp >= 0 && a.n0_qdp < QTL && e < (int)gridDim.x, a.err + 1,
                                  kBoundsTracerSlab);
  const double* lim0 = a.qlim + (size_t)e * a.Q * 2 * NLEV;
  if (tid == 0) {
    mbar_init(bar, 1);
    if (a.Q > 0 && slabs_ok) bulk_load2(q_buf, slab0, kSlab, q_lim, lim0, kLim, bar);
  }
  if (!slabs_ok) return;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const double spd = a.m.spheremp_d[(size_t)e * 16 + p];
  // AALSetupPhase (compute_2d_advection_step), per element here: the layer thickness
  // dp = derived_dp - rhs_multiplier dt divdp_proj, vstar = vn0 / dp, the limiter's
  // thickness dpdissk = dp - dt divdp (+ the biharmonic dp term), and f_dss spheremp for
  // the DSS of f_dss; then the tracer-independent part of div(vstar Qdp), the
  // contravariant flux per unit Qdp, (Dinv-contraction of vstar) * metdet
  const R rhsdt = R(a.rhs_multiplier * a.dt);
  const bool hvdk = a.nu_p > 0 && a.rhs_viss != 0.0;
  const R hvf = R(-a.rhs_viss * a.dt * a.nu_q) * recip(m.sp);  // over this element's spheremp
  R w0[NL], w1[NL];
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const size_t i3 = ((size_t)e * NLEV + l) * 16 + p;
    const size_t iv = ((size_t)e * NLEV + l) * 32 + p;
    const R dpt = cvt<R>(a.derived_dp[i3]) - rhsdt * cvt<R>(a.divdp_proj[i3]);
    const R rdpt = recip(dpt);
    const R vs0 = cvt<R>(a.vn0[iv]) * rdpt, vs1 = cvt<R>(a.vn0[iv + 16]) * rdpt;
    R dm = dpt - R(a.dt) * cvt<R>(a.divdp[i3]);
    if (hvdk) dm += hvf * cvt<R>(a.dpdiss_bih[i3]);
    a.fscr[i3] = a.f_dss[i3] * spd;
    w0[k] = m.dm00 * vs0 + m.dm10 * vs1;  // metdet folded into Dinv
    w1[k] = m.dm01 * vs0 + m.dm11 * vs1;
    s_dm[l * SROW + p] = dm;
    s_rdm[l * SROW + p] = recip(dm);
    s_c[l * SROW + p] = m.sp * dm;
  }
  // -dt times divergence_sphere's scale, folded into the derivative weights: the
  // advection below forms Qdp + q0 - dt div(vstar Qdp) as one multiply-add chain
  t.scale(R(-a.dt) * m.fdiv);
  __syncthreads();
  for (int l = tid; l < NLEV; l += blockDim.x) {
    R s1 = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) s1 += s_c[l * SROW + k];
    s_c1[l] = s1;
  }
  const bool add_hv = a.rhs_viss != 0.0;
  unsigned parity = 0;
#pragma unroll 1
  for (int q = 0; q < a.Q; ++q) {
    const size_t qb = ((size_t)e * a.Q + q) * NLEV * 16;
    // tracer q's slab: a bounded wait, then a block-wide vote, so that a copy that never
    // completes ends the kernel with an error flag instead of a hang
    const bool ok = __syncthreads_and(mbar_wait(bar, parity, 1 << 20));
    parity ^= 1u;
    if (!ok) {
      if (tid == 0) {
        atomicExch(a.err, 1);
        mbar_wait(bar, parity ^ 1u, 1 << 20);  // once more for the copy still in flight
      }
      return;
    }
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int l = lg + LG * k;
      const double qdd = q_buf[l * 16 + p];
      const R qd = cvt<R>(qdd);
      const double q0 = add_hv ? a.qtens[qb + l * 16 + p] : 0.0;
      if constexpr (kF32<R>) {
        s_q[l * SROW + p] = qdd + dbl(t.dxy(w0[k] * qd, w1[k] * qd)) + q0;  // -dt div(vstar Qdp)
      } else {
        const double acc = add_hv ? qdd + q0 : qdd;
        s_q[l * SROW + p] = t.dxy_acc(w0[k] * qd, w1[k] * qd, acc);
      }
    }
    __syncthreads();
    if (tid == 0 && q + 1 < a.Q) {  // the buffer is free: fetch the next tracer's slab and bounds
      fence_proxy_async_smem();
      bulk_load2(q_buf, slab0 + (size_t)(q + 1) * NLEV * 16, kSlab, q_lim + ((q + 1) & 1) * 2 * NLEV,
                 lim0 + (size_t)(q + 1) * 2 * NLEV, kLim, bar);
    }
    for (int l = tid; l < NLEV; l += blockDim.x) {
      if (s_c1[l] > R(0)) {
        R x[16], c[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          c[k] = s_c[l * SROW + k];
          x[k] = cvt<R>(s_q[l * SROW + k]) * s_rdm[l * SROW + k];
        }
        double* ql = a.qlim + ((size_t)e * a.Q + q) * 2 * NLEV;
        const double* qls = q_lim + (q & 1) * 2 * NLEV;  // the same bounds, prefetched
        double mn = qls[l], mx = qls[NLEV + l];
        const bool lim = limiter_level<R>(a.limiter_option, x, c, s_c1[l], mn, mx);
        ql[l] = mn;
        ql[NLEV + l] = mx;
        if (lim) {
#pragma unroll
          for (int k = 0; k < 16; ++k) s_q[l * SROW + k] = dbl(x[k] * s_dm[l * SROW + k]);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NL; ++k) {
      const int l = lg + LG * k;
      a.qscr[qb + l * 16 + p] = spd * s_q[l * SROW + p];
    }
    // (no barrier here: the next tracer's slab vote is one, and every thread reaches it
    // only after its stores of this tracer)
  }
}

template <typename R> constexpr size_t aal_smem() {
  // + the Qdp slab, two tracers' bounds and the barrier
  return aal_buf_offset<R>() + (NLEV * 16 + 4 * NLEV) * sizeof(double) + 16;
}

// The nine levels lo, lo + 8, ... of one point with N contributions from other elements
// at offsets so[] from the point's own value; N is uniform within a warp (warps grouped by
// point class), so each case is a branch, not a set of predicated adds.
template <int N, bool AVG>
__device__ __forceinline__ void dss_levels(const double* own, const long long* so, double* dst,
                                           const double* s0, double f, int lo) {
#pragma unroll
  for (int l = lo; l < NLEV; l += 8) {
    double acc = own[l * 16];
#pragma unroll
    for (int k = 0; k < N; ++k) acc += own[so[k] + l * 16];
    if constexpr (AVG) dst[l * 16] = fma(acc, f, s0[l * 16] * (1.0 / 3.0));
    else dst[l * 16] = acc * f;
  }
}

// DSS(rspheremp) of the tracer scratch into Qdp(np1); with time_avg the last RK2 stage
// also applies qdp_time_avg: Qdp(np1) = (Qdp(n0) + 2 Qdp(np1)) / 3, formed as
// Qdp(n0) / 3 + gather (2/3 rspheremp).  Grid E*Q, 128 threads: warps by point class
// over a group of 8 levels, each thread its point on the 9 levels lo, lo + 8, ..., so the
// point's table entries and factors are read once.
template <typename R>
__global__ void __launch_bounds__(EQ_THREADS) k_dss_tracers(EulerArgs<R> a, int time_avg) {
  const int eq = blockIdx.x, e = eq / a.Q, q = eq - e * a.Q;
  int lo, p;
  dss_thread_point(lo, p);
  const int ep = e * 16 + p;
  const double rs = a.m.rspheremp_d[ep];
  const long long es = (long long)a.Q * NLEV * 16;
  double* dst = a.qdp + (((size_t)e * QTL + a.np1_qdp) * a.Q + q) * NLEV * 16 + p;
  if (!in_bounds(ep < a.dss.npts, a.dss.flag, kBoundsDssPoint)) return;
  int n = a.dss.cnt[ep];
  if (!in_bounds(n >= 0 && n <= MAXSRC, a.dss.flag, kBoundsDssCount)) n = 0;
  long long so[MAXSRC] = {0, 0, 0};  // offsets of the sources' values from this point's
#pragma unroll
  for (int k = 0; k < MAXSRC; ++k) {
    if (k < n) {
      int sk = a.dss.src[ep * MAXSRC + k];
      if (!in_bounds(sk >= 0 && sk < a.dss.npts, a.dss.flag, kBoundsDssSource)) sk = ep;
      so[k] = ((long long)(sk >> 4) - e) * es + (sk & 15) - p;
    }
  }
  const double* own = a.qscr + (size_t)q * NLEV * 16 + (size_t)e * es + p;
  if (time_avg) {
    const double f = rs * (2.0 / 3.0);
    const double* s0 = a.qdp + (((size_t)e * QTL + a.avg_n0_qdp) * a.Q + q) * NLEV * 16 + p;
    switch (n) {
      case 0: dss_levels<0, true>(own, so, dst, s0, f, lo); break;
      case 1: dss_levels<1, true>(own, so, dst, s0, f, lo); break;
      case 2: dss_levels<2, true>(own, so, dst, s0, f, lo); break;
      default: dss_levels<3, true>(own, so, dst, s0, f, lo); break;
    }
  } else {
    switch (n) {
      case 0: dss_levels<0, false>(own, so, dst, nullptr, rs, lo); break;
      case 1: dss_levels<1, false>(own, so, dst, nullptr, rs, lo); break;
      case 2: dss_levels<2, false>(own, so, dst, nullptr, rs, lo); break;
      default: dss_levels<3, false>(own, so, dst, nullptr, rs, lo); break;
    }
  }
}

// Grid (E, 9), 128 threads: 8 levels per block, warps by point class.
__global__ void __launch_bounds__(128) k_dss_field(const double* __restrict__ src, double* dst,
                                                   const double* __restrict__ rsmp, DssTable tab) {
  int lo, p;
  dss_thread_point(lo, p);
  const int e = blockIdx.x, l = blockIdx.y * 8 + lo;
  double v = dss_gather(src, NLEV * 16, 16, e, l, p, tab);
  if (rsmp) v *= rsmp[e * 16 + p];
  dst[((size_t)e * NLEV + l) * 16 + p] = v;
}

// Generic in-place DSS through a scratch copy.
__global__ void __launch_bounds__(EQ_THREADS) k_copy_fields(int nf, const double* base, long long fs,
                                                             long long es, int ls, double* scr) {
  int e, f, l, p;
  eq_index(nf, e, f, l, p);
  scr[(((size_t)e * nf + f) * NLEV + l) * 16 + p] = base[(size_t)f * fs + (size_t)e * es + (size_t)l * ls + p];
}
__global__ void __launch_bounds__(EQ_THREADS) k_dss_from_copy(int nf, double* base, long long fs,
                                                               long long es, int ls, const double* scr,
                                                               const double* rsmp, DssTable tab) {
  int e, f, l, p;
  eq_index_dss(nf, e, f, l, p);
  double v = dss_gather(scr + (size_t)f * NLEV * 16, (long long)nf * NLEV * 16, 16, e, l, p, tab);
  if (rsmp) v *= rsmp[e * 16 + p];
  base[(size_t)f * fs + (size_t)e * es + (size_t)l * ls + p] = v;
}

// ======================================================================================
// PPM vertical remap (RemapFunctor + PpmVertRemap), four columns per warp.
// ======================================================================================
// A CTA is one warp holding four columns: lane (c = lane / 8, s = lane % 8) works on
// column c, owns its levels 9s .. 9s+8 (every lane busy in the level work; the column
// scans are 8-lane segmented shuffles) and its interfaces j = s, s+8, ..., s+72 of the
// grid and reconstruction work (74 interfaces on 80 lane slots).  Phases are separated
// by __syncwarp only.  Loads and stores of a level touch the four columns' consecutive
// points, so every 32-byte sector fetched is used.
constexpr int RCOLS = 4;  // columns per CTA
constexpr int RT = 32;    // threads per CTA
constexpr int RLV = 9;    // levels per lane
constexpr int RNI = 10;   // interface slots per lane (j = s + 8 i)
// Shared memory of one column, in doubles.  The reconstruction arrays hold R (double in
// the FP64 form, float in the mixed form, two to a double); the mixed form adds the FP32
// neighbour differences of v and T.  The arrays of the grid phase are reused once it is
// done: the cumulative thicknesses pio and pin hold the slopes and edge values, and the
// source reciprocals 1/D, which only the source-cell search reads (the lanes keep their
// own levels' in registers), the grid weights.  With that, 960 doubles a column in FP64
// (7.5 KB: seven CTAs of four columns per SM instead of six) and 705 in the mixed form.
template <typename R>
struct RemapLayout {
  static constexpr int RW = kF32<R> ? 2 : 1;
  static constexpr int D = 0;                           // D[-2 .. 73], source thickness with ghosts
  static constexpr int PIO = D + 76;                    // pio[0 .. 73]; then dma[0 .. 73], R
  static constexpr int PIN = PIO + 74;                  // pin[0 .. 72]; then ai[0 .. 72], R
  static constexpr int RDI = PIN + 74;                  // 1 / D[0 .. 71] in the grid phase; then G
  static constexpr int G = RDI;                         // combined grid weights [5][74], R
  static constexpr int MASS = G + (5 * 74 / RW > 72 ? 5 * 74 / RW : 72);  // mass[0 .. 73]
  static constexpr int A = MASS + 74;                   // cell means A[-2 .. 73], double
  static constexpr int DMA = PIO;
  static constexpr int AI = PIN;
  static constexpr int COEF = A + 76;                   // parabola coefficients [3][72], R
  static constexpr int DLF = COEF + 216 / RW;           // mixed: df[-1 .. 73], float
  static constexpr int END = DLF + (kF32<R> ? 38 : 0);
};

// (ar - cm) (cm - al) > 0, the parabola's monotonicity test: FP32 as is; FP64 as exact
// comparisons on the integer pipe (zeros of either sign compare equal).
template <typename T> __device__ __forceinline__ bool monotone(T al, T cm, T ar) {
  return (ar - cm) * (cm - al) > T(0);
}
template <> __device__ __forceinline__ bool monotone<double>(double al, double cm, double ar) {
  const long long kl = dkz(al), kc = dkz(cm), kr = dkz(ar);
  return (kr > kc && kc > kl) || (kr < kc && kc < kl);
}
// The slope limiter min(|da|, |2 y|, |2 x|) with the sign of da: FP32 as is; FP64 on the
// integer pipe, with min(|2x|, |2y|) formed as 2 min(|x|, |y|) (exact, dtwice).
template <typename T> __device__ __forceinline__ T slope_limit(T da, T x, T y) {
  return min3abs_signed(da, T(2) * y, T(2) * x, da);
}
template <> __device__ __forceinline__ double slope_limit<double>(double da, double x, double y) {
  const long long m = 0x7fffffffffffffffLL;
  const double t = dtwice(__longlong_as_double(kmin(__double_as_longlong(x) & m, __double_as_longlong(y) & m)));
  const long long k = kmin(__double_as_longlong(da) & m, __double_as_longlong(t));
  return __longlong_as_double(k | (__double_as_longlong(da) & ~m));
}
// A negative or NaN layer thickness (x < 0 or isnan(x)), on the integer pipe.
__device__ __forceinline__ bool bad_thickness(double x) {
  const long long b = __double_as_longlong(x);
  return (b < 0 && (b << 1) != 0) || b > 0x7ff0000000000000LL;
}

// compute_ppm at this lane's interfaces (PpmRemap.hpp:202-266): slopes dma[j]
// (j = 0 .. 73) and edge values ai[j] (j = 0 .. 72) of cell means A (ghosts included),
// with the grid weights combined per interface (k1 = g0 g1, k2 = g0 g2, h1 = g3 + g4 g5,
// h2 = g4 g8, h3 = g4 g9):
//   dma_j = limit(k1 (A_j - A_j-1) + k2 (A_j-1 - A_j-2)) if A_j-1 lies between its neighbours
//   ai_j  = A_j-1 + h1 (A_j - A_j-1) - h2 dma_j+1 + h3 dma_j.
template <typename T>
__device__ __forceinline__ void ppm_interfaces(int s, const T* A, const T* g, T* dma, T* ai) {
  T d1[RNI];
#pragma unroll
  for (int i = 0; i < RNI; ++i) {
    const int j = s + 8 * i;
    d1[i] = T(0);
    if (j < NLEV + 2) {
      const T am1 = A[j - 1];
      const T x = A[j] - am1, y = am1 - A[j - 2];
      d1[i] = x;
      T r = T(0);
      if (pos_prod(x, y)) r = slope_limit(g[j] * x + g[74 + j] * y, x, y);
      dma[j] = r;
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < RNI; ++i) {
    const int j = s + 8 * i;
    if (j < NLEV + 1) ai[j] = A[j - 1] + g[2 * 74 + j] * d1[i] - g[3 * 74 + j] * dma[j + 1] + g[4 * 74 + j] * dma[j];
  }
}

// The limited parabola of each of this lane's cells (PpmRemap.hpp:267-353):
// coef = (c0, c1, c2) = (1.5 A - (al + ar) / 4, ar - al, 3 (al + ar - 2 A)).
template <typename T>
__device__ __forceinline__ void ppm_cells(int l0, int remap_alg, const T* A, const T* ai, T* coef) {
  constexpr T sixth = T(1.0 / 6.0);
#pragma unroll
  for (int k3 = 0; k3 < RLV; ++k3) {
    const int jp = l0 + k3;
    T al = ai[jp], ar = ai[jp + 1];
    const T cm = A[jp];
    if (!monotone(al, cm, ar)) { al = cm; ar = cm; }
    // The two overshoot corrections are selected, not branched on: a warp whose lanes
    // disagree would otherwise run both bodies for all of them.  When the first applies
    // (al = 3 A - 2 ar) the second test is (ar - al)(A - (al + ar)/2) = 3/2 (ar - A)^2
    // < -3/2 (ar - A)^2, never true, so it is evaluated on the unmodified edges only.
    T d = ar - al, s2 = al + ar;
    const T q = d * d * sixth, r = d * (cm - s2 * T(0.5));
    const bool fix_l = less(q, r), fix_r = !fix_l && less(r, -q);
    const T c3 = T(3) * cm;
    al = fix_l ? c3 - T(2) * ar : al;
    ar = fix_r ? c3 - T(2) * al : ar;
    d = ar - al;
    s2 = al + ar;
    T c0 = T(1.5) * cm - s2 * T(0.25), c1 = d, c2 = T(3) * (s2 - T(2) * cm);
    if (remap_alg == 2 && (jp < 2 || jp >= NLEV - 2)) {  // PpmFixedParabola
      c0 = cm;
      c1 = T(0);
      c2 = T(0);
    }
    coef[jp] = c0;
    coef[72 + jp] = c1;
    coef[144 + jp] = c2;
  }
}

// The same reconstruction from the neighbour differences df[j] = A[j] - A[j-1]
// (j = -1 .. 73, ghosts included) alone, for the mixed form's v and T: slopes dma from
// df; edge offsets e[j] = ai[j] - A[j-1]; for cell k the parabola's offsets
// dl = al - A[k] = e[k] - df[k] and dr = ar - A[k] = e[k+1], limited as above, give
// coef = (c0 - A[k], c1, c2) = (-(dl + dr) / 4, dr - dl, 3 (dl + dr)).  FP32 carries only
// differences; A[k]'s share of a cell integral is added in FP64 by the caller.
__device__ __forceinline__ void ppm_interfaces_delta(int s, const float* df, const float* g, float* dma,
                                                     float* e) {
#pragma unroll
  for (int i = 0; i < RNI; ++i) {
    const int j = s + 8 * i;
    if (j < NLEV + 2) {
      const float d1 = df[j], d2 = df[j - 1];
      float r = 0.0f;
      if (d1 * d2 > 0.0f) r = min3abs_signed(g[j] * d1 + g[74 + j] * d2, 2.0f * d2, 2.0f * d1, g[j] * d1 + g[74 + j] * d2);
      dma[j] = r;
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < RNI; ++i) {
    const int j = s + 8 * i;
    if (j < NLEV + 1) e[j] = g[2 * 74 + j] * df[j] - g[3 * 74 + j] * dma[j + 1] + g[4 * 74 + j] * dma[j];
  }
}
__device__ __forceinline__ void ppm_cells_delta(int l0, int remap_alg, const float* df, const float* e,
                                                float* coef) {
  constexpr float sixth = 1.0f / 6.0f;
#pragma unroll
  for (int k3 = 0; k3 < RLV; ++k3) {
    const int jp = l0 + k3;
    float dl = e[jp] - df[jp], dr = e[jp + 1];
    if (!(dr * -dl > 0.0f)) { dl = 0.0f; dr = 0.0f; }
    // the overshoot corrections selected, not branched on (as in ppm_cells)
    float c1 = dr - dl;
    const float q = c1 * c1 * sixth, r = c1 * (-(dl + dr) * 0.5f);
    const bool fix_l = q < r, fix_r = !fix_l && r < -q;
    dl = fix_l ? -2.0f * dr : dl;
    dr = fix_r ? -2.0f * dl : dr;
    float d0 = -(dl + dr) * 0.25f, c2 = 3.0f * (dl + dr);
    c1 = dr - dl;
    if (remap_alg == 2 && (jp < 2 || jp >= NLEV - 2)) {  // PpmFixedParabola
      d0 = 0.0f;
      c1 = 0.0f;
      c2 = 0.0f;
    }
    coef[jp] = d0;
    coef[72 + jp] = c1;
    coef[144 + jp] = c2;
  }
}

// PPM vertical remap of v, T (rsplit > 0) and the tracers.  Everything runs in double in
// the FP64 form; the mixed form reconstructs in FP32 (v and T from their neighbour
// differences, the tracers from their FP32 cell means) and keeps the cell integrals, the
// cumulative masses and the grid in FP64, the bottom interface carrying the exact column
// mass (mass fixer).  Divisions are multiplications by Newton reciprocals.
template <typename R>
__global__ void __launch_bounds__(RT, 4) k_remap(RemapArgs a) {
  using LY = RemapLayout<R>;
  constexpr bool lo = kF32<R>;
  extern __shared__ double rsm[];
  const int lane = threadIdx.x, cw = lane >> 3, s = lane & 7;
  // A launch covers whole elements (16 columns each), so all four columns are live.
  const int cidx = blockIdx.x * RCOLS + cw;
  const int e = cidx >> 4, p = cidx & 15;
  double* sm = rsm + cw * LY::END;
  double* D = sm + LY::D + 2;
  double* pio = sm + LY::PIO;
  double* pin = sm + LY::PIN;
  double* rD = sm + LY::RDI;
  double* mass = sm + LY::MASS;
  double* A = sm + LY::A + 2;
  R* g = reinterpret_cast<R*>(sm + LY::G);  // g[c * 74 + j]
  R* dma = reinterpret_cast<R*>(sm + LY::DMA);
  R* ai = reinterpret_cast<R*>(sm + LY::AI);
  R* coef = reinterpret_cast<R*>(sm + LY::COEF);  // coef[c * 72 + k]
  float* dlf = reinterpret_cast<float*>(sm + LY::DLF) + 1;  // df[-1 .. 73]
  float* Af = reinterpret_cast<float*>(sm + LY::A) + 2;  // the tracers' FP32 cell means
  const int l0 = RLV * s;
  const size_t sb = ((size_t)e * NTL + a.np1) * NLEV * 16 + p;
  const size_t vb = ((size_t)e * NTL + a.np1) * NLEV * 32 + p;
  // ---- source thickness and surface pressure (compute_ps_v) ----
  double sv[RLV];
#pragma unroll
  for (int k = 0; k < RLV; ++k) sv[k] = a.dp[sb + (size_t)(l0 + k) * 16];
  double cs = 0.0;
#pragma unroll
  for (int k = 0; k < RLV; ++k) cs += sv[k];
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) cs += __shfl_xor_sync(FULL, cs, off, 8);  // same sum in all 8 lanes
  const double ps = cs + a.hyai0 * a.ps0;
  if (s == 0) a.ps_v[((size_t)e * NTL + a.np1) * 16 + p] = ps;
  // ---- target thickness; vertically Eulerian source thickness (RemapFunctor.hpp:42-100) ----
  double tg[RLV], rt[RLV], rdl[RLV];  // target thickness, its reciprocal, 1 / source thickness
  float rdf[RLV];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < RLV; ++k) {
    const int l = l0 + k;
    tg[k] = c_ai_delta[l] * a.ps0 + c_bi_delta[l] * ps;
    float rf;
    rt[k] = rcp_newton(tg[k], rf);
    if (a.rsplit == 0) {
      const size_t ie = ((size_t)e * NLEV + l) * 16 + p;
      const double en = l + 1 < NLEV ? a.eta[ie + 16] : 0.0;
      sv[k] = tg[k] + a.dt * (en - a.eta[ie]);
    }
    D[l] = sv[k];
    rdl[k] = rcp_newton(sv[k], rf);
    rD[l] = rdl[k];
    if constexpr (lo) rdf[k] = d2f_rn(rdl[k]);
    bad |= bad_thickness(sv[k]);
  }
  if (bad) atomicExch(a.invalid, 1);
  // ---- compute_partitions: cumulative source (pio) and target (pin) thickness ----
  {
    double ts = 0.0, tt = 0.0;
#pragma unroll
    for (int k = 0; k < RLV; ++k) {
      ts += sv[k];
      tt += tg[k];
    }
    double xo = seg_excl_prefix(ts, s), xn = seg_excl_prefix(tt, s);
#pragma unroll
    for (int k = 0; k < RLV; ++k) {
      pio[l0 + k] = xo;
      pin[l0 + k] = xn;
      xo += sv[k];
      xn += tg[k];
    }
    if (s == 7) {
      pio[NLEV] = xo;
      pio[NLEV + 1] = xo + 1.0;
      pin[NLEV] = xo;  // the column's total mass does not change
    }
  }
  __syncwarp();
  if (s == 0) {  // ghost cells of the source thickness: mirrored
    D[-1] = D[0];
    D[-2] = D[1];
    D[NLEV] = D[NLEV - 1];
    D[NLEV + 1] = D[NLEV - 2];
  }
  __syncwarp();
  // ---- compute_integral_bounds: the source cell holding each new interface, and the
  // partial-cell integral's weights x2 + 1/2, (x2^2 - 1/4) / 2, (x2^3 + 1/8) / 3 of this
  // lane's target levels (the search compares on the integer pipe) ----
  int kid[RLV];
  double wz[RLV][3];
  float wzf[RLV][3];
#pragma unroll
  for (int k3 = 0; k3 < RLV; ++k3) {
    const int k = l0 + k3;
    const double pk = pin[k + 1];
    const long long key = dkey(pk);
    int kk = k + 1;
    while (kk < NLEV + 2 && dkey(pio[kk - 1]) <= key) kk++;
    kk--;
    if (kk == NLEV + 1) kk = NLEV;
    if (kk < 1) {  // only reachable with a non-monotone (invalid) source grid
      kk = 1;
      atomicExch(a.invalid, 1);
    }
    if (!in_bounds(kk >= 1 && kk <= NLEV, a.invalid + 2, kBoundsRemapCell)) kk = 1;
    kid[k3] = kk - 1;
    const double x2 = (pk - (pio[kk - 1] + pio[kk]) * 0.5) * rD[kk - 1];
    wz[k3][0] = x2 + 0.5;
    wz[k3][1] = (x2 * x2 - 0.25) * 0.5;
    wz[k3][2] = (x2 * x2 * x2 + 0.125) * (1.0 / 3.0);
    if constexpr (lo) {
      const float xf = d2f_rn(x2);
      wzf[k3][0] = xf + 0.5f;
      wzf[k3][1] = (xf * xf - 0.25f) * 0.5f;
      wzf[k3][2] = (xf * xf * xf + 0.125f) * (1.0f / 3.0f);
    }
  }
  __syncwarp();  // every lane's search is done: 1/D's space takes the grid weights
  // ---- compute_grids (PpmRemap.hpp:367-413, 505-666) at this lane's interfaces, in
  // double; the weights are stored combined (ppm_interfaces), in R ----
#pragma unroll
  for (int i = 0; i < RNI; ++i) {
    const int j = s + 8 * i;
    if (j < NLEV + 2) {
      const double dm2 = D[j - 2], dm1 = D[j - 1], d0 = D[j];
      float rf;
      const double r10 = rcp_newton(dm1 + d0, rf);  // shared by g1, g3, g5
      const double g0 = dm1 * rcp_newton(dm2 + dm1 + d0, rf);
      g[j] = cvt<R>(g0 * ((dtwice(dm2) + dm1) * r10));                        // k1 = g0 g1
      g[74 + j] = cvt<R>(g0 * ((dm1 + dtwice(d0)) * rcp_newton(dm2 + dm1, rf)));  // k2 = g0 g2
      if (j < NLEV + 1) {
        const double dp1 = D[j + 1];
        const double r6 = rcp_newton(dtwice(dm1) + d0, rf);  // shared by g5, g8
        const double r7 = rcp_newton(dtwice(d0) + dm1, rf);  // shared by g5, g9
        const double g4 = rcp_newton(dm2 + dm1 + d0 + dp1, rf);
        const double g5 = (dtwice(dm1 * d0) * r10) * ((dm2 + dm1) * r6 - (dp1 + d0) * r7);
        g[2 * 74 + j] = cvt<R>(dm1 * r10 + g4 * g5);              // h1 = g3 + g4 g5
        g[3 * 74 + j] = cvt<R>(g4 * (dm1 * (dm2 + dm1) * r6));    // h2 = g4 g8
        g[4 * 74 + j] = cvt<R>(g4 * (d0 * (d0 + dp1) * r7));      // h3 = g4 g9
      }
    }
  }
  __syncwarp();
  const int nvar = 3 + a.Q;
  // The variable's values at this lane's levels: v (two components), T, then the
  // tracers.  Each variable's loads are issued one variable ahead, so their latency
  // overlaps the reconstruction of the previous one.
  auto load = [&](int var, double* y) {
#pragma unroll
    for (int k = 0; k < RLV; ++k) {
      const int l = l0 + k;
      if (var < 2) y[k] = a.v[vb + (size_t)l * 32 + var * 16];
      else if (var == 2) y[k] = a.T[sb + (size_t)l * 16];
      else y[k] = a.qdp[((((size_t)e * QTL + a.n0_qdp) * a.Q + (var - 3)) * NLEV + l) * 16 + p];
    }
  };
  const int var0 = a.rsplit == 0 ? 3 : 0;
  double xn[RLV];
  if (var0 < nvar) load(var0, xn);
#pragma unroll 1
  for (int var = var0; var < nvar; ++var) {
    // extrinsic values (v dp, T dp for the states; Qdp as is) and cell means
    double x[RLV];
#pragma unroll
    for (int k = 0; k < RLV; ++k) x[k] = var < 3 ? xn[k] * sv[k] : xn[k];
    if (var + 1 < nvar) load(var + 1, xn);
#pragma unroll
    for (int k = 0; k < RLV; ++k) {
      const int l = l0 + k;
      if (!lo || var < 3) A[l] = x[k] * rdl[k];
      else Af[l] = d2f_rn(x[k]) * rdf[k];
    }
    // mass[i + 1] = sum of x below cell i (mass[0] = mass[1] = 0, mass[73] = column total)
    {
      double tx = 0.0;
#pragma unroll
      for (int k = 0; k < RLV; ++k) tx += x[k];
      double ex = seg_excl_prefix(tx, s);
#pragma unroll
      for (int k = 0; k < RLV; ++k) {
        mass[l0 + k + 1] = ex;
        ex += x[k];
      }
      if (s == 7) mass[NLEV + 1] = ex;
      if (s == 0) mass[0] = 0.0;
    }
    __syncwarp();
    if constexpr (lo) {
      if (var < 3) {  // df[j] = A[j] - A[j-1]; ghosts: mirrored (remap_alg 1, 2) or constant (3) cells
#pragma unroll
        for (int k = 0; k < RLV; ++k) {
          const int j = l0 + k;
          if (j >= 1) dlf[j] = d2f_rn(A[j] - A[j - 1]);
        }
        __syncwarp();
        if (s == 0) {
          dlf[0] = 0.0f;
          dlf[-1] = a.remap_alg == 3 ? 0.0f : -dlf[1];
          dlf[NLEV] = 0.0f;
          dlf[NLEV + 1] = a.remap_alg == 3 ? 0.0f : -dlf[NLEV - 1];
        }
        __syncwarp();
        ppm_interfaces_delta(s, dlf, g, dma, ai);
        __syncwarp();
        ppm_cells_delta(l0, a.remap_alg, dlf, ai, coef);
      } else {
        if (s == 0) {
          Af[-1] = Af[0];
          Af[-2] = a.remap_alg == 3 ? Af[0] : Af[1];
          Af[NLEV] = Af[NLEV - 1];
          Af[NLEV + 1] = a.remap_alg == 3 ? Af[NLEV - 1] : Af[NLEV - 2];
        }
        __syncwarp();
        ppm_interfaces<float>(s, Af, g, dma, ai);
        __syncwarp();
        ppm_cells<float>(l0, a.remap_alg, Af, ai, coef);
      }
    } else {
      if (s == 0) {
        A[-1] = A[0];
        A[-2] = a.remap_alg == 3 ? A[0] : A[1];
        A[NLEV] = A[NLEV - 1];
        A[NLEV + 1] = a.remap_alg == 3 ? A[NLEV - 1] : A[NLEV - 2];
      }
      __syncwarp();
      ppm_interfaces<double>(s, A, g, dma, ai);
      __syncwarp();
      ppm_cells<double>(l0, a.remap_alg, A, ai, coef);
    }
    __syncwarp();
    // compute_remap: mass below each new interface, in double; new cell masses are
    // differences of consecutive interface masses (the lowest from the lane below)
    double m2[RLV];
#pragma unroll
    for (int k3 = 0; k3 < RLV; ++k3) {
      const int k = l0 + k3, kk = kid[k3];
      if constexpr (lo) {
        const float in = (coef[kk] * wzf[k3][0] + coef[72 + kk] * wzf[k3][1]) + coef[144 + kk] * wzf[k3][2];
        // v and T: the coefficients are offsets from the cell mean A[kk]
        const double ind = var < 3 ? fma(A[kk], wz[k3][0], dbl(in)) : dbl(in);
        m2[k3] = k == NLEV - 1 ? mass[NLEV + 1] : mass[kk + 1] + ind * D[kk];
      } else {
        const double in = (coef[kk] * wz[k3][0] + coef[72 + kk] * wz[k3][1]) + coef[144 + kk] * wz[k3][2];
        m2[k3] = mass[kk + 1] + in * D[kk];
      }
    }
    double below = __shfl_up_sync(FULL, m2[RLV - 1], 1, 8);
    if (s == 0) below = 0.0;
#pragma unroll
    for (int k3 = 0; k3 < RLV; ++k3) {
      const int k = l0 + k3;
      const double out = m2[k3] - (k3 == 0 ? below : m2[k3 - 1]);
      if (var < 2) a.v[vb + (size_t)k * 32 + var * 16] = out * rt[k3];
      else if (var == 2) a.T[sb + (size_t)k * 16] = out * rt[k3];
      else a.qdp[((((size_t)e * QTL + a.n0_qdp) * a.Q + (var - 3)) * NLEV + k) * 16 + p] = out;
    }
    __syncwarp();  // the next variable overwrites A, mass and coef
  }
}

// Dense weak Laplacian per element: column c is laplace_simple of the unit vector e_c
// (one half-warp per column), stored as out[e][row p][col c].
__global__ void __launch_bounds__(256) k_lap_matrix(MetricP<double> mp, double* out) {
  const int e = blockIdx.x, col = threadIdx.x >> 4, p = threadIdx.x & 15;
  Pt<double> t;
  t.init(p);
  PM<double> m;
  m.load(mp, e, p);
  out[((size_t)e * 16 + p) * 16 + col] = laplace_simple(t, m, p == col ? 1.0 : 0.0);
}

template <typename R> constexpr int LG_CAAR() { return 8; }
template <typename R> constexpr int LG_HV() { return 8; }
template <typename R> constexpr int LG_TR() { return 8; }

}  // namespace

namespace {
const char* g_last = "";
void (*g_before)(const char*, cudaStream_t) = nullptr;
void (*g_after)(const char*, cudaStream_t) = nullptr;
}  // namespace

void kernel_enter(const char* name, cudaStream_t s) {
  g_last = name;
  if (g_before) g_before(name, s);
}
void kernel_leave(const char* name, cudaStream_t s) {
  if (g_after) g_after(name, s);
}
const char* last_kernel_name() { return g_last; }
void set_kernel_hook(void (*b)(const char*, cudaStream_t), void (*a)(const char*, cudaStream_t)) {
  g_before = b;
  g_after = a;
}

void upload_constants(const double* dvv16, const double* hyai, const double* hybi, double ps0,
                      cudaStream_t s) {
  float f[16];
  for (int i = 0; i < 16; ++i) f[i] = (float)dvv16[i];
  double ad[NLEV], bd[NLEV];
  for (int l = 0; l < NLEV; ++l) {
    ad[l] = hyai[l + 1] - hyai[l];
    bd[l] = hybi[l + 1] - hybi[l];
  }
  double rdp0[NLEV];
  for (int l = 0; l < NLEV; ++l) rdp0[l] = 1.0 / (ad[l] * ps0 + bd[l] * ps0);
  cudaMemcpyToSymbolAsync(c_rdp0, rdp0, sizeof(double) * NLEV, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_dvv, dvv16, sizeof(double) * 16, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_dvvf, f, sizeof(float) * 16, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_hyai, hyai, sizeof(double) * (NLEV + 1), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_hybi, hybi, sizeof(double) * (NLEV + 1), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ai_delta, ad, sizeof(double) * NLEV, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_bi_delta, bd, sizeof(double) * NLEV, 0, cudaMemcpyHostToDevice, s);
  upload_adjoint_constants(dvv16, hyai, hybi, s);
  upload_tangent_constants(dvv16, hyai, hybi, s);
  cudaStreamSynchronize(s);
}

void launch_prim_step_init(int E, double* eta, double* vn0, double* omega_p, double* dpa, double* dpb,
                           double* derived_dp, const double* dp, int n0, int zero_diss, cudaStream_t s) {
  KScope k("prim_step_init", s);
  k_prim_step_init<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, eta, vn0, omega_p, dpa, dpb,
                                                                       derived_dp, dp, n0, zero_diss);
}

void launch_dp_from_ps(int E, double* dp, const double* ps_v, int n0, double ps0, cudaStream_t s) {
  KScope k("dp3d_from_ps", s);
  k_dp_from_ps<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, dp, ps_v, n0, ps0);
}

template <typename R>
void launch_caar(const CaarArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_CAAR<R>();
  // shared memory layouts of k_caar: FP64 form 7 double arrays; mixed form 3 double and
  // 4 float arrays, plus a double T_v array for moist runs
  constexpr size_t s64 = (6 * NLEV * SROW + 16) * sizeof(double);
  constexpr size_t s32 = (3 * NLEV * SROW + 16) * sizeof(double) + (NLEV * SROW + 3 * NLEV * 16) * sizeof(float);
  constexpr size_t stv = NLEV * SROW * sizeof(double);
  const size_t smem = kF32<R> ? s32 + (a.n0_qdp >= 0 ? stv : 0) : s64;
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_caar<R, LG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kF32<R> ? s32 + stv : s64));
    init = true;
  }
  KScope k("caar_stage", s);
  k_caar<R, LG><<<E, LG * 16, smem, s>>>(a);
}

void launch_dss_state(int E, const double* src, double* v, double* T, double* dp, int np1,
                      const double* rsmp, DssTable t, cudaStream_t s) {
  KScope k("dss_caar", s);
  k_dss_state<<<dim3(E, NLEV / 8), 128, 0, s>>>(src, v, T, dp, np1, rsmp, t);
}

template <typename R>
void launch_hv(const HvArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_HV<R>();
  for (int c = 0; c < a.ncyc; ++c) {
    {
      KScope k("hv_laplace1", s);
      k_hv_lap1<R, LG><<<E, LG * 16, 0, s>>>(a);
    }
    {
      KScope k("hv_laplace2", s);
      k_hv_lap2<R, LG><<<E, LG * 16, kF32<R> ? 4 * NLEV * 16 * sizeof(R) : 0, s>>>(a);
    }
    {
      KScope k("hv_dss_update", s);
      k_hv_update<R><<<dim3(E, NLEV / 8), 128, 0, s>>>(a);
    }
  }
}

template <typename R>
void launch_hv_laplacians(const HvArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_HV<R>();
  {
    KScope k("hv_laplace1", s);
    k_hv_lap1<R, LG><<<E, LG * 16, 0, s>>>(a);
  }
  KScope k("hv_laplace2", s);
  k_hv_lap2<R, LG><<<E, LG * 16, kF32<R> ? 4 * NLEV * 16 * sizeof(R) : 0, s>>>(a);
}

template <typename R>
void launch_hv_update(const HvArgs<R>& a, int E, cudaStream_t s) {
  KScope k("hv_dss_update", s);
  k_hv_update<R><<<dim3(E, NLEV / 8), 128, 0, s>>>(a);
}

template <typename R>
void launch_precompute_divdp(const EulerArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_TR<R>();
  KScope k("precompute_divdp", s);
  k_precompute_divdp<R, LG><<<E, LG * 16, 0, s>>>(a);
}

template <typename R>
void launch_euler_step(EulerArgs<R>& a, int E, int time_avg, cudaStream_t s) {
  constexpr int LG = LG_TR<R>();
  const int EQ = E * a.Q;
  a.rhs_viss = 0.0;
  if (a.Q > 0) {
    const bool nbr = (a.rhs_multiplier == 0.0 || a.rhs_multiplier == 2.0);
    {
      KScope k("euler_qminmax", s);
      k_qminmax<R><<<E, 96, 0, s>>>(a, nbr ? a.qlim_tmp : a.qlim, a.rhs_multiplier == 2.0);
    }
    if (a.rhs_multiplier == 2.0) {
      a.rhs_viss = 3.0;
      if (a.nu_p > 0) {
        KScope k("euler_bih_weight", s);
        k_bih_weight<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, a.dpdiss_ave, a.dpdissk);
      }
      {
        KScope k("euler_bih_pre", s);
        k_bih_pre<R, LG><<<EQ, LG * 16, 0, s>>>(a);
      }
      {
        KScope k("euler_bih_post", s);
        k_bih_post<R, LG><<<EQ, LG * 16, 0, s>>>(a);
      }
    }
    if (nbr) {
      KScope k("euler_minmax_nbr", s);
      k_minmax_nbr<<<nblk((long long)E * a.Q * NLEV, 256), 256, 0, s>>>(E, a.Q, a.qlim_tmp, a.qlim, a.conn);
    }
  }
  if (a.Q == 0) {  // with tracers, k_aal_tracer does the setup phase per element itself
    KScope k("euler_aal_setup", s);
    k_aal_setup<R><<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(a, E);
  }
  if (a.Q > 0) {
    {
      constexpr size_t smem = aal_smem<R>();
      static bool init = false;
      if (!init) {
        cudaFuncSetAttribute(k_aal_tracer<R, LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        init = true;
      }
      KScope k("euler_aal_tracer", s);
      k_aal_tracer<R, LG><<<E, LG * 16, smem, s>>>(a);
    }
    {
      KScope k("euler_dss_qdp", s);
      k_dss_tracers<R><<<E * a.Q, EQ_THREADS, 0, s>>>(a, time_avg);
    }
  }
  {
    KScope k("euler_dss_fvar", s);
    k_dss_field<<<dim3(E, NLEV / 8), 128, 0, s>>>(a.fscr, a.f_dss, a.m.rspheremp_d, a.dss);
  }
}

template <typename R>
size_t remap_smem() {
  const size_t smem = (size_t)RCOLS * RemapLayout<R>::END * sizeof(double);
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_remap<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    init = true;
  }
  return smem;
}

template <typename R>
void launch_remap(const RemapArgs& a, cudaStream_t s) {
  const size_t smem = remap_smem<R>();
  KScope k("ppm_remap", s);
  k_remap<R><<<a.nelem * 16 / RCOLS, RT, smem, s>>>(a);
}

template <typename R>
int remap_chunk_elements(int E, int parts) {
  const size_t smem = remap_smem<R>();
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_remap<R>, RT, smem) != cudaSuccess)
    per_sm = 0;
  const int wave = std::max(1, sms * per_sm * RCOLS / 16);
  const int want = std::max(1, (E + parts - 1) / parts);
  return std::max(1, want / wave) * wave;
}

void launch_update_q(int E, int Q, const double* qdp, double* Qc, const double* ps_v, int np1, int np1_qdp,
                     double ps0, cudaStream_t s) {
  if (Q == 0) return;
  KScope k("update_q", s);
  k_update_q<<<dim3(E, NLEV / 8), 128, 0, s>>>(Q, qdp, Qc, ps_v, np1, np1_qdp, ps0);
}

void launch_dss_inplace(int E, int nf, double* base, long long fs, long long es, int ls, double* scr,
                        const double* rsmp, DssTable t, cudaStream_t s) {
  if (nf <= 0) return;
  KScope k("dss_generic", s);
  k_copy_fields<<<dim3(E * nf, NLEV / EQ_LEVELS), EQ_THREADS, 0, s>>>(nf, base, fs, es, ls, scr);
  k_dss_from_copy<<<dim3(E * nf, NLEV / EQ_LEVELS), EQ_THREADS, 0, s>>>(nf, base, fs, es, ls, scr, rsmp, t);
}

void launch_cam_forcing(int E, int Q, double* T, double* v, const double* ft, const double* fm,
                        const double* fq, double* qdp, double* ps_v, double* Qc, int n0, int n0_qdp,
                        int moist, double dt, double ps0, cudaStream_t s) {
  {
    KScope k("cam_forcing_state", s);
    k_state_forcing<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, T, v, ft, fm, n0, dt);
  }
  if (fq == nullptr || Q == 0) return;
  KScope k("cam_forcing_tracers", s);
  if (moist) k_ps_forcing<<<nblk((long long)E * 16, 128), 128, 0, s>>>(E, Q, fq, qdp, ps_v, n0, n0_qdp, dt);
  k_tracer_forcing<<<dim3(E * Q, NLEV / EQ_LEVELS), EQ_THREADS, 0, s>>>(Q, fq, qdp, n0_qdp, dt);
  k_update_q<<<dim3(E, NLEV / 8), 128, 0, s>>>(Q, qdp, Qc, ps_v, n0, n0_qdp, ps0);
}

void launch_diag_scalars(int E, int Q, const double* qdp, const double* Qc, int tq, double* qvar,
                         double* qmass, cudaStream_t s) {
  if (Q == 0) return;
  KScope k("diag_scalars", s);
  k_diag_scalars<<<nblk((long long)E * Q * 16, 128), 128, 0, s>>>(E * Q, Q, qdp, Qc, tq, qvar, qmass);
}

void launch_diag_energy(int E, int Q, const double* T, const double* v, const double* ps_v, const double* phis,
                        const double* qdp, int t1, int t1q, int cpstar, double ps0, double* out,
                        cudaStream_t s) {
  // PhysicalConstants.hpp:18-20
  const double cp = 1005.0, cpwv = 1870.0;
  const double kq = cpwv / cp - 1.0;
  KScope k("diag_energy", s);
  k_diag_energy<<<nblk((long long)E * 16, 128), 128, 0, s>>>(E, Q, T, v, ps_v, phis, qdp, t1, t1q,
                                                               cpstar && Q > 0, ps0, cp, kq, out);
}

void launch_restart_checksum(const double* src, int E, int words, long long rec_words, long long off,
                             unsigned long long* out, cudaStream_t s) {
  if (words <= 0 || E <= 0) return;
  KScope k("restart_checksum", s);
  k_restart_checksum<<<E, 256, 0, s>>>(reinterpret_cast<const unsigned long long*>(src), words, rec_words, off,
                                       out);
}

void launch_lap_matrix(const MetricP<double>& m, int E, double* out, cudaStream_t s) {
  KScope k("lap_matrix", s);
  k_lap_matrix<<<E, 256, 0, s>>>(m, out);
}

#define HX_INST(R)                                                                  \
  template void launch_caar<R>(const CaarArgs<R>&, int, cudaStream_t);              \
  template void launch_hv<R>(const HvArgs<R>&, int, cudaStream_t);                  \
  template void launch_precompute_divdp<R>(const EulerArgs<R>&, int, cudaStream_t); \
  template void launch_euler_step<R>(EulerArgs<R>&, int, int, cudaStream_t);  \
  template void launch_remap<R>(const RemapArgs&, cudaStream_t);                  \
  template int remap_chunk_elements<R>(int, int);                                  \
  template void launch_hv_laplacians<R>(const HvArgs<R>&, int, cudaStream_t);        \
  template void launch_hv_update<R>(const HvArgs<R>&, int, cudaStream_t);
HX_INST(double)
HX_INST(float)

}  // namespace hx
