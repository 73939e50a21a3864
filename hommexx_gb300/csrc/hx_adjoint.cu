// hx_adjoint.cu — hand-written adjoint (vector-Jacobian product) kernels of the dry
// dynamics step: caar RK stage with its DSS, hyperviscosity subcycle, PPM remap.
//
// Each kernel reverses one forward kernel of hx_kernels.cu.  It reads the forward
// input from a checkpoint, recomputes the forward intermediates it needs (pressure,
// 1/p, the omega integral, gradients, vorticity; the PPM grids, slopes, edge values and
// parabolas) and then propagates the cotangents backwards through them:
//   * transposed sphere operators are the forward half-warp contractions with the
//     roles swapped (d/dx <-> weak row contraction, d/dy <-> weak column contraction);
//     the weak Laplacian applies the transposed element matrix (FP64 form) or the
//     contraction form, which is symmetric (mixed form);
//   * the DSS with rspheremp, R S with S the symmetric gather-sum, is transposed as
//     S R: a gather of rspheremp-weighted cotangents, fused into the consumer's load;
//   * the vertical scans reverse into scans in the opposite direction (segmented
//     warp scans in double, as in the forward);
//   * limiter branches (PPM slope and parabola limiters) follow the branch the forward
//     took, and the index search of the remap is kept fixed.
// The forward these reverse restates src/share/cxx/CaarFunctorImpl.hpp:97-889,
// SphereOperators.hpp:291-862, HyperviscosityFunctorImpl.{hpp:72-257,cpp:56-84},
// RemapFunctor.hpp:225-463 and PpmRemap.hpp:174-689.
#include <type_traits>

#include "hx_device.cuh"

namespace hx {
namespace {

// ---- transposed sphere operators on one point-level --------------------------------

// gradient_sphere^T: (g0, g1) -> scalar
template <typename R>
__device__ __forceinline__ R gradient_sphere_T(const Pt<R>& t, const PM<R>& m, R g0, R g1) {
  const R x = m.gr00 * g0 + m.gr10 * g1;  // gr = Dinv / rearth
  const R y = m.gr01 * g0 + m.gr11 * g1;
  return t.wrow(x) + t.wcol(y);
}

// divergence_sphere^T: scalar -> (v0, v1)
template <typename R>
__device__ __forceinline__ void divergence_sphere_T(const Pt<R>& t, const PM<R>& m, R db, R& v0,
                                                    R& v1) {
  const R s = db * m.fdiv;
  const R g0 = t.wrow(s), g1 = t.wcol(s);
  v0 = m.dm00 * g0 + m.dm01 * g1;  // dm = Dinv metdet
  v1 = m.dm10 * g0 + m.dm11 * g1;
}

// vorticity_sphere^T: scalar -> (v0, v1)
template <typename R>
__device__ __forceinline__ void vorticity_sphere_T(const Pt<R>& t, const PM<R>& m, R wb, R& v0,
                                                   R& v1) {
  const R s = wb * m.fdiv;
  const R c1 = t.wrow(s), c0 = -t.wcol(s);
  v0 = m.d00 * c0 + m.d10 * c1;
  v1 = m.d01 * c0 + m.d11 * c1;
}

// vlaplace_sphere_wk_contra^T (SphereOperators.hpp:816-862 reversed)
template <typename R>
__device__ __forceinline__ void vlaplace_contra_T(const Pt<R>& t, const PM<R>& m, R nu_ratio, R l0,
                                                  R l1, R& v0, R& v1) {
  // grad_sphere_wk_testcov reversed
  const R b0 = (m.d00 * l0 + m.d01 * l1) * rre<R>();
  const R b1 = (m.d10 * l0 + m.d11 * l1) * rre<R>();
  const R Xb = -(m.a00 * b0 + m.a10 * b1);
  const R Yb = -(m.a01 * b0 + m.a11 * b1);
  R divb = m.mp * (t.ddx(Xb) + t.ddy(Yb));
  if (nu_ratio > R(0) && nu_ratio != R(1)) divb *= nu_ratio;
  // curl_sphere_wk_testcov (factor -1) reversed: its covariant terms are -(b0, b1)
  const R vortb = m.mp * (t.ddy(b0) - t.ddx(b1));
  R a0, a1, c0, c1;
  vorticity_sphere_T(t, m, vortb, a0, a1);
  divergence_sphere_T(t, m, divb, c0, c1);
  const R f = R(2) * m.sp * rre<R>() * rre<R>();
  v0 = f * l0 + a0 + c0;
  v1 = f * l1 + a1 + c1;
}

// S R gather: the point's and its DSS partners' values weighted by their rspheremp,
// own first, then in table order (the transpose of the DSS with rspheremp).
__device__ __forceinline__ double dss_gather_w(const double* base, long long es, int ls, int e, int l,
                                               int p, const DssTable& tab, const double* w) {
  const int ep = e * 16 + p;
  if (!in_bounds(ep >= 0 && ep < tab.npts, tab.flag, kBoundsDssPoint)) return 0.0;
  double acc = w[ep] * base[(size_t)e * es + (size_t)l * ls + p];
  int n = tab.cnt[ep];
  if (!in_bounds(n >= 0 && n <= MAXSRC, tab.flag, kBoundsDssCount)) n = 0;
  for (int k = 0; k < n; ++k) {
    const int s = tab.src[ep * MAXSRC + k];
    if (!in_bounds(s >= 0 && s < tab.npts, tab.flag, kBoundsDssSource)) continue;
    acc += w[s] * base[(size_t)(s >> 4) * es + (size_t)l * ls + (s & 15)];
  }
  return acc;
}

// ======================================================================================
// caar stage reversed, one CTA per element.  Forward: out = R S (spheremp (xm + dt F(x))).
// ======================================================================================
// Shared memory of k_caar_vjp: four [72][17] double arrays and three in S (the FP64
// form: double; the mixed form: float, the operators' own type), 68.5 or 53.9 KB: three
// or four CTAs per SM.
template <typename R> using CaarVjpS = typename std::conditional<kF32<R>, float, double>::type;
template <typename R> constexpr size_t caar_vjp_smem() {
  return (4 * sizeof(double) + 3 * sizeof(CaarVjpS<R>)) * NLEV * SROW;
}
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_caar_vjp(CaarVjpArgs<R> a) {
  constexpr int NL = NLEV / LG;
  using S = CaarVjpS<R>;
  extern __shared__ double sm[];
  // (T and dp3d are read from the stage input, which stays in L1)
  double* s_p = sm;                       // pressure
  double* s_phib = sm + 1 * NLEV * SROW;  // cotangent of phi; then the scans' T cotangent
  double* s_pb = sm + 2 * NLEV * SROW;    // cotangent of p; then the scans' dp3d cotangent
  double* s_dvb = sm + 3 * NLEV * SROW;   // cotangent of div(v dp)
  S* s_div = reinterpret_cast<S*>(sm + 4 * NLEV * SROW);  // div(v dp); then the omega-integral cotangent
  S* s_rp = s_div + NLEV * SROW;          // 1 / pressure
  S* s_I = s_rp + NLEV * SROW;            // sum_{j<l} div_vdp_j
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const double* xv = a.x.v + (size_t)e * a.x.ev;
  const double* xT = a.x.T + (size_t)e * a.x.es;
  const double* xd = a.x.dp + (size_t)e * a.x.es;
  // ---- phase A: v dp and its divergence ----
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const R u = (R)xv[l * 32 + p], w = (R)xv[l * 32 + 16 + p];
    const double dd = xd[l * 16 + p];
    const R d = (R)dd;
    const R div = divergence_sphere(t, m, u * d, w * d);
    s_div[l * SROW + p] = (S)div;
  }
  __syncthreads();
  // ---- phase B: pressure, 1/p, omega integral (as the forward, in double) ----
  if (tid < 128) {
    const int col = tid >> 3, seg = tid & 7, l0 = seg * 9;
    double prev = seg == 0 ? 0.0 : xd[(l0 - 1) * 16 + col];
    double tot = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double d = xd[(l0 + k) * 16 + col];
      tot += 0.5 * (prev + d);
      prev = d;
    }
    double pr = a.p_top + seg_excl_prefix(tot, seg);
    prev = seg == 0 ? 0.0 : xd[(l0 - 1) * 16 + col];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double d = xd[(l0 + k) * 16 + col];
      pr = pr + 0.5 * (prev + d);
      prev = d;
      s_p[(l0 + k) * SROW + col] = pr;
      float rf;
      s_rp[(l0 + k) * SROW + col] = (S)rcp_newton(pr, rf);
    }
    double dt_ = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) dt_ += (double)s_div[(l0 + k) * SROW + col];
    double acc = seg_excl_prefix(dt_, seg);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      s_I[(l0 + k) * SROW + col] = (S)acc;
      acc = acc + (double)s_div[(l0 + k) * SROW + col];
    }
  }
  __syncthreads();
  // ---- phase C: the tendency's cotangents level by level ----
  const double spd = a.m.spheremp_d[(size_t)e * 16 + p];
  const R fcor = a.m.fcor[(size_t)e * 16 + p];
  const double* rsw = a.m.rspheremp_d;
  double* mv = a.xm_bar.v + (size_t)e * a.xm_bar.ev;
  double* mT = a.xm_bar.T + (size_t)e * a.xm_bar.es;
  double* md = a.xm_bar.dp + (size_t)e * a.xm_bar.es;
  double* ov = a.x0_bar.v + (size_t)e * a.x0_bar.ev;
  double* oT = a.x0_bar.T + (size_t)e * a.x0_bar.es;
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    // pre-DSS cotangent: S (rspheremp aout)
    const double pv0 = dss_gather_w(a.aout.v, a.aout.ev, 32, e, l, p, a.dss, rsw);
    const double pv1 = dss_gather_w(a.aout.v + 16, a.aout.ev, 32, e, l, p, a.dss, rsw);
    const double pT = dss_gather_w(a.aout.T, a.aout.es, 16, e, l, p, a.dss, rsw);
    const double pdp = dss_gather_w(a.aout.dp, a.aout.es, 16, e, l, p, a.dss, rsw);
    // xm_bar += spheremp pre
    mv[l * 32 + p] += spd * pv0;
    mv[l * 32 + 16 + p] += spd * pv1;
    mT[l * 16 + p] += spd * pT;
    md[l * 16 + p] += spd * pdp;
    const R gv0 = (R)(a.dt * spd * pv0), gv1 = (R)(a.dt * spd * pv1);
    const R gT = (R)(a.dt * spd * pT), gdp = (R)(a.dt * spd * pdp);
    // forward intermediates
    const double td = xT[l * 16 + p];
    const R u = (R)xv[l * 32 + p], w = (R)xv[l * 32 + 16 + p];
    const R T = (R)td;
    const R rp = (R)s_rp[l * SROW + p];
    R gp0, gp1, gt0, gt1;
    gradient_sphere(t, m, rel<R>(s_p[l * SROW + p]), gp0, gp1);
    gradient_sphere(t, m, rel<R>(td), gt0, gt1);
    const R div = (R)s_div[l * SROW + p];
    const R omega = (u * gp0 + w * gp1 - ((R)s_I[l * SROW + p] + R(0.5) * div)) * rp;
    const R vo = vorticity_sphere(t, m, u, w) + fcor;
    // F_T = -(v . grad T) + kappa T omega
    R vb0 = -gT * gt0, vb1 = -gT * gt1;
    const R gtb0 = -gT * u, gtb1 = -gT * w;
    R Tb = R(kKappa) * omega * gT;
    const R ob = R(kKappa) * T * gT;
    // F_v0 = -eg0 + v1 (vort + f), F_v1 = -eg1 - v0 (vort + f)
    vb1 += vo * gv0;
    vb0 -= vo * gv1;
    const R vob = w * gv0 - u * gv1;
    // eg = Rgas (T / p) grad p + grad(ke + phi), egb = -gv
    const R r = R(kRgas) * (T * rp);
    const R rb = -(gv0 * gp0 + gv1 * gp1);
    R gpb0 = -r * gv0, gpb1 = -r * gv1;
    Tb += R(kRgas) * rp * rb;
    R pb = -r * rp * rb;
    // omega = (v . grad p - (I + div / 2)) / p
    const R o = ob * rp;
    vb0 += o * gp0;
    vb1 += o * gp1;
    gpb0 += o * u;
    gpb1 += o * w;
    pb -= omega * o;
    // transposed operators
    R tv0, tv1;
    vorticity_sphere_T(t, m, vob, tv0, tv1);
    vb0 += tv0;
    vb1 += tv1;
    const R ephib = gradient_sphere_T(t, m, -gv0, -gv1);
    Tb += gradient_sphere_T(t, m, gtb0, gtb1);
    vb0 += u * ephib;  // ke = (u^2 + w^2) / 2
    vb1 += w * ephib;
    pb += gradient_sphere_T(t, m, gpb0, gpb1);
    s_phib[l * SROW + p] = (double)ephib;
    s_pb[l * SROW + p] = (double)pb;
    s_div[l * SROW + p] = (S)(-o);
    s_dvb[l * SROW + p] = (double)(-gdp - R(0.5) * o);
    ov[l * 32 + p] += (double)vb0;
    ov[l * 32 + 16 + p] += (double)vb1;
    oT[l * 16 + p] += (double)Tb;
  }
  __syncthreads();
  // ---- phase D: the scans reversed (double) ----
  if (tid < 128) {
    const int col = tid >> 3, seg = tid & 7, l0 = seg * 9;
    // phi_l = phis + 2 sum_{j>l} r_j + r_l  =>  rb_l = phib_l + 2 sum_{j<l} phib_j
    double tot = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) tot += s_phib[(l0 + k) * SROW + col];
    double acc = seg_excl_prefix(tot, seg);
    double Tb2[9], dpb2[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int i = (l0 + k) * SROW + col;
      const double phb = s_phib[i];
      const double rb = phb + 2.0 * acc;
      acc += phb;
      // 1 / p in double (the mixed form keeps only its FP32 image in shared memory)
      double rp;
      if constexpr (kF32<R>) {
        float rf;
        rp = rcp_newton(s_p[i], rf);
      } else {
        rp = s_rp[i];
      }
      const double T = xT[(l0 + k) * 16 + col], dp = xd[(l0 + k) * 16 + col];
      const double hr = dp * 0.5 * rp;  // r = Rgas T dp / (2 p)
      Tb2[k] = kRgas * hr * rb;
      dpb2[k] = kRgas * T * 0.5 * rp * rb;
      s_pb[i] -= kRgas * T * hr * rp * rb;
    }
    // p_l = p_top + sum_{j<l} dp_j + dp_l / 2  =>  dpb_l += pb_l / 2 + sum_{j>l} pb_j
    tot = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) tot += s_pb[(l0 + k) * SROW + col];
    acc = seg_excl_suffix(tot, seg);
#pragma unroll
    for (int k = 8; k >= 0; --k) {
      const double pbl = s_pb[(l0 + k) * SROW + col];
      dpb2[k] += 0.5 * pbl + acc;
      acc += pbl;
    }
    // omega integral I_l = sum_{j<l} div_j  =>  divb_l += sum_{j>l} Ib_j
    tot = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) tot += s_div[(l0 + k) * SROW + col];
    acc = seg_excl_suffix(tot, seg);
#pragma unroll
    for (int k = 8; k >= 0; --k) {
      const int i = (l0 + k) * SROW + col;
      const double ib = (double)s_div[i];
      s_dvb[i] += acc;
      acc += ib;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      s_phib[(l0 + k) * SROW + col] = Tb2[k];
      s_pb[(l0 + k) * SROW + col] = dpb2[k];
    }
  }
  __syncthreads();
  // ---- phase E: v dp reversed; the scans' T and dp3d cotangents ----
  double* od = a.x0_bar.dp + (size_t)e * a.x0_bar.es;
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    R vd0, vd1;
    divergence_sphere_T(t, m, (R)s_dvb[l * SROW + p], vd0, vd1);
    const double u = xv[l * 32 + p], w = xv[l * 32 + 16 + p];
    const double dd = xd[l * 16 + p];
    ov[l * 32 + p] += dd * (double)vd0;
    ov[l * 32 + 16 + p] += dd * (double)vd1;
    oT[l * 16 + p] += s_phib[l * SROW + p];
    od[l * 16 + p] += s_pb[l * SROW + p] + (u * (double)vd0 + w * (double)vd1);
  }
}

// ======================================================================================
// Hyperviscosity subcycle reversed: three kernels.
// ======================================================================================

// TagUpdateStates reversed, pointwise: v' = v + vt, T' = T + tt - (vt . v') / cp,
// dp' = R dpt; writes the input cotangent's direct part and pre = the cotangent of the
// DSS'd tendencies before their DSS.
__global__ void k_hvb_update(int E, DynV x, DynV xo, DynV a, DynV xb, double* pre,
                             const double* rsp, double dt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), l = (idx / 16) % NLEV, p = idx & 15;
  const double rs = rsp[e * 16 + p];
  const size_t iv = (size_t)e * a.ev + l * 32 + p, is = (size_t)e * a.es + l * 16 + p;
  const size_t xv_ = (size_t)e * x.ev + l * 32 + p, xov = (size_t)e * xo.ev + l * 32 + p;
  const size_t bv = (size_t)e * xb.ev + l * 32 + p, bs = (size_t)e * xb.es + l * 16 + p;
  double* pr = pre + ((size_t)e * NLEV + l) * 64 + p;
  const double tb = a.T[is];
  const double hb = -tb * (1.0 / kCp);
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const double vnew = xo.v[xov + c * 16];
    const double vt = vnew - x.v[xv_ + c * 16];
    const double vnb = a.v[iv + c * 16] + hb * vt;
    xb.v[bv + c * 16] = vnb;
    pr[c * 16] = dt * rs * (hb * vnew + vnb);
  }
  xb.T[bs] = tb;
  pr[32] = dt * rs * tb;
  pr[48] = rs * a.dp[is];
  xb.dp[bs] = 0.0;
}

// TagHyperPreExchange and the second Laplacian reversed: gathers S(pre); adds the
// dp3d and sponge (nu_top) parts to the input cotangent; writes mid = the cotangent of
// the first Laplacians after their DSS.
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_hvb_second(HvVjpArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const double spd = a.m.spheremp_d[(size_t)e * 16 + p];
  double* bv = a.xb.v + (size_t)e * a.xb.ev;
  double* bT = a.xb.T + (size_t)e * a.xb.es;
  double* bd = a.xb.dp + (size_t)e * a.xb.es;
  double* mo = a.mid + (size_t)e * NLEV * 64;
  const R r2 = R(a.nu_ratio2);
  LapOp<R> lap;
  lap.load(a.m, e, p, true);
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const double g0 = dss_gather(a.pre, NLEV * 64, 64, e, l, p, a.dss);
    const double g1 = dss_gather(a.pre + 16, NLEV * 64, 64, e, l, p, a.dss);
    const double gT = dss_gather(a.pre + 32, NLEV * 64, 64, e, l, p, a.dss);
    const double gd = dss_gather(a.pre + 48, NLEV * 64, 64, e, l, p, a.dss);
    bd[l * 16 + p] += spd * gd;
    const double xdt = gd * a.dt;
    R m0, m1;
    vlaplace_contra_T(t, m, r2, (R)(-a.nu * g0), (R)(-a.nu * g1), m0, m1);
    const R mT = lap(t, m, (R)(-a.nu_s * gT));
    const R md = lap(t, m, (R)(-a.nu_p * xdt));
    mo[l * 64 + p] = (double)m0;
    mo[l * 64 + 16 + p] = (double)m1;
    mo[l * 64 + 32 + p] = (double)mT;
    mo[l * 64 + 48 + p] = (double)md;
    // sponge layer: levels 0-2 (the other half-warp of the warp computes and discards)
    if (a.nu_top > 0.0 && __any_sync(FULL, l < 3)) {
      const double sc = l == 0 ? 4.0 * a.nu_top : l == 1 ? 2.0 * a.nu_top : l == 2 ? a.nu_top : 0.0;
      R s0, s1;
      vlaplace_contra_T(t, m, R(1), (R)(sc * g0), (R)(sc * g1), s0, s1);
      const R sT = lap(t, m, (R)(sc * gT));
      const R sd = lap(t, m, (R)(sc * xdt));
      if (l < 3) {
        bv[l * 32 + p] += (double)s0;
        bv[l * 32 + 16 + p] += (double)s1;
        bT[l * 16 + p] += (double)sT;
        bd[l * 16 + p] += (double)sd;
      }
    }
  }
}

// The first DSS (with rspheremp) and the first Laplacians reversed.
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_hvb_first(HvVjpArgs<R> a) {
  constexpr int NL = NLEV / LG;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const double* rsw = a.m.rspheremp_d;
  double* bv = a.xb.v + (size_t)e * a.xb.ev;
  double* bT = a.xb.T + (size_t)e * a.xb.es;
  double* bd = a.xb.dp + (size_t)e * a.xb.es;
  const R r1 = R(a.nu_ratio1);
  LapOp<R> lap;
  lap.load(a.m, e, p, true);
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const double g0 = dss_gather_w(a.mid, NLEV * 64, 64, e, l, p, a.dss, rsw);
    const double g1 = dss_gather_w(a.mid + 16, NLEV * 64, 64, e, l, p, a.dss, rsw);
    const double gT = dss_gather_w(a.mid + 32, NLEV * 64, 64, e, l, p, a.dss, rsw);
    const double gd = dss_gather_w(a.mid + 48, NLEV * 64, 64, e, l, p, a.dss, rsw);
    R v0, v1;
    vlaplace_contra_T(t, m, r1, (R)g0, (R)g1, v0, v1);
    const R lT = lap(t, m, (R)gT);
    const R ld = lap(t, m, (R)gd);
    bv[l * 32 + p] += (double)v0;
    bv[l * 32 + 16 + p] += (double)v1;
    bT[l * 16 + p] += (double)lT;
    bd[l * 16 + p] += (double)ld;
  }
}

// ======================================================================================
// Small pointwise kernels
// ======================================================================================
__global__ void k_rk5_comb_vjp(int E, DynV by, DynV b1, DynV b0) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), r = idx % (NLEV * 16), l = r / 16, p = r & 15;
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const double y = by.v[(size_t)e * by.ev + l * 32 + c * 16 + p];
    b1.v[(size_t)e * b1.ev + l * 32 + c * 16 + p] += 1.25 * y;
    b0.v[(size_t)e * b0.ev + l * 32 + c * 16 + p] -= 0.25 * y;
  }
  const double yt = by.T[(size_t)e * by.es + r], yd = by.dp[(size_t)e * by.es + r];
  b1.T[(size_t)e * b1.es + r] += 1.25 * yt;
  b0.T[(size_t)e * b0.es + r] -= 0.25 * yt;
  b1.dp[(size_t)e * b1.es + r] += 1.25 * yd;
  b0.dp[(size_t)e * b0.es + r] -= 0.25 * yd;
}

__global__ void k_copy_dyn(int E, DynV d, DynV s) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= E * NLEV * 16) return;
  const int e = idx / (NLEV * 16), r = idx % (NLEV * 16), l = r / 16, p = r & 15;
  d.v[(size_t)e * d.ev + l * 32 + p] = s.v[(size_t)e * s.ev + l * 32 + p];
  d.v[(size_t)e * d.ev + l * 32 + 16 + p] = s.v[(size_t)e * s.ev + l * 32 + 16 + p];
  d.T[(size_t)e * d.es + r] = s.T[(size_t)e * s.es + r];
  d.dp[(size_t)e * d.es + r] = s.dp[(size_t)e * s.es + r];
}

// ======================================================================================
// PPM remap of one column reversed (RemapFunctor + PpmVertRemap, rsplit > 0).  One warp
// per column; lane L owns cells 3L .. 3L+2 (L < 24) and grid interfaces j = 3L .. 3L+2
// (L < 25).  The forward is recomputed with the forward kernel's arithmetic (so every
// branch and index search matches it); contributions that a lane makes to another
// lane's index go through per-offset shared arrays that the owner sums afterwards.
// ======================================================================================
constexpr int VC = 1;  // columns (warps) per CTA: the shared memory (21.8 KB a column) sets the occupancy, and one-warp CTAs fill an SM best
// shared-memory slots of one column (doubles)
constexpr int V_D = 0;              // D[-2 .. 73]
constexpr int V_RD = V_D + 76;      // 1 / D[0 .. 71]
constexpr int V_PIO = V_RD + 72;    // pio[0 .. 73]
constexpr int V_PIN = V_PIO + 74;   // pin[0 .. 72]
constexpr int V_Z2 = V_PIN + 74;    // z2[0 .. 71]
constexpr int V_KID = V_Z2 + 72;    // kid[0 .. 71] (int)
constexpr int V_FIRST = V_KID + 36; // first interface of each source cell (int, -1: none)
constexpr int V_G = V_FIRST + 36;   // g[11][74]; row 10 = g5 (g6 - g7) as the forward forms it
constexpr int V_PINB = V_G + 814;   // cotangent of pin[0 .. 73]
constexpr int V_PIOL = V_PINB + 74; // cotangent of pio[kk] from the z2 of cell kk (by kk)
constexpr int V_A = V_PIOL + 74;    // A[-2 .. 73]
constexpr int V_MASS = V_A + 76;    // mass[0 .. 73]
constexpr int V_DMA = V_MASS + 74;  // dma[0 .. 73]
constexpr int V_AI = V_DMA + 74;    // ai[0 .. 72]
constexpr int V_COEF = V_AI + 74;   // coef[3][72]
constexpr int V_MB = V_COEF + 216;  // cotangent of the interface masses m(k)
constexpr int V_AIL = V_MB + 72;    // ai cotangent from cell jp's left edge (index jp)
constexpr int V_AIH = V_AIL + 74;   // ai cotangent from cell jp's right edge (index jp+1)
constexpr int V_DM9 = V_AIH + 74;   // dma cotangent from ai[j] (index j)
constexpr int V_DM8 = V_DM9 + 74;   // dma cotangent from ai[j] (index j+1)
constexpr int V_ACM = V_DM8 + 74;   // A cotangent from the parabola of cell k (index k)
constexpr int V_AID = V_ACM + 72;   // A cotangent from ai[j] (index j)
constexpr int V_AIM = V_AID + 74;   // A cotangent from ai[j] (index j-1)
constexpr int V_DD1 = V_AIM + 74;   // A cotangent from dma[j] (index j)
constexpr int V_DDM = V_DD1 + 74;   // A cotangent from dma[j] (index j-1)
constexpr int V_DD2 = V_DDM + 74;   // A cotangent from dma[j] (index j-2)
constexpr int V_COL = V_DD2 + 74;   // doubles per column
// after the variable loop the grid's D cotangent offsets reuse the per-variable slots
constexpr int V_GM2 = V_A, V_GM1 = V_MASS, V_G0 = V_DMA, V_GP1 = V_AI;

__device__ __forceinline__ double warp_excl_suffix(double v, int lane) {
  double incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double y = __shfl_down_sync(FULL, incl, off);
    if (lane + off < 32) incl += y;
  }
  const double ex = __shfl_down_sync(FULL, incl, 1);
  return lane == 31 ? 0.0 : ex;
}

__global__ void __launch_bounds__(VC * 32) k_remap_vjp(RemapVjpArgs a) {
  extern __shared__ double vsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cidx = blockIdx.x * VC + warp;
  if (cidx >= a.nelem * 16) return;  // whole warp leaves together; no CTA barriers below
  const int e = cidx >> 4, p = cidx & 15;
  double* sm = vsm + warp * V_COL;
  double* D = sm + V_D + 2;
  double* rD = sm + V_RD;
  double* pio = sm + V_PIO;
  double* pin = sm + V_PIN;
  double* z2 = sm + V_Z2;
  int* kid = reinterpret_cast<int*>(sm + V_KID);
  int* first = reinterpret_cast<int*>(sm + V_FIRST);
  double* g = sm + V_G;
  double* pinb = sm + V_PINB;
  double* piol = sm + V_PIOL;
  double* A = sm + V_A + 2;
  double* mass = sm + V_MASS;
  double* dma = sm + V_DMA;
  double* ai = sm + V_AI;
  double* coef = sm + V_COEF;
  double* mb = sm + V_MB;
  double* ail = sm + V_AIL;
  double* aih = sm + V_AIH;
  double* dm9 = sm + V_DM9;
  double* dm8 = sm + V_DM8;
  double* acm = sm + V_ACM;
  double* aid = sm + V_AID;
  double* aim = sm + V_AIM;
  double* dd1 = sm + V_DD1;
  double* ddm = sm + V_DDM;
  double* dd2 = sm + V_DD2;
  const bool own = lane < 24;
  const int l0 = 3 * lane;
  const double* xv = a.x.v + (size_t)e * a.x.ev + p;
  const double* xT = a.x.T + (size_t)e * a.x.es + p;
  const double* xd = a.x.dp + (size_t)e * a.x.es + p;
  double* bv = a.a.v + (size_t)e * a.a.ev + p;
  double* bT = a.a.T + (size_t)e * a.a.es + p;
  double* bd = a.a.dp + (size_t)e * a.a.es + p;
  // ---- grid (as the forward kernel) ----
  double s3[3] = {0.0, 0.0, 0.0}, t3[3] = {0.0, 0.0, 0.0}, rt3[3] = {0.0, 0.0, 0.0};
  if (own) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float rf;
      s3[k] = xd[(size_t)(l0 + k) * 16];
      D[l0 + k] = s3[k];
      rD[l0 + k] = rcp_newton(s3[k], rf);
    }
  }
  const double ps = warp_sum(s3[0] + s3[1] + s3[2]) + a.hyai0 * a.ps0;
  if (own) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int l = l0 + k;
      float rf;
      t3[k] = (c_hyai[l + 1] - c_hyai[l]) * a.ps0 + (c_hybi[l + 1] - c_hybi[l]) * ps;
      rt3[k] = rcp_newton(t3[k], rf);
    }
  }
  {
    double ex = warp_excl_scan(s3[0] + s3[1] + s3[2], lane);
    double ey = warp_excl_scan(t3[0] + t3[1] + t3[2], lane);
    if (own) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pio[l0 + k] = ex;
        pin[l0 + k] = ey;
        ex += s3[k];
        ey += t3[k];
      }
    }
    if (lane == 23) {
      pio[NLEV] = ex;
      pio[NLEV + 1] = ex + 1.0;
      pin[NLEV] = ex;
    }
  }
  for (int i = lane; i < 74; i += 32) {
    pinb[i] = 0.0;
    piol[i] = 0.0;
  }
  __syncwarp();
  if (lane == 0) {
    D[-1] = D[0];
    D[-2] = D[1];
    D[NLEV] = D[NLEV - 1];
    D[NLEV + 1] = D[NLEV - 2];
  }
  if (own)
    for (int k = 0; k < 3; ++k) first[l0 + k] = -1;
  __syncwarp();
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int k = l0 + k3;
      int kk = k + 1;
      while (kk < NLEV + 2 && pio[kk - 1] <= pin[k + 1]) kk++;
      kk--;
      if (kk == NLEV + 1) kk = NLEV;
      if (kk < 1) kk = 1;
      kid[k] = kk - 1;
      z2[k] = (pin[k + 1] - (pio[kk - 1] + pio[kk]) * 0.5) * rD[kk - 1];
    }
  }
  if (lane < 25) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int j = 3 * lane + k3;
      if (j < NLEV + 2) {
        // the forward's reciprocals (rcp_newton), so the weights are the forward's
        const double dm2 = D[j - 2], dm1 = D[j - 1], d0 = D[j];
        float rf;
        const double r10 = rcp_newton(dm1 + d0, rf);
        g[0 * 74 + j] = dm1 * rcp_newton(dm2 + dm1 + d0, rf);
        g[1 * 74 + j] = (2.0 * dm2 + dm1) * r10;
        g[2 * 74 + j] = (dm1 + 2.0 * d0) * rcp_newton(dm2 + dm1, rf);
        if (j < NLEV + 1) {
          const double dp1 = D[j + 1];
          const double r6 = rcp_newton(2.0 * dm1 + d0, rf);
          const double r7 = rcp_newton(2.0 * d0 + dm1, rf);
          g[3 * 74 + j] = dm1 * r10;
          g[4 * 74 + j] = rcp_newton(dm2 + dm1 + d0 + dp1, rf);
          g[5 * 74 + j] = (2.0 * dm1 * d0) * r10;
          g[6 * 74 + j] = (dm2 + dm1) * r6;
          g[7 * 74 + j] = (dp1 + d0) * r7;
          g[8 * 74 + j] = dm1 * (dm2 + dm1) * r6;
          g[9 * 74 + j] = d0 * (d0 + dp1) * r7;
          g[10 * 74 + j] = ((2.0 * dm1 * d0) * r10) * ((dm2 + dm1) * r6 - (dp1 + d0) * r7);
        }
      }
    }
  }
  __syncwarp();
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int k = l0 + k3;
      if (k == 0 || kid[k - 1] != kid[k]) first[kid[k]] = k;
    }
  }
  __syncwarp();
  // cotangent accumulators kept over the three variables
  double gb[3][10];
#pragma unroll
  for (int k3 = 0; k3 < 3; ++k3)
#pragma unroll
    for (int c = 0; c < 10; ++c) gb[k3][c] = 0.0;
  double Dbo[3] = {0.0, 0.0, 0.0}, srcb[3] = {0.0, 0.0, 0.0}, tgtb[3] = {0.0, 0.0, 0.0};
  double pioh[3] = {0.0, 0.0, 0.0};  // cotangent of pio[kk + 1] from the z2 of cell kk
  if (own) {
#pragma unroll
    for (int k = 0; k < 3; ++k) tgtb[k] = bd[(size_t)(l0 + k) * 16];
  }
  constexpr double sixth = 1.0 / 6.0;
#pragma unroll 1
  for (int var = 0; var < 3; ++var) {
    // ---- forward recompute ----
    double x[3] = {0.0, 0.0, 0.0}, q[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int l = l0 + k;
        x[k] = var < 2 ? xv[(size_t)l * 32 + var * 16] : xT[(size_t)l * 16];
        q[k] = x[k] * s3[k];
        A[l] = q[k] * rD[l];
      }
    }
    {
      double ex = warp_excl_scan(q[0] + q[1] + q[2], lane);
      if (own) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          mass[l0 + k + 1] = ex;
          ex += q[k];
        }
      }
    }
    __syncwarp();
    if (lane == 0) {
      A[-1] = A[0];
      A[-2] = A[1];
      A[NLEV] = A[NLEV - 1];
      A[NLEV + 1] = A[NLEV - 2];
    }
    __syncwarp();
    int dsel[3] = {0, 0, 0};
    double dsg[3] = {0.0, 0.0, 0.0};
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 2) {
          const double a0 = A[j], am1 = A[j - 1], am2 = A[j - 2];
          double r = 0.0;
          if (pos_prod(a0 - am1, am1 - am2)) {
            const double da = g[0 * 74 + j] * (g[1 * 74 + j] * (a0 - am1) + g[2 * 74 + j] * (am1 - am2));
            // the forward's min3abs_signed; magnitudes compared as bit patterns
            const double ya = 2.0 * (am1 - am2), za = 2.0 * (a0 - am1);
            const long long m = 0x7fffffffffffffffLL;
            const long long kx = __double_as_longlong(da) & m, ky = __double_as_longlong(ya) & m,
                            kz = __double_as_longlong(za) & m;
            long long mv = kx;
            dsel[k3] = 1;
            if (ky < mv) { mv = ky; dsel[k3] = 2; }
            if (kz < mv) dsel[k3] = 3;
            dsg[k3] = copysign(1.0, da);
            r = min3abs_signed(da, ya, za, da);
          }
          dma[j] = r;
        }
      }
    }
    __syncwarp();
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 1) {
          const double a0 = A[j], am1 = A[j - 1];
          ai[j] = am1 + g[3 * 74 + j] * (a0 - am1) +
                  g[4 * 74 + j] * (g[10 * 74 + j] * (a0 - am1) -
                                   g[8 * 74 + j] * dma[j + 1] + g[9 * 74 + j] * dma[j]);
        }
      }
    }
    __syncwarp();
    int br[3] = {0, 0, 0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int jp = l0 + k3;
        double al = ai[jp], ar = ai[jp + 1];
        const double cm = A[jp];
        if (!pos_prod(ar - cm, cm - al)) { al = cm; ar = cm; br[k3] |= 1; }
        if (less((ar - al) * (ar - al) * sixth, (ar - al) * (cm - (al + ar) * 0.5))) {
          al = 3.0 * cm - 2.0 * ar;
          br[k3] |= 2;
        }
        if (less((ar - al) * (cm - (al + ar) * 0.5), -(ar - al) * (ar - al) * sixth)) {
          ar = 3.0 * cm - 2.0 * al;
          br[k3] |= 4;
        }
        double c0 = 1.5 * cm - (al + ar) / 4.0, c1 = ar - al, c2 = 3.0 * (-2.0 * cm + (al + ar));
        if (a.remap_alg == 2 && (jp < 2 || jp >= NLEV - 2)) {
          c0 = cm;
          c1 = 0.0;
          c2 = 0.0;
        }
        coef[jp] = c0;
        coef[72 + jp] = c1;
        coef[144 + jp] = c2;
      }
    }
    __syncwarp();
    double m2[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int k = l0 + k3;
        const int kk = kid[k];
        const double x2 = z2[k], x1 = -0.5;
        const double in = (coef[kk] * (x2 - x1) + coef[72 + kk] * (x2 * x2 - x1 * x1) * 0.5) +
                          coef[144 + kk] * (x2 * x2 * x2 - x1 * x1 * x1) * (1.0 / 3.0);
        m2[k3] = mass[kk + 1] + in * D[kk];
      }
    }
    double below = __shfl_up_sync(FULL, m2[2], 1);
    if (lane == 0) below = 0.0;
    // ---- reverse: x_new = (m(k) - m(k-1)) / tgt ----
    double ob[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int k = l0 + k3;
        const double m1 = k3 == 0 ? below : m2[k3 - 1];
        const double xn = (m2[k3] - m1) * rt3[k3];
        const double xb = var < 2 ? bv[(size_t)k * 32 + var * 16] : bT[(size_t)k * 16];
        ob[k3] = xb * rt3[k3];
        tgtb[k3] -= ob[k3] * xn;
      }
    }
    {
      const double nxt = __shfl_down_sync(FULL, ob[0], 1);
      if (own) {
#pragma unroll
        for (int k3 = 0; k3 < 3; ++k3) {
          const int k = l0 + k3;
          const double o1 = k3 < 2 ? ob[k3 + 1] : (k + 1 < NLEV ? nxt : 0.0);
          mb[k] = ob[k3] - o1;
        }
      }
    }
    __syncwarp();
    // interface masses reversed, gathered per source cell in increasing k
    double cb[3][3], mbc[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int kk = l0 + k3;
        double c0b = 0.0, c1b = 0.0, c2b = 0.0;
        const double c0 = coef[kk], c1 = coef[72 + kk], c2 = coef[144 + kk];
        for (int k = first[kk]; k >= 0 && k < NLEV && kid[k] == kk; ++k) {
          const double b = mb[k];
          const double x2 = z2[k];
          const double in = (c0 * (x2 + 0.5) + c1 * (x2 * x2 - 0.25) * 0.5) +
                            c2 * (x2 * x2 * x2 + 0.125) * (1.0 / 3.0);
          mbc[k3] += b;
          Dbo[k3] += b * in;
          const double ib = b * D[kk];
          c0b += ib * (x2 + 0.5);
          c1b += ib * (x2 * x2 - 0.25) * 0.5;
          c2b += ib * (x2 * x2 * x2 + 0.125) * (1.0 / 3.0);
          // z2 = (pin[k+1] - (pio[kk] + pio[kk+1]) / 2) / D[kk]
          const double zb = ib * (c0 + c1 * x2 + c2 * x2 * x2);
          const double zr = zb * rD[kk];
          pinb[k + 1] += zr;
          piol[kk] -= 0.5 * zr;
          pioh[k3] -= 0.5 * zr;
          Dbo[k3] -= zr * x2;
        }
        cb[k3][0] = c0b;
        cb[k3][1] = c1b;
        cb[k3][2] = c2b;
      }
    }
    // parabola coefficients and their limiter reversed, per cell
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int jp = l0 + k3;
        double cmb, alb, arb;
        if (a.remap_alg == 2 && (jp < 2 || jp >= NLEV - 2)) {
          cmb = cb[k3][0];
          alb = arb = 0.0;
        } else {
          const double c0 = cb[k3][0], c1 = cb[k3][1], c2 = cb[k3][2];
          cmb = 1.5 * c0 - 6.0 * c2;
          alb = -c0 / 4.0 - c1 + 3.0 * c2;
          arb = -c0 / 4.0 + c1 + 3.0 * c2;
          if (br[k3] & 4) { cmb += 3.0 * arb; alb -= 2.0 * arb; arb = 0.0; }
          if (br[k3] & 2) { cmb += 3.0 * alb; arb -= 2.0 * alb; alb = 0.0; }
          if (br[k3] & 1) { cmb += alb + arb; alb = arb = 0.0; }
        }
        acm[jp] = cmb;
        ail[jp] = alb;
        aih[jp] = arb;
      }
    }
    __syncwarp();
    // edge values reversed, per interface j: ai_b[j] = right edge of cell j-1 + left of j
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 1) {
          const double b = (j >= 1 ? aih[j - 1] : 0.0) + (j < NLEV ? ail[j] : 0.0);
          const double d = A[j] - A[j - 1];
          const double gd = g[6 * 74 + j] - g[7 * 74 + j];
          const double g5 = g[5 * 74 + j], g8 = g[8 * 74 + j], g9 = g[9 * 74 + j];
          const double inner = g5 * gd * d - g8 * dma[j + 1] + g9 * dma[j];
          const double ib = b * g[4 * 74 + j];
          const double db = b * g[3 * 74 + j] + ib * g5 * gd;
          aim[j] = b - db;
          aid[j] = db;
          gb[k3][3] += b * d;
          gb[k3][4] += b * inner;
          gb[k3][5] += ib * gd * d;
          gb[k3][6] += ib * g5 * d;
          gb[k3][7] -= ib * g5 * d;
          gb[k3][8] -= ib * dma[j + 1];
          gb[k3][9] += ib * dma[j];
          dm8[j] = -ib * g8;  // for dma[j + 1]
          dm9[j] = ib * g9;   // for dma[j]
        }
      }
    }
    __syncwarp();
    // limited slopes reversed, per j: dma_b[j] = (from ai[j-1]) + (from ai[j])
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 2) {
          const double b = (j >= 1 ? dm8[j - 1] : 0.0) + (j < NLEV + 1 ? dm9[j] : 0.0);
          double d1b = 0.0, d2b = 0.0;
          if (dsel[k3] != 0) {
            const double d1 = A[j] - A[j - 1], d2 = A[j - 1] - A[j - 2];
            if (dsel[k3] == 1) {
              const double g0 = g[0 * 74 + j], g1 = g[1 * 74 + j], g2 = g[2 * 74 + j];
              gb[k3][0] += b * (g1 * d1 + g2 * d2);
              gb[k3][1] += b * g0 * d1;
              gb[k3][2] += b * g0 * d2;
              d1b = b * g0 * g1;
              d2b = b * g0 * g2;
            } else if (dsel[k3] == 2) {
              d2b = b * 2.0 * copysign(1.0, d2) * dsg[k3];
            } else {
              d1b = b * 2.0 * copysign(1.0, d1) * dsg[k3];
            }
          }
          dd1[j] = d1b;
          ddm[j] = d2b - d1b;
          dd2[j] = -d2b;
        }
      }
    }
    __syncwarp();
    // cell means: gather the A cotangents (with the mirrored ghost cells)
    double qb[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int k = l0 + k3;
        double ab = acm[k] + aid[k] + aim[k + 1] + dd1[k] + ddm[k + 1] + dd2[k + 2];
        if (k == 0) ab += aim[0] + ddm[0] + dd2[1];               // A[-1] = A[0]
        if (k == 1) ab += dd2[0];                                  // A[-2] = A[1]
        if (k == NLEV - 1) ab += aid[NLEV] + dd1[NLEV] + ddm[NLEV + 1];  // A[72] = A[71]
        if (k == NLEV - 2) ab += dd1[NLEV + 1];                    // A[73] = A[70]
        qb[k3] = ab * rD[k];
        Dbo[k3] -= ab * A[k] * rD[k];
      }
    }
    // mass[k + 1] = sum_{j<k} q_j  =>  qb_j += sum_{kk > j} mbc[kk]
    {
      double acc = warp_excl_suffix(mbc[0] + mbc[1] + mbc[2], lane);
#pragma unroll
      for (int k3 = 2; k3 >= 0; --k3) {
        qb[k3] += acc;
        acc += mbc[k3];
      }
    }
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int k = l0 + k3;
        srcb[k3] += qb[k3] * x[k3];
        const double xin = qb[k3] * s3[k3];
        if (var < 2) bv[(size_t)k * 32 + var * 16] = xin;
        else bT[(size_t)k * 16] = xin;
      }
    }
    __syncwarp();
  }
  // ---- grid reversed ----
  double* gm2 = sm + V_GM2;
  double* gm1 = sm + V_GM1;
  double* g0a = sm + V_G0;
  double* gp1 = sm + V_GP1;
  if (lane < 25) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int j = 3 * lane + k3;
      if (j < NLEV + 2) {
        const double a_ = D[j - 2], b_ = D[j - 1], c_ = D[j];
        double cm2 = 0.0, cm1 = 0.0, c0 = 0.0, cp1 = 0.0;
        // the reciprocals of the forward's weight denominators
        float rf;
        const double r3 = rcp_newton(a_ + b_ + c_, rf), r10 = rcp_newton(b_ + c_, rf),
                     r2 = rcp_newton(a_ + b_, rf);
        double v = gb[k3][0];  // b / (a + b + c)
        {
          const double sb = -v * g[0 * 74 + j] * r3;
          cm1 += v * r3 + sb;
          cm2 += sb;
          c0 += sb;
        }
        v = gb[k3][1];  // (2a + b) / (b + c)
        {
          const double nb = v * r10, sb = -nb * g[1 * 74 + j];
          cm2 += 2.0 * nb;
          cm1 += nb + sb;
          c0 += sb;
        }
        v = gb[k3][2];  // (b + 2c) / (a + b)
        {
          const double nb = v * r2, sb = -nb * g[2 * 74 + j];
          cm1 += nb + sb;
          c0 += 2.0 * nb;
          cm2 += sb;
        }
        if (j < NLEV + 1) {
          const double d_ = D[j + 1];
          const double r6 = rcp_newton(2.0 * b_ + c_, rf), r7 = rcp_newton(2.0 * c_ + b_, rf);
          v = gb[k3][3];  // b / (b + c)
          {
            const double nb = v * r10, sb = -nb * g[3 * 74 + j];
            cm1 += nb + sb;
            c0 += sb;
          }
          v = gb[k3][4];  // 1 / (a + b + c + d)
          {
            const double sb = -v * g[4 * 74 + j] * g[4 * 74 + j];
            cm2 += sb;
            cm1 += sb;
            c0 += sb;
            cp1 += sb;
          }
          v = gb[k3][5];  // 2 b c / (b + c)
          {
            const double nb = v * r10, sb = -nb * g[5 * 74 + j];
            cm1 += 2.0 * c_ * nb + sb;
            c0 += 2.0 * b_ * nb + sb;
          }
          v = gb[k3][6];  // (a + b) / (2b + c)
          {
            const double nb = v * r6, sb = -nb * g[6 * 74 + j];
            cm2 += nb;
            cm1 += nb + 2.0 * sb;
            c0 += sb;
          }
          v = gb[k3][7];  // (d + c) / (2c + b)
          {
            const double nb = v * r7, sb = -nb * g[7 * 74 + j];
            cp1 += nb;
            c0 += nb + 2.0 * sb;
            cm1 += sb;
          }
          v = gb[k3][8];  // b (a + b) / (2b + c)
          {
            const double nb = v * r6, sb = -nb * g[8 * 74 + j];
            cm2 += b_ * nb;
            cm1 += (a_ + 2.0 * b_) * nb + 2.0 * sb;
            c0 += sb;
          }
          v = gb[k3][9];  // c (c + d) / (b + 2c)
          {
            const double nb = v * r7, sb = -nb * g[9 * 74 + j];
            c0 += (2.0 * c_ + d_) * nb + 2.0 * sb;
            cp1 += c_ * nb;
            cm1 += sb;
          }
        }
        gm2[j] = cm2;
        gm1[j] = cm1;
        g0a[j] = c0;
        gp1[j] = cp1;  // zero for j = 73
      }
    }
  }
  __syncwarp();
  // D cotangent per cell (with the mirrored ghost thicknesses), pio / pin suffix sums
  double w3[3] = {0.0, 0.0, 0.0}, u3[3] = {0.0, 0.0, 0.0};
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int k = l0 + k3;
      double db = Dbo[k3] + g0a[k] + gm1[k + 1] + gm2[k + 2] + (k >= 1 ? gp1[k - 1] : 0.0);
      if (k == 0) db += gm1[0] + gm2[1];                          // D[-1] = D[0]
      if (k == 1) db += gm2[0];                                   // D[-2] = D[1]
      if (k == NLEV - 1) db += g0a[NLEV] + gm1[NLEV + 1] + gp1[NLEV - 1];  // D[72] = D[71]
      if (k == NLEV - 2) db += g0a[NLEV + 1] + gp1[NLEV];         // D[73] = D[70]
      srcb[k3] += db;
      // pio_b[k+1] = (z2 of cell k+1) + (z2 of cell k, upper end) [+ pin_b[72] at the bottom]
      w3[k3] = (k + 1 < NLEV ? piol[k + 1] : 0.0) + pioh[k3] + (k == NLEV - 1 ? pinb[NLEV] : 0.0);
      u3[k3] = k + 1 < NLEV ? pinb[k + 1] : 0.0;
    }
  }
  {
    double ws = warp_excl_suffix(w3[0] + w3[1] + w3[2], lane);
    double us = warp_excl_suffix(u3[0] + u3[1] + u3[2], lane);
#pragma unroll
    for (int k3 = 2; k3 >= 0; --k3) {
      ws += w3[k3];
      us += u3[k3];
      srcb[k3] += ws;  // src_b[j] += sum_{k>j} pio_b[k]
      tgtb[k3] += us;  // tgt_b[j] += sum_{j<k<72} pin_b[k]
    }
  }
  double psb = 0.0;
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) psb += (c_hybi[l0 + k3 + 1] - c_hybi[l0 + k3]) * tgtb[k3];
  }
  psb = warp_sum(psb);
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) bd[(size_t)(l0 + k3) * 16] = srcb[k3] + psb;
  }
}

template <typename R> constexpr int LG_ADJ() { return 8; }

}  // namespace

void upload_adjoint_constants(const double* dvv16, const double* hyai, const double* hybi,
                              cudaStream_t s) {
  float f[16];
  for (int i = 0; i < 16; ++i) f[i] = (float)dvv16[i];
  double ad[NLEV], bd[NLEV];
  for (int l = 0; l < NLEV; ++l) {
    ad[l] = hyai[l + 1] - hyai[l];
    bd[l] = hybi[l + 1] - hybi[l];
  }
  cudaMemcpyToSymbolAsync(c_dvv, dvv16, sizeof(double) * 16, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_dvvf, f, sizeof(float) * 16, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_hyai, hyai, sizeof(double) * (NLEV + 1), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_hybi, hybi, sizeof(double) * (NLEV + 1), 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_ai_delta, ad, sizeof(double) * NLEV, 0, cudaMemcpyHostToDevice, s);
  cudaMemcpyToSymbolAsync(c_bi_delta, bd, sizeof(double) * NLEV, 0, cudaMemcpyHostToDevice, s);
}

template <typename R>
void launch_caar_vjp(const CaarVjpArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_ADJ<R>();
  const size_t smem = caar_vjp_smem<R>();
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_caar_vjp<R, LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    init = true;
  }
  KScope k("caar_vjp", s);
  k_caar_vjp<R, LG><<<E, LG * 16, smem, s>>>(a);
}

template <typename R>
void launch_hv_vjp(const HvVjpArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = LG_ADJ<R>();
  {
    KScope k("hv_vjp_update", s);
    k_hvb_update<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, a.x, a.xo, a.a, a.xb, a.pre,
                                                                      a.m.rspheremp_d, a.dt);
  }
  {
    KScope k("hv_vjp_second", s);
    k_hvb_second<R, LG><<<E, LG * 16, 0, s>>>(a);
  }
  {
    KScope k("hv_vjp_first", s);
    k_hvb_first<R, LG><<<E, LG * 16, 0, s>>>(a);
  }
}

void launch_remap_vjp(const RemapVjpArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)VC * V_COL * sizeof(double);
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_remap_vjp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    init = true;
  }
  KScope k("remap_vjp", s);
  k_remap_vjp<<<(a.nelem * 16 + VC - 1) / VC, VC * 32, smem, s>>>(a);
}

void launch_rk5_comb_vjp(int E, DynV by, DynV b1, DynV b0, cudaStream_t s) {
  KScope k("rk5_comb_vjp", s);
  k_rk5_comb_vjp<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, by, b1, b0);
}

void launch_copy_dyn(int E, DynV dst, DynV src, cudaStream_t s) {
  KScope k("copy_state", s);
  k_copy_dyn<<<nblk((long long)E * NLEV * 16, 256), 256, 0, s>>>(E, dst, src);
}

#define HX_ADJ_INST(R)                                                              \
  template void launch_caar_vjp<R>(const CaarVjpArgs<R>&, int, cudaStream_t);       \
  template void launch_hv_vjp<R>(const HvVjpArgs<R>&, int, cudaStream_t);
HX_ADJ_INST(double)
HX_ADJ_INST(float)

}  // namespace hx
