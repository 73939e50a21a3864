// hx_tangent.cu — tangent-linear model (Jacobian-vector product) kernels of the dry
// dynamics step, the forward-mode companions of the adjoint in hx_adjoint.cu: Caar RK
// stage, hyperviscosity state update, PPM remap.
//
// A tangent kernel reads the primal input of its stage and the tangent of that input
// and writes the tangent of the stage's output; the forward kernel of hx_kernels.cu,
// launched after it on the same stream, then advances the primal.
//   * The sphere operators are linear: the tangent of an operator is the operator of
//     the tangent.  So is the DSS with rspheremp: the tangent of a Caar stage's
//     pre-DSS output goes through the forward DSS kernel.
//   * The vertical scans (pressure, geopotential, omega integral) are linear: their
//     tangent scans run beside the primal ones in double, with the same segmentation.
//   * The hyperviscosity Laplacians, the sponge and the dp3d term are linear, so the
//     forward Laplacian kernels run on the tangent as they are; the state update's
//     heating term, the one product of the subcycle, has its own kernel here.
//   * PPM remap: the primal recomputation follows the forward kernel's arithmetic
//     (reciprocals, compares on the integer pipe), so every slope and parabola limiter
//     branch and the index search are the forward's; the tangent follows the branch
//     taken, and the grid weights, the integral bounds and the target thickness carry
//     tangents of their own.
// The forward this linearises restates src/share/cxx/CaarFunctorImpl.hpp:97-889,
// SphereOperators.hpp:291-862, HyperviscosityFunctorImpl.hpp:134-158 and
// RemapFunctor.hpp:225-463 with PpmRemap.hpp:174-689.
#include "hx_device.cuh"

namespace hx {
namespace {

// ======================================================================================
// Caar RK stage, one CTA per element (the layout of k_caar): primal and tangent of
// div(v dp), pressure, geopotential and the omega integral in shared memory, then the
// tangent of the pre-DSS update level by level.
// ======================================================================================
template <typename R, int LG>
__global__ void __launch_bounds__(LG * 16) k_caar_jvp(CaarJvpArgs<R> a) {
  constexpr int NL = NLEV / LG;
  extern __shared__ double sm[];
  double* s_dp = sm;                      // dp3d, then phi
  double* s_div = sm + 1 * NLEV * SROW;   // div(v dp)
  double* s_p = sm + 2 * NLEV * SROW;     // pressure
  double* s_om = sm + 3 * NLEV * SROW;    // sum_{j<l} div(v dp)_j
  double* d_dp = sm + 4 * NLEV * SROW;    // their tangents
  double* d_div = sm + 5 * NLEV * SROW;
  double* d_p = sm + 6 * NLEV * SROW;
  double* d_om = sm + 7 * NLEV * SROW;
  const int e = blockIdx.x, tid = threadIdx.x, p = tid & 15, lg = tid >> 4;
  Pt<R> t;
  t.init(p);
  PM<R> m;
  m.load(a.m, e, p);
  const size_t vN0 = ((size_t)e * NTL + a.n0) * NLEV * 32;
  const size_t sN0 = ((size_t)e * NTL + a.n0) * NLEV * 16;
  // ---- phase A: div(v dp) and its tangent div(dv dp + v ddp) ----
#pragma unroll 1
  for (int k = 0; k < NL; ++k) {
    const int l = lg + LG * k;
    const R u = cvt_hw<R>(a.v[vN0 + l * 32 + p]), w = cvt_hw<R>(a.v[vN0 + l * 32 + 16 + p]);
    const R du = cvt_hw<R>(a.tv[vN0 + l * 32 + p]), dw = cvt_hw<R>(a.tv[vN0 + l * 32 + 16 + p]);
    const double dd = a.dp[sN0 + l * 16 + p], ddd = a.tdp[sN0 + l * 16 + p];
    const R d = cvt_hw<R>(dd), dD = cvt_hw<R>(ddd);
    const R div = divergence_sphere(t, m, u * d, w * d);
    const R ddiv = divergence_sphere(t, m, du * d + u * dD, dw * d + w * dD);
    s_dp[l * SROW + p] = dd;
    d_dp[l * SROW + p] = ddd;
    s_div[l * SROW + p] = dbl_hw(div);
    d_div[l * SROW + p] = dbl_hw(ddiv);
  }
  __syncthreads();
  // ---- phase B: the column scans and their tangents (double) ----
  if (tid < 128) {
    const int col = tid >> 3, seg = tid & 7, l0 = seg * 9;
    double prev = seg == 0 ? 0.0 : s_dp[(l0 - 1) * SROW + col];
    double dprev = seg == 0 ? 0.0 : d_dp[(l0 - 1) * SROW + col];
    double tot = 0.0, dtot = 0.0, tp[9], dtp[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double d = s_dp[(l0 + k) * SROW + col], dd = d_dp[(l0 + k) * SROW + col];
      tp[k] = 0.5 * (prev + d);
      dtp[k] = 0.5 * (dprev + dd);
      tot += tp[k];
      dtot += dtp[k];
      prev = d;
      dprev = dd;
    }
    double pr = a.p_top + seg_excl_prefix(tot, seg);
    double dpr = seg_excl_prefix(dtot, seg);
    double r[9], dr[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const int l = l0 + k;
      const double d = s_dp[l * SROW + col], dd = d_dp[l * SROW + col];
      pr = pr + tp[k];
      dpr = dpr + dtp[k];
      s_p[l * SROW + col] = pr;
      d_p[l * SROW + col] = dpr;
      const double rp = 1.0 / pr, drp = -dpr * rp * rp;
      // r = Rgas T dp / (2 p) (dry: T_v = T)
      const double Tl = a.T[sN0 + l * 16 + col], dTl = a.tT[sN0 + l * 16 + col];
      const double h = d * 0.5 * rp, dh = 0.5 * (dd * rp + d * drp);
      r[k] = kRgas * Tl * h;
      dr[k] = kRgas * (dTl * h + Tl * dh);
    }
    // geopotential: phi_k = phis + 2 sum_{j>k} r_j + r_k (phis has no tangent)
    double rt = 0.0, drt = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      rt += r[k];
      drt += dr[k];
    }
    double integ = seg_excl_suffix(rt, seg), dinteg = seg_excl_suffix(drt, seg);
    const double phis = dbl_hw(a.m.phis[(size_t)e * 16 + col]);
#pragma unroll
    for (int k = 8; k >= 0; --k) {
      s_dp[(l0 + k) * SROW + col] = phis + 2.0 * integ + r[k];
      d_dp[(l0 + k) * SROW + col] = 2.0 * dinteg + dr[k];
      integ = integ + r[k];
      dinteg = dinteg + dr[k];
    }
    // omega integral: exclusive prefix of div(v dp)
    double st = 0.0, dst = 0.0;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      st += s_div[(l0 + k) * SROW + col];
      dst += d_div[(l0 + k) * SROW + col];
    }
    double acc = seg_excl_prefix(st, seg), dacc = seg_excl_prefix(dst, seg);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      s_om[(l0 + k) * SROW + col] = acc;
      d_om[(l0 + k) * SROW + col] = dacc;
      acc = acc + s_div[(l0 + k) * SROW + col];
      dacc = dacc + d_div[(l0 + k) * SROW + col];
    }
  }
  __syncthreads();
  // ---- phase C: tangents of omega, T, v, dp3d at np1 (pre-DSS) ----
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
    const R u = cvt_hw<R>(a.v[vN0 + l * 32 + p]), w = cvt_hw<R>(a.v[vN0 + l * 32 + 16 + p]);
    const R du = cvt_hw<R>(a.tv[vN0 + l * 32 + p]), dw = cvt_hw<R>(a.tv[vN0 + l * 32 + 16 + p]);
    const double pd = s_p[l * SROW + p], dpd = d_p[l * SROW + p];
    const double rpd = 1.0 / pd;
    const R rp = cvt_hw<R>(rpd), drp = cvt_hw<R>(-dpd * rpd * rpd);
    R gp0, gp1, dgp0, dgp1;
    gradient_sphere(t, m, rel_hw<R>(pd), gp0, gp1);
    gradient_sphere(t, m, rel_hw<R>(dpd), dgp0, dgp1);
    const R div = cvt_hw<R>(s_div[l * SROW + p]), ddiv = cvt_hw<R>(d_div[l * SROW + p]);
    const R vgp = u * gp0 + w * gp1;
    const R dvgp = (du * gp0 + u * dgp0) + (dw * gp1 + w * dgp1);
    const R oin = cvt_hw<R>(s_om[l * SROW + p]) + R(0.5) * div;
    const R doin = cvt_hw<R>(d_om[l * SROW + p]) + R(0.5) * ddiv;
    const R omega = (vgp - oin) * rp;
    const R domega = (dvgp - doin) * rp + (vgp - oin) * drp;
    // tangent of the base level "nm1" (RK combine of stage 5 applied here too)
    double dtm = a.tT[sM + l * 16 + p], ddm = a.tdp[sM + l * 16 + p];
    double dvm0 = a.tv[vM + l * 32 + p], dvm1 = a.tv[vM + l * 32 + 16 + p];
    if (a.rk_combine) {
      dtm = (5.0 * dtm - a.tT[sO + l * 16 + p]) / 4.0;
      ddm = (5.0 * ddm - a.tdp[sO + l * 16 + p]) / 4.0;
      dvm0 = (5.0 * dvm0 - a.tv[vO + l * 32 + p]) / 4.0;
      dvm1 = (5.0 * dvm1 - a.tv[vO + l * 32 + 16 + p]) / 4.0;
      a.tT[sM + l * 16 + p] = dtm;
      a.tdp[sM + l * 16 + p] = ddm;
      a.tv[vM + l * 32 + p] = dvm0;
      a.tv[vM + l * 32 + 16 + p] = dvm1;
    }
    // temperature: F_T = -(v . grad T) + kappa T omega
    const double td = a.T[sN0 + l * 16 + p], dtd = a.tT[sN0 + l * 16 + p];
    R gt0, gt1, dgt0, dgt1;
    gradient_sphere(t, m, rel_hw<R>(td), gt0, gt1);
    gradient_sphere(t, m, rel_hw<R>(dtd), dgt0, dgt1);
    const R T = cvt_hw<R>(td), dT = cvt_hw<R>(dtd);
    const R dvgt = (du * gt0 + u * dgt0) + (dw * gt1 + w * dgt1);
    const R dttens = -dvgt + R(kKappa) * (dT * omega + T * domega);
    // velocity: F_v = -(R T / p) grad p - grad(KE + phi) +- v x (zeta + f)
    const R rr = R(kRgas) * (T * rp), drr = R(kRgas) * (dT * rp + T * drp);
    R dge0, dge1;
    gradient_sphere(t, m, (u * du + w * dw) + rel_hw<R>(d_dp[l * SROW + p]), dge0, dge1);
    R deg0 = (drr * gp0 + rr * dgp0) + dge0, deg1 = (drr * gp1 + rr * dgp1) + dge1;
    const R vort = vorticity_sphere(t, m, u, w) + fcor;
    const R dvort = vorticity_sphere(t, m, du, dw);
    deg0 = -deg0 + (dw * vort + w * dvort);
    deg1 = -deg1 - (du * vort + u * dvort);
    out[l * 64 + p] = spd * (dbl_hw(deg0 * dt) + dvm0);
    out[l * 64 + 16 + p] = spd * (dbl_hw(deg1 * dt) + dvm1);
    out[l * 64 + 32 + p] = spd * (dbl_hw(dttens * dt) + dtm);
    out[l * 64 + 48 + p] = spd * (ddm - dbl_hw(ddiv * dt));
  }
}

// ======================================================================================
// Hyperviscosity state update (the DSS and TagUpdateStates of k_hv_update) with the
// heating term linearised: T += dt tt rsmp - (vt . v_new) / cp with v_new = v + vt,
// so d(heating) = dvt . v_new + vt . (dv + dvt).  Grid (E, 9), 128 threads.
// ======================================================================================
template <typename R>
__global__ void __launch_bounds__(128) k_hv_update_jvp(HvJvpArgs<R> a) {
  int lo, p;
  dss_thread_point(lo, p);
  const int e = blockIdx.x, l = blockIdx.y * 8 + lo;
  const double rsd = a.m.rspheremp_d[e * 16 + p];
  const R rs = cvt<R>(rsd);
  const R dt = R(a.dt);
  const size_t vb = (((size_t)e * NTL + a.np1) * NLEV + l) * 32 + p;
  const size_t sb = (((size_t)e * NTL + a.np1) * NLEV + l) * 16 + p;
  // primal velocity increment and updated velocity, as k_hv_update computes them
  R vt0 = cvt<R>(dss_gather(a.bufB, NLEV * 64, 64, e, l, p, a.dss));
  R vt1 = cvt<R>(dss_gather(a.bufB + 16, NLEV * 64, 64, e, l, p, a.dss));
  vt0 = dt * vt0 * rs;
  vt1 = dt * vt1 * rs;
  const double v0 = a.v[vb] + dbl(vt0), v1 = a.v[vb + 16] + dbl(vt1);
  // tangents
  R dvt0 = cvt<R>(dss_gather(a.tbufB, NLEV * 64, 64, e, l, p, a.dss));
  R dvt1 = cvt<R>(dss_gather(a.tbufB + 16, NLEV * 64, 64, e, l, p, a.dss));
  R dtt = cvt<R>(dss_gather(a.tbufB + 32, NLEV * 64, 64, e, l, p, a.dss));
  const double ddpt = dss_gather(a.tbufB + 48, NLEV * 64, 64, e, l, p, a.dss);
  dvt0 = dt * dvt0 * rs;
  dvt1 = dt * dvt1 * rs;
  dtt = dt * dtt * rs;
  const double dv0 = a.tv[vb] + dbl(dvt0), dv1 = a.tv[vb + 16] + dbl(dvt1);
  a.tv[vb] = dv0;
  a.tv[vb + 16] = dv1;
  const R dheat = (dvt0 * cvt<R>(v0) + dvt1 * cvt<R>(v1)) + (vt0 * cvt<R>(dv0) + vt1 * cvt<R>(dv1));
  a.tT[sb] = a.tT[sb] + dbl(dtt - dheat * R(1.0 / kCp));
  a.tdp[sb] = ddpt * rsd;
}

// ======================================================================================
// PPM remap of v and T (rsplit > 0) with tangents, one warp per column: lane L owns
// levels 3L .. 3L+2 (L < 24) and grid interfaces j = 3L .. 3L+2 (L < 25), as k_remap.
// The tangent of ps_v (the sum of the source thicknesses) is written for the dp3d
// reset that follows the remap.
// ======================================================================================
constexpr int JC = 4;  // columns (warps) per CTA
// shared-memory slots of one column (doubles): primal, then tangents
constexpr int J_D = 0;                // D[-2 .. 73]
constexpr int J_RD = J_D + 76;        // 1 / D[0 .. 71]
constexpr int J_PIO = J_RD + 72;      // pio[0 .. 73]
constexpr int J_PIN = J_PIO + 74;     // pin[0 .. 72]
constexpr int J_KID = J_PIN + 74;     // kid[0 .. 71] (int)
constexpr int J_G = J_KID + 36;       // g[10][74] (rows 6 and 7 unused, row 5 = g5 (g6 - g7))
constexpr int J_A = J_G + 740;        // A[-2 .. 73]
constexpr int J_MASS = J_A + 76;      // mass[0 .. 72]
constexpr int J_DMA = J_MASS + 74;    // dma[0 .. 73]
constexpr int J_AI = J_DMA + 74;      // ai[0 .. 72]
constexpr int J_COEF = J_AI + 74;     // coef[3][72]
constexpr int J_TD = J_COEF + 216;    // tangents of D, pio, pin, g, A, mass, dma, ai, coef
constexpr int J_TPIO = J_TD + 76;
constexpr int J_TPIN = J_TPIO + 74;
constexpr int J_TG = J_TPIN + 74;
constexpr int J_TA = J_TG + 740;
constexpr int J_TMASS = J_TA + 76;
constexpr int J_TDMA = J_TMASS + 74;
constexpr int J_TAI = J_TDMA + 74;
constexpr int J_TCOEF = J_TAI + 74;
constexpr int J_COL = J_TCOEF + 216;  // doubles per column

__device__ __forceinline__ double sgn(double x) { return x < 0.0 ? -1.0 : 1.0; }

__global__ void __launch_bounds__(JC * 32) k_remap_jvp(RemapJvpArgs a) {
  extern __shared__ double jsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cidx = blockIdx.x * JC + warp;
  if (cidx >= a.nelem * 16) return;  // whole warp leaves together; no CTA barriers below
  const int e = cidx >> 4, p = cidx & 15;
  double* sm = jsm + warp * J_COL;
  double* D = sm + J_D + 2;
  double* rD = sm + J_RD;
  double* pio = sm + J_PIO;
  double* pin = sm + J_PIN;
  int* kid = reinterpret_cast<int*>(sm + J_KID);
  double* g = sm + J_G;
  double* A = sm + J_A + 2;
  double* mass = sm + J_MASS;
  double* dma = sm + J_DMA;
  double* ai = sm + J_AI;
  double* coef = sm + J_COEF;
  double* tD = sm + J_TD + 2;
  double* tpio = sm + J_TPIO;
  double* tpin = sm + J_TPIN;
  double* tg = sm + J_TG;
  double* tA = sm + J_TA + 2;
  double* tmass = sm + J_TMASS;
  double* tdma = sm + J_TDMA;
  double* tai = sm + J_TAI;
  double* tcoef = sm + J_TCOEF;
  const bool own = lane < 24;
  const int l0 = 3 * lane;
  const size_t sb = ((size_t)e * NTL + a.np1) * NLEV * 16 + p;
  const size_t vb = ((size_t)e * NTL + a.np1) * NLEV * 32 + p;
  // source thickness, surface pressure, target thickness
  double s3[3] = {0.0, 0.0, 0.0}, ds3[3] = {0.0, 0.0, 0.0};
  if (own) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      s3[k] = a.dp[sb + (size_t)(l0 + k) * 16];
      ds3[k] = a.tdp[sb + (size_t)(l0 + k) * 16];
    }
  }
  const double ps = warp_sum(s3[0] + s3[1] + s3[2]) + a.hyai0 * a.ps0;
  const double dps = warp_sum(ds3[0] + ds3[1] + ds3[2]);
  if (lane == 0) a.tps[((size_t)e * NTL + a.np1) * 16 + p] = dps;
  double t3[3] = {0.0, 0.0, 0.0}, dt3[3] = {0.0, 0.0, 0.0}, rt3[3] = {0.0, 0.0, 0.0};
  if (own) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int l = l0 + k;
      const double db = c_hybi[l + 1] - c_hybi[l];
      t3[k] = (c_hyai[l + 1] - c_hyai[l]) * a.ps0 + db * ps;
      dt3[k] = db * dps;
      float rf;
      rt3[k] = rcp_newton(t3[k], rf);
      D[l] = s3[k];
      tD[l] = ds3[k];
      rD[l] = rcp_newton(s3[k], rf);
    }
  }
  // cumulative source and target thickness
  {
    double ex = warp_excl_scan(s3[0] + s3[1] + s3[2], lane);
    double ey = warp_excl_scan(t3[0] + t3[1] + t3[2], lane);
    double dex = warp_excl_scan(ds3[0] + ds3[1] + ds3[2], lane);
    double dey = warp_excl_scan(dt3[0] + dt3[1] + dt3[2], lane);
    if (own) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pio[l0 + k] = ex;
        pin[l0 + k] = ey;
        tpio[l0 + k] = dex;
        tpin[l0 + k] = dey;
        ex += s3[k];
        ey += t3[k];
        dex += ds3[k];
        dey += dt3[k];
      }
    }
    if (lane == 23) {
      pio[NLEV] = ex;
      pio[NLEV + 1] = ex + 1.0;
      pin[NLEV] = ex;
      tpio[NLEV] = dex;
      tpio[NLEV + 1] = dex;
      tpin[NLEV] = dex;
    }
  }
  __syncwarp();
  if (lane == 0) {
    D[-1] = D[0];
    D[-2] = D[1];
    D[NLEV] = D[NLEV - 1];
    D[NLEV + 1] = D[NLEV - 2];
    tD[-1] = tD[0];
    tD[-2] = tD[1];
    tD[NLEV] = tD[NLEV - 1];
    tD[NLEV + 1] = tD[NLEV - 2];
  }
  __syncwarp();
  // integral bounds: the index search is the forward's; z2 and its tangent
  double z2[3] = {0.0, 0.0, 0.0}, dz2[3] = {0.0, 0.0, 0.0};
  if (own) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int k = l0 + k3;
      int kk = k + 1;
      while (kk < NLEV + 2 && pio[kk - 1] <= pin[k + 1]) kk++;
      kk--;
      if (kk == NLEV + 1) kk = NLEV;
      if (kk < 1) kk = 1;  // only with a non-monotone source grid, which the forward flags
      kid[k] = kk - 1;
      const double num = pin[k + 1] - (pio[kk - 1] + pio[kk]) * 0.5;
      const double dnum = tpin[k + 1] - (tpio[kk - 1] + tpio[kk]) * 0.5;
      z2[k3] = num * rD[kk - 1];
      dz2[k3] = (dnum - z2[k3] * tD[kk - 1]) * rD[kk - 1];
    }
  }
  // grid weights (the forward's reciprocals) and their tangents by the quotient rule
  if (lane < 25) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3) {
      const int j = 3 * lane + k3;
      if (j < NLEV + 2) {
        const double dm2 = D[j - 2], dm1 = D[j - 1], d0 = D[j];
        const double em2 = tD[j - 2], em1 = tD[j - 1], e0 = tD[j];
        float rf;
        const double r10 = rcp_newton(dm1 + d0, rf);
        const double r3 = rcp_newton(dm2 + dm1 + d0, rf);
        const double r2 = rcp_newton(dm2 + dm1, rf);
        const double g0 = dm1 * r3, g1 = (2.0 * dm2 + dm1) * r10, g2 = (dm1 + 2.0 * d0) * r2;
        g[0 * 74 + j] = g0;
        g[1 * 74 + j] = g1;
        g[2 * 74 + j] = g2;
        tg[0 * 74 + j] = (em1 - g0 * (em2 + em1 + e0)) * r3;
        tg[1 * 74 + j] = ((2.0 * em2 + em1) - g1 * (em1 + e0)) * r10;
        tg[2 * 74 + j] = ((em1 + 2.0 * e0) - g2 * (em2 + em1)) * r2;
        if (j < NLEV + 1) {
          const double dp1 = D[j + 1], ep1 = tD[j + 1];
          const double r6 = rcp_newton(2.0 * dm1 + d0, rf);
          const double r7 = rcp_newton(2.0 * d0 + dm1, rf);
          const double g3 = dm1 * r10;
          const double g4 = rcp_newton(dm2 + dm1 + d0 + dp1, rf);
          const double a5 = (2.0 * dm1 * d0) * r10;
          const double g6 = (dm2 + dm1) * r6, g7 = (dp1 + d0) * r7;
          g[3 * 74 + j] = g3;
          g[4 * 74 + j] = g4;
          g[5 * 74 + j] = a5 * ((dm2 + dm1) * r6 - (dp1 + d0) * r7);
          g[8 * 74 + j] = dm1 * (dm2 + dm1) * r6;
          g[9 * 74 + j] = d0 * (d0 + dp1) * r7;
          const double ta5 = (2.0 * (em1 * d0 + dm1 * e0) - a5 * (em1 + e0)) * r10;
          const double tg6 = ((em2 + em1) - g6 * (2.0 * em1 + e0)) * r6;
          const double tg7 = ((ep1 + e0) - g7 * (2.0 * e0 + em1)) * r7;
          tg[3 * 74 + j] = (em1 - g3 * (em1 + e0)) * r10;
          tg[4 * 74 + j] = -g4 * g4 * (em2 + em1 + e0 + ep1);
          tg[5 * 74 + j] = ta5 * (g6 - g7) + a5 * (tg6 - tg7);
          tg[8 * 74 + j] = em1 * g6 + dm1 * tg6;
          tg[9 * 74 + j] = e0 * g7 + d0 * tg7;
        }
      }
    }
  }
  __syncwarp();
  // partial-cell integral weights of this lane's target levels and their tangents
  double wz[3][3], dwz[3][3];
#pragma unroll
  for (int k3 = 0; k3 < 3; ++k3) {
    const double x2 = z2[k3], dx = dz2[k3];
    wz[k3][0] = x2 + 0.5;
    wz[k3][1] = (x2 * x2 - 0.25) * 0.5;
    wz[k3][2] = (x2 * x2 * x2 + 0.125) * (1.0 / 3.0);
    dwz[k3][0] = dx;
    dwz[k3][1] = x2 * dx;
    dwz[k3][2] = x2 * x2 * dx;
  }
  constexpr double sixth = 1.0 / 6.0;
#pragma unroll 1
  for (int var = 0; var < 3; ++var) {
    // extrinsic values x dp, cell means, masses below each source interface
    double x3[3] = {0.0, 0.0, 0.0}, dx3[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int l = l0 + k;
        const size_t ix = var < 2 ? vb + (size_t)l * 32 + var * 16 : sb + (size_t)l * 16;
        const double x = var < 2 ? a.v[ix] : a.T[ix];
        const double dx = var < 2 ? a.tv[ix] : a.tT[ix];
        x3[k] = x * s3[k];
        dx3[k] = dx * s3[k] + x * ds3[k];
        A[l] = x3[k] * rD[l];
        tA[l] = (dx3[k] - A[l] * ds3[k]) * rD[l];
      }
    }
    {
      double ex = warp_excl_scan(x3[0] + x3[1] + x3[2], lane);
      double dex = warp_excl_scan(dx3[0] + dx3[1] + dx3[2], lane);
      if (own) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          mass[l0 + k + 1] = ex;
          tmass[l0 + k + 1] = dex;
          ex += x3[k];
          dex += dx3[k];
        }
      }
      if (lane == 0) {
        mass[0] = 0.0;
        tmass[0] = 0.0;
      }
    }
    __syncwarp();
    if (lane == 0) {  // ghost cells: mirrored (remap_alg 1, 2) or constant (3)
      const bool c3 = a.remap_alg == 3;
      A[-1] = A[0];
      A[-2] = c3 ? A[0] : A[1];
      A[NLEV] = A[NLEV - 1];
      A[NLEV + 1] = c3 ? A[NLEV - 1] : A[NLEV - 2];
      tA[-1] = tA[0];
      tA[-2] = c3 ? tA[0] : tA[1];
      tA[NLEV] = tA[NLEV - 1];
      tA[NLEV + 1] = c3 ? tA[NLEV - 1] : tA[NLEV - 2];
    }
    __syncwarp();
    // slopes: dma = sign(da) min(|da|, 2|A_{j-1} - A_{j-2}|, 2|A_j - A_{j-1}|) where the
    // differences have one sign; the tangent follows the first minimum in that order
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 2) {
          const double d1 = A[j] - A[j - 1], d2 = A[j - 1] - A[j - 2];
          const double e1 = tA[j] - tA[j - 1], e2 = tA[j - 1] - tA[j - 2];
          double r = 0.0, dr = 0.0;
          if (pos_prod(d1, d2)) {
            const double b = g[1 * 74 + j] * d1 + g[2 * 74 + j] * d2;
            const double db = tg[1 * 74 + j] * d1 + g[1 * 74 + j] * e1 + tg[2 * 74 + j] * d2 + g[2 * 74 + j] * e2;
            const double da = g[0 * 74 + j] * b;
            const double dda = tg[0 * 74 + j] * b + g[0 * 74 + j] * db;
            r = min3abs_signed(da, 2.0 * d2, 2.0 * d1, da);
            double mv = fabs(da);
            dr = dda;
            if (fabs(2.0 * d2) < mv) {
              mv = fabs(2.0 * d2);
              dr = sgn(da) * sgn(d2) * 2.0 * e2;
            }
            if (fabs(2.0 * d1) < mv) dr = sgn(da) * sgn(d1) * 2.0 * e1;
          }
          dma[j] = r;
          tdma[j] = dr;
        }
      }
    }
    __syncwarp();
    // edge values
    if (lane < 25) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int j = 3 * lane + k3;
        if (j < NLEV + 1) {
          const double d = A[j] - A[j - 1], ed = tA[j] - tA[j - 1];
          const double in = g[5 * 74 + j] * d - g[8 * 74 + j] * dma[j + 1] + g[9 * 74 + j] * dma[j];
          const double din = (tg[5 * 74 + j] * d + g[5 * 74 + j] * ed) -
                             (tg[8 * 74 + j] * dma[j + 1] + g[8 * 74 + j] * tdma[j + 1]) +
                             (tg[9 * 74 + j] * dma[j] + g[9 * 74 + j] * tdma[j]);
          ai[j] = A[j - 1] + g[3 * 74 + j] * d + g[4 * 74 + j] * in;
          tai[j] = tA[j - 1] + (tg[3 * 74 + j] * d + g[3 * 74 + j] * ed) +
                   (tg[4 * 74 + j] * in + g[4 * 74 + j] * din);
        }
      }
    }
    __syncwarp();
    // limited parabolas
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int jp = l0 + k3;
        double al = ai[jp], ar = ai[jp + 1], tal = tai[jp], tar = tai[jp + 1];
        const double cm = A[jp], tcm = tA[jp];
        if (!pos_prod(ar - cm, cm - al)) {
          al = cm;
          ar = cm;
          tal = tcm;
          tar = tcm;
        }
        if (less((ar - al) * (ar - al) * sixth, (ar - al) * (cm - (al + ar) * 0.5))) {
          al = 3.0 * cm - 2.0 * ar;
          tal = 3.0 * tcm - 2.0 * tar;
        }
        if (less((ar - al) * (cm - (al + ar) * 0.5), -(ar - al) * (ar - al) * sixth)) {
          ar = 3.0 * cm - 2.0 * al;
          tar = 3.0 * tcm - 2.0 * tal;
        }
        double c0 = 1.5 * cm - (al + ar) / 4.0, c1 = ar - al, c2 = 3.0 * (-2.0 * cm + (al + ar));
        double t0 = 1.5 * tcm - (tal + tar) / 4.0, t1 = tar - tal, t2 = 3.0 * (-2.0 * tcm + (tal + tar));
        if (a.remap_alg == 2 && (jp < 2 || jp >= NLEV - 2)) {  // PpmFixedParabola
          c0 = cm;
          c1 = 0.0;
          c2 = 0.0;
          t0 = tcm;
          t1 = 0.0;
          t2 = 0.0;
        }
        coef[jp] = c0;
        coef[72 + jp] = c1;
        coef[144 + jp] = c2;
        tcoef[jp] = t0;
        tcoef[72 + jp] = t1;
        tcoef[144 + jp] = t2;
      }
    }
    __syncwarp();
    // mass below each new interface; new cell values from consecutive differences
    double m2[3] = {0.0, 0.0, 0.0}, dm2[3] = {0.0, 0.0, 0.0};
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int kk = kid[l0 + k3];
        const double c0 = coef[kk], c1 = coef[72 + kk], c2 = coef[144 + kk];
        const double in = (c0 * wz[k3][0] + c1 * wz[k3][1]) + c2 * wz[k3][2];
        const double din = (tcoef[kk] * wz[k3][0] + c0 * dwz[k3][0]) + (tcoef[72 + kk] * wz[k3][1] + c1 * dwz[k3][1]) +
                           (tcoef[144 + kk] * wz[k3][2] + c2 * dwz[k3][2]);
        m2[k3] = mass[kk + 1] + in * D[kk];
        dm2[k3] = tmass[kk + 1] + din * D[kk] + in * tD[kk];
      }
    }
    double below = __shfl_up_sync(FULL, m2[2], 1), dbelow = __shfl_up_sync(FULL, dm2[2], 1);
    if (lane == 0) {
      below = 0.0;
      dbelow = 0.0;
    }
    if (own) {
#pragma unroll
      for (int k3 = 0; k3 < 3; ++k3) {
        const int k = l0 + k3;
        const double m1 = k3 == 0 ? below : m2[k3 - 1], dm1 = k3 == 0 ? dbelow : dm2[k3 - 1];
        const double xn = (m2[k3] - m1) * rt3[k3];
        const double dxn = ((dm2[k3] - dm1) - xn * dt3[k3]) * rt3[k3];
        if (var < 2) a.tv[vb + (size_t)k * 32 + var * 16] = dxn;
        else a.tT[sb + (size_t)k * 16] = dxn;
      }
    }
    __syncwarp();
  }
}

}  // namespace

template <typename R>
void launch_caar_jvp(const CaarJvpArgs<R>& a, int E, cudaStream_t s) {
  constexpr int LG = 8;
  const size_t smem = (size_t)8 * NLEV * SROW * sizeof(double);
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_caar_jvp<R, LG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    init = true;
  }
  KScope k("caar_jvp", s);
  k_caar_jvp<R, LG><<<E, LG * 16, smem, s>>>(a);
}

template <typename R>
void launch_hv_update_jvp(const HvJvpArgs<R>& a, int E, cudaStream_t s) {
  KScope k("hv_update_jvp", s);
  k_hv_update_jvp<R><<<dim3(E, NLEV / 8), 128, 0, s>>>(a);
}

void launch_remap_jvp(const RemapJvpArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)JC * J_COL * sizeof(double);
  static bool init = false;
  if (!init) {
    cudaFuncSetAttribute(k_remap_jvp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    init = true;
  }
  KScope k("remap_jvp", s);
  k_remap_jvp<<<(a.nelem * 16 + JC - 1) / JC, JC * 32, smem, s>>>(a);
}

void upload_tangent_constants(const double* dvv16, const double* hyai, const double* hybi,
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

template void launch_caar_jvp<double>(const CaarJvpArgs<double>&, int, cudaStream_t);
template void launch_caar_jvp<float>(const CaarJvpArgs<float>&, int, cudaStream_t);
template void launch_hv_update_jvp<double>(const HvJvpArgs<double>&, int, cudaStream_t);
template void launch_hv_update_jvp<float>(const HvJvpArgs<float>&, int, cudaStream_t);

}  // namespace hx
