// hx_device.cuh — device-side building blocks shared by the kernel translation units
// (hx_kernels.cu: the forward step; hx_adjoint.cu: its adjoint): constant-memory
// tables, the per-point metric, the half-warp sphere-operator contractions, the DSS
// gather, the column scans and the per-launch timing scope.  Each translation unit
// that includes this file has its own copy of the __constant__ tables and uploads it
// (upload_constants / upload_adjoint_constants).
#pragma once
#include "hx_kernels.cuh"

namespace hx {

// Per-kernel timing hooks (defined in hx_kernels.cu).
void kernel_enter(const char* name, cudaStream_t s);
void kernel_leave(const char* name, cudaStream_t s);

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SROW = 17;  // padded shared-memory row of 16 points

__constant__ double c_dvv[16];
__constant__ float c_dvvf[16];
__constant__ double c_hyai[NLEV + 1];
__constant__ double c_hybi[NLEV + 1];
__constant__ double c_ai_delta[NLEV];
__constant__ double c_bi_delta[NLEV];
__constant__ double c_rdp0[NLEV];  // 1 / reference layer thickness (hybrid coordinate at ps0)

template <typename R> __device__ __forceinline__ R dvv_at(int a, int b);
template <> __device__ __forceinline__ double dvv_at<double>(int a, int b) { return c_dvv[a * 4 + b]; }
template <> __device__ __forceinline__ float dvv_at<float>(int a, int b) { return c_dvvf[a * 4 + b]; }

template <typename R> __device__ __forceinline__ R sh16(R v, int src) {
  return __shfl_sync(FULL, v, src, 16);
}

template <typename R> __device__ __forceinline__ R rre() { return R(kRrearth); }

template <typename R> constexpr bool kF32 = sizeof(R) == 4;

// A double field value as operator input.  In the mixed form the value at point 0 of the
// same level and element is subtracted first (in double): the sphere operators annihilate
// constants, and the FP32 operand then carries the horizontal variation instead of the
// large mean (pressure, geopotential, temperature, layer thickness).  In the FP64 form the
// value is used as is, so the arithmetic follows the reference formulas.
template <typename R> __device__ __forceinline__ R rel(double x);

// Per-thread GLL point data: index, dvv rows/columns for the four contractions.
template <typename R>
struct Pt {
  int p, i, j;
  R dx[4], dy[4], tx[4], ty[4];
  __device__ __forceinline__ void init(int p_) {
    p = p_;
    i = p >> 2;
    j = p & 3;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dx[k] = dvv_at<R>(j, k);
      dy[k] = dvv_at<R>(i, k);
      tx[k] = dvv_at<R>(k, j);
      ty[k] = dvv_at<R>(k, i);
    }
  }
  // sum_k dvv[j][k] s(i,k)  — derivative along jgp (x1)
  __device__ __forceinline__ R ddx(R s) const {
    R a = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) a += dx[k] * sh16(s, 4 * i + k);
    return a;
  }
  // sum_k dvv[i][k] s(k,j)  — derivative along igp (x2)
  __device__ __forceinline__ R ddy(R s) const {
    R a = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) a += dy[k] * sh16(s, 4 * k + j);
    return a;
  }
  // ddx(s0) + ddy(s1) and ddx(s0) - ddy(s1) as one chain of eight multiply-adds
  __device__ __forceinline__ R dxy(R s0, R s1) const {
    R a = dx[0] * sh16(s0, 4 * i);
#pragma unroll
    for (int k = 1; k < 4; ++k) a += dx[k] * sh16(s0, 4 * i + k);
#pragma unroll
    for (int k = 0; k < 4; ++k) a += dy[k] * sh16(s1, 4 * k + j);
    return a;
  }
  // acc + ddx(s0) + ddy(s1), the same chain started from acc
  __device__ __forceinline__ R dxy_acc(R s0, R s1, R acc) const {
    R a = acc;
#pragma unroll
    for (int k = 0; k < 4; ++k) a += dx[k] * sh16(s0, 4 * i + k);
#pragma unroll
    for (int k = 0; k < 4; ++k) a += dy[k] * sh16(s1, 4 * k + j);
    return a;
  }
  // the derivative weights times a per-point factor (folds a scale of the result)
  __device__ __forceinline__ void scale(R f) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dx[k] *= f;
      dy[k] *= f;
    }
  }
  __device__ __forceinline__ R dxmy(R s0, R s1) const {
    R a = dx[0] * sh16(s0, 4 * i);
#pragma unroll
    for (int k = 1; k < 4; ++k) a += dx[k] * sh16(s0, 4 * i + k);
#pragma unroll
    for (int k = 0; k < 4; ++k) a -= dy[k] * sh16(s1, 4 * k + j);
    return a;
  }
  // sum_k w(i,k) dvv[k][j]  — weak-form row contraction
  __device__ __forceinline__ R wrow(R w) const {
    R a = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) a += sh16(w, 4 * i + k) * tx[k];
    return a;
  }
  // sum_k w(k,j) dvv[k][i]  — weak-form column contraction
  __device__ __forceinline__ R wcol(R w) const {
    R a = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) a += sh16(w, 4 * k + j) * ty[k];
    return a;
  }
};

// Metric of one GLL point of one element.
template <typename R>
struct PM {
  R di00, di01, di10, di11, d00, d01, d10, d11, md, fdiv, sp, mp, a00, a01, a10, a11, rsp;
  R gr00, gr01, gr10, gr11;  // Dinv * rrearth, for gradient_sphere
  R dm00, dm01, dm10, dm11;  // Dinv * metdet, for divergence_sphere
  R l00, l01, l10, l11;  // spheremp * (Dinv Dinv^T) * rrearth, for laplace_simple
  R e00, e01, e10, e11;  // D * rrearth, mp / metdet / rrearth and 2 spheremp rrearth^2, for
  R mpf, f2;             // vlaplace_sphere_wk_contra
  __device__ __forceinline__ void load(const MetricP<R>& m, int e, int p) {
    const R* Di = m.Dinv + (size_t)e * 64;
    const R* D = m.D + (size_t)e * 64;
    const R* Mi = m.metinv + (size_t)e * 64;
    di00 = Di[p]; di01 = Di[16 + p]; di10 = Di[32 + p]; di11 = Di[48 + p];
    gr00 = di00 * rre<R>(); gr01 = di01 * rre<R>(); gr10 = di10 * rre<R>(); gr11 = di11 * rre<R>();
    d00 = D[p]; d01 = D[16 + p]; d10 = D[32 + p]; d11 = D[48 + p];
    md = m.metdet[(size_t)e * 16 + p];
    fdiv = R(1.0) / md * rre<R>();
    sp = m.spheremp[(size_t)e * 16 + p];
    rsp = m.rspheremp[(size_t)e * 16 + p];
    mp = m.mp[(size_t)e * 16 + p];
    dm00 = di00 * md; dm01 = di01 * md; dm10 = di10 * md; dm11 = di11 * md;
    a00 = Mi[p] * md; a01 = Mi[16 + p] * md; a10 = Mi[32 + p] * md; a11 = Mi[48 + p] * md;
    // c = (Dinv^T-contraction of the Dinv-contraction): c_a = sum_b K_ab v_b with
    // K_ab = sum_c Dinv(c,a) Dinv(c,b) in the reference's C++ indices.
    l00 = sp * (di00 * di00 + di10 * di10) * rre<R>();
    l01 = sp * (di00 * di01 + di10 * di11) * rre<R>();
    l10 = sp * (di01 * di00 + di11 * di10) * rre<R>();
    l11 = sp * (di01 * di01 + di11 * di11) * rre<R>();
    e00 = d00 * rre<R>(); e01 = d01 * rre<R>(); e10 = d10 * rre<R>(); e11 = d11 * rre<R>();
    mpf = mp * fdiv;
    f2 = R(2) * sp * rre<R>() * rre<R>();
  }
};

// ---- sphere operators on one point-level (SphereOperators.hpp) ------------------------
// The 1/rearth of the derivatives is folded into the metric factors (m.gr = Dinv / a).
template <typename R>
__device__ __forceinline__ void gradient_sphere(const Pt<R>& t, const PM<R>& m, R s, R& g0, R& g1) {
  const R v0 = t.ddx(s), v1 = t.ddy(s);
  g0 = m.gr00 * v0 + m.gr01 * v1;
  g1 = m.gr10 * v0 + m.gr11 * v1;
}

// metdet folded into the metric factors (m.dm = Dinv metdet)
template <typename R>
__device__ __forceinline__ R divergence_sphere(const Pt<R>& t, const PM<R>& m, R v0, R v1) {
  const R gv0 = m.dm00 * v0 + m.dm10 * v1;
  const R gv1 = m.dm01 * v0 + m.dm11 * v1;
  return t.dxy(gv0, gv1) * m.fdiv;
}

template <typename R>
__device__ __forceinline__ R vorticity_sphere(const Pt<R>& t, const PM<R>& m, R v0, R v1) {
  const R c0 = m.d00 * v0 + m.d01 * v1;
  const R c1 = m.d10 * v0 + m.d11 * v1;
  return t.dxmy(c1, c0) * m.fdiv;
}

// divergence_sphere_wk of the vector (g0, g1)
template <typename R>
__device__ __forceinline__ R divergence_sphere_wk(const Pt<R>& t, const PM<R>& m, R g0, R g1) {
  const R w0 = m.sp * (m.di00 * g0 + m.di10 * g1);
  const R w1 = m.sp * (m.di01 * g0 + m.di11 * g1);
  return -(t.wrow(w0) + t.wcol(w1)) * rre<R>();
}

// laplace_simple = divergence_sphere_wk(gradient_sphere(s)).  The two metric
// transforms compose to Dinv Dinv^T = metinv, so the weak-form operands are
// spheremp metinv rrearth (d s/dx, d s/dy); m.l00/l01/l10/l11 hold that product.
template <typename R>
__device__ __forceinline__ R laplace_simple(const Pt<R>& t, const PM<R>& m, R s) {
  const R sx = t.ddx(s), sy = t.ddy(s);
  const R w0 = m.l00 * sx + m.l01 * sy;
  const R w1 = m.l10 * sx + m.l11 * sy;
  return -(t.wrow(w0) + t.wcol(w1)) * rre<R>();
}

// The weak Laplacian of the thread's point on one level.  FP64 form: the element's dense
// 16x16 matrix (laplace_simple applied to the unit vectors once at initialisation), row p
// in registers, the level's 16 inputs by shuffles: 16 DFMA instead of the contractions'
// 22 FP64 instructions.  transpose = true loads column p (the adjoint's L^T).  Mixed
// form: the contractions in FP32.
template <typename R>
struct LapOp {
  double w[kF32<R> ? 1 : 16];
  __device__ __forceinline__ void load(const MetricP<R>& mp, int e, int p, bool transpose = false) {
    if constexpr (!kF32<R>) {
      const double* L = mp.lapm + (size_t)e * 256;
#pragma unroll
      for (int q = 0; q < 16; ++q) w[q] = transpose ? L[q * 16 + p] : L[p * 16 + q];
    }
  }
  __device__ __forceinline__ R operator()(const Pt<R>& t, const PM<R>& m, R s) const {
    if constexpr (kF32<R>) {
      return laplace_simple(t, m, s);
    } else {
      double a = 0.0;
#pragma unroll
      for (int q = 0; q < 16; ++q) a = fma(w[q], sh16(s, q), a);
      return a;
    }
  }
};

template <typename R>
__device__ __forceinline__ R laplace_tensor(const Pt<R>& t, const PM<R>& m, const R* tv, R s) {
  R g0, g1;
  gradient_sphere(t, m, s, g0, g1);
  const R t0 = tv[0] * g0 + tv[2] * g1;
  const R t1 = tv[1] * g0 + tv[3] * g1;
  return divergence_sphere_wk(t, m, t0, t1);
}

// vlaplace_sphere_wk_contra (SphereOperators.hpp:816-862): grad_sphere_wk_testcov of the
// divergence (times nu_ratio when it applies) minus curl_sphere_wk_testcov of the
// vorticity, plus 2 spheremp v / rearth^2.  Factors are folded per point: mp times the
// divergence and the vorticity take mp / metdet / rearth (m.mpf), and the two weak
// operators' covariant results are combined before D / rearth (m.e) is applied once.
template <typename R>
__device__ __forceinline__ void vlaplace_contra(const Pt<R>& t, const PM<R>& m, R nu_ratio, R v0, R v1,
                                                R& l0, R& l1) {
  const R gv0 = m.dm00 * v0 + m.dm10 * v1;
  const R gv1 = m.dm01 * v0 + m.dm11 * v1;
  R w = t.dxy(gv0, gv1) * m.mpf;  // mp div
  if (nu_ratio > R(0) && nu_ratio != R(1)) w *= nu_ratio;
  const R c0 = m.d00 * v0 + m.d01 * v1;
  const R c1 = m.d10 * v0 + m.d11 * v1;
  const R wv = t.dxmy(c1, c0) * m.mpf;  // mp vort
  const R X = t.wrow(w), Y = t.wcol(w);
  // (grad_wk_testcov - curl_wk_testcov) in covariant components
  const R q0 = t.wcol(wv) - (m.a00 * X + m.a01 * Y);
  const R q1 = -(m.a10 * X + m.a11 * Y) - t.wrow(wv);
  l0 = m.f2 * v0 + (m.e00 * q0 + m.e10 * q1);
  l1 = m.f2 * v1 + (m.e01 * q0 + m.e11 * q1);
}

// vlaplace_sphere_wk_cartesian (SphereOperators.hpp:750-814); tv = tensorVisc[0..3],
// s2c = vec_sph2cart[2][3] of this point.
template <typename R>
__device__ __forceinline__ void vlaplace_cartesian(const Pt<R>& t, const PM<R>& m, const R* tv, const R* s2c,
                                                   R v0, R v1, R& l0, R& l1) {
  R lc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) lc[c] = laplace_tensor(t, m, tv, s2c[c] * v0 + s2c[3 + c] * v1);
  const R f = R(2) * m.sp * rre<R>() * rre<R>();
  l0 = s2c[0] * lc[0] + s2c[1] * lc[1] + s2c[2] * lc[2] + f * v0;
  l1 = s2c[3] * lc[0] + s2c[4] * lc[1] + s2c[5] * lc[2] + f * v1;
}

// Index checks of the debug build (compiled with -DHX_BOUNDS_CHECK, the library's
// stand-in for a memory checker): an index outside its array records `code` in the flag
// word (the first violation wins) and the caller skips the access; the host reports the
// code after the interval (HX_ERR_CUDA).  In the regular build the check is the constant
// true and costs nothing.
__device__ __forceinline__ bool in_bounds(bool ok, int* flag, int code) {
#ifdef HX_BOUNDS_CHECK
  if (!ok) {
    if (flag) atomicCAS(flag, 0, code);
    return false;
  }
#else
  (void)ok;
  (void)flag;
  (void)code;
#endif
  return true;
}

// DSS gather of one point-level: own value plus the table's sources, in order, in double.
template <typename T>
__device__ __forceinline__ double dss_gather(const T* base, long long es, int ls, int e, int l, int p,
                                             const DssTable& tab) {
  const int ep = e * 16 + p;
  if (!in_bounds(ep >= 0 && ep < tab.npts, tab.flag, kBoundsDssPoint)) return 0.0;
  double acc = (double)base[(size_t)e * es + (size_t)l * ls + p];
  int n = tab.cnt[ep];
  if (!in_bounds(n >= 0 && n <= MAXSRC, tab.flag, kBoundsDssCount)) n = 0;
  for (int k = 0; k < n; ++k) {
    const int s = tab.src[ep * MAXSRC + k];
    if (!in_bounds(s >= 0 && s < tab.npts, tab.flag, kBoundsDssSource)) continue;
    acc += (double)base[(size_t)(s >> 4) * es + (size_t)l * ls + (s & 15)];
  }
  return acc;
}

// Thread -> (level in a group of 8, point) for a 128-thread block of a standalone DSS:
// each warp holds one class of points over the 8 levels -- interior {5,6,9,10} (no
// contribution from other elements), edge {1,2,4,7} and {8,11,13,14} (one), corner
// {0,3,12,15} (two or three) -- so the gather loop has one trip count per warp instead
// of every warp running the longest.  Each point still sums in its own fixed order.
__device__ __forceinline__ void dss_thread_point(int& lo, int& p) {
  constexpr unsigned long long kPerm = 0x5ull | 0x6ull << 4 | 0x9ull << 8 | 0xAull << 12 | 0x1ull << 16 |
                                       0x2ull << 20 | 0x4ull << 24 | 0x7ull << 28 | 0x8ull << 32 |
                                       0xBull << 36 | 0xDull << 40 | 0xEull << 44 | 0x0ull << 48 |
                                       0x3ull << 52 | 0xCull << 56 | 0xFull << 60;
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  lo = lane >> 2;
  p = (int)((kPerm >> (4 * (w * 4 + (lane & 3)))) & 15);
}

// ---- segmented column scans (128 threads: 16 columns x 8 segments of 9 levels) ------
// Exclusive prefix of the per-segment totals within an 8-lane group.
template <typename T>
__device__ __forceinline__ T seg_excl_prefix(T tot, int seg) {
  T incl = tot;
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    const T y = __shfl_up_sync(FULL, incl, off, 8);
    if (seg >= off) incl += y;
  }
  T ex = __shfl_up_sync(FULL, incl, 1, 8);
  return seg == 0 ? T(0) : ex;
}
// Exclusive suffix (sum of later segments).
__device__ __forceinline__ double seg_excl_suffix(double tot, int seg) {
  double incl = tot;
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    const double y = __shfl_down_sync(FULL, incl, off, 8);
    if (seg + off < 8) incl += y;
  }
  double ex = __shfl_down_sync(FULL, incl, 1, 8);
  return seg == 7 ? 0.0 : ex;
}

// Exclusive prefix over the warp of one value per lane.
__device__ __forceinline__ double warp_excl_scan(double v, int lane) {
  double incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const double y = __shfl_up_sync(FULL, incl, off);
    if (lane >= off) incl += y;
  }
  const double ex = __shfl_up_sync(FULL, incl, 1);
  return lane == 0 ? 0.0 : ex;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
  return v;
}

// ---- exact FP64 operations on the integer pipe ------------------------------------
// The GB300's FP64 pipe issues 2 thread-instructions per cycle per SM (1/64 of FP32),
// and min/max and compares issue there like arithmetic.  Exact ones move to the integer
// pipe: a non-NaN double's bit pattern, with the magnitude bits flipped when the sign
// bit is set, orders like the value as a signed 64-bit integer (-0 below +0).
__device__ __forceinline__ long long dkey(double x) {
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double dkey_value(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}
__device__ __forceinline__ long long kmin(long long a, long long b) { return b < a ? b : a; }
__device__ __forceinline__ long long kmax(long long a, long long b) { return b > a ? b : a; }

// Exact sign tests and orderings of T values: FP32 as is, FP64 on the integer pipe.
template <typename T> __device__ __forceinline__ bool pos(T x) { return x > T(0); }
template <> __device__ __forceinline__ bool pos<double>(double x) {
  return __double_as_longlong(x) > 0;  // > +0 (non-NaN)
}
// x == 0 (either sign): FP32 as is; FP64 on the integer pipe.
template <typename T> __device__ __forceinline__ bool is_zero(T x) { return x == T(0); }
template <> __device__ __forceinline__ bool is_zero<double>(double x) {
  return (__double_as_longlong(x) << 1) == 0;
}
// a b > 0 for non-NaN a, b: FP32 as is; FP64 on the integer pipe as "the same sign and
// neither zero" (differs from the product's test only where a b would underflow to 0).
template <typename T> __device__ __forceinline__ bool pos_prod(T a, T b) { return a * b > T(0); }
template <> __device__ __forceinline__ bool pos_prod<double>(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return (x ^ y) >= 0 && (x << 1) != 0 && (y << 1) != 0;
}
template <typename T> __device__ __forceinline__ bool less(T a, T b) { return a < b; }
template <> __device__ __forceinline__ bool less<double>(double a, double b) {
  return dkey(a) < dkey(b);  // exact for non-NaN except that -0 < +0
}
// a < b for non-NaN values, zeros of either sign equal (the IEEE comparison): FP32 as is,
// FP64 on the integer pipe.
__device__ __forceinline__ long long dkz(double x) {
  const long long k = dkey(x);
  return k == -1 ? 0 : k;  // -0 -> +0
}
template <typename T> __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
template <> __device__ __forceinline__ bool lt<double>(double a, double b) { return dkz(a) < dkz(b); }
// min(|a|, |b|, |c|) with the sign of s.
template <typename T> __device__ __forceinline__ T min3abs_signed(T a, T b, T c, T s) {
  return fmin(fmin(fabs(a), fabs(b)), fabs(c)) * copysign(T(1), s);
}
template <> __device__ __forceinline__ double min3abs_signed<double>(double a, double b, double c,
                                                                    double s) {
  const long long m = 0x7fffffffffffffffLL;
  long long k = __double_as_longlong(a) & m;
  k = kmin(k, __double_as_longlong(b) & m);
  k = kmin(k, __double_as_longlong(c) & m);
  return __longlong_as_double(k | (__double_as_longlong(s) & ~m));
}

// ---- double <-> float conversions on the integer pipe --------------------------------
// F2F conversions issue to the FP64 pipe at the cost of an FP64 multiply-add; the mixed
// form converts at every load and store of a double field.  These restate the IEEE 754
// binary64 <-> binary32 conversions (round to nearest, ties to even) as integer field
// manipulation; zeros are handled inline and the rare subnormal, overflowing, infinite and
// NaN cases fall back to the hardware conversion, so the results equal the hardware's for
// every input.  The inlined fallback compiles to a predicated conversion that each warp
// still issues; an out-of-line fallback (a branch around a call) removes that, and pays
// off in d2f_seed and dtwice below (FP64 kernels), but here it measured slower in the
// mixed form's tracer advection (more FP64-pipe instructions, 6.9 vs 6.2 ms per ne30
// interval), so these two keep the inline form.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;  // binary32 biased exponent
  if (e <= 0 || e >= 255) {
    if (((hi & 0x7FFFFFFFu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return __double2float_rn(x);
  }
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // top 23 of the 52 mantissa bits
  const unsigned rest = lo & 0x1FFFFFFFu;                   // the 29 dropped bits
  unsigned r = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
  r += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // carry is exact
  return __uint_as_float(r);
}
__device__ __forceinline__ double f2d(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e == 0u || e == 255u) {
    if ((u << 1) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)x;
  }
  return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3)),
                          (int)(u << 29));
}
// The out-of-line rare cases of d2f_seed and dtwice: a uniform branch around a call
// instead of a predicated FP64-pipe instruction in every warp.
__device__ __noinline__ float d2f_slow(double x) { return __double2float_rn(x); }
__device__ __noinline__ double dtwice_slow(double x) { return x * 2.0; }
// double -> R and R -> double (identities in the FP64 form)
template <typename R> __device__ __forceinline__ R cvt(double x);
template <> __device__ __forceinline__ double cvt<double>(double x) { return x; }
template <> __device__ __forceinline__ float cvt<float>(double x) { return d2f_rn(x); }
__device__ __forceinline__ double dbl(double x) { return x; }
__device__ __forceinline__ double dbl(float x) { return f2d(x); }

template <typename R> __device__ __forceinline__ R rel(double x) {
  if constexpr (kF32<R>) return d2f_rn(x - sh16(x, 0));
  else return x;
}
// The same conversions on the hardware path, for kernels whose instruction issue (not
// the FP64 pipe) limits them.
template <typename R> __device__ __forceinline__ R cvt_hw(double x) { return (R)x; }
__device__ __forceinline__ double dbl_hw(double x) { return x; }
__device__ __forceinline__ double dbl_hw(float x) { return (double)x; }
template <typename R> __device__ __forceinline__ R rel_hw(double x) {
  if constexpr (kF32<R>) return (R)(x - sh16(x, 0));
  else return x;
}

// x as a float with the mantissa truncated to 23 bits (relative error below 2^-23), on
// the integer pipe: the exponent rebiased and the top mantissa bits moved, for |x| in
// the float normal range, else the hardware conversion.  A seed for reciprocals, whose
// Newton refinement removes the truncation.
__device__ __forceinline__ float d2f_seed(double x) {
  const unsigned hi = (unsigned)__double2hiint(x);
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;
  if (e <= 0 || e >= 255) return d2f_slow(x);
  const unsigned lo = (unsigned)__double2loint(x);
  return __uint_as_float((hi & 0x80000000u) | ((unsigned)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}

// 2 x, exact, on the integer pipe (the exponent field incremented) for normal x below
// 2^1022 in magnitude and for zeros; subnormals and larger values take the FP64 product
// (out of line, as the conversions' rare cases).
__device__ __forceinline__ double dtwice(double x) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const bool zero = (b << 1) == 0;
  if ((e == 0 || e >= 0x7FE) && !zero) return dtwice_slow(x);
  return zero ? x : __longlong_as_double(b + (1LL << 52));
}

// 1/x in FP64 from the approximate FP32 reciprocal of x (__fdividef of the truncated
// float image, within 3 ulp of a float) refined by two Newton-Raphson steps
// r <- r + r (1 - x r), each of which squares the relative error (below 3 * 2^-23 ->
// 2^-42 -> below one ulp of the result); rf returns the FP32 reciprocal.  For x of magnitude
// 2^-125 .. 2^125; within one ulp of 1.0 / x.
__device__ __forceinline__ double rcp_newton(double x, float& rf) {
  rf = __fdividef(1.0f, d2f_seed(x));
  double r = f2d(rf);  // exact; on the integer pipe
  r = fma(r, fma(-x, r, 1.0), r);
  return fma(r, fma(-x, r, 1.0), r);
}

// One Newton-Raphson step from the same seed: relative error below 2^-42 (the seed's
// 3 * 2^-23 squared; about 2.3e-13), for the mixed form's FP64 integrands next to FP32
// operators.
__device__ __forceinline__ double rcp_newton1(double x, float& rf) {
  rf = __fdividef(1.0f, d2f_seed(x));
  const double r = f2d(rf);
  return fma(r, fma(-x, r, 1.0), r);
}

// 1 / x in R: the FP32 quotient in FP32; in FP64 rcp_newton (four FMAs instead of the
// IEEE division's longer sequence; within one ulp, for |x| in 2^-125 .. 2^125).
template <typename R> __device__ __forceinline__ R recip(R x) {
  if constexpr (kF32<R>) {
    return R(1) / x;
  } else {
    float rf;
    return rcp_newton(x, rf);
  }
}

// a / b from r = rcp_newton(b): the product a r corrected once by its residual,
// q + r (a - q b) (the final step of Markstein's division, IBM J. Res. Dev. 34 (1990)
// 111-119), within one ulp of the IEEE quotient.  Same domain for b as rcp_newton.
__device__ __forceinline__ double div_newton(double a, double b, double r) {
  const double q = a * r;
  return fma(fma(-q, b, a), r, q);
}

// ---- bulk asynchronous copies into shared memory (the TMA engine, untiled) ---------
// One thread arms an mbarrier with the expected byte count and issues
// cp.async.bulk global -> shared; the copy completes the barrier's phase, which the
// threads that read the data wait for.  Addresses 16-byte aligned, sizes multiples of
// 16 bytes.
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's earlier generic-proxy accesses of shared memory before later
// async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// Two copies completing one phase of the barrier (one arrival expecting both sizes).
__device__ __forceinline__ void bulk_load2(void* dst1, const void* src1, unsigned bytes1, void* dst2,
                                           const void* src2, unsigned bytes2, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes1 + bytes2)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst1)),
               "l"(src1), "r"(bytes1), "r"(smem_addr(bar))
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst2)),
               "l"(src2), "r"(bytes2), "r"(smem_addr(bar))
               : "memory");
}
// Waits for the completion of phase `parity` of the barrier; false after `tries` polls
// (each poll may suspend the thread for a short, hardware-chosen time).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int tries) {
  for (int i = 0; i < tries; ++i) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Brackets one launch for the per-kernel timing hooks.
struct KScope {
  const char* n;
  cudaStream_t s;
  KScope(const char* name, cudaStream_t st) : n(name), s(st) { kernel_enter(name, st); }
  ~KScope() { kernel_leave(n, s); }
};

inline int nblk(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace
}  // namespace hx
