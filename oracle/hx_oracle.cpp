// hx_oracle.cpp — CPU oracle for the preqx dycore step.  TEST INFRASTRUCTURE ONLY.
//
// This file is the checker the GPU library is compared against.  It is a plain C++17
// (+OpenMP over elements) restatement, loop for loop, of the reference HOMMEXX C++
// functors, in FP64, compiled without FMA contraction so the result does not depend on
// the host CPU.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// load it; nothing in the product links or calls it.
//
// Parity status: the reference cannot be built here (its hot path needs Kokkos, which
// is not vendored — cmake/Trilinos.cmake:103-108 — and its Fortran twins need gfortran
// and MPI) and it ships no golden vectors, so this restatement is pinned by the
// reference's own property tests (limiter bounds/mass/1-norm, preqx_ut.cpp:1330-1527),
// analytic operator identities and conservation checks, not by reference outputs.
//
// It exports the same C symbols as libhxgpu.so (include/hxgpu.h), so one driver can
// run either library.  Internal arrays use the reference device layout, level index
// fastest: v [E][3][2][16][72], T/dp3d [E][3][16][72], Qdp [E][2][Q][16][72]
// (src/share/cxx/Elements.hpp:44-67, Tracers.hpp:26-30); the Fortran arrays are
// transposed on init/push as in src/share/cxx/utilities/SyncUtils.hpp.
//
// Point index p = igp*4 + jgp with the reference C++ names (igp = Fortran j,
// jgp = Fortran i).

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "hxgpu.h"

namespace {

constexpr int NP = 4;
constexpr int NP2 = 16;
constexpr int NLEV = 72;
constexpr int NTL = 3;
constexpr int QTL = 2;

// src/share/cxx/PhysicalConstants.hpp:17-22
constexpr double Rwater_vapor = 461.5;
constexpr double Rgas = 287.04;
constexpr double cp = 1005.0;
constexpr double kappa = Rgas / cp;
constexpr double rrearth = 1.0 / 6.376e6;

// Forward-mode dual number: the element and column routines below are templates over
// the field scalar, so instantiating them with Dual gives the exact tangent-linear model
// of the same code (value part bit-identical to the double instantiation).  Branches and
// index searches follow the value part.
struct Dual {
  double v, d;
  Dual(double a = 0.0) : v(a), d(0.0) {}
  Dual(double a, double b) : v(a), d(b) {}
  Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
  Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
  Dual& operator*=(const Dual& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
  Dual& operator/=(const Dual& o) {
    const double q = v / o.v;
    d = (d - q * o.d) / o.v;
    v = q;
    return *this;
  }
};
inline Dual operator+(Dual a, const Dual& b) { return a += b; }
inline Dual operator-(Dual a, const Dual& b) { return a -= b; }
inline Dual operator*(Dual a, const Dual& b) { return a *= b; }
inline Dual operator/(Dual a, const Dual& b) { return a /= b; }
inline Dual operator-(const Dual& a) { return {-a.v, -a.d}; }
inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
inline double val(double x) { return x; }
inline double val(const Dual& x) { return x.v; }
inline double sabs(double x) { return std::fabs(x); }
inline Dual sabs(const Dual& x) { return x.v < 0.0 ? -x : x; }

struct Params {
  int remap_alg = 1, limiter_option = 8, rsplit = 1, qsplit = 1, time_step_type = 5;
  int qsize = 0, state_frequency = 1, hypervis_order = 2, hypervis_subcycle = 1, ftype = -1;
  double nu = 0, nu_p = 0, nu_q = 0, nu_s = 0, nu_div = 0, nu_top = 0, hypervis_scaling = 0;
  double nu_ratio1 = 1, nu_ratio2 = 1;
  bool moist = false, disable_diagnostics = true, use_cpstar = false, set = false;
};

struct TimeLevel {
  int nm1 = 0, n0 = 1, np1 = 2, nstep = 0, nstep0 = 0, n0_qdp = 0, np1_qdp = 1;
  void update_dynamics_levels() {  // LEAPFROG, TimeLevel.hpp:37-52
    int tmp = np1;
    np1 = nm1;
    nm1 = n0;
    n0 = tmp;
    ++nstep;
  }
  void update_tracers_levels(int qsplit) {  // TimeLevel.hpp:58-67
    int i_temp = nstep / qsplit;
    if (i_temp % 2 == 0) { n0_qdp = 0; np1_qdp = 1; }
    else { n0_qdp = 1; np1_qdp = 0; }
  }
};

struct Ctx {
  Params prm;
  TimeLevel tl;
  int E = 0, Q = 0;
  bool consthv = true;
  double dvv[NP][NP] = {};
  // hybrid coordinate
  double ps0 = 0, hyai[NLEV + 1] = {}, hybi[NLEV + 1] = {}, ai_delta[NLEV] = {},
         bi_delta[NLEV] = {}, dp0[NLEV] = {}, hyai0 = 0;
  // metric, C++ index order == Fortran memory
  std::vector<double> D, Dinv, metinv, tensorvisc, vec_sph2cart;
  std::vector<double> fcor, mp, spheremp, rspheremp, metdet, phis;
  // state
  std::vector<double> v, t, dp3d, ps_v, qdp, Qc;
  std::vector<double> fm, ft, fq;  // CAM forcing: FM [E][2][16][NLEV], FT/FQ level-contiguous
  // init_diagnostics_c host arrays: Q, Qvar, Qmass, Q1mass, IEner, IEner_wet, KEner, PEner
  double* diag[8] = {};
  double* stream_to[7] = {};  // hx_stream_results destinations
  bool streamed = false;
  std::vector<double> phi, omega_p, eta_dot_dpdn, derived_dp, divdp, divdp_proj,
      dpdiss_ave, dpdiss_bih, vn0;
  // buffers
  std::vector<double> vtens, ttens, dptens, qtens_bih, qlim, vstar, dpdissk, dp_buf;
  // connectivity: conn[e][slot] = {remote elem, remote slot}
  std::vector<int> conn;
  std::vector<int> g_src_e, g_src_p, g_cnt;  // gather table [E][16][3], [E][16]
  bool conn_final = false, tables = false;
  int last_err = 0;
  std::string last_msg;
  bool abort_on_error = true;
  int valid_remap = 1;
};

Ctx* g = nullptr;
Ctx& C() {
  if (!g) g = new Ctx();
  return *g;
}

void set_error(int code, const std::string& msg) {
  Ctx& c = C();
  c.last_err = code;
  c.last_msg = msg;
  if (c.abort_on_error) {
    std::fprintf(stderr, "%s\nExiting...\n", msg.c_str());
    std::exit(code);
  }
}

inline size_t IV(int e, int tl, int comp, int p, int k) {
  return ((((size_t)e * NTL + tl) * 2 + comp) * NP2 + p) * NLEV + k;
}
inline size_t IS(int e, int tl, int p, int k) {  // T, dp3d
  return (((size_t)e * NTL + tl) * NP2 + p) * NLEV + k;
}
inline size_t IQ(int e, int qtl, int q, int p, int k, int Q) {
  return ((((size_t)e * QTL + qtl) * Q + q) * NP2 + p) * NLEV + k;
}
inline size_t I3(int e, int p, int k) { return ((size_t)e * NP2 + p) * NLEV + k; }
inline size_t I3V(int e, int comp, int p, int k) {
  return (((size_t)e * 2 + comp) * NP2 + p) * NLEV + k;
}

// ----------------------------------------------------------------------------------
// Sphere operators (src/share/cxx/SphereOperators.hpp:291-862), multi-level form.
// Fields are [16][NLEV] (point, level); vectors [2][16][NLEV].  Operators act on the
// first nl levels.
// ----------------------------------------------------------------------------------
struct EM {  // metric of one element
  const double *D, *Dinv, *metinv, *metdet, *spheremp, *mp, *tensor, *sph2cart;
  const double (*dvv)[NP];
  double d(int a, int b, int p) const { return D[(a * 2 + b) * NP2 + p]; }
  double di(int a, int b, int p) const { return Dinv[(a * 2 + b) * NP2 + p]; }
  double mi(int a, int b, int p) const { return metinv[(a * 2 + b) * NP2 + p]; }
  double tv(int a, int b, int p) const { return tensor[(a * 2 + b) * NP2 + p]; }
  double s2c(int a, int b, int p) const { return sph2cart[(a * 3 + b) * NP2 + p]; }
};

inline int P(int i, int j) { return i * NP + j; }
#define F(arr, p, k) (arr)[(p) * NLEV + (k)]
#define FV(arr, c, p, k) (arr)[((c) * NP2 + (p)) * NLEV + (k)]

// SphereOperators.hpp:291-319
template <class S>
void gradient_sphere(const EM& m, const S* s, S* g, int nl) {
  for (int igp = 0; igp < NP; ++igp)
    for (int jgp = 0; jgp < NP; ++jgp)
      for (int l = 0; l < nl; ++l) {
        S v0 = 0.0, v1 = 0.0;
        for (int k = 0; k < NP; ++k) {
          v0 += m.dvv[jgp][k] * F(s, P(igp, k), l);
          v1 += m.dvv[igp][k] * F(s, P(k, jgp), l);
        }
        v0 *= rrearth;
        v1 *= rrearth;
        const int p = P(igp, jgp);
        FV(g, 0, p, l) = m.di(0, 0, p) * v0 + m.di(0, 1, p) * v1;
        FV(g, 1, p, l) = m.di(1, 0, p) * v0 + m.di(1, 1, p) * v1;
      }
}

// SphereOperators.hpp:321-348
template <class S>
void gradient_sphere_update(const EM& m, const S* s, S* g, int nl) {
  for (int igp = 0; igp < NP; ++igp)
    for (int jgp = 0; jgp < NP; ++jgp)
      for (int l = 0; l < nl; ++l) {
        S dsdx = 0.0, dsdy = 0.0;
        for (int k = 0; k < NP; ++k) {
          dsdx += m.dvv[jgp][k] * F(s, P(igp, k), l);
          dsdy += m.dvv[igp][k] * F(s, P(k, jgp), l);
        }
        dsdx *= rrearth;
        dsdy *= rrearth;
        const int p = P(igp, jgp);
        FV(g, 0, p, l) += m.di(0, 0, p) * dsdx + m.di(0, 1, p) * dsdy;
        FV(g, 1, p, l) += m.di(1, 0, p) * dsdx + m.di(1, 1, p) * dsdy;
      }
}

// SphereOperators.hpp:350-392
template <class S>
void divergence_sphere(const EM& m, const S* v, S* div, int nl) {
  std::vector<S> gv(2 * NP2 * NLEV);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const S v0 = FV(v, 0, p, l), v1 = FV(v, 1, p, l);
      FV(gv.data(), 0, p, l) = (m.di(0, 0, p) * v0 + m.di(1, 0, p) * v1) * m.metdet[p];
      FV(gv.data(), 1, p, l) = (m.di(0, 1, p) * v0 + m.di(1, 1, p) * v1) * m.metdet[p];
    }
  for (int igp = 0; igp < NP; ++igp)
    for (int jgp = 0; jgp < NP; ++jgp)
      for (int l = 0; l < nl; ++l) {
        S dudx = 0.0, dvdy = 0.0;
        for (int k = 0; k < NP; ++k) {
          dudx += m.dvv[jgp][k] * FV(gv.data(), 0, P(igp, k), l);
          dvdy += m.dvv[igp][k] * FV(gv.data(), 1, P(k, jgp), l);
        }
        const int p = P(igp, jgp);
        F(div, p, l) = (dudx + dvdy) * (1.0 / m.metdet[p] * rrearth);
      }
}

// SphereOperators.hpp:394-444: qtens = qdp + alpha*div(vstar*qdp) [+ qtens]
template <class S>
void divergence_sphere_update(const EM& m, double alpha, bool add_hv, const S* vstar,
                              const S* qdp, S* qtens, int nl) {
  std::vector<S> gv(2 * NP2 * NLEV);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const S q = F(qdp, p, l);
      const S v0 = FV(vstar, 0, p, l) * q;
      const S v1 = FV(vstar, 1, p, l) * q;
      FV(gv.data(), 0, p, l) = (m.di(0, 0, p) * v0 + m.di(1, 0, p) * v1) * m.metdet[p];
      FV(gv.data(), 1, p, l) = (m.di(0, 1, p) * v0 + m.di(1, 1, p) * v1) * m.metdet[p];
    }
  for (int igp = 0; igp < NP; ++igp)
    for (int jgp = 0; jgp < NP; ++jgp)
      for (int l = 0; l < nl; ++l) {
        S dudx = 0.0, dvdy = 0.0;
        for (int k = 0; k < NP; ++k) {
          dudx += m.dvv[jgp][k] * FV(gv.data(), 0, P(igp, k), l);
          dvdy += m.dvv[igp][k] * FV(gv.data(), 1, P(k, jgp), l);
        }
        const int p = P(igp, jgp);
        const S q0 = add_hv ? F(qtens, p, l) : S(0.0);
        F(qtens, p, l) =
            (F(qdp, p, l) + alpha * ((dudx + dvdy) * (1.0 / m.metdet[p] * rrearth)) + q0);
      }
}

// SphereOperators.hpp:492-533
template <class S>
void vorticity_sphere(const EM& m, const S* v, S* vort, int nl) {
  std::vector<S> vc(2 * NP2 * NLEV);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const S v0 = FV(v, 0, p, l), v1 = FV(v, 1, p, l);
      FV(vc.data(), 0, p, l) = m.d(0, 0, p) * v0 + m.d(0, 1, p) * v1;
      FV(vc.data(), 1, p, l) = m.d(1, 0, p) * v0 + m.d(1, 1, p) * v1;
    }
  for (int igp = 0; igp < NP; ++igp)
    for (int jgp = 0; jgp < NP; ++jgp)
      for (int l = 0; l < nl; ++l) {
        S dudy = 0.0, dvdx = 0.0;
        for (int k = 0; k < NP; ++k) {
          dvdx += m.dvv[jgp][k] * FV(vc.data(), 1, P(igp, k), l);
          dudy += m.dvv[igp][k] * FV(vc.data(), 0, P(k, jgp), l);
        }
        const int p = P(igp, jgp);
        F(vort, p, l) = (dvdx - dudy) * (1.0 / m.metdet[p] * rrearth);
      }
}

// SphereOperators.hpp:536-583 (the input vector is overwritten, as in the reference)
template <class S>
void divergence_sphere_wk(const EM& m, S* v, S* div, int nl) {
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const S v0 = FV(v, 0, p, l), v1 = FV(v, 1, p, l);
      FV(v, 0, p, l) = m.di(0, 0, p) * v0 + m.di(1, 0, p) * v1;
      FV(v, 1, p, l) = m.di(0, 1, p) * v0 + m.di(1, 1, p) * v1;
    }
  for (int ngp = 0; ngp < NP; ++ngp)
    for (int mgp = 0; mgp < NP; ++mgp)
      for (int l = 0; l < nl; ++l) {
        S dd = 0.0;
        for (int jgp = 0; jgp < NP; ++jgp) {
          dd -= (m.spheremp[P(ngp, jgp)] * FV(v, 0, P(ngp, jgp), l) * m.dvv[jgp][mgp] +
                 m.spheremp[P(jgp, mgp)] * FV(v, 1, P(jgp, mgp), l) * m.dvv[jgp][ngp]) *
                rrearth;
        }
        F(div, P(ngp, mgp), l) = dd;
      }
}

// SphereOperators.hpp:585-597
template <class S>
void laplace_simple(const EM& m, const S* field, S* lap, int nl) {
  std::vector<S> gs(2 * NP2 * NLEV);
  gradient_sphere(m, field, gs.data(), nl);
  divergence_sphere_wk(m, gs.data(), lap, nl);
}

// SphereOperators.hpp:599-635
void laplace_tensor(const EM& m, const double* field, double* lap, int nl) {
  std::vector<double> gs(2 * NP2 * NLEV), sb(2 * NP2 * NLEV);
  gradient_sphere(m, field, gs.data(), nl);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const double g0 = FV(gs.data(), 0, p, l), g1 = FV(gs.data(), 1, p, l);
      FV(sb.data(), 0, p, l) = m.tv(0, 0, p) * g0 + m.tv(1, 0, p) * g1;
      FV(sb.data(), 1, p, l) = m.tv(0, 1, p) * g0 + m.tv(1, 1, p) * g1;
    }
  divergence_sphere_wk(m, sb.data(), lap, nl);
}

// SphereOperators.hpp:680-710: curls = beta*curls + alpha*curl(scalar)
template <class S>
void curl_sphere_wk_testcov_update(const EM& m, double alpha, double beta,
                                   const S* scalar, S* curls, int nl) {
  for (int ngp = 0; ngp < NP; ++ngp)
    for (int mgp = 0; mgp < NP; ++mgp)
      for (int l = 0; l < nl; ++l) {
        S sb0 = 0.0, sb1 = 0.0;
        for (int j = 0; j < NP; ++j) {
          sb0 -= m.mp[P(j, mgp)] * F(scalar, P(j, mgp), l) * m.dvv[j][ngp];
          sb1 += m.mp[P(ngp, j)] * F(scalar, P(ngp, j), l) * m.dvv[j][mgp];
        }
        const int p = P(ngp, mgp);
        FV(curls, 0, p, l) = beta * FV(curls, 0, p, l) +
                             alpha * (m.d(0, 0, p) * sb0 + m.d(1, 0, p) * sb1) * rrearth;
        FV(curls, 1, p, l) = beta * FV(curls, 1, p, l) +
                             alpha * (m.d(0, 1, p) * sb0 + m.d(1, 1, p) * sb1) * rrearth;
      }
}

// SphereOperators.hpp:712-748
template <class S>
void grad_sphere_wk_testcov(const EM& m, const S* scalar, S* grads, int nl) {
  for (int ngp = 0; ngp < NP; ++ngp)
    for (int mgp = 0; mgp < NP; ++mgp)
      for (int l = 0; l < nl; ++l) {
        S b0 = 0.0, b1 = 0.0;
        const int p = P(ngp, mgp);
        for (int j = 0; j < NP; ++j) {
          const double mpnj = m.mp[P(ngp, j)];
          const double mpjm = m.mp[P(j, mgp)];
          const double md = m.metdet[p];
          const S snj = F(scalar, P(ngp, j), l);
          const S sjm = F(scalar, P(j, mgp), l);
          const double djm = m.dvv[j][mgp];
          const double djn = m.dvv[j][ngp];
          b0 -= (mpnj * m.mi(0, 0, p) * md * snj * djm + mpjm * m.mi(0, 1, p) * md * sjm * djn);
          b1 -= (mpnj * m.mi(1, 0, p) * md * snj * djm + mpjm * m.mi(1, 1, p) * md * sjm * djn);
        }
        FV(grads, 0, p, l) = (m.d(0, 0, p) * b0 + m.d(1, 0, p) * b1) * rrearth;
        FV(grads, 1, p, l) = (m.d(0, 1, p) * b0 + m.d(1, 1, p) * b1) * rrearth;
      }
}

// SphereOperators.hpp:816-862 (input and output may alias)
template <class S>
void vlaplace_sphere_wk_contra(const EM& m, double nu_ratio, const S* vec, S* lap,
                               int nl) {
  std::vector<S> div(NP2 * NLEV), gcc(2 * NP2 * NLEV);
  divergence_sphere(m, vec, div.data(), nl);
  if (nu_ratio > 0 && nu_ratio != 1.0)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < nl; ++l) F(div.data(), p, l) *= nu_ratio;
  grad_sphere_wk_testcov(m, div.data(), gcc.data(), nl);
  std::vector<S>& vort = div;
  vorticity_sphere(m, vec, vort.data(), nl);
  curl_sphere_wk_testcov_update(m, -1.0, 1.0, vort.data(), gcc.data(), nl);
  const double re2 = rrearth * rrearth;
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const double f = 2.0 * m.spheremp[p];
      const S a0 = f * FV(vec, 0, p, l) * re2 + FV(gcc.data(), 0, p, l);
      const S a1 = f * FV(vec, 1, p, l) * re2 + FV(gcc.data(), 1, p, l);
      FV(lap, 0, p, l) = a0;
      FV(lap, 1, p, l) = a1;
    }
}

// SphereOperators.hpp:750-814 (input and output may alias)
void vlaplace_sphere_wk_cartesian(const EM& m, const double* vec, double* lap, int nl) {
  std::vector<double> l0(NP2 * NLEV), l1(NP2 * NLEV), l2(NP2 * NLEV), vin(2 * NP2 * NLEV);
  std::copy(vec, vec + 2 * NP2 * NLEV, vin.begin());
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      const double v0 = FV(vin.data(), 0, p, l), v1 = FV(vin.data(), 1, p, l);
      F(l0.data(), p, l) = m.s2c(0, 0, p) * v0 + m.s2c(1, 0, p) * v1;
      F(l1.data(), p, l) = m.s2c(0, 1, p) * v0 + m.s2c(1, 1, p) * v1;
      F(l2.data(), p, l) = m.s2c(0, 2, p) * v0 + m.s2c(1, 2, p) * v1;
    }
  laplace_tensor(m, l0.data(), l0.data(), nl);
  laplace_tensor(m, l1.data(), l1.data(), nl);
  laplace_tensor(m, l2.data(), l2.data(), nl);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < nl; ++l) {
      FV(lap, 0, p, l) = m.s2c(0, 0, p) * F(l0.data(), p, l) + m.s2c(0, 1, p) * F(l1.data(), p, l) +
                         m.s2c(0, 2, p) * F(l2.data(), p, l) +
                         2.0 * m.spheremp[p] * FV(vin.data(), 0, p, l) * (rrearth) * (rrearth);
      FV(lap, 1, p, l) = m.s2c(1, 0, p) * F(l0.data(), p, l) + m.s2c(1, 1, p) * F(l1.data(), p, l) +
                         m.s2c(1, 2, p) * F(l2.data(), p, l) +
                         2.0 * m.spheremp[p] * FV(vin.data(), 1, p, l) * (rrearth) * (rrearth);
    }
}

EM metric(int e) {
  Ctx& c = C();
  EM m;
  m.D = &c.D[(size_t)e * 64];
  m.Dinv = &c.Dinv[(size_t)e * 64];
  m.metinv = &c.metinv[(size_t)e * 64];
  m.metdet = &c.metdet[(size_t)e * 16];
  m.spheremp = &c.spheremp[(size_t)e * 16];
  m.mp = &c.mp[(size_t)e * 16];
  m.tensor = c.tensorvisc.empty() ? nullptr : &c.tensorvisc[(size_t)e * 64];
  m.sph2cart = c.vec_sph2cart.empty() ? nullptr : &c.vec_sph2cart[(size_t)e * 96];
  m.dvv = c.dvv;
  return m;
}

// ----------------------------------------------------------------------------------
// DSS (src/share/cxx/mpi/BoundaryExchange.cpp:285-618, ConnectivityHelpers.hpp)
// ----------------------------------------------------------------------------------
const int PTS_FWD[8][4] = {{0, 1, 2, 3}, {12, 13, 14, 15}, {0, 4, 8, 12}, {3, 7, 11, 15},
                           {0, -1, -1, -1}, {3, -1, -1, -1}, {12, -1, -1, -1}, {15, -1, -1, -1}};
const int PTS_BWD[8][4] = {{3, 2, 1, 0}, {15, 14, 13, 12}, {12, 8, 4, 0}, {15, 11, 7, 3},
                           {0, -1, -1, -1}, {3, -1, -1, -1}, {12, -1, -1, -1}, {15, -1, -1, -1}};
// 0 = forward, 1 = backward (ConnectivityHelpers.hpp:129-139)
const int DIRECTION[4][4] = {{1, 0, 0, 1}, {0, 1, 1, 0}, {0, 1, 1, 0}, {1, 0, 0, 1}};

void build_tables() {
  Ctx& c = C();
  const int E = c.E;
  c.g_src_e.assign((size_t)E * 16 * 3, 0);
  c.g_src_p.assign((size_t)E * 16 * 3, 0);
  c.g_cnt.assign((size_t)E * 16, 0);
  auto add = [&](int e, int p, int se, int sp) {
    int& n = c.g_cnt[(size_t)e * 16 + p];
    c.g_src_e[((size_t)e * 16 + p) * 3 + n] = se;
    c.g_src_p[((size_t)e * 16 + p) * 3 + n] = sp;
    ++n;
  };
  for (int e = 0; e < E; ++e) {
    for (int k = 0; k < NP; ++k)
      for (int slot = 0; slot < 4; ++slot) {  // S, N, W, E
        const int r = c.conn[(e * 8 + slot) * 2], rs = c.conn[(e * 8 + slot) * 2 + 1];
        if (r < 0) continue;
        const int dir = DIRECTION[rs][slot];
        add(e, PTS_FWD[slot][k], r, dir == 0 ? PTS_FWD[rs][k] : PTS_BWD[rs][k]);
      }
    for (int slot = 4; slot < 8; ++slot) {  // SW, SE, NW, NE
      const int r = c.conn[(e * 8 + slot) * 2], rs = c.conn[(e * 8 + slot) * 2 + 1];
      if (r < 0) continue;
      add(e, PTS_FWD[slot][0], r, PTS_FWD[rs][0]);
    }
  }
  c.tables = true;
}

// One registered 3-D field: element block of [16][NLEV] at base + e*estride.
template <class S>
struct FieldRefT {
  S* base;
  size_t estride;
};
using FieldRef = FieldRefT<double>;

// BoundaryExchange::exchange: pack all (pre-exchange values), unpack in the fixed order,
// then optionally multiply by rspheremp.
template <class S>
void dss_t(const std::vector<FieldRefT<S>>& fields, bool rsmp) {
  Ctx& c = C();
  const int E = c.E;
  for (const FieldRefT<S>& f : fields) {
    std::vector<S> pre((size_t)E * NP2 * NLEV);
#pragma omp parallel for
    for (int e = 0; e < E; ++e)
      std::copy(f.base + (size_t)e * f.estride, f.base + (size_t)e * f.estride + NP2 * NLEV,
                &pre[(size_t)e * NP2 * NLEV]);
#pragma omp parallel for
    for (int e = 0; e < E; ++e) {
      S* dst = f.base + (size_t)e * f.estride;
      for (int p = 0; p < NP2; ++p) {
        const int n = c.g_cnt[(size_t)e * 16 + p];
        for (int s = 0; s < n; ++s) {
          const int se = c.g_src_e[((size_t)e * 16 + p) * 3 + s];
          const int sp = c.g_src_p[((size_t)e * 16 + p) * 3 + s];
          const S* src = &pre[((size_t)se * NP2 + sp) * NLEV];
          for (int l = 0; l < NLEV; ++l) dst[p * NLEV + l] += src[l];
        }
      }
      if (rsmp)
        for (int p = 0; p < NP2; ++p) {
          const double r = c.rspheremp[(size_t)e * 16 + p];
          for (int l = 0; l < NLEV; ++l) dst[p * NLEV + l] *= r;
        }
    }
  }
}
void dss(const std::vector<FieldRef>& fields, bool rsmp) { dss_t<double>(fields, rsmp); }

// BoundaryExchange.cpp:620-849 on qlim [E][Q][2][NLEV]
void dss_minmax() {
  Ctx& c = C();
  const int E = c.E, Q = c.Q;
  std::vector<double> pre(c.qlim);
#pragma omp parallel for
  for (int e = 0; e < E; ++e)
    for (int q = 0; q < Q; ++q)
      for (int l = 0; l < NLEV; ++l)
        for (int slot = 0; slot < 8; ++slot) {
          const int r = c.conn[(e * 8 + slot) * 2];
          if (r < 0) continue;
          double& mx = c.qlim[(((size_t)e * Q + q) * 2 + 1) * NLEV + l];
          double& mn = c.qlim[(((size_t)e * Q + q) * 2 + 0) * NLEV + l];
          mx = std::max(mx, pre[(((size_t)r * Q + q) * 2 + 1) * NLEV + l]);
          mn = std::min(mn, pre[(((size_t)r * Q + q) * 2 + 0) * NLEV + l]);
        }
}

// ----------------------------------------------------------------------------------
// Caar (src/share/cxx/CaarFunctorImpl.hpp), one element.
// ----------------------------------------------------------------------------------
// Element constants the caar tendency reads.
struct CaarElem {
  const EM* m;
  const double* phis;      // [16]
  const double* fcor;      // [16]
  const double* spheremp;  // [16]
  double p_top;            // hyai(0) * ps0
  int rsplit;              // 0: vertically Eulerian
  const double* hybi;      // [NLEV + 1]
};

CaarElem caar_elem(const EM& m, int e) {
  Ctx& c = C();
  return {&m, &c.phis[(size_t)e * 16], &c.fcor[(size_t)e * 16], &c.spheremp[(size_t)e * 16],
          c.hyai0 * c.ps0, c.prm.rsplit, c.hybi};
}

// One caar stage of one element (CaarFunctorImpl.hpp:97-597):
// new = spheremp * (state(nm1) + dt * tendency(state(n0))), before the DSS.  TV is the
// virtual temperature (T itself when dry).  The outputs must not alias the inputs; vn0,
// omega_p, phi_out and eta_acc (diagnostics) may be null.  With rsplit == 0 the vertical
// velocity eta_dot_dpdn and the vertical advection of T and v enter the tendencies and
// eta_dot_dpdn accumulates into eta_acc.
template <class S>
void caar_core(const CaarElem& ce, const S* V0, const S* T0, const S* DP0, const S* TV,
               const S* Vm, const S* Tm, const S* DPm, double dt, S* v_new, S* t_new,
               S* dp_new, double eta_ave_w, S* vn0, S* omega_p, S* phi_out, S* eta_acc = nullptr) {
  const EM& m = *ce.m;
  const size_t N3 = NP2 * NLEV;
  std::vector<S> vdp(2 * N3), div_vdp(N3), pressure(N3), gradp(2 * N3), omega(N3),
      gradt(2 * N3), eg(2 * N3), ephi(N3), vort(N3), phi(N3), eta(N3, S(0.0)), t_vadv(N3, S(0.0)),
      v_vadv(2 * N3, S(0.0));
  // compute_temperature_div_vdp: CaarFunctorImpl.hpp:330-409
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      FV(vdp.data(), 0, p, l) = FV(V0, 0, p, l) * F(DP0, p, l);
      FV(vdp.data(), 1, p, l) = FV(V0, 1, p, l) * F(DP0, p, l);
      if (vn0) {
        FV(vn0, 0, p, l) += eta_ave_w * FV(vdp.data(), 0, p, l);
        FV(vn0, 1, p, l) += eta_ave_w * FV(vdp.data(), 1, p, l);
      }
    }
  divergence_sphere(m, vdp.data(), div_vdp.data(), NLEV);
  // compute_pressure (serial form, CaarFunctorImpl.hpp:618-647)
  for (int p = 0; p < NP2; ++p) {
    S dp_prev = 0.0;
    S p_prev = ce.p_top;
    for (int l = 0; l < NLEV; ++l) {
      F(pressure.data(), p, l) = p_prev + 0.5 * (dp_prev + F(DP0, p, l));
      p_prev = F(pressure.data(), p, l);
      dp_prev = F(DP0, p, l);
    }
  }
  // preq_hydrostatic (serial form, :686-730)
  for (int p = 0; p < NP2; ++p) {
    const double phis = ce.phis[p];
    S integration = 0.0;
    for (int l = NLEV - 1; l >= 0; --l) {
      const S r = Rgas * F(TV, p, l) * (F(DP0, p, l) * 0.5 / F(pressure.data(), p, l));
      F(phi.data(), p, l) = phis + 2.0 * integration + r;
      integration = integration + r;
    }
  }
  if (phi_out) std::copy(phi.begin(), phi.end(), phi_out);
  // preq_omega_ps (serial form, :848-889)
  gradient_sphere(m, pressure.data(), gradp.data(), NLEV);
  for (int p = 0; p < NP2; ++p) {
    S integration = 0.0;
    for (int l = 0; l < NLEV; ++l) {
      const S vgrad_p = FV(V0, 0, p, l) * FV(gradp.data(), 0, p, l) +
                        FV(V0, 1, p, l) * FV(gradp.data(), 1, p, l);
      const S dv = F(div_vdp.data(), p, l);
      F(omega.data(), p, l) = (vgrad_p - (integration + 0.5 * dv)) / F(pressure.data(), p, l);
      integration = integration + dv;
    }
  }
  // compute_phase_3 (:136-148): with rsplit == 0 first eta_dot_dpdn
  // (compute_eta_dot_dpdn_vertadv_euler, :262-300), preq_vertadv (:496-597) and
  // accumulate_eta_dot_dpdn (:236-248); then omega_p, T, v, dp3d
  if (ce.rsplit == 0) {
    for (int p = 0; p < NP2; ++p) {
      S sdot = 0.0;
      for (int k = 0; k < NLEV - 1; ++k) {
        sdot += F(div_vdp.data(), p, k);
        F(eta.data(), p, k + 1) = sdot;
      }
      sdot += F(div_vdp.data(), p, NLEV - 1);
      for (int k = 1; k < NLEV; ++k) F(eta.data(), p, k) = ce.hybi[k] * sdot - F(eta.data(), p, k);
      F(eta.data(), p, 0) = 0.0;
      // first level
      S facp = (0.5 * 1 / F(DP0, p, 0)) * F(eta.data(), p, 1);
      F(t_vadv.data(), p, 0) = facp * (F(T0, p, 1) - F(T0, p, 0));
      for (int c2 = 0; c2 < 2; ++c2)
        FV(v_vadv.data(), c2, p, 0) = facp * (FV(V0, c2, p, 1) - FV(V0, c2, p, 0));
      for (int k = 1; k < NLEV - 1; ++k) {
        facp = 0.5 * (1 / F(DP0, p, k)) * F(eta.data(), p, k + 1);
        const S facm = 0.5 * (1 / F(DP0, p, k)) * F(eta.data(), p, k);
        F(t_vadv.data(), p, k) = facp * (F(T0, p, k + 1) - F(T0, p, k)) +
                                 facm * (F(T0, p, k) - F(T0, p, k - 1));
        for (int c2 = 0; c2 < 2; ++c2)
          FV(v_vadv.data(), c2, p, k) = facp * (FV(V0, c2, p, k + 1) - FV(V0, c2, p, k)) +
                                        facm * (FV(V0, c2, p, k) - FV(V0, c2, p, k - 1));
      }
      const int kl = NLEV - 1;
      const S facm = (0.5 * (1 / F(DP0, p, kl))) * F(eta.data(), p, kl);
      F(t_vadv.data(), p, kl) = facm * (F(T0, p, kl) - F(T0, p, kl - 1));
      for (int c2 = 0; c2 < 2; ++c2)
        FV(v_vadv.data(), c2, p, kl) = facm * (FV(V0, c2, p, kl) - FV(V0, c2, p, kl - 1));
      if (eta_acc)
        for (int k = 0; k < NLEV; ++k) F(eta_acc, p, k) += eta_ave_w * F(eta.data(), p, k);
    }
  }
  if (omega_p)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l) F(omega_p, p, l) += eta_ave_w * F(omega.data(), p, l);
  // compute_temperature_np1 (:424-460)
  gradient_sphere(m, T0, gradt.data(), NLEV);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      const S vgrad_t = FV(V0, 0, p, l) * FV(gradt.data(), 0, p, l) +
                        FV(V0, 1, p, l) * FV(gradt.data(), 1, p, l);
      const S lead = ce.rsplit == 0 ? -F(t_vadv.data(), p, l) : S(0.0);
      const S ttens = (lead - vgrad_t) + kappa * F(TV, p, l) * F(omega.data(), p, l);
      S temp_np1 = ttens * dt + F(Tm, p, l);
      temp_np1 *= ce.spheremp[p];
      F(t_new, p, l) = temp_np1;
    }
  // compute_velocity_np1 (:183-232) with compute_energy_grad (:97-132)
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      const S r = Rgas * (F(TV, p, l) / F(pressure.data(), p, l));
      FV(eg.data(), 0, p, l) = r * FV(gradp.data(), 0, p, l);
      FV(eg.data(), 1, p, l) = r * FV(gradp.data(), 1, p, l);
      const S ke = 0.5 * (FV(V0, 0, p, l) * FV(V0, 0, p, l) + FV(V0, 1, p, l) * FV(V0, 1, p, l));
      F(ephi.data(), p, l) = ke + F(phi.data(), p, l);
    }
  gradient_sphere_update(m, ephi.data(), eg.data(), NLEV);
  vorticity_sphere(m, V0, vort.data(), NLEV);
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      F(vort.data(), p, l) += ce.fcor[p];
      S e0 = FV(eg.data(), 0, p, l), e1 = FV(eg.data(), 1, p, l);
      const S vo = F(vort.data(), p, l);
      const S va0 = ce.rsplit == 0 ? -FV(v_vadv.data(), 0, p, l) : S(0.0);
      const S va1 = ce.rsplit == 0 ? -FV(v_vadv.data(), 1, p, l) : S(0.0);
      e0 *= -1.0;
      e0 += va0 + FV(V0, 1, p, l) * vo;
      e1 *= -1.0;
      e1 += va1 - FV(V0, 0, p, l) * vo;
      e0 *= dt;
      e0 += FV(Vm, 0, p, l);
      e1 *= dt;
      e1 += FV(Vm, 1, p, l);
      const double smp = ce.spheremp[p];
      FV(v_new, 0, p, l) = smp * e0;
      FV(v_new, 1, p, l) = smp * e1;
    }
  // compute_dp3d_np1 (:462-493); eta_dot_dpdn is zero when rsplit > 0
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      S tmp = l + 1 < NLEV ? F(eta.data(), p, l + 1) : S(0.0);
      tmp += F(div_vdp.data(), p, l);
      tmp -= F(eta.data(), p, l);
      tmp = F(DPm, p, l) - tmp * dt;
      F(dp_new, p, l) = ce.spheremp[p] * tmp;
    }
}

void caar_element(int e, int nm1, int n0, int np1, double dt, double eta_ave_w, int n0_qdp) {
  Ctx& c = C();
  const EM m = metric(e);
  const size_t N3 = NP2 * NLEV;
  std::vector<double> tv(N3), t_new(N3), v_new(2 * N3), dp_new(N3);
  const double* T0 = &c.t[IS(e, n0, 0, 0)];
  const double* DP0 = &c.dp3d[IS(e, n0, 0, 0)];
  // virtual temperature (CaarFunctorImpl.hpp:330-360)
  for (int p = 0; p < NP2; ++p)
    for (int l = 0; l < NLEV; ++l) {
      if (n0_qdp < 0) {
        F(tv.data(), p, l) = F(T0, p, l);
      } else {
        double Qt = c.qdp[IQ(e, n0_qdp, 0, p, l, c.Q)] / F(DP0, p, l);
        Qt *= (Rwater_vapor / Rgas - 1.0);
        Qt += 1.0;
        F(tv.data(), p, l) = F(T0, p, l) * Qt;
      }
    }
  caar_core<double>(caar_elem(m, e), &c.v[IV(e, n0, 0, 0, 0)], T0, DP0, tv.data(),
                    &c.v[IV(e, nm1, 0, 0, 0)], &c.t[IS(e, nm1, 0, 0)], &c.dp3d[IS(e, nm1, 0, 0)],
                    dt, v_new.data(), t_new.data(), dp_new.data(), eta_ave_w,
                    &c.vn0[I3V(e, 0, 0, 0)], &c.omega_p[I3(e, 0, 0)], &c.phi[I3(e, 0, 0)],
                    &c.eta_dot_dpdn[I3(e, 0, 0)]);
  std::memcpy(&c.t[IS(e, np1, 0, 0)], t_new.data(), sizeof(double) * N3);
  std::memcpy(&c.v[IV(e, np1, 0, 0, 0)], v_new.data(), sizeof(double) * 2 * N3);
  std::memcpy(&c.dp3d[IS(e, np1, 0, 0)], dp_new.data(), sizeof(double) * N3);
}

void caar_run(int nm1, int n0, int np1, double dt, double eta_ave_w, int n0_qdp) {
  Ctx& c = C();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < c.E; ++e) caar_element(e, nm1, n0, np1, dt, eta_ave_w, n0_qdp);
  // BoundaryExchange registered in CaarFunctorImpl.hpp:68-79: v(2), T, dp3d
  const size_t sv = (size_t)NTL * 2 * NP2 * NLEV, ss = (size_t)NTL * NP2 * NLEV;
  dss({{&c.v[IV(0, np1, 0, 0, 0)], sv}, {&c.v[IV(0, np1, 1, 0, 0)], sv},
       {&c.t[IS(0, np1, 0, 0)], ss}, {&c.dp3d[IS(0, np1, 0, 0)], ss}},
      true);
}

// prim_advance_exp.cpp:113-161
void u3_5stage(int nm1, int n0, int np1, int n0_qdp, double dt, double w) {
  Ctx& c = C();
  caar_run(n0, n0, nm1, dt / 5.0, w / 4.0, n0_qdp);
  caar_run(n0, nm1, np1, dt / 5.0, 0.0, n0_qdp);
  caar_run(n0, np1, np1, dt / 3.0, 0.0, n0_qdp);
  caar_run(n0, np1, np1, 2.0 * dt / 3.0, 0.0, n0_qdp);
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l) {
        double& t = c.t[IS(e, nm1, p, l)];
        t = (5.0 * t - c.t[IS(e, n0, p, l)]) / 4.0;
        double& v0 = c.v[IV(e, nm1, 0, p, l)];
        v0 = (5.0 * v0 - c.v[IV(e, n0, 0, p, l)]) / 4.0;
        double& v1 = c.v[IV(e, nm1, 1, p, l)];
        v1 = (5.0 * v1 - c.v[IV(e, n0, 1, p, l)]) / 4.0;
        double& d = c.dp3d[IS(e, nm1, p, l)];
        d = (5.0 * d - c.dp3d[IS(e, n0, p, l)]) / 4.0;
      }
  caar_run(nm1, np1, np1, 3.0 * dt / 4.0, 3.0 * w / 4.0, n0_qdp);
}

// ----------------------------------------------------------------------------------
// Hyperviscosity (src/share/cxx/HyperviscosityFunctorImpl.{hpp,cpp})
// ----------------------------------------------------------------------------------
// TagFirstLaplaceHV, one element (HyperviscosityFunctorImpl.hpp:72-90).
template <class S>
void hv_first_laplace(const EM& m, double nu_ratio1, const S* T, const S* DP, const S* V,
                      S* ttens, S* dptens, S* vtens) {
  laplace_simple(m, T, ttens, NLEV);
  laplace_simple(m, DP, dptens, NLEV);
  vlaplace_sphere_wk_contra(m, nu_ratio1, V, vtens, NLEV);
}

// TagSecondLaplaceConstHV, one element, in place (HyperviscosityFunctorImpl.hpp:92-109).
template <class S>
void hv_second_laplace_const(const EM& m, double nu_ratio2, S* ttens, S* dptens, S* vtens) {
  laplace_simple(m, ttens, ttens, NLEV);
  laplace_simple(m, dptens, dptens, NLEV);
  vlaplace_sphere_wk_contra(m, nu_ratio2, vtens, vtens, NLEV);
}

// TagHyperPreExchange without the dpdiss diagnostics (HyperviscosityFunctorImpl.hpp:
// 161-257): scale by -nu, add the nu_top sponge on the top 3 levels, and form the
// spheremp-weighted dp3d update.
template <class S>
void hv_pre_exchange(const EM& m, const Params& pr, double dt, const S* T, const S* DP,
                     const S* V, S* ttens, S* dptens, S* vtens) {
  const size_t N3 = NP2 * NLEV;
  const double nu_scale_top[3] = {4.0 * pr.nu_top, 2.0 * pr.nu_top, 1.0 * pr.nu_top};
  std::vector<S> lap_v(2 * N3), lap_t(N3), lap_dp(N3);
  if (pr.nu_top > 0) {
    vlaplace_sphere_wk_contra(m, 1.0, V, lap_v.data(), 3);
    laplace_simple(m, T, lap_t.data(), 3);
    laplace_simple(m, DP, lap_dp.data(), 3);
  }
  for (int p = 0; p < NP2; ++p) {
    for (int l = 0; l < NLEV; ++l) {
      FV(vtens, 0, p, l) *= -pr.nu;
      FV(vtens, 1, p, l) *= -pr.nu;
      F(ttens, p, l) *= -pr.nu_s;
      F(dptens, p, l) *= -pr.nu_p;
    }
    if (pr.nu_top > 0)
      for (int l = 0; l < 3; ++l) {
        FV(vtens, 0, p, l) += nu_scale_top[l] * FV(lap_v.data(), 0, p, l);
        FV(vtens, 1, p, l) += nu_scale_top[l] * FV(lap_v.data(), 1, p, l);
        F(ttens, p, l) += nu_scale_top[l] * F(lap_t.data(), p, l);
        F(dptens, p, l) += nu_scale_top[l] * F(lap_dp.data(), p, l);
      }
    for (int l = 0; l < NLEV; ++l) {
      F(dptens, p, l) *= dt;
      F(dptens, p, l) += F(DP, p, l) * m.spheremp[p];
    }
  }
}

// TagUpdateStates, one element (HyperviscosityFunctorImpl.hpp:134-158), after the DSS.
template <class S>
void hv_update(const double* rsmp_e, double dt, S* V, S* T, S* DP, S* vtens, S* ttens,
               const S* dptens) {
  for (int p = 0; p < NP2; ++p) {
    const double rsmp = rsmp_e[p];
    for (int l = 0; l < NLEV; ++l) {
      S& vt0 = FV(vtens, 0, p, l);
      S& vt1 = FV(vtens, 1, p, l);
      vt0 = (dt * vt0 * rsmp);
      vt1 = (dt * vt1 * rsmp);
      S& v0 = FV(V, 0, p, l);
      S& v1 = FV(V, 1, p, l);
      v0 += vt0;
      v1 += vt1;
      S& tt = F(ttens, p, l);
      tt = (dt * tt * rsmp);
      const S heating = vt0 * v0 + vt1 * v1;
      S& t = F(T, p, l);
      t = t + tt - heating / cp;
      F(DP, p, l) = (F(dptens, p, l) * rsmp);
    }
  }
}

void hypervis_run(int np1, double dt_in, double eta_ave_w) {
  Ctx& c = C();
  const Params& pr = c.prm;
  const int hsub = pr.hypervis_subcycle;
  const double dt = dt_in / hsub;
  const size_t N3 = NP2 * NLEV;
  for (int icycle = 0; icycle < hsub; ++icycle) {
    // TagFirstLaplaceHV
#pragma omp parallel for
    for (int e = 0; e < c.E; ++e)
      hv_first_laplace(metric(e), pr.nu_ratio1, &c.t[IS(e, np1, 0, 0)],
                       &c.dp3d[IS(e, np1, 0, 0)], &c.v[IV(e, np1, 0, 0, 0)],
                       &c.ttens[I3(e, 0, 0)], &c.dptens[I3(e, 0, 0)], &c.vtens[I3V(e, 0, 0, 0)]);
    const std::vector<FieldRef> tens = {{&c.vtens[I3V(0, 0, 0, 0)], 2 * N3},
                                        {&c.vtens[I3V(0, 1, 0, 0)], 2 * N3},
                                        {&c.ttens[0], N3},
                                        {&c.dptens[0], N3}};
    dss(tens, true);
    // TagSecondLaplaceConstHV / TensorHV
#pragma omp parallel for
    for (int e = 0; e < c.E; ++e) {
      const EM m = metric(e);
      if (c.consthv) {
        hv_second_laplace_const(m, pr.nu_ratio2, &c.ttens[I3(e, 0, 0)], &c.dptens[I3(e, 0, 0)],
                                &c.vtens[I3V(e, 0, 0, 0)]);
      } else {
        laplace_tensor(m, &c.ttens[I3(e, 0, 0)], &c.ttens[I3(e, 0, 0)], NLEV);
        laplace_tensor(m, &c.dptens[I3(e, 0, 0)], &c.dptens[I3(e, 0, 0)], NLEV);
        vlaplace_sphere_wk_cartesian(m, &c.vtens[I3V(e, 0, 0, 0)], &c.vtens[I3V(e, 0, 0, 0)],
                                     NLEV);
      }
    }
    // TagHyperPreExchange (HyperviscosityFunctorImpl.hpp:161-257)
#pragma omp parallel for
    for (int e = 0; e < c.E; ++e) {
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l) {
          c.dpdiss_ave[I3(e, p, l)] += eta_ave_w * c.dp3d[IS(e, np1, p, l)] / hsub;
          c.dpdiss_bih[I3(e, p, l)] += eta_ave_w * c.dptens[I3(e, p, l)] / hsub;
        }
      hv_pre_exchange(metric(e), pr, dt, &c.t[IS(e, np1, 0, 0)], &c.dp3d[IS(e, np1, 0, 0)],
                      &c.v[IV(e, np1, 0, 0, 0)], &c.ttens[I3(e, 0, 0)], &c.dptens[I3(e, 0, 0)],
                      &c.vtens[I3V(e, 0, 0, 0)]);
    }
    dss(tens, false);
    // TagUpdateStates (HyperviscosityFunctorImpl.hpp:134-158)
#pragma omp parallel for
    for (int e = 0; e < c.E; ++e)
      hv_update(&c.rspheremp[(size_t)e * 16], dt, &c.v[IV(e, np1, 0, 0, 0)],
                &c.t[IS(e, np1, 0, 0)], &c.dp3d[IS(e, np1, 0, 0)], &c.vtens[I3V(e, 0, 0, 0)],
                &c.ttens[I3(e, 0, 0)], &c.dptens[I3(e, 0, 0)]);
  }
}

// ----------------------------------------------------------------------------------
// Euler step (src/share/cxx/EulerStepFunctorImpl.hpp)
// ----------------------------------------------------------------------------------

// with_limiter_shell + Limit functors (EulerStepFunctorImpl.hpp:693-884); team form,
// reductions in k order.  x, c are [16]; returns with x limited.
void limiter_level(int option, double* x, const double* cw, double& minp_io, double& maxp_io) {
  double s0 = 0, s1 = 0;
  for (int k = 0; k < NP2; ++k) {
    s0 += x[k] * cw[k];
    s1 += cw[k];
  }
  if (s1 <= 0) return;
  double minp = minp_io, maxp = maxp_io;
  if (minp < 0) minp = minp_io = 0;
  if (s0 < minp * s1) minp = minp_io = s0 / s1;
  if (s0 > maxp * s1) maxp = maxp_io = s0 / s1;
  const double mass = s0;
  if (option == 8) {
    const int maxiter = NP2 - 1;
    const double tol_limiter = 5e-14;
    for (int iter = 0; iter < maxiter; ++iter) {
      double addmass = 0;
      for (int k = 0; k < NP2; ++k) {
        double delta = 0;
        if (x[k] > maxp) {
          delta = x[k] - maxp;
          x[k] = maxp;
        } else if (x[k] < minp) {
          delta = x[k] - minp;
          x[k] = minp;
        }
        addmass += delta * cw[k];
      }
      if (std::abs(addmass) <= tol_limiter * std::abs(mass)) break;
      if (addmass > 0) {
        double weightssum = 0;
        for (int k = 0; k < NP2; ++k)
          if (x[k] < maxp) weightssum += cw[k];
        if (weightssum == 0) break;  // see the serial limiter's f != 0 guard
        const double adw = addmass / weightssum;
        for (int k = 0; k < NP2; ++k) x[k] += (x[k] < maxp) ? adw : 0;
      } else {
        double weightssum = 0;
        for (int k = 0; k < NP2; ++k)
          if (x[k] > minp) weightssum += cw[k];
        if (weightssum == 0) break;
        const double adw = addmass / weightssum;
        for (int k = 0; k < NP2; ++k) x[k] += (x[k] > minp) ? adw : 0;
      }
    }
  } else {  // option 9, clip and assured sum
    double addmass = 0;
    for (int k = 0; k < NP2; ++k) {
      double delta = 0;
      if (x[k] > maxp) {
        delta = x[k] - maxp;
        x[k] = maxp;
      } else if (x[k] < minp) {
        delta = x[k] - minp;
        x[k] = minp;
      }
      addmass += delta * cw[k];
    }
    if (addmass == 0) return;
    if (addmass > 0) {
      double fac = 0;
      for (int k = 0; k < NP2; ++k) fac += cw[k] * (maxp - x[k]);
      if (fac > 0) {
        fac = addmass / fac;
        for (int k = 0; k < NP2; ++k) x[k] += fac * (maxp - x[k]);
      }
    } else {
      double fac = 0;
      for (int k = 0; k < NP2; ++k) fac += cw[k] * (x[k] - minp);
      if (fac > 0) {
        fac = addmass / fac;
        for (int k = 0; k < NP2; ++k) x[k] += fac * (x[k] - minp);
      }
    }
  }
}

void euler_step(int np1_qdp, int n0_qdp, double dt, double rhs_multiplier, int dssopt) {
  Ctx& c = C();
  const Params& pr = c.prm;
  const int E = c.E, Q = c.Q;
  double rhs_viss = 0.0;
  const size_t N3 = NP2 * NLEV;
  // compute_dp (EulerStepFunctorImpl.hpp:405-435): buffer "pressure" holds dp
#pragma omp parallel for
  for (int e = 0; e < E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l)
        c.dp_buf[I3(e, p, l)] =
            c.derived_dp[I3(e, p, l)] - (rhs_multiplier * dt) * c.divdp_proj[I3(e, p, l)];
  // compute_qmin_qmax (:437-482)
#pragma omp parallel for collapse(2)
  for (int e = 0; e < E; ++e)
    for (int q = 0; q < Q; ++q) {
      double* qb = &c.qtens_bih[((size_t)e * Q + q) * N3];
      double* ql = &c.qlim[((size_t)e * Q + q) * 2 * NLEV];
      for (int l = 0; l < NLEV; ++l) {
        if (rhs_multiplier != 1.0) {
          const double v = c.qdp[IQ(e, n0_qdp, q, 0, l, Q)] / c.dp_buf[I3(e, 0, l)];
          qb[l] = v;
          ql[l] = v;
          ql[NLEV + l] = v;
        }
        for (int p = 0; p < NP2; ++p) {
          const double v = c.qdp[IQ(e, n0_qdp, q, p, l, Q)] / c.dp_buf[I3(e, p, l)];
          qb[p * NLEV + l] = v;
          ql[l] = std::min(ql[l], v);
          ql[NLEV + l] = std::max(ql[NLEV + l], v);
        }
      }
    }
  if (rhs_multiplier == 0.0) {
    dss_minmax();
  } else if (rhs_multiplier == 2.0) {
    // minmax_and_biharmonic (:493-499); min/max of the pre-biharmonic qlim
    rhs_viss = 3.0;
    // compute_biharmonic_pre (BIHPreNup / BIHPreNoNup)
#pragma omp parallel for collapse(2)
    for (int e = 0; e < E; ++e)
      for (int q = 0; q < Q; ++q) {
        const EM m = metric(e);
        double* qb = &c.qtens_bih[((size_t)e * Q + q) * N3];
        if (pr.nu_p > 0)
          for (int p = 0; p < NP2; ++p)
            for (int l = 0; l < NLEV; ++l)
              qb[p * NLEV + l] = qb[p * NLEV + l] * c.dpdiss_ave[I3(e, p, l)] / c.dp0[l];
        laplace_simple(m, qb, qb, NLEV);
      }
    std::vector<FieldRef> f;
    for (int q = 0; q < Q; ++q) f.push_back({&c.qtens_bih[(size_t)q * N3], (size_t)Q * N3});
    dss(f, true);
    // compute_biharmonic_post (BIHPostConstHV / TensorHV + rhsviss_adjustment)
    const double fac = -rhs_viss * dt * pr.nu_q;
#pragma omp parallel for collapse(2)
    for (int e = 0; e < E; ++e)
      for (int q = 0; q < Q; ++q) {
        const EM m = metric(e);
        double* qb = &c.qtens_bih[((size_t)e * Q + q) * N3];
        if (c.consthv) laplace_simple(m, qb, qb, NLEV);
        else laplace_tensor(m, qb, qb, NLEV);
        for (int p = 0; p < NP2; ++p)
          for (int l = 0; l < NLEV; ++l)
            qb[p * NLEV + l] = (fac * c.dp0[l] * qb[p * NLEV + l] / m.spheremp[p]);
      }
    dss_minmax();
  }
  // advect_and_limit: AALSetupPhase (compute_2d_advection_step, :585-631)
  const bool add_ps_diss = pr.nu_p > 0 && rhs_viss != 0.0;
  const double diss_fac = add_ps_diss ? -rhs_viss * dt * pr.nu_q : 0;
  std::vector<double>& f_dss = dssopt == 0 ? c.eta_dot_dpdn : dssopt == 1 ? c.omega_p : c.divdp_proj;
#pragma omp parallel for
  for (int e = 0; e < E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l) {
        const double dp = c.dp_buf[I3(e, p, l)];
        c.vstar[I3V(e, 0, p, l)] = c.vn0[I3V(e, 0, p, l)] / dp;
        c.vstar[I3V(e, 1, p, l)] = c.vn0[I3V(e, 1, p, l)] / dp;
        c.dpdissk[I3(e, p, l)] = dp - dt * c.divdp[I3(e, p, l)];
        if (add_ps_diss)
          c.dpdissk[I3(e, p, l)] +=
              diss_fac * c.dpdiss_bih[I3(e, p, l)] / c.spheremp[(size_t)e * 16 + p];
        f_dss[I3(e, p, l)] *= c.spheremp[(size_t)e * 16 + p];
      }
  // AALTracerPhase: compute_qtens, limiter, apply_spheremp (:563-582, 633-687)
#pragma omp parallel for collapse(2)
  for (int e = 0; e < E; ++e)
    for (int q = 0; q < Q; ++q) {
      const EM m = metric(e);
      double* qt = &c.qtens_bih[((size_t)e * Q + q) * N3];
      divergence_sphere_update(m, -dt, rhs_viss != 0.0, &c.vstar[I3V(e, 0, 0, 0)],
                               &c.qdp[IQ(e, n0_qdp, q, 0, 0, Q)], qt, NLEV);
      if (pr.limiter_option == 8 || pr.limiter_option == 9) {
        double* ql = &c.qlim[((size_t)e * Q + q) * 2 * NLEV];
        for (int l = 0; l < NLEV; ++l) {
          double x[NP2], cw[NP2];
          for (int k = 0; k < NP2; ++k) {
            const double dpm = c.dpdissk[I3(e, k, l)];
            cw[k] = m.spheremp[k] * dpm;
            x[k] = qt[k * NLEV + l] / dpm;
          }
          double s1 = 0;
          for (int k = 0; k < NP2; ++k) s1 += cw[k];
          if (s1 <= 0) continue;
          limiter_level(pr.limiter_option, x, cw, ql[l], ql[NLEV + l]);
          for (int k = 0; k < NP2; ++k) qt[k * NLEV + l] = x[k] * c.dpdissk[I3(e, k, l)];
        }
      }
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l)
          c.qdp[IQ(e, np1_qdp, q, p, l, Q)] = m.spheremp[p] * qt[p * NLEV + l];
    }
  // exchange_qdp_dss_var (:501-504): Qdp(np1) and the DSS-option field, rspheremp
  std::vector<FieldRef> f;
  for (int q = 0; q < Q; ++q) f.push_back({&c.qdp[IQ(0, np1_qdp, q, 0, 0, Q)], (size_t)QTL * Q * N3});
  f.push_back({f_dss.data(), N3});
  dss(f, true);
}

void precompute_divdp() {  // EulerStepFunctorImpl.hpp:348-377
  Ctx& c = C();
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e) {
    const EM m = metric(e);
    divergence_sphere(m, &c.vn0[I3V(e, 0, 0, 0)], &c.divdp[I3(e, 0, 0)], NLEV);
    std::memcpy(&c.divdp_proj[I3(e, 0, 0)], &c.divdp[I3(e, 0, 0)], sizeof(double) * NP2 * NLEV);
  }
}

void qdp_time_avg(int n0_qdp, int np1_qdp) {  // EulerStepFunctorImpl.hpp:379-403
  Ctx& c = C();
  const double rkstage = 3.0;
#pragma omp parallel for collapse(2)
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < c.Q; ++q)
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l) {
          double& a = c.qdp[IQ(e, np1_qdp, q, p, l, c.Q)];
          a = (c.qdp[IQ(e, n0_qdp, q, p, l, c.Q)] + (rkstage - 1) * a) / rkstage;
        }
}

void tracers_rk2(double dt) {  // prim_advec_tracers_remap.cpp:32-90
  Ctx& c = C();
  c.tl.update_tracers_levels(c.prm.qsplit);
  precompute_divdp();
  euler_step(c.tl.np1_qdp, c.tl.n0_qdp, dt / 2.0, 0.0, 2);
  euler_step(c.tl.np1_qdp, c.tl.np1_qdp, dt / 2.0, 1.0, 0);
  euler_step(c.tl.np1_qdp, c.tl.np1_qdp, dt / 2.0, 2.0, 1);
  qdp_time_avg(c.tl.n0_qdp, c.tl.np1_qdp);
}

// ----------------------------------------------------------------------------------
// PPM vertical remap (src/share/cxx/RemapFunctor.hpp, PpmRemap.hpp); rsplit > 0.
// Padded arrays use A(m) = a[m + 2] for m in [-2, NLEV+1].
// ----------------------------------------------------------------------------------
template <class S>
struct ColumnGridT {
  S pio[NLEV + 2], pin[NLEV + 1], dpo[NLEV + 4], z2[NLEV];
  int kid[NLEV];
  S g[10][NLEV + 2];
};
using ColumnGrid = ColumnGridT<double>;

template <class S>
void ppm_grids(const S* src, const S* tgt, ColumnGridT<S>& G) {
  // compute_partitions (PpmRemap.hpp:488-575)
  S acc = 0.0;
  for (int k = 0; k < NLEV; ++k) {
    G.pio[k] = acc;
    acc += src[k];
  }
  acc = 0.0;
  for (int k = 0; k < NLEV; ++k) {
    G.pin[k] = acc;
    acc += tgt[k];
  }
  G.pio[NLEV] = G.pio[NLEV - 1] + src[NLEV - 1];
  G.pin[NLEV] = G.pin[NLEV - 1] + tgt[NLEV - 1];
  G.pio[NLEV + 1] = G.pio[NLEV] + 1.0;
  G.pin[NLEV] = G.pio[NLEV];
  S* D = G.dpo + 2;
  for (int k = 0; k < NLEV; ++k) D[k] = src[k];
  for (int k = 0; k < 2; ++k) {
    D[-1 - k] = D[k];
    D[NLEV + k] = D[NLEV - 1 - k];
  }
  // compute_integral_bounds (:577-648)
  for (int k = 0; k < NLEV; ++k) {
    int kk = k + 1;
    while (kk < NLEV + 2 && G.pio[kk - 1] <= G.pin[k + 1]) kk++;
    kk--;
    if (kk == NLEV + 1) kk = NLEV;
    if (kk < 1) kk = 1;  // invalid (non-monotone) source grid; flagged by the caller
    G.kid[k] = kk - 1;
    G.z2[k] = (G.pin[k + 1] - (G.pio[kk - 1] + G.pio[kk]) * 0.5) / D[kk - 1];
  }
  // compute_grids (:355-413); dx(j + 1 + off) = D(j - 1)
  for (int j = 0; j < NLEV + 2; ++j) {
    G.g[0][j] = D[j - 1] / (D[j - 2] + D[j - 1] + D[j]);
    G.g[1][j] = (2.0 * D[j - 2] + D[j - 1]) / (D[j - 1] + D[j]);
    G.g[2][j] = (D[j - 1] + 2.0 * D[j]) / (D[j - 2] + D[j - 1]);
  }
  for (int j = 0; j < NLEV + 1; ++j) {
    G.g[3][j] = D[j - 1] / (D[j - 1] + D[j]);
    G.g[4][j] = 1.0 / (D[j - 2] + D[j - 1] + D[j] + D[j + 1]);
    G.g[5][j] = (2.0 * D[j - 1] * D[j]) / (D[j - 1] + D[j]);
    G.g[6][j] = (D[j - 2] + D[j - 1]) / (2.0 * D[j - 1] + D[j]);
    G.g[7][j] = (D[j + 1] + D[j]) / (2.0 * D[j] + D[j - 1]);
    G.g[8][j] = D[j - 1] * (D[j - 2] + D[j - 1]) / (2.0 * D[j - 1] + D[j]);
    G.g[9][j] = D[j] * (D[j] + D[j + 1]) / (D[j - 1] + 2.0 * D[j]);
  }
}

template <class S>
inline S integrate_parabola(const S& sq, const S& lin, const S& cst, double x1, const S& x2) {
  return (cst * (x2 - x1) + lin * (x2 * x2 - x1 * x1) / 2.0) + sq * (x2 * x2 * x2 - x1 * x1 * x1) / 3.0;
}

// compute_remap_phase + compute_ppm + compute_remap (PpmRemap.hpp:202-483)
template <class S>
void ppm_remap_column(const ColumnGridT<S>& G, int remap_alg, S* q /* [NLEV] */) {
  const S* D = G.dpo + 2;
  S a_[NLEV + 4];
  S* A = a_ + 2;
  S mass[NLEV + 2];
  S dma[NLEV + 2], ai[NLEV + 1], coef[3][NLEV];
  for (int k = 0; k < NLEV; ++k) A[k] = q[k] / D[k];
  if (remap_alg == 3) {
    for (int k = 0; k < 2; ++k) {
      A[-1 - k] = A[0];
      A[NLEV + k] = A[NLEV - 1];
    }
  } else {
    for (int k = 0; k < 2; ++k) {
      A[-1 - k] = A[k];
      A[NLEV + k] = A[NLEV - 1 - k];
    }
  }
  S acc = 0.0;
  for (int k = 0; k < NLEV; ++k) {
    mass[k + 1] = acc;
    acc += q[k];
  }
  mass[0] = 0.0;
  mass[NLEV + 1] = mass[NLEV] + q[NLEV - 1];
  for (int j = 0; j < NLEV + 2; ++j) {
    if ((A[j] - A[j - 1]) * (A[j - 1] - A[j - 2]) > 0.0) {
      const S da = G.g[0][j] * (G.g[1][j] * (A[j] - A[j - 1]) + G.g[2][j] * (A[j - 1] - A[j - 2]));
      dma[j] = std::min(std::min(sabs(da), 2.0 * sabs(A[j - 1] - A[j - 2])),
                        2.0 * sabs(A[j] - A[j - 1])) *
               std::copysign(1.0, val(da));
    } else {
      dma[j] = 0.0;
    }
  }
  for (int j = 0; j < NLEV + 1; ++j) {
    ai[j] = A[j - 1] + G.g[3][j] * (A[j] - A[j - 1]) +
            G.g[4][j] * (G.g[5][j] * (G.g[6][j] - G.g[7][j]) * (A[j] - A[j - 1]) -
                         G.g[8][j] * dma[j + 1] + G.g[9][j] * dma[j]);
  }
  for (int jp = 0; jp < NLEV; ++jp) {
    const int j = jp + 1;
    S al = ai[j - 1], ar = ai[j];
    const S cm = A[j - 1];
    if ((ar - cm) * (cm - al) <= 0.) {
      al = cm;
      ar = cm;
    }
    if ((ar - al) * (cm - (al + ar) / 2.0) > (ar - al) * (ar - al) / 6.0) al = 3.0 * cm - 2.0 * ar;
    if ((ar - al) * (cm - (al + ar) / 2.0) < -(ar - al) * (ar - al) / 6.0) ar = 3.0 * cm - 2.0 * al;
    coef[0][jp] = 1.5 * cm - (al + ar) / 4.0;
    coef[1][jp] = ar - al;
    coef[2][jp] = 3.0 * (-2.0 * cm + (al + ar));
  }
  if (remap_alg == 2) {  // PpmFixedParabola::apply_ppm_boundary
    coef[0][0] = A[0];
    coef[0][1] = A[1];
    coef[0][NLEV - 2] = A[NLEV - 2];
    coef[0][NLEV - 1] = A[NLEV - 1];
    coef[1][0] = coef[1][1] = coef[2][0] = coef[2][1] = 0.0;
    coef[1][NLEV - 2] = coef[1][NLEV - 1] = coef[2][NLEV - 2] = coef[2][NLEV - 1] = 0.0;
  }
  // compute_remap, GPU form (each level recomputes the lower interface mass)
  auto cmass = [&](int kk, const S& x2) {
    const S integral = integrate_parabola(coef[2][kk], coef[1][kk], coef[0][kk], -0.5, x2);
    return mass[kk + 1] + integral * D[kk];
  };
  S out[NLEV];
  for (int k = 0; k < NLEV; ++k) {
    const S m1 = k > 0 ? cmass(G.kid[k - 1], G.z2[k - 1]) : S(0.0);
    const S m2 = cmass(G.kid[k], G.z2[k]);
    out[k] = m2 - m1;
  }
  for (int k = 0; k < NLEV; ++k) q[k] = out[k];
}

// compute_ps_v, the target thicknesses from the hybrid coordinate and the PPM grids of
// one column (RemapFunctor.hpp:225-240, 364-384; PpmRemap.hpp:488-648); returns ps.
template <class S>
S remap_target(const S* src, S* tgt, ColumnGridT<S>& G) {
  Ctx& c = C();
  S ps = 0.0;
  for (int l = 0; l < NLEV; ++l) ps += src[l];
  ps += c.hyai0 * c.ps0;
  for (int l = 0; l < NLEV; ++l)
    tgt[l] = (c.hyai[l + 1] - c.hyai[l]) * c.ps0 + (c.hybi[l + 1] - c.hybi[l]) * ps;
  ppm_grids(src, tgt, G);
  return ps;
}

// Remap of one state variable of a column as a mass-weighted quantity: v and T are
// multiplied by dp3d before and divided by the target thickness after
// (RemapFunctor.hpp:243-256, 285-297, 386-420).
template <class S>
void remap_state_var(const ColumnGridT<S>& G, int remap_alg, const S* src, const S* tgt,
                     S* x) {
  S col[NLEV];
  for (int l = 0; l < NLEV; ++l) col[l] = x[l] * src[l];
  ppm_remap_column(G, remap_alg, col);
  for (int l = 0; l < NLEV; ++l) x[l] = col[l] / tgt[l];
}

void remap_run(int np1, int n0_qdp, double dt) {  // RemapFunctor::run_remap
  Ctx& c = C();
  const int E = c.E, Q = c.Q;
  int valid = 1;
#pragma omp parallel for reduction(& : valid)
  for (int e = 0; e < E; ++e) {
    for (int p = 0; p < NP2; ++p) {
      double src[NLEV], tgt[NLEV];
      ColumnGrid G;
      if (c.prm.rsplit > 0) {
        for (int l = 0; l < NLEV; ++l) {
          src[l] = c.dp3d[IS(e, np1, p, l)];
          if (std::isnan(src[l]) || src[l] < 0.0) valid = 0;
        }
        c.ps_v[((size_t)e * NTL + np1) * NP2 + p] = remap_target(src, tgt, G);
        remap_state_var(G, c.prm.remap_alg, src, tgt, &c.v[IV(e, np1, 0, p, 0)]);
        remap_state_var(G, c.prm.remap_alg, src, tgt, &c.v[IV(e, np1, 1, p, 0)]);
        remap_state_var(G, c.prm.remap_alg, src, tgt, &c.t[IS(e, np1, p, 0)]);
      } else {
        // vertically Eulerian: ps from dp3d(np1), tracers only, from the source
        // thickness tgt + dt (eta_dot_dpdn(k+1) - eta_dot_dpdn(k)) (RemapFunctor.hpp:42-100)
        double ps = 0.0;
        for (int l = 0; l < NLEV; ++l) ps += c.dp3d[IS(e, np1, p, l)];
        ps += c.hyai0 * c.ps0;
        c.ps_v[((size_t)e * NTL + np1) * NP2 + p] = ps;
        for (int l = 0; l < NLEV; ++l) {
          tgt[l] = (c.hyai[l + 1] - c.hyai[l]) * c.ps0 + (c.hybi[l + 1] - c.hybi[l]) * ps;
          const double en = l + 1 < NLEV ? c.eta_dot_dpdn[I3(e, p, l + 1)] : 0.0;
          src[l] = tgt[l] + dt * (en - c.eta_dot_dpdn[I3(e, p, l)]);
          if (std::isnan(src[l]) || src[l] < 0.0) valid = 0;
        }
        ppm_grids(src, tgt, G);
      }
      double col[NLEV];
      for (int q = 0; q < Q; ++q) {
        double* base = &c.qdp[IQ(e, n0_qdp, q, p, 0, Q)];
        for (int l = 0; l < NLEV; ++l) col[l] = base[l];
        ppm_remap_column(G, c.prm.remap_alg, col);
        for (int l = 0; l < NLEV; ++l) base[l] = col[l];
      }
    }
  }
  c.valid_remap = valid;
}

// prim_step.cpp:20-103
void prim_step(double dt) {
  Ctx& c = C();
  const Params& pr = c.prm;
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l) {
        c.eta_dot_dpdn[I3(e, p, l)] = 0;
        c.vn0[I3V(e, 0, p, l)] = 0;
        c.vn0[I3V(e, 1, p, l)] = 0;
        c.omega_p[I3(e, p, l)] = 0;
        if (pr.nu_p > 0) {
          c.dpdiss_ave[I3(e, p, l)] = 0;
          c.dpdiss_bih[I3(e, p, l)] = 0;
        }
        c.derived_dp[I3(e, p, l)] = c.dp3d[IS(e, c.tl.n0, p, l)];
      }
  for (int n = 0; n < pr.qsplit; ++n) {
    if (n > 0) c.tl.update_dynamics_levels();
    int n0_qdp = -1;
    if (pr.moist) {
      c.tl.update_tracers_levels(pr.qsplit);
      n0_qdp = c.tl.n0_qdp;
    }
    const double w = 1.0 / pr.qsplit;
    u3_5stage(c.tl.nm1, c.tl.n0, c.tl.np1, n0_qdp, dt, w);
    hypervis_run(c.tl.np1, dt, w);
  }
  if (pr.qsize > 0) tracers_rk2(dt * pr.qsplit);
}

// CAM forcing (CamForcing.cpp:20-170): state_forcing adds dt FT, dt FM to T, v at n0;
// with tracers (ftype 0) tracer_forcing adds dt FQ to Qdp at n0_qdp, clipped so that no
// forcing makes Qdp negative, moves ps_v by the clipped increments of tracer 0 when
// moist, and recomputes Q.
void apply_cam_forcing(double dt, bool tracers) {
  Ctx& c = C();
  if (c.ft.empty()) return;  // no forcing pushed
  const int n0 = c.tl.n0, nq = c.tl.n0_qdp, Q = c.Q;
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l) {
        c.t[IS(e, n0, p, l)] += dt * c.ft[I3(e, p, l)];
        c.v[IV(e, n0, 0, p, l)] += dt * c.fm[I3V(e, 0, p, l)];
        c.v[IV(e, n0, 1, p, l)] += dt * c.fm[I3V(e, 1, p, l)];
      }
  if (!tracers || Q == 0) return;
  auto clip = [](double qdp_s, double v1) {
    if (qdp_s + v1 < 0.0 && v1 < 0.0) v1 = qdp_s < 0.0 ? 0.0 : -qdp_s;
    return v1;
  };
  auto FQ = [&](int e, int q, int p, int l) -> double& {
    return c.fq[(((size_t)e * Q + q) * NP2 + p) * NLEV + l];
  };
  if (c.prm.moist) {
#pragma omp parallel for
    for (int e = 0; e < c.E; ++e)
      for (int p = 0; p < NP2; ++p) {
        double acc = 0.0;
        for (int l = 0; l < NLEV; ++l) acc += clip(c.qdp[IQ(e, nq, 0, p, l, Q)], dt * FQ(e, 0, p, l));
        c.ps_v[((size_t)e * NTL + n0) * NP2 + p] += acc;
      }
  }
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < Q; ++q)
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l) {
          double& qd = c.qdp[IQ(e, nq, q, p, l, Q)];
          qd += clip(qd, dt * FQ(e, q, p, l));
        }
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < Q; ++q)
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l) {
          const double dp = c.ai_delta[l] * c.ps0 + c.bi_delta[l] * c.ps_v[((size_t)e * NTL + n0) * NP2 + p];
          c.Qc[(((size_t)e * Q + q) * NP2 + p) * NLEV + l] = c.qdp[IQ(e, nq, q, p, l, Q)] / dp;
        }
}

void push_block(const double* in, double* f, int ncomp);

// Tracer mass diagnostics (Diagnostics.cpp:37-84): the mixing ratio is copied into the
// host array Q (np,np,nlev,qsize,nelemd); per tracer and GLL point the column sums of
// Qdp*Q and of Qdp at the call's tracer level go to Qvar(:,:,q,ivar), Qmass(:,:,q,ivar)
// and Q1mass(:,:,q).
void diag_scalars(bool before_advance, int ivar) {
  Ctx& c = C();
  c.tl.update_tracers_levels(c.prm.qsplit);
  const int t2 = before_advance ? c.tl.n0_qdp : c.tl.np1_qdp;
  if (c.prm.time_step_type <= 0) return;
  const int Q = c.Q;
  const size_t B = (size_t)NP2 * NLEV;
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < Q; ++q)
      push_block(&c.Qc[((size_t)e * Q + q) * B], c.diag[0] + ((size_t)e * Q + q) * B, 1);
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < Q; ++q)
      for (int p = 0; p < NP2; ++p) {
        double sqq = 0.0, sq = 0.0;
        for (int l = 0; l < NLEV; ++l) {
          const double qd = c.qdp[IQ(e, t2, q, p, l, Q)];
          sqq += qd * c.Qc[(((size_t)e * Q + q) * NP2 + p) * NLEV + l];
          sq += qd;
        }
        const size_t k = (((size_t)e * 4 + ivar) * Q + q) * NP2 + p;
        c.diag[1][k] = sqq;
        c.diag[2][k] = sq;
        c.diag[3][((size_t)e * Q + q) * NP2 + p] = sq;
      }
}

// Column energies (Diagnostics.cpp:86-185) at the call's dynamics level, with the layer
// thickness taken from ps_v: IEner = sum cp* T dp, IEner_wet = sum (cp* - cp) T dp,
// KEner = sum (u^2 + v^2)/2 dp, PEner = sum phis dp; cp* = cp (1 + (cpv/cp - 1) q0) with
// q0 = Qdp(tracer 1)/dp when use_cpstar, else cp.  cp = 1005, cpv = 1870
// (PhysicalConstants.hpp:18-20).
void energy_halftimes(bool before_advance, int ivar) {
  Ctx& c = C();
  c.tl.update_tracers_levels(c.prm.qsplit);
  const int t1 = before_advance ? c.tl.n0 : c.tl.np1;
  const int t1q = before_advance ? c.tl.n0_qdp : c.tl.np1_qdp;
  const double cp = 1005.0, cpwv = 1870.0;
  const bool cpstar = c.prm.use_cpstar && c.Q > 0;
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int p = 0; p < NP2; ++p) {
      double ie = 0.0, iew = 0.0, ke = 0.0, pe = 0.0;
      const double ps = c.ps_v[((size_t)e * NTL + t1) * NP2 + p], phis = c.phis[(size_t)e * NP2 + p];
      for (int l = 0; l < NLEV; ++l) {
        const double dp = c.ai_delta[l] * c.ps0 + c.bi_delta[l] * ps;
        double cps = cp;
        if (cpstar) cps = cp * (1.0 + (cpwv / cp - 1.0) * (c.qdp[IQ(e, t1q, 0, p, l, c.Q)] / dp));
        const double T = c.t[IS(e, t1, p, l)];
        const double u = c.v[IV(e, t1, 0, p, l)], v = c.v[IV(e, t1, 1, p, l)];
        ie += cps * T * dp;
        iew += (cps - cp) * T * dp;
        ke += (u * u + v * v) * 0.5 * dp;
        pe += phis * dp;
      }
      const size_t k = ((size_t)e * 4 + ivar) * NP2 + p;
      c.diag[4][k] = ie;
      c.diag[5][(size_t)e * NP2 + p] = iew;
      c.diag[6][k] = ke;
      c.diag[7][k] = pe;
    }
}

void prim_run_subcycle(double dt, int& nstep, int& nm1, int& n0, int& np1,
                       int last_time_step) {  // prim_driver.cpp:31-156
  Ctx& c = C();
  const Params& pr = c.prm;
  const double dt_q = dt * pr.qsplit;
  double dt_remap = dt_q;
  int nstep_end = c.tl.nstep + pr.qsplit;
  if (pr.rsplit > 0) {
    dt_remap = dt_q * pr.rsplit;
    nstep_end = c.tl.nstep + pr.qsplit * pr.rsplit;
  }
  // prim_driver.cpp:49-58; the arrays of init_diagnostics_c must be set
  bool diag = (pr.state_frequency > 0 && nstep_end % pr.state_frequency == 0) ||
              nstep_end == c.tl.nstep0 || nstep_end >= last_time_step;
  if (pr.disable_diagnostics || !c.diag[0]) diag = false;
  if (diag) {
    diag_scalars(true, 3);
    energy_halftimes(true, 2);
  }
  c.tl.update_tracers_levels(pr.qsplit);
  if (pr.ftype == 0) apply_cam_forcing(dt_remap, true);
  else if (pr.ftype == 2) apply_cam_forcing(dt_remap, false);
  if (diag) {
    energy_halftimes(true, 0);
    diag_scalars(true, 0);
  }
  // dp3d from ps_v
  const int tn0 = c.tl.n0;
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e)
    for (int p = 0; p < NP2; ++p)
      for (int l = 0; l < NLEV; ++l)
        c.dp3d[IS(e, tn0, p, l)] =
            c.ai_delta[l] * c.ps0 + c.bi_delta[l] * c.ps_v[((size_t)e * NTL + tn0) * NP2 + p];
  prim_step(dt);
  for (int r = 1; r < pr.rsplit; ++r) {
    c.tl.update_dynamics_levels();
    prim_step(dt);
  }
  c.tl.update_tracers_levels(pr.qsplit);
  remap_run(c.tl.np1, c.tl.np1_qdp, dt_remap);
  if (!c.valid_remap) {
    set_error(101, "Negative (or nan) layer thickness detected, aborting!");
    return;
  }
  // update_q (prim_driver.cpp:171-206)
  const int tnp1 = c.tl.np1, np1_qdp = c.tl.np1_qdp;
#pragma omp parallel for collapse(2)
  for (int e = 0; e < c.E; ++e)
    for (int q = 0; q < c.Q; ++q)
      for (int p = 0; p < NP2; ++p)
        for (int l = 0; l < NLEV; ++l) {
          const double dp = c.ai_delta[l] * c.ps0 + c.bi_delta[l] * c.ps_v[((size_t)e * NTL + tnp1) * NP2 + p];
          c.Qc[(((size_t)e * c.Q + q) * NP2 + p) * NLEV + l] = c.qdp[IQ(e, np1_qdp, q, p, l, c.Q)] / dp;
        }
  if (diag) {
    diag_scalars(false, 1);
    energy_halftimes(false, 1);
  }
  c.tl.update_dynamics_levels();
  nstep = c.tl.nstep;
  nm1 = c.tl.nm1;
  n0 = c.tl.n0;
  np1 = c.tl.np1;
}

// Fortran <-> internal transposes (SyncUtils.hpp).  Fortran per-element/time-level
// blocks are [lev][comp][16]; internal blocks are [comp][16][lev].
void pull_block(const double* f, double* in, int ncomp) {
  for (int l = 0; l < NLEV; ++l)
    for (int cc = 0; cc < ncomp; ++cc)
      for (int p = 0; p < NP2; ++p) in[(cc * NP2 + p) * NLEV + l] = f[(l * ncomp + cc) * NP2 + p];
}
void push_block(const double* in, double* f, int ncomp) {
  for (int l = 0; l < NLEV; ++l)
    for (int cc = 0; cc < ncomp; ++cc)
      for (int p = 0; p < NP2; ++p) f[(l * ncomp + cc) * NP2 + p] = in[(cc * NP2 + p) * NLEV + l];
}

#include "hx_oracle_traj.inc"

}  // namespace

// ====================================================================================
// Exported C ABI (same names as libhxgpu.so; see include/hxgpu.h)
// ====================================================================================
extern "C" {

void initialize_hommexx_session(void) { C(); }
void finalize_hommexx_session(void) {
  delete g;
  g = nullptr;
  TC() = TrajCtx();
}
void reset_cxx_comm(const int*) {}

void init_connectivity(const int* n) {
  Ctx& c = C();
  c.conn.assign((size_t)(*n) * 16, -1);
  c.conn_final = false;
}

void add_connection(const int* fl, const int*, const int* fp, const int*, const int* sl,
                    const int*, const int* sp, const int*) {
  Ctx& c = C();
  auto convert = [](int fpos) { return fpos <= 4 ? (((fpos - 1) + 2) % 4) : (fpos - 1); };
  const int e = *fl - 1, s = convert(*fp);
  c.conn[(e * 8 + s) * 2] = *sl - 1;
  c.conn[(e * 8 + s) * 2 + 1] = convert(*sp);
}
void finalize_connectivity(void) { C().conn_final = true; }

void init_derivative_c(const double* const* dvv) {
  Ctx& c = C();
  for (int i = 0; i < NP; ++i)
    for (int j = 0; j < NP; ++j) c.dvv[i][j] = (*dvv)[i * NP + j];
}

void init_simulation_params_c(const int* remap_alg, const int* limiter_option, const int* rsplit,
                              const int* qsplit, const int* time_step_type, const int*,
                              const int* qsize, const int* state_frequency, const double* nu,
                              const double* nu_p, const double* nu_q, const double* nu_s,
                              const double* nu_div, const double* nu_top,
                              const int* hypervis_order, const int* hypervis_subcycle,
                              const double* hypervis_scaling, const int* ftype,
                              const bool* prescribed_wind, const bool* moisture,
                              const bool* disable_diagnostics, const bool* use_cpstar,
                              const bool* use_semi_lagrangian_transport) {
  Ctx& c = C();
  c.last_err = 0;
  auto bad = [&](const char* opt) {
    set_error(11, std::string("Error in init_simulation_params_c: unsupported value for input parameter '") + opt + "'.");
  };
  if (*remap_alg != 1 && *remap_alg != 2) return bad("vert_remap_q_alg");
  if (*prescribed_wind) return bad("prescribed_wind");
  if (*hypervis_order != 2) return bad("hypervis_order");
  if (*use_semi_lagrangian_transport) return bad("use_semi_lagrangian_transport");
  if (*time_step_type != 5) return bad("time_step_type");
  if (*limiter_option != 8 && *limiter_option != 9) return bad("limiter_option");
  if (*ftype != -1 && *ftype != 0 && *ftype != 2) return bad("ftype");
  if (!(*nu_p > 0)) return bad("nu_p");
  if (!(*nu > 0)) return bad("nu");
  if (!(*nu_div > 0)) return bad("nu_div");
  Params& p = c.prm;
  p.remap_alg = *remap_alg;
  p.limiter_option = *limiter_option;
  p.rsplit = *rsplit;
  p.qsplit = *qsplit;
  p.time_step_type = *time_step_type;
  p.qsize = *qsize;
  p.state_frequency = *state_frequency;
  p.nu = *nu;
  p.nu_p = *nu_p;
  p.nu_q = *nu_q;
  p.nu_s = *nu_s;
  p.nu_div = *nu_div;
  p.nu_top = *nu_top;
  p.hypervis_order = *hypervis_order;
  p.hypervis_subcycle = *hypervis_subcycle;
  p.hypervis_scaling = *hypervis_scaling;
  p.ftype = *ftype;
  p.moist = *moisture;
  p.disable_diagnostics = *disable_diagnostics;
  p.use_cpstar = *use_cpstar;
  if (p.nu != p.nu_div) {
    const double ratio = p.nu_div / p.nu;
    if (p.hypervis_scaling != 0.0) {
      p.nu_ratio1 = ratio * ratio;
      p.nu_ratio2 = 1.0;
    } else {
      p.nu_ratio1 = ratio;
      p.nu_ratio2 = ratio;
    }
  } else {
    p.nu_ratio1 = 1.0;
    p.nu_ratio2 = 1.0;
  }
  p.set = true;
}

void init_hvcoord_c(const double* ps0, const double* const*, const double* const* hyai,
                    const double* const*, const double* const* hybi) {
  Ctx& c = C();
  c.ps0 = *ps0;
  for (int k = 0; k <= NLEV; ++k) {
    c.hyai[k] = (*hyai)[k];
    c.hybi[k] = (*hybi)[k];
  }
  c.hyai0 = c.hyai[0];
  for (int l = 0; l < NLEV; ++l) {  // HybridVCoord::compute_deltas
    c.ai_delta[l] = c.hyai[l + 1] - c.hyai[l];
    c.bi_delta[l] = c.hybi[l + 1] - c.hybi[l];
    c.dp0[l] = c.ai_delta[l] * c.ps0 + c.bi_delta[l] * c.ps0;
  }
}

void init_elements_2d_c(const int* nelemd, const double* const* D, const double* const* Dinv,
                        const double* const* fcor, const double* const* mp,
                        const double* const* spheremp, const double* const* rspheremp,
                        const double* const* metdet, const double* const* metinv,
                        const double* const* phis, const double* const* tensorvisc,
                        const double* const* vec_sph2cart, const bool* consthv) {
  Ctx& c = C();
  const int E = *nelemd;
  c.E = E;
  c.Q = c.prm.qsize;
  c.consthv = *consthv;
  auto cp = [](std::vector<double>& dst, const double* src, size_t n) { dst.assign(src, src + n); };
  cp(c.D, *D, (size_t)E * 64);
  cp(c.Dinv, *Dinv, (size_t)E * 64);
  cp(c.metinv, *metinv, (size_t)E * 64);
  cp(c.fcor, *fcor, (size_t)E * 16);
  cp(c.mp, *mp, (size_t)E * 16);
  cp(c.spheremp, *spheremp, (size_t)E * 16);
  cp(c.rspheremp, *rspheremp, (size_t)E * 16);
  cp(c.metdet, *metdet, (size_t)E * 16);
  cp(c.phis, *phis, (size_t)E * 16);
  if (!c.consthv) {
    cp(c.tensorvisc, *tensorvisc, (size_t)E * 64);
    cp(c.vec_sph2cart, *vec_sph2cart, (size_t)E * 96);
  }
  const size_t N3 = (size_t)E * NP2 * NLEV;
  const int Q = c.Q;
  c.v.assign(N3 * NTL * 2, 0.0);
  c.t.assign(N3 * NTL, 0.0);
  c.dp3d.assign(N3 * NTL, 0.0);
  c.ps_v.assign((size_t)E * NTL * NP2, 0.0);
  c.qdp.assign(N3 * QTL * Q, 0.0);
  c.Qc.assign(N3 * Q, 0.0);
  for (auto* f : {&c.phi, &c.omega_p, &c.eta_dot_dpdn, &c.derived_dp, &c.divdp, &c.divdp_proj,
                  &c.dpdiss_ave, &c.dpdiss_bih, &c.ttens, &c.dptens, &c.dpdissk, &c.dp_buf})
    f->assign(N3, 0.0);
  c.vn0.assign(2 * N3, 0.0);
  c.vtens.assign(2 * N3, 0.0);
  c.vstar.assign(2 * N3, 0.0);
  c.qtens_bih.assign(N3 * Q, 0.0);
  c.qlim.assign((size_t)E * Q * 2 * NLEV, 0.0);
}

void init_elements_states_c(const double* const* v, const double* const* T,
                            const double* const* dp3d, const double* const* Qdp,
                            const double* const* ps_v) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  for (int e = 0; e < c.E; ++e)
    for (int tl = 0; tl < NTL; ++tl) {
      pull_block(*v + ((size_t)e * NTL + tl) * 2 * B, &c.v[IV(e, tl, 0, 0, 0)], 2);
      pull_block(*T + ((size_t)e * NTL + tl) * B, &c.t[IS(e, tl, 0, 0)], 1);
      pull_block(*dp3d + ((size_t)e * NTL + tl) * B, &c.dp3d[IS(e, tl, 0, 0)], 1);
    }
  for (int e = 0; e < c.E; ++e)
    for (int qt = 0; qt < QTL; ++qt)
      for (int q = 0; q < c.Q; ++q)
        pull_block(*Qdp + (((size_t)e * QTL + qt) * c.Q + q) * B, &c.qdp[IQ(e, qt, q, 0, 0, c.Q)], 1);
  std::memcpy(c.ps_v.data(), *ps_v, sizeof(double) * c.E * NTL * NP2);
}

void init_diagnostics_c(double* const* q, double* const* qvar, double* const* qmass,
                        double* const* q1mass, double* const* iener, double* const* iener_wet,
                        double* const* kener, double* const* pener) {
  double* const* a[8] = {q, qvar, qmass, q1mass, iener, iener_wet, kener, pener};
  for (int i = 0; i < 8; ++i) C().diag[i] = *a[i];
}

void init_boundary_exchanges_c(void) { build_tables(); }

void init_time_level_c(const int* nm1, const int* n0, const int* np1, const int* nstep,
                       const int* nstep0) {
  Ctx& c = C();
  c.tl.nm1 = *nm1 - 1;
  c.tl.n0 = *n0 - 1;
  c.tl.np1 = *np1 - 1;
  c.tl.nstep = *nstep;
  c.tl.nstep0 = *nstep0;
}

void prim_run_subcycle_c(const double* dt, int* nstep, int* nm1, int* n0, int* np1,
                         const int* last_time_step) {
  Ctx& c = C();
  c.last_err = 0;
  c.streamed = false;
  prim_run_subcycle(*dt, *nstep, *nm1, *n0, *np1, last_time_step ? *last_time_step : INT_MAX);
  if (c.stream_to[0] && c.last_err == 0) {
    double* const* p = c.stream_to;
    cxx_push_results_to_f90(&p[0], &p[1], &p[2], &p[3], &p[4], &p[5], &p[6]);
    c.streamed = true;
  }
}

void cxx_push_results_to_f90(double* const* v, double* const* T, double* const* dp3d,
                             double* const* Qdp, double* const* Q, double* const* ps_v,
                             double* const* omega_p) {
  Ctx& c = C();
  {
    double* const p[7] = {*v, *T, *dp3d, *Qdp, *Q, *ps_v, *omega_p};
    bool same = c.streamed;
    for (int i = 0; i < 7; ++i) same = same && p[i] == c.stream_to[i];
    if (same) return;
  }
  const size_t B = (size_t)NP2 * NLEV;
  for (int e = 0; e < c.E; ++e)
    for (int tl = 0; tl < NTL; ++tl) {
      push_block(&c.v[IV(e, tl, 0, 0, 0)], *v + ((size_t)e * NTL + tl) * 2 * B, 2);
      push_block(&c.t[IS(e, tl, 0, 0)], *T + ((size_t)e * NTL + tl) * B, 1);
      push_block(&c.dp3d[IS(e, tl, 0, 0)], *dp3d + ((size_t)e * NTL + tl) * B, 1);
    }
  for (int e = 0; e < c.E; ++e)
    for (int qt = 0; qt < QTL; ++qt)
      for (int q = 0; q < c.Q; ++q)
        push_block(&c.qdp[IQ(e, qt, q, 0, 0, c.Q)], *Qdp + (((size_t)e * QTL + qt) * c.Q + q) * B, 1);
  for (int e = 0; e < c.E; ++e) {
    for (int q = 0; q < c.Q; ++q)
      push_block(&c.Qc[(((size_t)e * c.Q + q) * NP2) * NLEV], *Q + ((size_t)e * c.Q + q) * B, 1);
    push_block(&c.omega_p[I3(e, 0, 0)], *omega_p + (size_t)e * B, 1);
  }
  std::memcpy(*ps_v, c.ps_v.data(), sizeof(double) * c.E * NTL * NP2);
}

// cxx_f90_interface.cpp:180-205: forcing in (FQ only for ftype 0) and the tracer mass.
void f90_push_forcing_to_cxx(const double* FM, const double* FT, const double* FQ,
                             const double* Qdp) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  c.fm.resize((size_t)c.E * 2 * B);
  c.ft.resize((size_t)c.E * B);
  for (int e = 0; e < c.E; ++e) {
    pull_block(FM + (size_t)e * 2 * B, &c.fm[I3V(e, 0, 0, 0)], 2);
    pull_block(FT + (size_t)e * B, &c.ft[I3(e, 0, 0)], 1);
  }
  if (c.prm.ftype == 0) {
    c.fq.resize((size_t)c.E * c.Q * B);
    for (int e = 0; e < c.E; ++e)
      for (int q = 0; q < c.Q; ++q)
        pull_block(FQ + ((size_t)e * c.Q + q) * B, &c.fq[((size_t)e * c.Q + q) * B], 1);
  }
  for (int e = 0; e < c.E; ++e)
    for (int qt = 0; qt < QTL; ++qt)
      for (int q = 0; q < c.Q; ++q)
        pull_block(Qdp + (((size_t)e * QTL + qt) * c.Q + q) * B, &c.qdp[IQ(e, qt, q, 0, 0, c.Q)], 1);
}

// cxx_f90_interface.cpp:157-178
void cxx_push_forcing_to_f90(double* FM, double* FT, double* FQ) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  if (c.ft.empty()) {  // nothing pushed: zero forcing
    std::memset(FM, 0, sizeof(double) * c.E * 2 * B);
    std::memset(FT, 0, sizeof(double) * c.E * B);
  } else {
    for (int e = 0; e < c.E; ++e) {
      push_block(&c.fm[I3V(e, 0, 0, 0)], FM + (size_t)e * 2 * B, 2);
      push_block(&c.ft[I3(e, 0, 0)], FT + (size_t)e * B, 1);
    }
  }
  if (c.prm.ftype == 0) {
    if (c.fq.empty()) c.fq.assign((size_t)c.E * c.Q * B, 0.0);
    for (int e = 0; e < c.E; ++e)
      for (int q = 0; q < c.Q; ++q)
        push_block(&c.fq[((size_t)e * c.Q + q) * B], FQ + ((size_t)e * c.Q + q) * B, 1);
  }
}

// Restart files (format and checksum as documented in include/hxgpu.h): records
// restate the prognostic elem_state_t of src/share/element_mod.F90:103-115, the header
// the TimeLevel_t and the size checks of src/restart_io_mod.F90:401-471.
static unsigned long long splitmix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static size_t restart_record_words(int Q) {
  return (size_t)NTL * NLEV * 32 + 2 * (size_t)NTL * NLEV * 16 + NTL * 16 + 16 + (size_t)Q * NLEV * 16 +
         (size_t)QTL * Q * NLEV * 16;
}
static unsigned long long restart_sum(const double* rec, size_t words, unsigned long long k0) {
  unsigned long long acc = 0;
  for (size_t j = 0; j < words; ++j) {
    unsigned long long w;
    std::memcpy(&w, rec + j, 8);
    acc += splitmix64(w + (k0 + j + 1) * 0x9E3779B97F4A7C15ull);
  }
  return acc;
}
static void pack_record(int e, double* r) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  for (int tl = 0; tl < NTL; ++tl) push_block(&c.v[IV(e, tl, 0, 0, 0)], r + tl * 2 * B, 2);
  r += NTL * 2 * B;
  for (int tl = 0; tl < NTL; ++tl) push_block(&c.t[IS(e, tl, 0, 0)], r + tl * B, 1);
  r += NTL * B;
  for (int tl = 0; tl < NTL; ++tl) push_block(&c.dp3d[IS(e, tl, 0, 0)], r + tl * B, 1);
  r += NTL * B;
  std::memcpy(r, &c.ps_v[(size_t)e * NTL * NP2], sizeof(double) * NTL * NP2);
  r += NTL * NP2;
  std::memcpy(r, &c.phis[(size_t)e * NP2], sizeof(double) * NP2);
  r += NP2;
  for (int q = 0; q < c.Q; ++q) push_block(&c.Qc[((size_t)e * c.Q + q) * B], r + q * B, 1);
  r += (size_t)c.Q * B;
  for (int qt = 0; qt < QTL; ++qt)
    for (int q = 0; q < c.Q; ++q) push_block(&c.qdp[IQ(e, qt, q, 0, 0, c.Q)], r + ((size_t)qt * c.Q + q) * B, 1);
}
static void unpack_record(int e, const double* r) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  for (int tl = 0; tl < NTL; ++tl) pull_block(r + tl * 2 * B, &c.v[IV(e, tl, 0, 0, 0)], 2);
  r += NTL * 2 * B;
  for (int tl = 0; tl < NTL; ++tl) pull_block(r + tl * B, &c.t[IS(e, tl, 0, 0)], 1);
  r += NTL * B;
  for (int tl = 0; tl < NTL; ++tl) pull_block(r + tl * B, &c.dp3d[IS(e, tl, 0, 0)], 1);
  r += NTL * B;
  std::memcpy(&c.ps_v[(size_t)e * NTL * NP2], r, sizeof(double) * NTL * NP2);
  r += NTL * NP2;
  std::memcpy(&c.phis[(size_t)e * NP2], r, sizeof(double) * NP2);
  r += NP2;
  for (int q = 0; q < c.Q; ++q) pull_block(r + q * B, &c.Qc[((size_t)e * c.Q + q) * B], 1);
  r += (size_t)c.Q * B;
  for (int qt = 0; qt < QTL; ++qt)
    for (int q = 0; q < c.Q; ++q) pull_block(r + ((size_t)qt * c.Q + q) * B, &c.qdp[IQ(e, qt, q, 0, 0, c.Q)], 1);
}

int hx_write_restart(const char* path) {
  Ctx& c = C();
  c.last_err = 0;
  if (c.E == 0) { set_error(HX_ERR_STATE, "library not initialised"); return HX_ERR_STATE; }
  const size_t rw = restart_record_words(c.Q);
  hx_restart_header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, HX_RESTART_MAGIC, 8);
  h.version = HX_RESTART_VERSION;
  h.header_bytes = sizeof(h);
  h.nelem = c.E; h.np = NP; h.nlev = NLEV; h.qsize = c.Q; h.timelevels = NTL; h.qsize_timelevels = QTL;
  h.nm1 = c.tl.nm1 + 1; h.n0 = c.tl.n0 + 1; h.np1 = c.tl.np1 + 1; h.nstep = c.tl.nstep; h.nstep0 = c.tl.nstep0;
  h.record_bytes = rw * 8;
  std::vector<double> all((size_t)c.E * rw);
  unsigned long long sum = 0;
  for (int e = 0; e < c.E; ++e) {
    pack_record(e, &all[(size_t)e * rw]);
    sum += restart_sum(&all[(size_t)e * rw], rw, (unsigned long long)e * rw);
  }
  h.checksum = sum;
  FILE* f = path ? std::fopen(path, "wb") : nullptr;
  if (!f) { set_error(HX_ERR_IO, "cannot open restart file for writing"); return HX_ERR_IO; }
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(all.data(), 8, all.size(), f) == all.size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) { set_error(HX_ERR_IO, "write error on restart file"); return HX_ERR_IO; }
  return 0;
}

int hx_read_restart(const char* path) {
  Ctx& c = C();
  c.last_err = 0;
  if (c.E == 0) { set_error(HX_ERR_STATE, "library not initialised"); return HX_ERR_STATE; }
  auto err = [&](const std::string& m) { set_error(HX_ERR_IO, m); return HX_ERR_IO; };
  FILE* f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) return err("cannot open restart file");
  const size_t rw = restart_record_words(c.Q);
  hx_restart_header h;
  std::vector<double> all;
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1;
  if (ok && (std::memcmp(h.magic, HX_RESTART_MAGIC, 8) != 0 || h.header_bytes != sizeof(h))) {
    std::fclose(f);
    return err("not a restart file");
  }
  if (ok && h.version != HX_RESTART_VERSION) { std::fclose(f); return err("restart version does not match"); }
  if (ok && (h.nelem != c.E || h.np != NP || h.nlev != NLEV || h.qsize != c.Q || h.timelevels != NTL ||
             h.qsize_timelevels != QTL || h.record_bytes != rw * 8)) {
    std::fclose(f);
    return err("restart file does not match the session");
  }
  if (ok) {
    all.resize((size_t)c.E * rw);
    ok = std::fread(all.data(), 8, all.size(), f) == all.size();
  }
  std::fclose(f);
  if (!ok) return err("short read on restart file");
  for (int t : {h.nm1, h.n0, h.np1})
    if (t < 1 || t > NTL) return err("bad time level in restart header");
  unsigned long long sum = 0;
  for (int e = 0; e < c.E; ++e) sum += restart_sum(&all[(size_t)e * rw], rw, (unsigned long long)e * rw);
  if (sum != h.checksum) return err("checksum mismatch");
  for (int e = 0; e < c.E; ++e) unpack_record(e, &all[(size_t)e * rw]);
  c.tl.nm1 = h.nm1 - 1; c.tl.n0 = h.n0 - 1; c.tl.np1 = h.np1 - 1;
  c.tl.nstep = h.nstep; c.tl.nstep0 = h.nstep0;
  return 0;
}

// Copies that overlap the step: on the CPU the input is read at once (the flag has no
// effect) and the streamed results are pushed when each interval ends.
int hx_set_async_copies(int) { return 0; }
int hx_stream_results(double* v, double* T, double* dp3d, double* Qdp, double* Q, double* ps_v,
                      double* omega_p) {
  Ctx& c = C();
  double* const p[7] = {v, T, dp3d, Qdp, Q, ps_v, omega_p};
  int n = 0;
  for (int i = 0; i < 7; ++i) n += p[i] != nullptr;
  if (n != 0 && n != 7) {
    set_error(13, "hx_stream_results: give all seven destinations or none");
    return 13;
  }
  for (int i = 0; i < 7; ++i) c.stream_to[i] = p[i];
  c.streamed = false;
  return 0;
}

int hx_last_error(char* buf, int buflen) {
  Ctx& c = C();
  if (buf && buflen > 0) {
    std::strncpy(buf, c.last_msg.c_str(), buflen - 1);
    buf[buflen - 1] = 0;
  }
  return c.last_err;
}
void hx_set_abort_on_error(int a) { C().abort_on_error = a != 0; }
int hx_set_precision(int mode) {
  if (mode != 0) {
    set_error(12, "the oracle computes in FP64 only");
    return 12;
  }
  return 0;
}

static double* field_ptr(const std::string& n, int tl, int& ncomp, size_t& estride, int& nblocks) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
  ncomp = 1;
  nblocks = 1;
  if (n == "v") { ncomp = 2; estride = NTL * 2 * B; return &c.v[IV(0, tl, 0, 0, 0)]; }
  if (n == "T") { estride = NTL * B; return &c.t[IS(0, tl, 0, 0)]; }
  if (n == "dp3d") { estride = NTL * B; return &c.dp3d[IS(0, tl, 0, 0)]; }
  if (n == "Qdp") { nblocks = c.Q; estride = (size_t)QTL * c.Q * B; return &c.qdp[IQ(0, tl, 0, 0, 0, c.Q)]; }
  if (n == "Q") { nblocks = c.Q; estride = (size_t)c.Q * B; return c.Qc.data(); }
  if (n == "vn0") { ncomp = 2; estride = 2 * B; return c.vn0.data(); }
  estride = B;
  if (n == "omega_p") return c.omega_p.data();
  if (n == "phi") return c.phi.data();
  if (n == "eta_dot_dpdn") return c.eta_dot_dpdn.data();
  if (n == "derived_dp") return c.derived_dp.data();
  if (n == "divdp") return c.divdp.data();
  if (n == "divdp_proj") return c.divdp_proj.data();
  if (n == "dpdiss_ave") return c.dpdiss_ave.data();
  if (n == "dpdiss_biharmonic") return c.dpdiss_bih.data();
  return nullptr;
}

int hx_get_field(const char* name, int tl, double* out) {
  Ctx& c = C();
  const std::string n(name);
  if (n == "ps_v") {
    for (int e = 0; e < c.E; ++e)
      std::memcpy(out + (size_t)e * NP2, &c.ps_v[((size_t)e * NTL + tl) * NP2], sizeof(double) * NP2);
    return 0;
  }
  int ncomp, nb;
  size_t es;
  double* base = field_ptr(n, tl, ncomp, es, nb);
  if (!base) return HX_ERR_STATE;
  const size_t B = (size_t)NP2 * NLEV * ncomp;
  for (int e = 0; e < c.E; ++e)
    for (int b = 0; b < nb; ++b) push_block(base + e * es + b * B, out + ((size_t)e * nb + b) * B, ncomp);
  return 0;
}

int hx_set_field(const char* name, int tl, const double* in) {
  Ctx& c = C();
  const std::string n(name);
  if (n == "ps_v") {
    for (int e = 0; e < c.E; ++e)
      std::memcpy(&c.ps_v[((size_t)e * NTL + tl) * NP2], in + (size_t)e * NP2, sizeof(double) * NP2);
    return 0;
  }
  int ncomp, nb;
  size_t es;
  double* base = field_ptr(n, tl, ncomp, es, nb);
  if (!base) return HX_ERR_STATE;
  const size_t B = (size_t)NP2 * NLEV * ncomp;
  for (int e = 0; e < c.E; ++e)
    for (int b = 0; b < nb; ++b) pull_block(in + ((size_t)e * nb + b) * B, base + e * es + b * B, ncomp);
  return 0;
}

int hx_run_caar_stage(int nm1, int n0, int np1, double dt, double w) {
  caar_run(nm1, n0, np1, dt, w, -1);
  return 0;
}
int hx_run_rk5(int nm1, int n0, int np1, int n0_qdp, double dt, double w) {
  u3_5stage(nm1, n0, np1, n0_qdp, dt, w);
  return 0;
}
int hx_run_hypervis(int np1, double dt, double w) {
  hypervis_run(np1, dt, w);
  return 0;
}
int hx_run_euler_step(int np1_qdp, int n0_qdp, double dt, double rhs, int dssopt) {
  euler_step(np1_qdp, n0_qdp, dt, rhs, dssopt);
  return 0;
}
int hx_run_tracers_rk2(double dt) {
  tracers_rk2(dt);
  return 0;
}
int hx_run_remap(int np1, int np1_qdp, double dt) {
  remap_run(np1, np1_qdp, dt);
  return C().valid_remap ? 0 : 101;
}
int hx_run_prim_step(double dt) {
  prim_step(dt);
  return 0;
}
int hx_run_dss(const char* name, int tl, int rsmp) {
  int ncomp, nb;
  size_t es;
  double* base = field_ptr(name, tl, ncomp, es, nb);
  if (!base) return HX_ERR_STATE;
  std::vector<FieldRef> f;
  for (int b = 0; b < nb * ncomp; ++b) f.push_back({base + (size_t)b * NP2 * NLEV, es});
  dss(f, rsmp != 0);
  return 0;
}
int hx_num_elems(void) { return C().E; }
int hx_qsize(void) { return C().Q; }
int hx_enable_timing(int) { return 0; }
int hx_kernel_stats(char*, int, long long*, double*, int) { return 0; }
long long hx_launch_count(void) { return 0; }
int hx_synchronize(void) { return 0; }
int hx_timer_start(void) { return 0; }
int hx_timer_stop(double* ms) {
  *ms = 0.0;
  return 0;
}
int hx_host_register(void*, size_t) { return 0; }
int hx_host_unregister(void*) { return 0; }
// Test hooks of the oracle only (no counterpart in the GPU library).

// One level of the quasi-monotone limiter exactly as with_limiter_shell applies it
// (EulerStepFunctorImpl.hpp:693-757): ptens[16] (mass), sphweights[16], dpmass[16],
// qlim[2] (min, max) in/out.
void hx_oracle_limiter(int option, double* ptens, const double* sphweights,
                       const double* dpmass, double* qlim) {
  double x[NP2], cw[NP2], s1 = 0;
  for (int k = 0; k < NP2; ++k) {
    cw[k] = sphweights[k] * dpmass[k];
    x[k] = ptens[k] / dpmass[k];
    s1 += cw[k];
  }
  if (s1 <= 0) return;
  limiter_level(option, x, cw, qlim[0], qlim[1]);
  for (int k = 0; k < NP2; ++k) ptens[k] = x[k] * dpmass[k];
}

// Apply a sphere operator to every level of a field given in the Fortran layout of
// one time level ([E][72][16]; vectors [E][72][2][16]):
//   op 0: laplace_simple (weak), 1: divergence_sphere, 2: vorticity_sphere,
//   3: gradient_sphere (out is a vector), 4: vlaplace_sphere_wk_contra (in/out vectors).
int hx_oracle_sphere_op(int op, const double* in, double* out) {
  Ctx& c = C();
  const size_t B = (size_t)NP2 * NLEV;
#pragma omp parallel for
  for (int e = 0; e < c.E; ++e) {
    const EM m = metric(e);
    std::vector<double> a(2 * B), b(2 * B);
    const int nin = (op == 1 || op == 2 || op == 4) ? 2 : 1;
    const int nout = (op == 3 || op == 4) ? 2 : 1;
    pull_block(in + (size_t)e * nin * B, a.data(), nin);
    switch (op) {
      case 0: laplace_simple(m, a.data(), b.data(), NLEV); break;
      case 1: divergence_sphere(m, a.data(), b.data(), NLEV); break;
      case 2: vorticity_sphere(m, a.data(), b.data(), NLEV); break;
      case 3: gradient_sphere(m, a.data(), b.data(), NLEV); break;
      default: vlaplace_sphere_wk_contra(m, 1.0, a.data(), b.data(), NLEV); break;
    }
    push_block(b.data(), out + (size_t)e * nout * B, nout);
  }
  return 0;
}

// Dry-dynamics trajectory (include/hxgpu.h).  The oracle keeps the input state of every
// step and recomputes each step's stage inputs on the way back.
int hx_traj_forward(const double* v, const double* T, const double* dp3d, int nsteps,
                    double dt, double* v_out, double* T_out, double* dp3d_out) {
  C().last_err = 0;
  if (!traj_ready(false)) return C().last_err;
  if (nsteps < 0 || !(dt > 0)) {
    set_error(HX_ERR_STATE, "hx_traj_forward: nsteps must be >= 0 and dt > 0");
    return C().last_err;
  }
  TrajCtx& tc = TC();
  tc.have = false;
  tc.steps.clear();
  DryState<double> x;
  traj_pull(v, T, dp3d, x);
  for (int s = 0; s < nsteps; ++s) {
    tc.steps.push_back(x);
    if (!dry_step(x, dt, traj_remaps_after(s), (std::vector<DryState<double>>*)nullptr)) {
      set_error(101, "Negative (or nan) layer thickness detected, aborting!");
      return C().last_err;
    }
  }
  tc.nsteps = nsteps;
  tc.dt = dt;
  tc.have = true;
  traj_push(x, v_out, T_out, dp3d_out);
  return 0;
}

int hx_traj_vjp(const double* v_bar, const double* T_bar, const double* dp3d_bar,
                double* v_grad, double* T_grad, double* dp3d_grad) {
  C().last_err = 0;
  if (!traj_ready(true)) return C().last_err;
  TrajCtx& tc = TC();
  DryState<double> a;
  traj_pull(v_bar, T_bar, dp3d_bar, a);
  for (int s = tc.nsteps - 1; s >= 0; --s)
    dry_step_vjp(tc.steps[(size_t)s], tc.dt, traj_remaps_after(s), a);
  traj_push(a, v_grad, T_grad, dp3d_grad);
  return 0;
}

int hx_traj_jvp(const double* dv, const double* dT, const double* ddp3d, double* v_tan,
                double* T_tan, double* dp3d_tan) {
  C().last_err = 0;
  if (!traj_ready(true)) return C().last_err;
  TrajCtx& tc = TC();
  DryState<double> d;
  traj_pull(dv, dT, ddp3d, d);
  if (tc.nsteps == 0) {
    traj_push(d, v_tan, T_tan, dp3d_tan);
    return 0;
  }
  DryState<Dual> x;
  x.alloc(C().E);
  const DryState<double>& x0 = tc.steps[0];
  for (size_t i = 0; i < x.v.size(); ++i) x.v[i] = Dual(x0.v[i], d.v[i]);
  for (size_t i = 0; i < x.t.size(); ++i) {
    x.t[i] = Dual(x0.t[i], d.t[i]);
    x.dp[i] = Dual(x0.dp[i], d.dp[i]);
  }
  for (int s = 0; s < tc.nsteps; ++s)
    dry_step(x, tc.dt, traj_remaps_after(s), (std::vector<DryState<Dual>>*)nullptr);
  DryState<double> out;
  out.alloc(C().E);
  for (size_t i = 0; i < x.v.size(); ++i) out.v[i] = x.v[i].d;
  for (size_t i = 0; i < x.t.size(); ++i) {
    out.t[i] = x.t[i].d;
    out.dp[i] = x.dp[i].d;
  }
  traj_push(out, v_tan, T_tan, dp3d_tan);
  return 0;
}

int hx_traj_set_checkpointing(int mode) {
  if (mode < 0 || mode > 2) {
    set_error(HX_ERR_STATE, "hx_traj_set_checkpointing: mode must be 0, 1 or 2");
    return C().last_err;
  }
  return 0;  // the oracle always keeps step states and recomputes the stages
}

int hx_oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
