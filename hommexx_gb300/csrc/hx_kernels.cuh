// hx_kernels.cuh — launch interface of the preqx kernels (implemented in hx_kernels.cu).
//
// Every field lives in HBM in double.  Kernels are templated on R, the type of the
// sphere-operator arithmetic: double for the FP64 plain form, float for the mixed
// form.  In both forms the vertical scans (pressure, geopotential, omega), the DSS
// accumulation, the PPM remap and the final state updates x = spheremp (x0 + dt f)
// run in double; only tendencies and operators are computed in R.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "hx_common.h"

namespace hx {

// Uploads dvv (C++ order), the hybrid coordinate and nu_top scaling to constant memory.
void upload_constants(const double* dvv16, const double* hyai73, const double* hybi73,
                      double ps0, cudaStream_t s);

template <typename R>
struct CaarArgs {
  MetricP<R> m;
  double* v;        // [E][3][72][2][16]
  double* T;        // [E][3][72][16]
  double* dp;       // [E][3][72][16]
  double* vn0;      // [E][72][2][16]
  double* omega_p;  // [E][72][16]
  double* phi;      // [E][72][16]
  const double* qdp;  // [E][2][Q][72][16] (moist only)
  int qsize, n0_qdp;  // n0_qdp < 0: dry
  double* out;      // pre-DSS result [E][72][4][16]: v0, v1, T, dp3d
  int nm1, n0;
  double dt, eta_ave_w, p_top;  // p_top = hyai(0)*ps0
  int rk_combine, n0orig;       // stage 5: nm1 := (5 nm1 - n0orig)/4 first
  int rsplit;                   // 0: vertically Eulerian (eta_dot_dpdn, vertical advection)
  double* eta_acc;              // [E][72][16] eta_dot_dpdn accumulation (rsplit == 0)
};

template <typename R>
struct HvArgs {
  MetricP<R> m;
  DssTable dss;
  double* v;
  double* T;
  double* dp;
  double* dpdiss_ave;
  double* dpdiss_bih;
  double* bufA;   // [E][72][4][16]
  double* bufB;
  int np1, hsub, consthv;
  int ncyc;  // subcycles this launch runs (hsub for a whole HyperviscosityFunctorImpl::run)
  double dt, eta_ave_w, nu, nu_s, nu_p, nu_top, nu_ratio1, nu_ratio2;
};

template <typename R>
struct EulerArgs {
  MetricP<R> m;
  DssTable dss;
  const double* derived_dp;
  double* divdp;
  double* divdp_proj;
  double* vn0;
  double* dpdiss_ave;
  double* dpdiss_bih;
  double* f_dss;     // eta_dot_dpdn / omega_p / divdp_proj selected by the DSS option
  double* vstar;     // [E][72][2][16]
  double* dpdissk;   // [E][72][16]
  double* fscr;      // [E][72][16] scratch for the DSS of f_dss
  double* qdp;  // [E][2][Q][72][16]
  double* qtens;     // [E][Q][72][16] qtens_biharmonic
  double* qscr;      // [E][Q][72][16] pre-DSS scratch
  double* qlim;     // [E][Q][2][72]
  double* qlim_tmp;
  const double* dp0;  // [72] device
  const int* conn;    // [E][8] neighbour element per connection slot, -1 if missing
  int Q, n0_qdp, np1_qdp, limiter_option, consthv;
  int avg_n0_qdp;  // level averaged with np1 when the last RK2 stage fuses qdp_time_avg
  double dt, rhs_multiplier, rhs_viss, nu_p, nu_q;
  int* err;  // set to 1 when a kernel gives up waiting for its asynchronous copies
};

struct RemapArgs {
  double* v;
  double* T;
  const double* dp;
  double* qdp;
  double* ps_v;   // [E][3][16]
  int np1, n0_qdp, Q, remap_alg, nelem;
  double ps0, hyai0;
  int* invalid;   // set to 1 on a negative or NaN source thickness
  int rsplit;     // 0: tracers only, from the source thickness tgt + dt d(eta_dot_dpdn)
  const double* eta;  // [E][72][16] eta_dot_dpdn (rsplit == 0)
  double dt;
};

// CAM forcing (CamForcing.cpp:20-170): T, v at level n0 += dt FT, dt FM; with fq,
// Qdp at n0_qdp += dt FQ clipped at zero, ps_v(n0) moved by tracer 0's clipped increments
// when moist, Q = Qdp / dp.
void launch_cam_forcing(int E, int Q, double* T, double* v, const double* ft, const double* fm,
                        const double* fq, double* qdp, double* ps_v, double* Qc, int n0, int n0_qdp,
                        int moist, double dt, double ps0, cudaStream_t s);
// Dense weak Laplacian per element ([E][16][16]) from the FP64 metric.
void launch_lap_matrix(const MetricP<double>& m, int E, double* out, cudaStream_t s);
// Cubed-sphere mesh generation (hx_mesh.cu).  Device outputs in the init_elements_2d_c
// layouts (any may be null); status carries the CUDA error and the area correction.
struct CubeMeshDev {
  double *D, *Dinv, *metinv, *metdet, *mp, *spheremp, *fcor, *vec, *tens, *lat, *lon;
};
struct CubeMeshStatus {
  cudaError_t err;
  double alpha_c;
};
CubeMeshStatus cube_metric(int ne, double hypervis_scaling, const CubeMeshDev& out, cudaStream_t s);
// [E][8][2] (remote element, remote slot), 0-based slots S N W E SW SE NW NE, -1 if none.
std::vector<int> cube_connectivity(int ne);
// Restart-file checksum of E element segments (segment e at src + e*words, its word j at
// record word index e*rec_words + off + j), added to *out.
void launch_restart_checksum(const double* src, int E, int words, long long rec_words, long long off,
                             unsigned long long* out, cudaStream_t s);
void launch_prim_step_init(int E, double* eta, double* vn0, double* omega_p, double* dpa,
                           double* dpb, double* derived_dp, const double* dp, int n0, int zero_diss,
                           cudaStream_t s);
void launch_dp_from_ps(int E, double* dp, const double* ps_v, int n0, double ps0, cudaStream_t s);
template <typename R> void launch_caar(const CaarArgs<R>& a, int E, cudaStream_t s);
void launch_dss_state(int E, const double* src, double* v, double* T, double* dp, int np1,
                      const double* rsmp, DssTable t, cudaStream_t s);
template <typename R> void launch_hv(const HvArgs<R>& a, int E, cudaStream_t s);
template <typename R> void launch_precompute_divdp(const EulerArgs<R>& a, int E, cudaStream_t s);
template <typename R> void launch_euler_step(EulerArgs<R>& a, int E, int time_avg, cudaStream_t s);
template <typename R> void launch_remap(const RemapArgs& a, cudaStream_t s);
// Elements per launch when a remap over E elements is split into about `parts` launches:
// a whole number of full waves (SMs x resident CTAs x 4 columns / 16 points), at least one.
template <typename R> int remap_chunk_elements(int E, int parts);
void launch_update_q(int E, int Q, const double* qdp, double* Qc, const double* ps_v, int np1,
                     int np1_qdp, double ps0, cudaStream_t s);
// Energy and tracer mass diagnostics (Diagnostics.cpp): qvar/qmass [E][Q][16] at tracer
// level tq; out = IEner, IEner_wet, KEner, PEner, each [E][16], at dynamics level t1.
void launch_diag_scalars(int E, int Q, const double* qdp, const double* Qc, int tq, double* qvar,
                         double* qmass, cudaStream_t s);
void launch_diag_energy(int E, int Q, const double* T, const double* v, const double* ps_v, const double* phis,
                        const double* qdp, int t1, int t1q, int cpstar, double ps0, double* out,
                        cudaStream_t s);
// Generic DSS of nf fields (field f at base + f*fs, element stride es, level stride ls).
void launch_dss_inplace(int E, int nf, double* base, long long fs, long long es, int ls,
                        double* scratch, const double* rsmp, DssTable t, cudaStream_t s);

// ---- adjoint of the dry dynamics (hx_adjoint.cu) ------------------------------------

void upload_adjoint_constants(const double* dvv16, const double* hyai73, const double* hybi73,
                              cudaStream_t s);

// One time level of the dynamics state: v component c of element e, level l, point p
// at v[e*ev + l*32 + c*16 + p]; T and dp3d at T[e*es + l*16 + p].  A time level tl of
// the [E][3][72]... state arrays is (base + tl*72*32, base + tl*72*16, ev = 3*72*32,
// es = 3*72*16); a stand-alone level has ev = 72*32, es = 72*16.
struct DynV {
  double* v;
  double* T;
  double* dp;
  long long ev, es;
};

template <typename R>
struct CaarVjpArgs {
  MetricP<R> m;
  DssTable dss;
  DynV x;       // stage input (its n0 state)
  DynV aout;    // cotangent of the stage output (after its DSS)
  DynV xm_bar;  // += spheremp * pre-DSS cotangent
  DynV x0_bar;  // += tendency^T (dt spheremp pre-DSS cotangent); may alias xm_bar
  double dt, p_top;
};

template <typename R>
struct HvVjpArgs {
  MetricP<R> m;
  DssTable dss;
  DynV x;      // subcycle input
  DynV xo;     // subcycle output (recomputed)
  DynV a;      // cotangent of the output
  DynV xb;     // cotangent of the input (written)
  double* pre; // scratch [E][72][4][16]
  double* mid; // scratch [E][72][4][16]
  double dt, nu, nu_s, nu_p, nu_top, nu_ratio1, nu_ratio2;
};

struct RemapVjpArgs {
  DynV x;   // remap input
  DynV a;   // in: cotangent of the remapped v, T and of dp3d = target thickness;
            // out (in place): cotangent of the remap input
  int remap_alg, nelem;
  double ps0, hyai0;
};

template <typename R> void launch_caar_vjp(const CaarVjpArgs<R>& a, int E, cudaStream_t s);
template <typename R> void launch_hv_vjp(const HvVjpArgs<R>& a, int E, cudaStream_t s);
void launch_remap_vjp(const RemapVjpArgs& a, cudaStream_t s);
// b1 += 5/4 by, b0 -= 1/4 by (reverse of the RK5 combination (5 X1 - X0)/4).
void launch_rk5_comb_vjp(int E, DynV by, DynV b1, DynV b0, cudaStream_t s);
// Copy one time level (dst and src may have different element strides).
void launch_copy_dyn(int E, DynV dst, DynV src, cudaStream_t s);

// ---- tangent-linear model of the dry step (hx_tangent.cu) ----------------------------
// Each tangent kernel reads the primal stage input, which the forward kernel launched
// after it then advances.
void upload_tangent_constants(const double* dvv16, const double* hyai73, const double* hybi73,
                              cudaStream_t s);

template <typename R>
struct CaarJvpArgs {
  MetricP<R> m;
  const double *v, *T, *dp;  // primal state [E][3][...] (levels nm1, n0, n0orig read)
  double *tv, *tT, *tdp;     // tangent state [E][3][...]; level nm1 rewritten when rk_combine
  double* out;               // tangent of the pre-DSS result [E][72][4][16]
  int nm1, n0, n0orig, rk_combine;
  double dt, p_top;
};

template <typename R>
struct HvJvpArgs {
  MetricP<R> m;
  DssTable dss;
  const double* v;      // primal v [E][3][72][2][16] before the update
  const double* bufB;   // primal pre-DSS tendencies of the subcycle
  double *tv, *tT, *tdp;  // tangent state, level np1 updated
  const double* tbufB;  // tangent pre-DSS tendencies
  int np1;
  double dt;            // subcycle step
};

struct RemapJvpArgs {
  const double *v, *T, *dp;  // primal state [E][3][...], source at level np1
  double *tv, *tT, *tdp;     // tangent state; v and T of level np1 remapped in place
  double* tps;               // tangent ps_v [E][3][16], level np1 written
  int np1, remap_alg, nelem;
  double ps0, hyai0;
};

template <typename R> void launch_caar_jvp(const CaarJvpArgs<R>& a, int E, cudaStream_t s);
template <typename R> void launch_hv_update_jvp(const HvJvpArgs<R>& a, int E, cudaStream_t s);
void launch_remap_jvp(const RemapJvpArgs& a, cudaStream_t s);
// The two halves of one hyperviscosity subcycle (launch_hv with ncyc = 1): the
// Laplacians into bufB, then the DSS and state update.
template <typename R> void launch_hv_laplacians(const HvArgs<R>& a, int E, cudaStream_t s);
template <typename R> void launch_hv_update(const HvArgs<R>& a, int E, cudaStream_t s);

// Name of the last kernel launched by the wrappers above (for per-kernel timing).
const char* last_kernel_name();
void set_kernel_hook(void (*before)(const char*, cudaStream_t), void (*after)(const char*, cudaStream_t));

}  // namespace hx
