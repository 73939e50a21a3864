/*
 * hxgpu.h — C ABI of the GB300 preqx dycore step (libhxgpu.so).
 *
 * The first block keeps the symbol names and by-reference argument conventions of the
 * HOMMEXX C++ entry points that the Fortran driver binds with ISO_C_BINDING, so that
 * linking libhxgpu.so in place of the reference's C++ library is a drop-in for the
 * preqx step.  Fortran passes every argument by reference: scalars arrive as pointers,
 * and `type(c_ptr)` arrays arrive as a pointer to the c_ptr (the reference's
 * `CF90Ptr&` / `F90Ptr&`, here `const double* const*` / `double* const*`).
 * Arrays are in Fortran column-major layout, e.g. state T is (np,np,nlev,3,nelemd).
 *
 * On a bad option or a negative layer thickness the reference aborts the process with
 * codes 11/12/13/101 (src/share/cxx/ErrorDefs.hpp:51-57).  These symbols do the same by
 * default; after hx_set_abort_on_error(0) they record the error instead, and
 * hx_last_error() returns it.
 *
 * The second block (hx_*) has no counterpart in the reference: status reporting,
 * precision selection, per-phase entry points used by the parity tests, field
 * access and timing.
 */
#ifndef HXGPU_H
#define HXGPU_H

#ifdef __cplusplus
#include <cstddef>
extern "C" {
#else
#include <stdbool.h>
#include <stddef.h>
#endif

/* ---- Reference entry points ------------------------------------------------------ */

/* src/share/cxx/Hommexx_Session.cpp:35 — selects the GPU, creates the stream. */
void initialize_hommexx_session(void);
/* src/share/cxx/Hommexx_Session.cpp:75 — frees all device memory. */
void finalize_hommexx_session(void);

/* src/share/cxx/mpi/mpi_cxx_f90_interface.cpp:20 — single GPU, whole mesh resident:
 * the communicator is recorded and otherwise unused. */
void reset_cxx_comm(const int* f_comm);
/* src/share/cxx/mpi/mpi_cxx_f90_interface.cpp:27-60 — 1-based ids, F90 positions
 * W=1 E=2 S=3 N=4 SW=5 SE=6 NW=7 NE=8. */
void init_connectivity(const int* num_local_elems);
void add_connection(const int* first_elem_lid, const int* first_elem_gid,
                    const int* first_elem_pos, const int* first_elem_pid,
                    const int* second_elem_lid, const int* second_elem_gid,
                    const int* second_elem_pos, const int* second_elem_pid);
void finalize_connectivity(void);

/* src/share/cxx/cxx_f90_interface.cpp:207 — dvv(np,np). */
void init_derivative_c(const double* const* dvv);

/* src/share/cxx/cxx_f90_interface.cpp:33-117 — same option checks. */
void init_simulation_params_c(const int* remap_alg, const int* limiter_option,
                              const int* rsplit, const int* qsplit,
                              const int* time_step_type, const int* energy_fixer,
                              const int* qsize, const int* state_frequency,
                              const double* nu, const double* nu_p, const double* nu_q,
                              const double* nu_s, const double* nu_div, const double* nu_top,
                              const int* hypervis_order, const int* hypervis_subcycle,
                              const double* hypervis_scaling, const int* ftype,
                              const bool* prescribed_wind, const bool* moisture,
                              const bool* disable_diagnostics, const bool* use_cpstar,
                              const bool* use_semi_lagrangian_transport);

/* src/share/cxx/cxx_f90_interface.cpp:119-124 — hyam/hybm(nlev), hyai/hybi(nlev+1). */
void init_hvcoord_c(const double* ps0, const double* const* hybrid_am,
                    const double* const* hybrid_ai, const double* const* hybrid_bm,
                    const double* const* hybrid_bi);

/* src/share/cxx/cxx_f90_interface.cpp:224-233 — D/Dinv/metinv (np,np,2,2,nelemd),
 * 2-D fields (np,np,nelemd), tensorvisc (np,np,2,2,nelemd),
 * vec_sph2cart (np,np,3,2,nelemd). */
void init_elements_2d_c(const int* nelemd, const double* const* D,
                        const double* const* Dinv, const double* const* fcor,
                        const double* const* mp, const double* const* spheremp,
                        const double* const* rspheremp, const double* const* metdet,
                        const double* const* metinv, const double* const* phis,
                        const double* const* tensorvisc, const double* const* vec_sph2cart,
                        const bool* consthv);

/* src/share/cxx/cxx_f90_interface.cpp:235-251 — v (np,np,2,nlev,3,nelemd),
 * T/dp3d (np,np,nlev,3,nelemd), Qdp (np,np,nlev,qsize_d,2,nelemd),
 * ps_v (np,np,3,nelemd).  Host -> device copies. */
void init_elements_states_c(const double* const* v, const double* const* T,
                            const double* const* dp3d, const double* const* Qdp,
                            const double* const* ps_v);

/* src/share/cxx/cxx_f90_interface.cpp:253-262 — host arrays elem%state%Q
 * (np,np,nlev,qsize_d,nelemd) and elem%accum Qvar, Qmass (np,np,qsize_d,4,nelemd), Q1mass
 * (np,np,qsize_d,nelemd), IEner, KEner, PEner (np,np,4,nelemd), IEner_wet (np,np,nelemd);
 * qsize_d is qsize, as for Qdp.  A remap interval that computes diagnostics
 * (prim_driver.cpp:49-58: nstep_end a multiple of state_frequency, equal to nstep0, or
 * >= last_time_step; never with disable_diagnostics) writes them as Diagnostics.cpp does:
 * Q and Qvar/Qmass slots 4, 1, 2 and IEner/KEner/PEner slots 3, 1, 2 (1-based), before
 * forcing, after forcing and after the remap.  Until this is called, no interval computes
 * diagnostics. */
void init_diagnostics_c(double* const* q, double* const* qvar, double* const* qmass,
                        double* const* q1mass, double* const* iener,
                        double* const* iener_wet, double* const* kener,
                        double* const* pener);

/* src/share/cxx/cxx_f90_interface.cpp:264-280 — builds the DSS gather tables. */
void init_boundary_exchanges_c(void);

/* src/share/cxx/cxx_f90_interface.cpp:213-222 — 1-based in, stored 0-based. */
void init_time_level_c(const int* nm1, const int* n0, const int* np1,
                       const int* nstep, const int* nstep0);

/* src/share/cxx/prim_driver.cpp:31-156 — one remap interval; time levels return
 * 0-based as in the reference. */
void prim_run_subcycle_c(const double* dt, int* nstep, int* nm1, int* n0, int* np1,
                         const int* last_time_step);

/* src/share/cxx/cxx_f90_interface.cpp:126-154 — device -> host copies; Q and omega_p
 * are (np,np,nlev,qsize_d,nelemd) and (np,np,nlev,nelemd). */
void cxx_push_results_to_f90(double* const* v, double* const* T, double* const* dp3d,
                             double* const* Qdp, double* const* Q, double* const* ps_v,
                             double* const* omega_p);

/* These two take the arrays themselves (the Fortran interface declares them as
 * real(c_double) arrays, prim_driver_mod.F90:1328-1343), not c_ptr by reference.
 * src/share/cxx/cxx_f90_interface.cpp:180-205 — CAM forcing in: FM (np,np,2,nlev,nelemd),
 * FT (np,np,nlev,nelemd), FQ (np,np,nlev,qsize_d,nelemd; read for ftype 0 only) and the
 * tracer mass Qdp (np,np,nlev,qsize_d,2,nelemd).  The Fortran prim_run_subcycle calls it
 * before every prim_run_subcycle_c (src/share/prim_driver_mod.F90:1380).  The forcing is
 * applied at the start of each remap interval: ftype 0 forces T, v and the tracers
 * (CamForcing.cpp apply_cam_forcing), ftype 2 T and v (apply_cam_forcing_dynamics). */
void f90_push_forcing_to_cxx(const double* FM, const double* FT, const double* FQ,
                             const double* Qdp);
/* src/share/cxx/cxx_f90_interface.cpp:157-178 — the forcing back (FQ for ftype 0 only). */
void cxx_push_forcing_to_f90(double* FM, double* FT, double* FQ);

/* ---- Additions (no counterpart in the reference) ------------------------------------ */

/* Status of the last call: 0 on success, else the reference's error code
 * (11, 12, 13, 101), HX_ERR_CUDA, HX_ERR_STATE or HX_ERR_IO; the message is copied into
 * buf. */
#define HX_ERR_CUDA 200
#define HX_ERR_STATE 201
int hx_last_error(char* buf, int buflen);
/* 1 (default) = exit the process with the reference's code on error; 0 = record. */
void hx_set_abort_on_error(int abort_on_error);

/* 0 = FP64 plain form (default); 1 = mixed form: sphere operators, caar,
 * hyperviscosity and tracer advection in FP32; pressure/geopotential scans, DSS
 * accumulation and PPM remap integrals in FP64.  Call before init_elements_2d_c. */
int hx_set_precision(int mode);

/* Field access in the Fortran layout of one time level, e.g. "T" is
 * (np,np,nlev,nelemd) for time level tl (0-based).  Names: v T dp3d ps_v Qdp Q
 * omega_p phi vn0 eta_dot_dpdn derived_dp divdp divdp_proj dpdiss_ave
 * dpdiss_biharmonic.  tl is ignored for fields without time levels. */
int hx_get_field(const char* name, int tl, double* out);
int hx_set_field(const char* name, int tl, const double* in);

/* Per-phase entry points (0-based time levels), each one reference routine:
 *  CaarFunctor::run + DSS (src/share/cxx/CaarFunctor.cpp:96-116),
 *  u3_5stage_timestep (src/share/cxx/prim_advance_exp.cpp:113-161),
 *  HyperviscosityFunctorImpl::run (src/share/cxx/HyperviscosityFunctorImpl.cpp:56-84),
 *  EulerStepFunctorImpl::euler_step (src/share/cxx/EulerStepFunctorImpl.hpp:514-561)
 *    with dss_opt 0 = ETA, 1 = OMEGA, 2 = DIV_VDP_AVE,
 *  prim_advec_tracers_remap_RK2 (src/share/cxx/prim_advec_tracers_remap.cpp:32-90),
 *  RemapFunctor::run_remap (src/share/cxx/RemapFunctor.hpp:299-331),
 *  prim_step (src/share/cxx/prim_step.cpp:20-103). */
int hx_run_caar_stage(int nm1, int n0, int np1, double dt, double eta_ave_w);
int hx_run_rk5(int nm1, int n0, int np1, int n0_qdp, double dt, double eta_ave_w);
int hx_run_hypervis(int np1, double dt, double eta_ave_w);
int hx_run_euler_step(int np1_qdp, int n0_qdp, double dt, double rhs_multiplier,
                      int dss_opt);
int hx_run_tracers_rk2(double dt);
int hx_run_remap(int np1, int np1_qdp, double dt);
int hx_run_prim_step(double dt);
/* DSS of one registered field at time level tl, optionally scaled by rspheremp. */
int hx_run_dss(const char* name, int tl, int apply_rspheremp);

/* Sizes the library was initialised with. */
int hx_num_elems(void);
int hx_qsize(void);

/* Device kernel timing: when enabled, every launch is bracketed by CUDA events and
 * its time accumulated per kernel name; hx_kernel_stats fills up to max entries of
 * (name, launches, total ms) and returns the number of kernels seen. */
int hx_enable_timing(int on);
int hx_kernel_stats(char* names, int name_len, long long* launches, double* total_ms,
                    int max);
/* No counterpart in the reference.  Bit 0: the library was built with device index
 * checks (HX_BOUNDS_CHECK=1 at build time: DSS table sources, the remap's source-cell
 * search and the tracer slabs are checked, a violation is reported as HX_ERR_CUDA by the
 * interval that met it, and the access is skipped). */
int hx_build_flags(void);
/* Number of kernels this library launched since initialisation. */
long long hx_launch_count(void);
/* Block the host until all device work of the session has finished. */
int hx_synchronize(void);
/* CUDA-event timer on the library's stream: start records an event, stop records a
 * second one, waits for it and returns the elapsed device time in *ms. */
int hx_timer_start(void);
int hx_timer_stop(double* ms);
/* No counterpart in the reference.  Measured FP64 throughput of the current device in
 * TFLOP/s (2 per fused multiply-add): a kernel of independent FMA chains at full
 * occupancy, timed with CUDA events after a warm-up launch (~0.1 s).  The roof of the
 * FP64 form's kernels, which the FP64 pipe bounds rather than HBM.  Returns 0 or
 * HX_ERR_CUDA; needs no session. */
int hx_fp64_peak(double* tflops);
/* No counterpart in the reference.  DSS of one caller-owned device field
 * [nelem][nlev][np*np] (in and out may alias) without allocating device memory, for
 * callers that cannot call cudaMalloc when they need it (a host model that reserves
 * its GPU memory budget up front, code where allocation is forbidden).  Scratch is a
 * fixed 4 MiB __device__ array (at most 455 elements of 72 levels); larger fields are
 * rejected with code 13.  The array is made resident on the session's device during
 * init_boundary_exchanges_c (its address is looked up there, which loads it under
 * CUDA's lazy module loading), so the call itself loads and allocates nothing; it
 * holds those 4 MiB until the process exits.  It must be made with the session's
 * device current (HX_ERR_STATE otherwise).  Calls share the array, so calls that
 * overlap on the GPU race; the array keeps the last call's contents and needs no
 * clearing because every call overwrites what it reads.  Enqueued on the session's
 * stream; returns 0, 13 or HX_ERR_STATE/HX_ERR_CUDA. */
int hx_dss_noalloc(const double* in, double* out, int nelem, int apply_rspheremp);

/* ---- Dry-dynamics trajectory and its adjoint (no counterpart in the reference) ----
 * A trajectory of nsteps steps, each the dynamics part of prim_step for rsplit > 0:
 * u3_5stage caar with DSS (src/share/cxx/prim_advance_exp.cpp:113-161), the
 * hyperviscosity subcycles (src/share/cxx/HyperviscosityFunctorImpl.cpp:56-84) and,
 * after every rsplit-th step, the PPM remap of v and T (src/share/cxx/RemapFunctor.hpp:
 * 299-331) with dp3d reset to the hybrid thickness from ps, as the next remap interval
 * starts (src/share/cxx/prim_driver.cpp:90-113).  Dry: tracers are not advected, T_v = T.
 * Uses the session's mesh, hybrid coordinate and namelist values (nu, nu_p, nu_s,
 * nu_top, hypervis_subcycle, rsplit, remap_alg); tensor hyperviscosity is rejected
 * with code 12.  States are one time level in the Fortran layout: v (np,np,2,nlev,
 * nelemd), T and dp3d (np,np,nlev,nelemd); pointers may be host or device memory.
 *
 * hx_traj_forward runs the trajectory from (v, T, dp3d), writes the final state and
 * keeps the checkpoints its adjoint needs (returns 101 on a negative layer
 * thickness).  hx_traj_vjp takes the cotangent of the final state and returns the
 * gradient with respect to the initial state (a vector-Jacobian product), reversing
 * the last forward trajectory: each caar stage, hyperviscosity subcycle and remap is
 * differentiated by hand, with its inputs checkpointed and its intermediates
 * recomputed.  hx_traj_jvp is the tangent-linear model along the same trajectory (a
 * Jacobian-vector product: the tangent of the final state from a tangent of the
 * initial one), run forward from the trajectory's checkpointed initial state with
 * hand-written tangent kernels beside the forward ones.
 * hx_traj_set_checkpointing: 0 = automatic (every RK stage and hyperviscosity
 * subcycle input of every step when that fits in device memory, else mode 2), 1 =
 * keep every stage input, 2 = keep the step inputs only and recompute each step's
 * stage inputs when reversing it (one extra forward step of work per step). */
int hx_traj_forward(const double* v, const double* T, const double* dp3d, int nsteps,
                    double dt, double* v_out, double* T_out, double* dp3d_out);
int hx_traj_vjp(const double* v_bar, const double* T_bar, const double* dp3d_bar,
                double* v_grad, double* T_grad, double* dp3d_grad);
int hx_traj_jvp(const double* dv, const double* dT, const double* ddp3d, double* v_tan,
                double* T_tan, double* dp3d_tan);
int hx_traj_set_checkpointing(int mode);

/* ---- Cubed-sphere mesh generated on the GPU (no counterpart in the reference's C++
 * layer) ----
 * The inputs the Fortran driver builds before it calls init_derivative_c,
 * init_elements_2d_c and add_connection, for an equiangular gnomonic cubed sphere of
 * 6 ne^2 elements with np = 4 GLL points: dvv (derivative_mod_base.F90:437-475), the
 * metric of metric_atomic (cube_mod.F90:215-454) rescaled to a total area of 4 pi as
 * prim_driver_mod.F90:403-418 does, mp and spheremp = mp metdet, rspheremp = 1/DSS
 * (spheremp) (mass_matrix_mod.F90:98-115), fcor = 2 Omega sin(lat), vec_sphere2cart and,
 * when hypervis_scaling != 0, tensorVisc (cube_mod.F90:310-440); Omega = 7.292e-5,
 * rearth = 6.376e6.  Host outputs in the layouts init_elements_2d_c takes: D, Dinv,
 * metinv, tensorvisc (np,np,2,2,nelemd); vec_sph2cart (np,np,3,2,nelemd); fcor, mp,
 * spheremp, rspheremp, metdet, lat, lon (np,np,nelemd); dvv (np,np).  connections
 * (2,8,nelemd): for element e and add_connection position k (W=1 E=2 S=3 N=4 SW=5 SE=6
 * NW=7 NE=8) the 1-based remote element and its position, or 0 0 where there is no
 * neighbour (the missing corner of the elements at the eight cube corners).  Elements
 * are ordered face by face, then row by row.  Any output may be null.  The metric is
 * computed on the GPU, one thread per GLL point; the connectivity on the host from exact
 * integer corner positions.  Needs no session.  Returns 0, 13 (ne outside [1, 1024]) or
 * HX_ERR_CUDA. */
int hx_cube_mesh(int ne, double hypervis_scaling, double* dvv, double* D, double* Dinv,
                 double* fcor, double* mp, double* spheremp, double* rspheremp,
                 double* metdet, double* metinv, double* tensorvisc, double* vec_sph2cart,
                 double* lat, double* lon, int* connections);

/* ---- Restart files (no counterpart in the reference's C++ layer) ------------------
 * A binary restart format in place of the Fortran restart_io_mod.F90 (WriteRestart /
 * ReadRestart, src/restart_io_mod.F90:626-698): a 128-byte header, then one record per
 * element holding the prognostic elem_state_t of src/share/element_mod.F90:103-115 in
 * its Fortran layouts, in this order:
 *   v (np,np,2,nlev,3)  T (np,np,nlev,3)  dp3d (np,np,nlev,3)  ps_v (np,np,3)
 *   phis (np,np)  Q (np,np,nlev,qsize)  Qdp (np,np,nlev,qsize,2)
 * All numbers little-endian; doubles are IEEE binary64.  The header keeps the
 * reference's TimeLevel_t (nm1, n0, np1 1-based; nstep, nstep0) and is checked on
 * read against the session (nelem, np, nlev, qsize), as CheckRestartHeader checks ne,
 * np and nlev (src/restart_io_mod.F90:440-471).  checksum is the sum modulo 2^64, over
 * the 64-bit words w_k of all records (k = 0, 1, ... from the first record), of
 * splitmix64(w_k + (k + 1) * 0x9E3779B97F4A7C15), splitmix64 being the output
 * function z ^= z >> 30; z *= 0xBF58476D1CE4E5B9; z ^= z >> 27; z *= 0x94D049BB133111EB;
 * z ^= z >> 31 (Steele, Lea and Flood, OOPSLA 2014).
 * hx_write_restart writes the session's state and time levels; hx_read_restart
 * replaces them (phis included).  Both stream the records through host buffers of at
 * most 256 MiB, so device memory use does not grow.  hx_read_restart reads the file
 * twice: it verifies the checksum on the host first, so a failed read (damaged,
 * truncated or mismatched file) leaves the session's state and time levels unchanged.
 * Errors: HX_ERR_IO (open, read, write, bad magic or version, size mismatch,
 * checksum), HX_ERR_STATE (no session). */
#define HX_ERR_IO 202
#define HX_RESTART_MAGIC "HXRESTRT"
#define HX_RESTART_VERSION 1
typedef struct hx_restart_header {
  char magic[8];         /* HX_RESTART_MAGIC, not NUL-terminated */
  unsigned int version;  /* HX_RESTART_VERSION */
  unsigned int header_bytes;  /* 128 */
  int nelem, np, nlev, qsize, timelevels, qsize_timelevels;  /* -, 4, 72, -, 3, 2 */
  int nm1, n0, np1, nstep, nstep0;  /* TimeLevel_t, levels 1-based */
  int reserved0;
  unsigned long long record_bytes;  /* bytes of one element record */
  unsigned long long checksum;
  char reserved[48];
} hx_restart_header;
int hx_write_restart(const char* path);
int hx_read_restart(const char* path);

/* Copies that overlap the step (no counterpart in the reference).  Host<->device
 * traffic runs on the host link (about 210 GB/s in, 190 GB/s out on a GB300), so the
 * state copied in and out every interval costs as much as a third of a mixed-form
 * interval unless it overlaps the step's kernels.
 * hx_set_async_copies(1): init_elements_states_c returns once v, T, dp3d and ps_v are on
 * the device (one contiguous copy each); Qdp keeps streaming in on a copy stream and the
 * first kernel that reads it (the first tracer step) waits for it.  The caller must
 * leave the Qdp host array unchanged until the next prim_run_subcycle_c (or any other
 * call of this library) returns.  Default 0.
 * hx_stream_results(v, T, dp3d, Qdp, Q, ps_v, omega_p): host destinations in the
 * layouts of cxx_push_results_to_f90 (all seven, or all NULL to stop).  Every following
 * prim_run_subcycle_c copies its results there before it returns, each piece as soon as
 * it is final: dynamics level n0 while the interval's last dynamics step runs (it only
 * reads it), level nm1 once that step's RK stages are done, the tracer level the last
 * tracer step only reads before that step, omega_p after it, and level np1, the other
 * tracer level and Q chunk by chunk of elements from a final remap and update_q split
 * into launches of whole waves, so most of the copy overlaps the step's kernels; a
 * cxx_push_results_to_f90 with the same seven pointers right after it returns at once.
 * The destinations should be page-locked (hx_host_register) for the copies to overlap. */
int hx_set_async_copies(int on);
int hx_stream_results(double* v, double* T, double* dp3d, double* Qdp, double* Q,
                      double* ps_v, double* omega_p);

/* Page-lock (pin) host memory so init/push copies run at full link bandwidth. */
int hx_host_register(void* ptr, size_t bytes);
int hx_host_unregister(void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* HXGPU_H */
