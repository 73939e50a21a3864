/* A C driver of libhxgpu.so that makes the Fortran driver's call sequence: the
 * initialisation of prim_driver_mod.F90 (prim_init2 -> prim_create_c_data_structures /
 * prim_init_elements_views / prim_init_state_views / init_boundary_exchanges_c /
 * init_time_level_c, src/share/prim_driver_mod.F90:1045-1104, with the connectivity of
 * prim_cxx_driver_mod.F90:131-140) and the time loop of prim_main.F90:297-317
 * (prim_run_subcycle_c each remap interval, then cxx_push_results_to_f90), passing
 * every argument by reference as ISO_C_BINDING does and every array in its Fortran
 * layout.
 *
 * Usage: prim_main_from_c <input file> <output file>.  The input holds, in this order
 * (little-endian): int32 nelem, qsize, nconn, nint, rsplit, hypervis_subcycle,
 * limiter_option, remap_alg; double dt, nu, nu_top, ps0; int32 connections[nconn][8]
 * (the add_connection arguments); double dvv[16], hyam[72], hyai[73], hybm[72],
 * hybi[73]; the init_elements_2d_c arrays D, Dinv (nelem*64), fcor, mp, spheremp,
 * rspheremp, metdet (nelem*16), metinv (nelem*64), phis (nelem*16), tensorvisc
 * (nelem*64), vec_sph2cart (nelem*96); the state v (nelem*3*72*32), T, dp3d
 * (nelem*3*72*16), Qdp (nelem*2*qsize*72*16), ps_v (nelem*3*16).  The output holds the
 * arrays cxx_push_results_to_f90 returns (v, T, dp3d, Qdp, Q, ps_v, omega_p) after nint
 * remap intervals, then int32 nstep, nm1, n0, np1 as prim_run_subcycle_c returned them.
 * Exit status 0, or the library's error code. */
#include <stdio.h>
#include <stdlib.h>

#include "hxgpu.h"

static FILE* fin;

static void* take(size_t n, size_t size) {
  void* p = malloc(n > 0 ? n * size : 1);
  if (!p || fread(p, size, n, fin) != n) {
    fprintf(stderr, "short input\n");
    exit(2);
  }
  return p;
}

static int status(const char* what) {
  char msg[512];
  const int code = hx_last_error(msg, (int)sizeof msg);
  if (code) fprintf(stderr, "%s: error %d: %s\n", what, code, msg);
  return code;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  fin = fopen(argv[1], "rb");
  if (!fin) return 2;
  int* hd = (int*)take(8, sizeof(int));
  const int nelem = hd[0], qsize = hd[1], nconn = hd[2], nint = hd[3];
  int rsplit = hd[4], hsub = hd[5], limiter = hd[6], remap_alg = hd[7];
  double* par = (double*)take(4, sizeof(double));
  double dt = par[0], nu = par[1], nu_top = par[2], ps0 = par[3];
  int* conn = (int*)take((size_t)nconn * 8, sizeof(int));
  double* dvv = (double*)take(16, sizeof(double));
  double* hyam = (double*)take(72, sizeof(double));
  double* hyai = (double*)take(73, sizeof(double));
  double* hybm = (double*)take(72, sizeof(double));
  double* hybi = (double*)take(73, sizeof(double));
  const size_t E = (size_t)nelem;
  double* D = (double*)take(E * 64, sizeof(double));
  double* Dinv = (double*)take(E * 64, sizeof(double));
  double* fcor = (double*)take(E * 16, sizeof(double));
  double* mp = (double*)take(E * 16, sizeof(double));
  double* spheremp = (double*)take(E * 16, sizeof(double));
  double* rspheremp = (double*)take(E * 16, sizeof(double));
  double* metdet = (double*)take(E * 16, sizeof(double));
  double* metinv = (double*)take(E * 64, sizeof(double));
  double* phis = (double*)take(E * 16, sizeof(double));
  double* tensorvisc = (double*)take(E * 64, sizeof(double));
  double* vec = (double*)take(E * 96, sizeof(double));
  const size_t n3 = E * 72 * 16;
  double* v = (double*)take(n3 * 3 * 2, sizeof(double));
  double* T = (double*)take(n3 * 3, sizeof(double));
  double* dp3d = (double*)take(n3 * 3, sizeof(double));
  double* Qdp = (double*)take(n3 * 2 * (size_t)qsize, sizeof(double));
  double* ps_v = (double*)take(E * 3 * 16, sizeof(double));
  fclose(fin);

  hx_set_abort_on_error(0);
  /* prim_driver_mod.F90:143 */
  initialize_hommexx_session();
  if (status("initialize_hommexx_session")) return 1;
  int comm = 0;
  reset_cxx_comm(&comm);
  /* prim_cxx_driver_mod.F90:131-140 */
  init_connectivity(&nelem);
  for (int c = 0; c < nconn; ++c) {
    const int* t = conn + (size_t)c * 8;
    add_connection(&t[0], &t[1], &t[2], &t[3], &t[4], &t[5], &t[6], &t[7]);
  }
  finalize_connectivity();
  if (status("connectivity")) return 1;
  /* prim_driver_mod.F90:82, 1045-1054 */
  const double* pdvv = dvv;
  init_derivative_c(&pdvv);
  int qsplit = 1, tstep = 5, efix = 0, freq = 1000000, hvo = 2, ftype = -1;
  double nu_p = nu, nu_q = nu, nu_s = nu, nu_div = nu, hvs = 0.0;
  bool pw = false, moist = false, nodiag = true, cpstar = false, sl = false;
  init_simulation_params_c(&remap_alg, &limiter, &rsplit, &qsplit, &tstep, &efix, &qsize, &freq, &nu, &nu_p,
                           &nu_q, &nu_s, &nu_div, &nu_top, &hvo, &hsub, &hvs, &ftype, &pw, &moist, &nodiag,
                           &cpstar, &sl);
  if (status("init_simulation_params_c")) return 1;
  /* prim_driver_mod.F90:1068-1072 */
  const double *pD = D, *pDinv = Dinv, *pf = fcor, *pmp = mp, *psp = spheremp, *prsp = rspheremp, *pmd = metdet,
               *pmi = metinv, *pph = phis, *ptv = tensorvisc, *pvec = vec;
  const bool consthv = true;
  init_elements_2d_c(&nelem, &pD, &pDinv, &pf, &pmp, &psp, &prsp, &pmd, &pmi, &pph, &ptv, &pvec, &consthv);
  if (status("init_elements_2d_c")) return 1;
  /* prim_driver_mod.F90:1079-1080 */
  const double *pv = v, *pT = T, *pdp = dp3d, *pq = Qdp, *pps = ps_v;
  init_elements_states_c(&pv, &pT, &pdp, &pq, &pps);
  if (status("init_elements_states_c")) return 1;
  /* prim_driver_mod.F90:1100-1104 */
  const double *pam = hyam, *pai = hyai, *pbm = hybm, *pbi = hybi;
  init_hvcoord_c(&ps0, &pam, &pai, &pbm, &pbi);
  init_boundary_exchanges_c();
  if (status("init_boundary_exchanges_c")) return 1;
  int nm1 = 1, n0 = 2, np1 = 3, nstep = 0, nstep0 = 0;
  init_time_level_c(&nm1, &n0, &np1, &nstep, &nstep0);
  /* prim_main.F90:297-317: prim_run_subcycle each interval, results to Fortran */
  for (int it = 0; it < nint; ++it) {
    const int last = 1 << 30;
    prim_run_subcycle_c(&dt, &nstep, &nm1, &n0, &np1, &last);
    if (status("prim_run_subcycle_c")) return 1;
  }
  double* Q = (double*)malloc(n3 * (size_t)(qsize ? qsize : 1) * sizeof(double));
  double* omega_p = (double*)malloc(n3 * sizeof(double));
  double *ov = v, *oT = T, *odp = dp3d, *oq = Qdp, *oQ = Q, *ops = ps_v, *oom = omega_p;
  cxx_push_results_to_f90(&ov, &oT, &odp, &oq, &oQ, &ops, &oom);
  if (status("cxx_push_results_to_f90")) return 1;
  finalize_hommexx_session();

  FILE* fo = fopen(argv[2], "wb");
  if (!fo) return 2;
  fwrite(v, sizeof(double), n3 * 6, fo);
  fwrite(T, sizeof(double), n3 * 3, fo);
  fwrite(dp3d, sizeof(double), n3 * 3, fo);
  fwrite(Qdp, sizeof(double), n3 * 2 * (size_t)qsize, fo);
  fwrite(Q, sizeof(double), n3 * (size_t)qsize, fo);
  fwrite(ps_v, sizeof(double), E * 48, fo);
  fwrite(omega_p, sizeof(double), n3, fo);
  const int tl[4] = {nstep, nm1, n0, np1};
  fwrite(tl, sizeof(int), 4, fo);
  fclose(fo);
  printf("prim_main_from_c: %d elements, %d tracers, %d remap intervals, time levels %d %d %d, nstep %d\n", nelem,
         qsize, nint, nm1, n0, np1, nstep);
  return 0;
}
