/* A C driver of libhxgpu.so, run on a host without a GPU: includes include/hxgpu.h as
 * C, passes arguments the way Fortran's ISO_C_BINDING does (scalars by reference), and
 * checks the status path: the session reports HX_ERR_CUDA, a step without a session
 * HX_ERR_STATE (nothing runs on the host instead), and the reference's option check
 * still answers 11.  Prints the codes; exit status 0 when they are the expected ones. */
#include <stdio.h>

#include "hxgpu.h"

int main(void) {
  char msg[256];
  hx_set_abort_on_error(0);
  initialize_hommexx_session();
  const int init_code = hx_last_error(msg, (int)sizeof msg);
  /* a session-less step: state error, never a CPU fallback */
  const int step_code = hx_run_prim_step(300.0);
  /* the reference's option checks (cxx_f90_interface.cpp:43-52): limiter 4 -> 11 */
  int remap_alg = 1, limiter = 4, rsplit = 3, qsplit = 1, tstep = 5, efix = 0, qsize = 4, freq = 1;
  double nu = 1e15, nu_p = -1, nu_q = -1, nu_s = -1, nu_div = -1, nu_top = 2.5e5, hvs = 0;
  int hvo = 2, hsub = 3, ftype = -1;
  bool pw = false, moist = false, nodiag = true, cpstar = false, sl = false;
  init_simulation_params_c(&remap_alg, &limiter, &rsplit, &qsplit, &tstep, &efix, &qsize, &freq, &nu, &nu_p,
                           &nu_q, &nu_s, &nu_div, &nu_top, &hvo, &hsub, &hvs, &ftype, &pw, &moist, &nodiag,
                           &cpstar, &sl);
  const int opt_code = hx_last_error(msg, (int)sizeof msg);
  printf("init %d, prim_step without a session %d, limiter_option 4 %d\n", init_code, step_code, opt_code);
  return (init_code == HX_ERR_CUDA && step_code == HX_ERR_STATE && opt_code == 11) ? 0 : 1;
}
