/*
 * qd_mex.c - MATLAB MEX shim: cudaOpenMPEvolution(FH2Data) on top of libqd.
 *
 * Replaces the reference's mexFunction (cudaOpenMPEvolution.C:15-79) and its
 * struct views (matlabStructures.C:17-153): every field is read from the
 * MATLAB struct as a borrowed pointer, exactly as the reference does, and the
 * outputs are written in place (OmegaStates.wave_packets, time.steps, CRP.CRP).
 * insist() failures and CUDA errors come back as mexErrMsgTxt, like
 * MatlabCrashLoc (matlabUtils.C:8-13); nothing calls exit().  The
 * options.wave_to_matlab script is run through mexCallMATLAB when script.m
 * exists (wave2matlab.C:19-26).
 *
 * Build (needs MATLAB; not part of the default build):
 *   mex -I<repo>/include qd_mex.c -L<repo>/qd-openmp-cuda_gb300 -lqd \
 *       -output cudaOpenMPEvolution
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <mex.h>

#include "qd.h"

static const mxArray *req(const mxArray *s, const char *name) {
  const mxArray *f = mxGetField(s, 0, name);
  if (!f) {
    char buf[160];
    snprintf(buf, sizeof buf, "insist failed: field %s", name);
    mexErrMsgTxt(buf);
  }
  return f;
}

static void *dat(const mxArray *s, const char *name) {
  const mxArray *f = mxGetField(s, 0, name);
  return f ? mxGetData(f) : NULL;
}

static int i32(const mxArray *s, const char *name) {
  const void *p = dat(s, name);
  if (!p) mexErrMsgTxt("insist failed: int32 field missing");
  return *(const int32_t *)p;
}

static double f64(const mxArray *s, const char *name) {
  const void *p = dat(s, name);
  if (!p) mexErrMsgTxt("insist failed: double field missing");
  return *(const double *)p;
}

static char *str(const mxArray *s, const char *name) {
  const mxArray *f = mxGetField(s, 0, name);
  return f ? mxArrayToString(f) : NULL;
}

/* mexCallMATLAB(options.wave_to_matlab) if <script>.m exists */
static int call_script(qd_fh2data *d, void *user) {
  (void)d;
  const char *script = (const char *)user;
  char file[1024];
  snprintf(file, sizeof file, "%s.m", script);
  if (access(file, F_OK) != 0) return 0;
  return mexCallMATLAB(0, NULL, 0, NULL, script) != 0;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  (void)nlhs;
  (void)plhs;
  if (nrhs != 1) mexErrMsgTxt("insist failed: nrhs == 1");
  const mxArray *D = prhs[0];
  qd_fh2data q;
  memset(&q, 0, sizeof q);

  const mxArray *r1 = req(D, "r1"), *r2 = req(D, "r2"), *th = req(D, "theta");
  q.r1.n = i32(r1, "n");
  q.r1.left = f64(r1, "left");
  q.r1.dr = f64(r1, "dr");
  q.r1.mass = f64(r1, "mass");
  q.r2.n = i32(r2, "n");
  q.r2.left = f64(r2, "left");
  q.r2.dr = f64(r2, "dr");
  q.r2.mass = f64(r2, "mass");
  q.theta.n = i32(th, "n");
  q.theta.m = i32(th, "m");
  q.theta.x = (const double *)dat(th, "x");
  q.theta.w = (const double *)dat(th, "w");
  q.theta.associated_legendre = (const double *)dat(th, "associated_legendre");
  q.pot = (const double *)mxGetData(req(D, "pot"));

  const mxArray *tm = req(D, "time");
  int32_t *steps = (int32_t *)dat(tm, "steps");   /* in/out, as matlabStructures.C:42 */
  q.time.total_steps = i32(tm, "total_steps");
  q.time.time_step = f64(tm, "time_step");
  q.time.steps = *steps;

  const mxArray *op = req(D, "options");
  char *script = str(op, "wave_to_matlab");
  if (script) {   /* remove_matlab_script_extension (matlabStructures.C:5-12) */
    const size_t n = strlen(script);
    if (n > 2 && strcmp(script + n - 2, ".m") == 0) script[n - 2] = '\0';
  }
  char *test_name = str(op, "test_name");
  q.options.wave_to_matlab = script;
  q.options.test_name = test_name;
  q.options.steps_to_copy_psi_from_device_to_host = i32(op, "steps_to_copy_psi_from_device_to_host");
  q.options.use_p2p_async = i32(op, "use_p2p_async");
  if (dat(op, "precision")) q.options.precision = i32(op, "precision");

  const mxArray *d1 = mxGetField(D, 0, "dump1"), *d2 = mxGetField(D, 0, "dump2");
  q.dump1.dump = d1 ? (const double *)dat(d1, "dump") : NULL;
  q.dump2.dump = d2 ? (const double *)dat(d2, "dump") : NULL;

  const mxArray *crp = req(D, "CRP");
  q.CRP.n_dividing_surface = i32(crp, "n_dividing_surface");
  q.CRP.n_gradient_points = i32(crp, "n_gradient_points");
  q.CRP.n_energies = i32(crp, "n_energies");
  q.CRP.calculate_CRP = i32(crp, "calculate_CRP");
  q.CRP.energies = (const double *)dat(crp, "energies");
  q.CRP.eta_sq = (const double *)dat(crp, "eta_sq");
  q.CRP.CRP = (double *)dat(crp, "CRP");

  const mxArray *om = req(D, "OmegaStates");
  const mxArray *omegas = req(om, "omegas");
  const mxArray *al = req(om, "associated_legendres");
  const mxArray *wp = req(om, "wave_packets");
  q.OmegaStates.J = i32(om, "J");
  q.OmegaStates.parity = i32(om, "parity");
  q.OmegaStates.l_max = i32(om, "l_max");
  q.OmegaStates.n_omegas_max = i32(om, "n_omegas_max");
  q.OmegaStates.n_omegas = (int32_t)mxGetNumberOfElements(omegas);
  q.OmegaStates.omegas = (const int32_t *)mxGetData(omegas);
  q.OmegaStates.associated_legendres = (const double *)mxGetData(al);
  q.OmegaStates.n_cols = (int32_t)mxGetDimensions(al)[1];
  q.OmegaStates.wave_packets = (double *)mxGetData(wp);

  const int st = qd_evolve(&q, script ? call_script : NULL, script);
  *steps = q.time.steps;
  if (script) mxFree(script);
  if (test_name) mxFree(test_name);
  if (st != QD_OK) mexErrMsgTxt(qd_last_error());
}
