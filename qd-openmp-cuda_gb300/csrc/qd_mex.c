/*
 * qd_mex.c - MATLAB MEX shim: cudaOpenMPEvolution(FH2Data) on top of libqd.
 *
 * Replaces the reference's mexFunction (cudaOpenMPEvolution.C:15-79) and its
 * struct views (matlabStructures.C:17-153): every field is read from the
 * MATLAB struct as a borrowed pointer, exactly as the reference does, and the
 * outputs are written in place (OmegaStates.wave_packets, time.steps, CRP.CRP).
 * insist() failures and CUDA errors come back as mexErrMsgTxt, like
 * MatlabCrashLoc (matlabUtils.C:8-13); nothing calls exit().
 *
 * The options.wave_to_matlab script runs when script.m exists
 * (wave2matlab.C:19-26), after the wave packets have been copied into
 * OmegaStates.wave_packets and with time.steps already holding the step
 * counter in MATLAB's memory: the reference binds time.steps by reference
 * (matlabStructures.C:42) and its plotting script reads it (FH2Matlab.m:18).
 * The script runs through mexCallMATLABWithTrap, so a MATLAB error inside it
 * returns here instead of unwinding through libqd's frames (which would skip
 * the release of its device memory and stream); libqd returns
 * QD_ERR_CALLBACK, and the script's own MATLAB exception is rethrown once
 * libqd has returned.
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

static void fail(const char *what, const char *name) {
  char buf[200];
  snprintf(buf, sizeof buf, "insist failed: %s %s", what, name);
  mexErrMsgTxt(buf);
}

static const mxArray *req(const mxArray *s, const char *name) {
  const mxArray *f = mxGetField(s, 0, name);
  if (!f) fail("field", name);
  return f;
}

/* a required numeric field of the given class with at least `min_elems` elements */
static void *num(const mxArray *s, const char *name, mxClassID cls, size_t min_elems) {
  const mxArray *f = req(s, name);
  if (mxGetClassID(f) != cls || mxIsComplex(f)) fail("class of field", name);
  if (mxGetNumberOfElements(f) < min_elems) fail("size of field", name);
  return mxGetData(f);
}

static int32_t i32(const mxArray *s, const char *name) { return *(const int32_t *)num(s, name, mxINT32_CLASS, 1); }
static double f64(const mxArray *s, const char *name) { return *(const double *)num(s, name, mxDOUBLE_CLASS, 1); }

static char *str(const mxArray *s, const char *name) {
  const mxArray *f = mxGetField(s, 0, name);
  return f ? mxArrayToString(f) : NULL;
}

/* what the callback needs: the script and MATLAB's own time.steps */
typedef struct script_ctx {
  const char *script;
  int32_t *steps;       /* MATLAB memory of FH2Data.time.steps */
  mxArray *exception;   /* MException raised by the script, rethrown after qd_evolve */
} script_ctx;

/* wavepacket_to_matlab(options.wave_to_matlab) if <script>.m exists */
static int call_script(qd_fh2data *d, void *user) {
  script_ctx *ctx = (script_ctx *)user;
  char file[1024];
  snprintf(file, sizeof file, "%s.m", ctx->script);
  if (access(file, F_OK) != 0) return 0;
  *ctx->steps = d->time.steps;   /* the script sees the live counter */
  ctx->exception = mexCallMATLABWithTrap(0, NULL, 0, NULL, ctx->script);
  return ctx->exception != NULL;
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
  if (q.r1.n <= 0 || q.r2.n <= 0 || q.theta.n <= 0) mexErrMsgTxt("insist failed: grid sizes > 0");
  const size_t n1 = (size_t)q.r1.n, n2 = (size_t)q.r2.n, nth = (size_t)q.theta.n;
  q.theta.x = (const double *)num(th, "x", mxDOUBLE_CLASS, nth);
  q.theta.w = (const double *)num(th, "w", mxDOUBLE_CLASS, nth);
  if (mxGetField(th, 0, "associated_legendre"))
    q.theta.associated_legendre = (const double *)num(th, "associated_legendre", mxDOUBLE_CLASS, 0);
  q.pot = (const double *)num(D, "pot", mxDOUBLE_CLASS, n1 * n2 * nth);

  const mxArray *tm = req(D, "time");
  int32_t *steps = (int32_t *)num(tm, "steps", mxINT32_CLASS, 1);   /* in/out, as matlabStructures.C:42 */
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
  if (mxGetField(op, 0, "precision")) q.options.precision = i32(op, "precision");
  char *autotune_cache = str(op, "autotune_cache");   /* optional extension */
  q.options.autotune_cache = autotune_cache;

  /* masks: optional, active only when both are present (matlabData.h:27) */
  const mxArray *d1 = mxGetField(D, 0, "dump1"), *d2 = mxGetField(D, 0, "dump2");
  if (d1 && mxGetField(d1, 0, "dump")) q.dump1.dump = (const double *)num(d1, "dump", mxDOUBLE_CLASS, n1);
  if (d2 && mxGetField(d2, 0, "dump")) q.dump2.dump = (const double *)num(d2, "dump", mxDOUBLE_CLASS, n2);

  const mxArray *crp = req(D, "CRP");
  q.CRP.n_dividing_surface = i32(crp, "n_dividing_surface");
  q.CRP.n_gradient_points = i32(crp, "n_gradient_points");
  q.CRP.n_energies = i32(crp, "n_energies");
  q.CRP.calculate_CRP = i32(crp, "calculate_CRP");
  if (q.CRP.calculate_CRP) {
    const size_t ne = q.CRP.n_energies > 0 ? (size_t)q.CRP.n_energies : 0;
    q.CRP.energies = (const double *)num(crp, "energies", mxDOUBLE_CLASS, ne);
    q.CRP.eta_sq = (const double *)num(crp, "eta_sq", mxDOUBLE_CLASS, ne);
    q.CRP.CRP = (double *)num(crp, "CRP", mxDOUBLE_CLASS, ne);
  }

  const mxArray *om = req(D, "OmegaStates");
  const mxArray *omegas = req(om, "omegas");
  const mxArray *al = req(om, "associated_legendres");
  const mxArray *wp = req(om, "wave_packets");
  if (mxGetClassID(omegas) != mxINT32_CLASS) fail("class of field", "omegas");
  q.OmegaStates.J = i32(om, "J");
  q.OmegaStates.parity = i32(om, "parity");
  q.OmegaStates.l_max = i32(om, "l_max");
  q.OmegaStates.n_omegas_max = i32(om, "n_omegas_max");
  q.OmegaStates.n_omegas = (int32_t)mxGetNumberOfElements(omegas);
  q.OmegaStates.omegas = (const int32_t *)mxGetData(omegas);
  if (mxGetClassID(al) != mxDOUBLE_CLASS || mxGetNumberOfDimensions(al) < 2)
    fail("class of field", "associated_legendres");
  q.OmegaStates.associated_legendres = (const double *)mxGetData(al);
  q.OmegaStates.n_cols = (int32_t)mxGetDimensions(al)[1];
  const size_t n_om = (size_t)q.OmegaStates.n_omegas;
  /* every block's [n_theta][n_cols] Legendre matrix, and its [2 n1][n2][n_theta]
     packet (the reference's insist(2*size == n1*n2*n3), matlabStructures.C:146):
     libqd reads and writes exactly these extents */
  if (mxGetNumberOfElements(al) < nth * (size_t)q.OmegaStates.n_cols * n_om)
    fail("size of field", "associated_legendres");
  if (mxGetClassID(wp) != mxDOUBLE_CLASS || mxIsComplex(wp) || mxGetNumberOfElements(wp) != 2 * n1 * n2 * nth * n_om)
    fail("size of field", "wave_packets (2 n1 x n2 x n_theta x n_omegas doubles)");
  q.OmegaStates.wave_packets = (double *)mxGetData(wp);

  script_ctx ctx = {script, steps, NULL};
  const int st = qd_evolve(&q, script ? call_script : NULL, &ctx);
  *steps = q.time.steps;
  if (script) mxFree(script);
  if (test_name) mxFree(test_name);
  if (autotune_cache) mxFree(autotune_cache);
  if (ctx.exception) mexCallMATLAB(0, NULL, 1, &ctx.exception, "rethrow");   /* the script's own error */
  if (st != QD_OK) mexErrMsgTxt(qd_last_error());
}
