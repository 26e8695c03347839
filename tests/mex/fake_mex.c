/*
 * fake_mex.c - a minimal MEX runtime for testing the MEX shim without MATLAB.
 *
 * TEST INFRASTRUCTURE.  mxArrays are small in-memory records: structs (named
 * fields), numeric arrays that borrow caller memory (so in-place writes by the
 * shim are visible to the caller, as in MATLAB), and char arrays.
 * mexErrMsgTxt longjmps back to fm_run, as MATLAB unwinds a MEX call.  MATLAB
 * scripts are a callback into the test (fm_set_script_handler); a script that
 * fails makes mexCallMATLABWithTrap return an exception object, which
 * mexCallMATLAB(..., "rethrow") raises.  Counters report how many errors were
 * raised and how many mxArrayToString strings are still allocated.
 */
#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"

#define FM_MAX_FIELDS 32
#define FM_MAX_ARRAYS 4096

struct mxArray_tag {
  mxClassID cls;
  size_t ndims;
  size_t dims[4];
  void *data;                       /* borrowed (numeric) */
  int n_fields;
  char names[FM_MAX_FIELDS][64];
  mxArray *values[FM_MAX_FIELDS];   /* struct fields */
  char *text;                       /* char arrays and exception messages */
};

static mxArray *g_arrays[FM_MAX_ARRAYS];
static int g_n_arrays = 0;
static jmp_buf g_env;
static int g_in_run = 0;
static char g_msg[1024];
static int g_errors = 0, g_rethrows = 0, g_live_strings = 0;
static int (*g_script)(const char *name) = NULL;

static mxArray *fm_new(mxClassID cls) {
  if (g_n_arrays >= FM_MAX_ARRAYS) return NULL;
  mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
  a->cls = cls;
  g_arrays[g_n_arrays++] = a;
  return a;
}

/* ---- test-side constructors */
mxArray *fm_struct(void) { return fm_new(mxSTRUCT_CLASS); }

int fm_set(mxArray *s, const char *name, mxArray *v) {
  if (!s || s->cls != mxSTRUCT_CLASS || s->n_fields >= FM_MAX_FIELDS) return 1;
  for (int i = 0; i < s->n_fields; i++)
    if (strcmp(s->names[i], name) == 0) {
      s->values[i] = v;
      return 0;
    }
  snprintf(s->names[s->n_fields], sizeof s->names[0], "%s", name);
  s->values[s->n_fields++] = v;
  return 0;
}

int fm_remove(mxArray *s, const char *name) {
  for (int i = 0; i < s->n_fields; i++)
    if (strcmp(s->names[i], name) == 0) {
      for (int k = i + 1; k < s->n_fields; k++) {
        memcpy(s->names[k - 1], s->names[k], sizeof s->names[0]);
        s->values[k - 1] = s->values[k];
      }
      s->n_fields--;
      return 0;
    }
  return 1;
}

mxArray *fm_numeric(int cls, int ndims, const size_t *dims, void *data) {
  mxArray *a = fm_new((mxClassID)cls);
  a->ndims = (size_t)ndims;
  for (int i = 0; i < ndims && i < 4; i++) a->dims[i] = dims[i];
  a->data = data;
  return a;
}

mxArray *fm_string(const char *s) {
  mxArray *a = fm_new(mxCHAR_CLASS);
  a->ndims = 2;
  a->dims[0] = 1;
  a->dims[1] = strlen(s);
  a->text = strdup(s);
  return a;
}

void fm_set_script_handler(int (*h)(const char *name)) { g_script = h; }

/* runs mexFunction(FH2Data); returns 0, or 1 with the error message in msg */
int fm_run(const mxArray *D, char *msg, size_t cap) {
  g_msg[0] = '\0';
  g_in_run = 1;
  int rc = 0;
  if (setjmp(g_env) == 0) {
    const mxArray *prhs[1] = {D};
    mexFunction(0, NULL, 1, prhs);
  } else {
    rc = 1;
  }
  g_in_run = 0;
  if (msg && cap) snprintf(msg, cap, "%s", g_msg);
  return rc;
}

int fm_errors(void) { return g_errors; }
int fm_rethrows(void) { return g_rethrows; }
int fm_live_strings(void) { return g_live_strings; }

void fm_reset(void) {
  for (int i = 0; i < g_n_arrays; i++) {
    free(g_arrays[i]->text);
    free(g_arrays[i]);
  }
  g_n_arrays = 0;
  g_errors = g_rethrows = g_live_strings = 0;
}

/* ---- the MEX/MX API used by the shim */
mxArray *mxGetField(const mxArray *pm, size_t index, const char *fieldname) {
  if (!pm || pm->cls != mxSTRUCT_CLASS || index != 0) return NULL;
  for (int i = 0; i < pm->n_fields; i++)
    if (strcmp(pm->names[i], fieldname) == 0) return pm->values[i];
  return NULL;
}

void *mxGetData(const mxArray *pm) { return pm ? pm->data : NULL; }

size_t mxGetNumberOfElements(const mxArray *pm) {
  if (!pm) return 0;
  if (pm->cls == mxSTRUCT_CLASS) return 1;
  size_t n = 1;
  for (size_t i = 0; i < pm->ndims; i++) n *= pm->dims[i];
  return n;
}

mwSize mxGetNumberOfDimensions(const mxArray *pm) { return pm ? pm->ndims : 0; }
const mwSize *mxGetDimensions(const mxArray *pm) { return pm ? pm->dims : NULL; }
mxClassID mxGetClassID(const mxArray *pm) { return pm ? pm->cls : mxUNKNOWN_CLASS; }
int mxIsComplex(const mxArray *pm) {
  (void)pm;
  return 0;
}

char *mxArrayToString(const mxArray *a) {
  if (!a || a->cls != mxCHAR_CLASS || !a->text) return NULL;
  g_live_strings++;
  return strdup(a->text);
}

void mxFree(void *ptr) {
  if (ptr) g_live_strings--;
  free(ptr);
}

void mexErrMsgTxt(const char *errormsg) {
  g_errors++;
  snprintf(g_msg, sizeof g_msg, "%s", errormsg ? errormsg : "");
  if (g_in_run) longjmp(g_env, 1);
  abort();   /* an error outside fm_run is a harness bug */
}

mxArray *mexCallMATLABWithTrap(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name) {
  (void)nlhs;
  (void)plhs;
  (void)nrhs;
  (void)prhs;
  if (g_script && g_script(name) != 0) {
    mxArray *e = fm_new(mxUNKNOWN_CLASS);   /* an MException */
    char buf[256];
    snprintf(buf, sizeof buf, "error in script %s", name);
    e->text = strdup(buf);
    return e;
  }
  return NULL;
}

int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name) {
  (void)nlhs;
  (void)plhs;
  if (strcmp(name, "rethrow") == 0 && nrhs == 1 && prhs[0] && prhs[0]->text) {
    g_rethrows++;
    mexErrMsgTxt(prhs[0]->text);   /* MATLAB raises the exception: unwinds like an error */
    return 1;
  }
  /* a plain script call: an error in it unwinds through the caller, as in MATLAB */
  if (g_script && g_script(name) != 0) mexErrMsgTxt("error in script (untrapped)");
  return 0;
}
