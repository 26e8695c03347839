/*
 * mex.h - test stand-in for MATLAB's MEX/MX API header.
 *
 * Declares only the documented MEX/MX calls that the shim qd_mex.c uses, with
 * their C signatures.  fake_mex.c implements them over a minimal in-memory
 * mxArray so that the shim's mexFunction can run without MATLAB.
 */
#ifndef QD_TEST_FAKE_MEX_H
#define QD_TEST_FAKE_MEX_H
#include <stddef.h>

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxCELL_CLASS,
  mxSTRUCT_CLASS,
  mxLOGICAL_CLASS,
  mxCHAR_CLASS,
  mxVOID_CLASS,
  mxDOUBLE_CLASS,
  mxSINGLE_CLASS,
  mxINT8_CLASS,
  mxUINT8_CLASS,
  mxINT16_CLASS,
  mxUINT16_CLASS,
  mxINT32_CLASS,
  mxUINT32_CLASS,
  mxINT64_CLASS,
  mxUINT64_CLASS
} mxClassID;

mxArray *mxGetField(const mxArray *pm, size_t index, const char *fieldname);
void *mxGetData(const mxArray *pm);
size_t mxGetNumberOfElements(const mxArray *pm);
mwSize mxGetNumberOfDimensions(const mxArray *pm);
const mwSize *mxGetDimensions(const mxArray *pm);
mxClassID mxGetClassID(const mxArray *pm);
int mxIsComplex(const mxArray *pm);
char *mxArrayToString(const mxArray *array_ptr);
void mxFree(void *ptr);
void mexErrMsgTxt(const char *errormsg);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *functionName);
mxArray *mexCallMATLABWithTrap(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *functionName);
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#endif
