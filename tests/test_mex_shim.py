"""The MATLAB MEX shim compiles against the public MEX interface (a stub header declaring only
the calls it uses: no MATLAB is installed) and the C ABI header."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

# declarations of the documented MEX/MX API entry points the shim calls, with their C signatures
MEX_STUB = """
#pragma once
#include <stddef.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
mxArray *mxGetField(const mxArray *pm, size_t index, const char *fieldname);
void *mxGetData(const mxArray *pm);
size_t mxGetNumberOfElements(const mxArray *pm);
const mwSize *mxGetDimensions(const mxArray *pm);
char *mxArrayToString(const mxArray *array_ptr);
void mxFree(void *ptr);
void mexErrMsgTxt(const char *errormsg);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *functionName);
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
"""


def test_mex_shim_compiles(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    (tmp_path / "mex.h").write_text(MEX_STUB)
    r = subprocess.run([cc, "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-Wall", "-Werror", "-fsyntax-only",
                        "-I", str(tmp_path), "-I", str(ROOT / "include"),
                        str(ROOT / "qd-openmp-cuda_gb300" / "csrc" / "qd_mex.c")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
