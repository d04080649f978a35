"""The MEX / oct-file gateway (festung_gb300/matlab/dgadv_mex.c) compiles: neither Matlab nor Octave
is installed, so it is checked against a stub of the MEX API (declarations only) and the real
include/dgadv.h, with warnings as errors.  A mistyped call or a missing C-ABI entry fails here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# declarations of the MEX API calls the gateway makes (names and signatures of the public API)
MEX_STUB = r'''
#pragma once
#include <stdbool.h>
#include <stddef.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef bool mxLogical;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef enum { mxUNKNOWN_CLASS = 0, mxUINT8_CLASS = 9, mxUINT64_CLASS = 15 } mxClassID;
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);
int mexAtExit(void (*fn)(void));
bool mxIsChar(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsComplex(const mxArray *a);
bool mxIsEmpty(const mxArray *a);
bool mxIsLogical(const mxArray *a);
bool mxIsUint64(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetNumberOfElements(const mxArray *a);
mwSize mxGetNumberOfDimensions(const mxArray *a);
const mwSize *mxGetDimensions(const mxArray *a);
void *mxGetData(const mxArray *a);
double *mxGetPr(const mxArray *a);
mxLogical *mxGetLogicals(const mxArray *a);
double mxGetScalar(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, mwSize len);
void *mxMalloc(size_t n);
void mxFree(void *p);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID id, mxComplexity c);
void mxDestroyArray(mxArray *a);
'''


def test_gateway_compiles_against_the_header(tmp_path):
    cc = shutil.which('gcc') or shutil.which('cc')
    if not cc:
        pytest.skip('no C compiler')
    (tmp_path / 'mex.h').write_text(MEX_STUB)
    src = os.path.join(ROOT, 'festung_gb300', 'matlab', 'dgadv_mex.c')
    cmd = [cc, '-std=c11', '-fsyntax-only', '-Wall', '-Werror', '-I', str(tmp_path),
           '-I', os.path.join(ROOT, 'include'), src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr



def test_matlab_problem_folder_is_complete():
    """The advection_gpu folder holds every step function main.m and iterateSubSteps look up
    (core/getStepLists.m) and configures every test case of the Python mirror."""
    from festung_gb300.testcases import TESTCASES
    d = os.path.join(ROOT, 'festung_gb300', 'matlab', 'advection_gpu')
    steps = ('configureProblem', 'preprocessProblem', 'initializeProblem', 'preprocessStep', 'solveStep',
             'postprocessStep', 'outputStep', 'postprocessProblem', 'preprocessSubStep', 'solveSubStep',
             'postprocessSubStep')
    for f in steps:
        src = open(os.path.join(d, f + '.m')).read()
        assert 'function problemData = %s(' % f in src, f
    conf = open(os.path.join(d, 'configureProblem.m')).read()
    for tc in TESTCASES:
        assert "'%s'" % tc in conf, tc
