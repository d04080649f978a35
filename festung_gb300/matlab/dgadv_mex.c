/*
 * dgadv_mex.c -- MEX / oct-file gateway over the C-ABI of libdgadv (include/dgadv.h).
 *
 * Build (Matlab):  mex -I<repo>/include dgadv_mex.c -L<repo>/festung_gb300 -ldgadv
 * Build (Octave):  mkoctfile --mex -I<repo>/include dgadv_mex.c -L<repo>/festung_gb300 -ldgadv
 *
 * Usage from the advection_gpu problem folder:
 *   h = dgadv_mex('create', coordV, V0T, idE0T, markE0TbdrD, markE0TbdrN, [p ordRK prec lim limType dev flags])
 *   dgadv_mex('set_velocity', h, u1Disc, u2Disc, vNormalOnQuadEdge)
 *   dgadv_mex('set_source_terms', h, timeFn, rhsTerms, cDV0T)
 *   dgadv_mex('set_state', h, cDisc)
 *   dgadv_mex('limit_state', h, t)
 *   dgadv_mex('step', h, nSteps, nStep0, tau)
 *   cDisc = dgadv_mex('get_state', h)
 *   dgadv_mex('destroy', h)
 * Launch options and the discrete adjoint (no counterpart in the reference):
 *   dgadv_mex('set_option', h, option, value);  value = dgadv_mex('get_option', h, option)
 *   dgadv_mex('set_velocity_modes', h, u1Modes, u2Modes, vNModes)   % K x N x M, K x N x M, K x 3R x M
 *   dgadv_mex('set_velocity_theta', h, theta)                       % M coefficients
 *   dgadv_mex('forward_record', h, nSteps, tau, nSnapshots)         % 0: every stage stored
 *   [dJdc0, dJdtheta] = dgadv_mex('backward', h, dJdcT)             % dJdcT: K x N
 * Arrays keep Matlab's layout (column-major), integer inputs are converted from 1-based doubles
 * to 0-based int32 here.  Every non-zero status becomes a Matlab error with the library's
 * message.  Handles are uint64 scalars; mexAtExit destroys the ones still open.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mex.h"
#include "dgadv.h"

#define MAX_HANDLES 64
static dgadv_handle *g_open[MAX_HANDLES];
static int32_t g_nmodes[MAX_HANDLES];   /* velocity modes set on each open handle */

static int slot_of(const dgadv_handle *h) {
  for (int i = 0; i < MAX_HANDLES; ++i)
    if (g_open[i] == h) return i;
  return -1;
}

static void cleanup(void) {
  for (int i = 0; i < MAX_HANDLES; ++i)
    if (g_open[i]) { dgadv_destroy(g_open[i]); g_open[i] = NULL; }
}

static void check(int st, dgadv_handle *h) {
  if (st != DGADV_OK)
    mexErrMsgIdAndTxt("dgadv:status", "%s: %s", dgadv_status_string(st), h ? dgadv_last_error(h) : "");
}

static dgadv_handle *get_handle(const mxArray *a) {
  if (!mxIsUint64(a) || mxGetNumberOfElements(a) != 1) mexErrMsgIdAndTxt("dgadv:arg", "bad handle");
  dgadv_handle *h = (dgadv_handle *)(uintptr_t)(*(uint64_t *)mxGetData(a));
  for (int i = 0; i < MAX_HANDLES; ++i)
    if (g_open[i] == h) return h;
  mexErrMsgIdAndTxt("dgadv:arg", "unknown or destroyed handle");
  return NULL;
}

static const double *dbl(const mxArray *a, size_t n, const char *what) {
  if (!mxIsDouble(a) || mxIsComplex(a) || mxGetNumberOfElements(a) != n)
    mexErrMsgIdAndTxt("dgadv:arg", "%s must be a real double array with %zu elements", what, n);
  return mxGetPr(a);
}

/* 1-based double ids -> 0-based int32 (caller frees) */
static int32_t *ids0(const mxArray *a, size_t n, const char *what) {
  const double *d = dbl(a, n, what);
  int32_t *o = (int32_t *)mxMalloc(n * sizeof(int32_t));
  for (size_t i = 0; i < n; ++i) o[i] = (int32_t)d[i] - 1;
  return o;
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
  static int registered = 0;
  if (!registered) { mexAtExit(cleanup); registered = 1; }
  if (nrhs < 1 || !mxIsChar(prhs[0])) mexErrMsgIdAndTxt("dgadv:arg", "first argument: command");
  char cmd[32];
  mxGetString(prhs[0], cmd, sizeof cmd);

  if (!strcmp(cmd, "create")) {
    if (nrhs != 7) mexErrMsgIdAndTxt("dgadv:arg", "create: 6 arguments");
    const size_t numV = mxGetM(prhs[1]), numT = mxGetM(prhs[2]);
    dgadv_mesh m;
    memset(&m, 0, sizeof m);
    m.numT = (int32_t)numT; m.numV = (int32_t)numV;
    m.coordV = dbl(prhs[1], 2 * numV, "coordV");
    int32_t *V0T = ids0(prhs[2], 3 * numT, "V0T");
    m.V0T = V0T;
    int32_t *idE0T = NULL; uint8_t *bD = NULL, *bN = NULL;
    if (!mxIsEmpty(prhs[3])) {
      const double *d = dbl(prhs[3], 3 * numT, "idE0T");
      idE0T = (int32_t *)mxMalloc(3 * numT * sizeof(int32_t));
      for (size_t i = 0; i < 3 * numT; ++i) idE0T[i] = (int32_t)d[i];
      m.idE0T = idE0T;
    }
    if (!mxIsEmpty(prhs[4])) {
      if (mxGetNumberOfElements(prhs[4]) != 3 * numT) mexErrMsgIdAndTxt("dgadv:arg", "markE0TbdrD size");
      bD = (uint8_t *)mxMalloc(3 * numT);
      for (size_t i = 0; i < 3 * numT; ++i) bD[i] = mxIsLogical(prhs[4]) ? mxGetLogicals(prhs[4])[i] : (mxGetPr(prhs[4])[i] != 0);
      m.markE0TbdrD = bD;
    }
    if (!mxIsEmpty(prhs[5])) {
      if (mxGetNumberOfElements(prhs[5]) != 3 * numT) mexErrMsgIdAndTxt("dgadv:arg", "markE0TbdrN size");
      bN = (uint8_t *)mxMalloc(3 * numT);
      for (size_t i = 0; i < 3 * numT; ++i) bN[i] = mxIsLogical(prhs[5]) ? mxGetLogicals(prhs[5])[i] : (mxGetPr(prhs[5])[i] != 0);
      m.markE0TbdrN = bN;
    }
    const double *o = dbl(prhs[6], 7, "options");
    dgadv_params prm = {(int32_t)o[0], (int32_t)o[1], (int32_t)o[2], (int32_t)o[3], (int32_t)o[4],
                        (int32_t)o[5], (int32_t)o[6]};
    dgadv_handle *h = NULL;
    const int st = dgadv_create(&m, &prm, &h);
    mxFree(V0T); if (idE0T) mxFree(idE0T); if (bD) mxFree(bD); if (bN) mxFree(bN);
    if (st != DGADV_OK) {
      char msg[512];
      snprintf(msg, sizeof msg, "%s: %s", dgadv_status_string(st), h ? dgadv_last_error(h) : "");
      dgadv_destroy(h);
      mexErrMsgIdAndTxt("dgadv:status", "%s", msg);
    }
    int slot = -1;
    for (int i = 0; i < MAX_HANDLES; ++i) if (!g_open[i]) { slot = i; break; }
    if (slot < 0) { dgadv_destroy(h); mexErrMsgIdAndTxt("dgadv:arg", "too many open handles"); }
    g_open[slot] = h;
    g_nmodes[slot] = 0;
    plhs[0] = mxCreateNumericMatrix(1, 1, mxUINT64_CLASS, mxREAL);
    *(uint64_t *)mxGetData(plhs[0]) = (uint64_t)(uintptr_t)h;
    return;
  }
  if (nrhs < 2) mexErrMsgIdAndTxt("dgadv:arg", "%s: missing handle", cmd);
  dgadv_handle *h = get_handle(prhs[1]);
  if (!strcmp(cmd, "set_velocity")) {
    check(dgadv_set_velocity(h, mxGetPr(prhs[2]), mxGetPr(prhs[3]), mxGetPr(prhs[4])), h);
  } else if (!strcmp(cmd, "set_source_terms")) {
    const size_t n = mxGetNumberOfElements(prhs[2]);
    int32_t fn[4] = {0, 0, 0, 0};
    for (size_t i = 0; i < n && i < 4; ++i) fn[i] = (int32_t)mxGetPr(prhs[2])[i];
    check(dgadv_set_source_terms(h, (int32_t)n, fn, n ? mxGetPr(prhs[3]) : NULL,
                                 (nrhs > 4 && !mxIsEmpty(prhs[4])) ? mxGetPr(prhs[4]) : NULL), h);
  } else if (!strcmp(cmd, "set_state")) {
    check(dgadv_set_state(h, mxGetPr(prhs[2])), h);
  } else if (!strcmp(cmd, "limit_state")) {
    check(dgadv_limit_state(h, mxGetScalar(prhs[2])), h);
  } else if (!strcmp(cmd, "step")) {
    check(dgadv_step(h, (int32_t)mxGetScalar(prhs[2]), (int32_t)mxGetScalar(prhs[3]), mxGetScalar(prhs[4])), h);
  } else if (!strcmp(cmd, "get_state")) {
    const mwSize K = (mwSize)mxGetScalar(prhs[2]), N = (mwSize)mxGetScalar(prhs[3]);
    plhs[0] = mxCreateDoubleMatrix(K, N, mxREAL);
    check(dgadv_get_state(h, mxGetPr(plhs[0])), h);
  } else if (!strcmp(cmd, "step_implicit") || !strcmp(cmd, "solve_stationary")) {
    /* [iters, relres] = dgadv_mex('step_implicit', h, nSteps, nStep0, tau, ordRK, [tol maxIter restart])
     * [iters, relres] = dgadv_mex('solve_stationary', h, [tol maxIter restart])
     * (handles created with flags DGADV_FLAG_IMPLICIT in the options' last entry) */
    const int stat = !strcmp(cmd, "solve_stationary");
    const int ko = stat ? 2 : 6;
    dgadv_krylov kr = {1e-12, 2000, 50};
    if (nrhs > ko && !mxIsEmpty(prhs[ko])) {
      const double *k = dbl(prhs[ko], 3, "krylov options");
      kr.tol = k[0]; kr.maxIter = (int32_t)k[1]; kr.restart = (int32_t)k[2];
    }
    int32_t it = 0;
    double rr = 0.0;
    if (stat)
      check(dgadv_solve_stationary(h, &kr, &it, &rr), h);
    else
      check(dgadv_step_implicit(h, (int32_t)mxGetScalar(prhs[2]), (int32_t)mxGetScalar(prhs[3]), mxGetScalar(prhs[4]),
                                (int32_t)mxGetScalar(prhs[5]), &kr, &it, &rr), h);
    plhs[0] = mxCreateDoubleScalar((double)it);
    if (nlhs > 1) plhs[1] = mxCreateDoubleScalar(rr);
  } else if (!strcmp(cmd, "transport_init")) {
    /* dgadv_mex('transport_init', h, hDisc, cH0, maskTol, isMask): cH0 is K x N x nSpecies */
    const mwSize nd = mxGetNumberOfDimensions(prhs[3]);
    const int32_t ns = nd > 2 ? (int32_t)mxGetDimensions(prhs[3])[2] : 1;
    check(dgadv_transport_init(h, ns, mxGetPr(prhs[2]), mxGetPr(prhs[3]), mxGetScalar(prhs[4]),
                               (int32_t)mxGetScalar(prhs[5])), h);
  } else if (!strcmp(cmd, "transport_step")) {
    check(dgadv_transport_step(h, (int32_t)mxGetScalar(prhs[2]), (int32_t)mxGetScalar(prhs[3]),
                               mxGetScalar(prhs[4])), h);
  } else if (!strcmp(cmd, "transport_get")) {
    /* [cH, c, mask] = dgadv_mex('transport_get', h, species (1-based), K, N) */
    const mwSize K = (mwSize)mxGetScalar(prhs[3]), N = (mwSize)mxGetScalar(prhs[4]);
    plhs[0] = mxCreateDoubleMatrix(K, N, mxREAL);
    mxArray *c = mxCreateDoubleMatrix(K, N, mxREAL);
    mxArray *m = mxCreateNumericMatrix(K, 1, mxUINT8_CLASS, mxREAL);
    check(dgadv_transport_get(h, (int32_t)mxGetScalar(prhs[2]) - 1, mxGetPr(plhs[0]), mxGetPr(c),
                              (uint8_t *)mxGetData(m)), h);
    if (nlhs > 1) plhs[1] = c; else mxDestroyArray(c);
    if (nlhs > 2) plhs[2] = m; else mxDestroyArray(m);
  } else if (!strcmp(cmd, "output")) {
    /* dgadv_mex('output', h, varName, fileName, tLvl, fileTypes): fileTypes 1 vtk, 2 tec, 3 both */
    char var[256], file[4096];
    if (nrhs < 6 || mxGetString(prhs[2], var, sizeof var) || mxGetString(prhs[3], file, sizeof file))
      mexErrMsgIdAndTxt("dgadv:arg", "output: varName, fileName, tLvl, fileTypes expected");
    check(dgadv_output(h, var, file, (int32_t)mxGetScalar(prhs[4]), (int32_t)mxGetScalar(prhs[5])), h);
  } else if (!strcmp(cmd, "output_wait")) {
    check(dgadv_output_wait(h), h);
  } else if (!strcmp(cmd, "set_option")) {
    check(dgadv_set_option(h, (int32_t)mxGetScalar(prhs[2]), (int32_t)mxGetScalar(prhs[3])), h);
  } else if (!strcmp(cmd, "get_option")) {
    int32_t v = 0;
    check(dgadv_get_option(h, (int32_t)mxGetScalar(prhs[2]), &v), h);
    plhs[0] = mxCreateDoubleScalar((double)v);
  } else if (!strcmp(cmd, "set_velocity_modes")) {
    /* the modes run along the third dimension of each array */
    const mwSize nd = mxGetNumberOfDimensions(prhs[2]);
    const int32_t nm = nd > 2 ? (int32_t)mxGetDimensions(prhs[2])[2] : 1;
    check(dgadv_set_velocity_modes(h, nm, mxGetPr(prhs[2]), mxGetPr(prhs[3]), mxGetPr(prhs[4])), h);
    g_nmodes[slot_of(h)] = nm;
  } else if (!strcmp(cmd, "set_velocity_theta")) {
    check(dgadv_set_velocity_theta(h, mxGetPr(prhs[2])), h);
  } else if (!strcmp(cmd, "forward_record")) {
    check(dgadv_forward_record(h, (int32_t)mxGetScalar(prhs[2]), mxGetScalar(prhs[3]),
                               (int32_t)mxGetScalar(prhs[4])), h);
  } else if (!strcmp(cmd, "backward")) {
    /* dJdc0 has dJdcT's shape; dJdtheta one entry per velocity mode (empty without modes) */
    const mwSize K = (mwSize)mxGetM(prhs[2]), N = (mwSize)(mxGetNumberOfElements(prhs[2]) / (K ? K : 1));
    const int32_t nm = g_nmodes[slot_of(h)];
    plhs[0] = mxCreateDoubleMatrix(K, N, mxREAL);
    mxArray *g = mxCreateDoubleMatrix((mwSize)nm, nm ? 1 : 0, mxREAL);
    check(dgadv_backward(h, dbl(prhs[2], (size_t)K * N, "dJdcT"), mxGetPr(plhs[0]), nm ? mxGetPr(g) : NULL), h);
    if (nlhs > 1) plhs[1] = g; else mxDestroyArray(g);
  } else if (!strcmp(cmd, "destroy")) {
    for (int i = 0; i < MAX_HANDLES; ++i) if (g_open[i] == h) { g_open[i] = NULL; g_nmodes[i] = 0; }
    dgadv_destroy(h);
  } else {
    mexErrMsgIdAndTxt("dgadv:arg", "unknown command %s", cmd);
  }
}
