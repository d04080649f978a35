// C-ABI entry points of the host helpers (grid, quadrature, basis) and status strings.
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "dgadv_guard.h"
#include "../../include/dgadv.h"
#include "dgadv_host.h"

using namespace dgadv;

extern "C" int dgadv_grid_build(int32_t numV, const double *coordV, int32_t numT, const int32_t *V0T,
                                dgadv_grid **out) {
  return guarded(nullptr, [&]() -> int {
  if (!out || !coordV || !V0T || numV <= 0 || numT <= 0) return DGADV_EINVAL;
  *out = nullptr;
  Grid g;
  std::string err;
  if (!build_grid(numV, coordV, numT, V0T, g, err)) return DGADV_EMESH;
  dgadv_grid *r = (dgadv_grid *)std::calloc(1, sizeof(dgadv_grid));
  if (!r) return DGADV_ENOMEM;
  r->numT = g.numT; r->numV = g.numV; r->numE = g.numE;
  const size_t T = g.numT, E = g.numE;
  bool ok = true;
  auto ai = [&](size_t n) { int32_t *p = (int32_t *)std::malloc(n * sizeof(int32_t) + 4); ok = ok && p; return p; };
  auto ad = [&](size_t n) { double *p = (double *)std::malloc(n * sizeof(double) + 8); ok = ok && p; return p; };
  r->V0E = ai(2 * E); r->T0E = ai(2 * E); r->E0T = ai(3 * T); r->E0E = ai(2 * E);
  r->areaE = ad(E); r->nuE = ad(2 * E); r->baryE = ad(2 * E); r->areaT = ad(T); r->baryT = ad(2 * T);
  r->B = ad(4 * T); r->areaE0T = ad(3 * T); r->nuE0T = ad(6 * T); r->coordV0T = ad(6 * T); r->detJ0T = ad(T);
  if (!ok) { dgadv_grid_free(r); return DGADV_ENOMEM; }
  // column-major outputs with the reference's conventions
  for (size_t e = 0; e < E; ++e)
    for (int c = 0; c < 2; ++c) {
      r->V0E[c * E + e] = g.V0E[2 * e + c];
      r->T0E[c * E + e] = g.T0E[2 * e + c] + 1;            // 1-based, 0 = none
      r->E0E[c * E + e] = g.E0E[2 * e + c] + 1;            // 1-based, 0 = none
      r->nuE[c * E + e] = g.nuE[2 * e + c];
      r->baryE[c * E + e] = g.baryE[2 * e + c];
    }
  for (size_t e = 0; e < E; ++e) r->areaE[e] = g.areaE[e];
  for (size_t t = 0; t < T; ++t) {
    r->areaT[t] = g.areaT[t];
    r->detJ0T[t] = g.detJ0T[t];
    for (int c = 0; c < 2; ++c) r->baryT[c * T + t] = g.baryT[2 * t + c];
    // B(t, m, n) at t + T*m + 2T*n
    r->B[t + 0 * T + 0 * T] = g.B[4 * t + 0];   // B(:,1,1)
    r->B[t + 0 * T + 2 * T] = g.B[4 * t + 1];   // B(:,1,2)
    r->B[t + 1 * T + 0 * T] = g.B[4 * t + 2];   // B(:,2,1)
    r->B[t + 1 * T + 2 * T] = g.B[4 * t + 3];   // B(:,2,2)
    for (int n = 0; n < 3; ++n) {
      r->E0T[n * T + t] = g.E0T[3 * t + n];
      r->areaE0T[n * T + t] = g.areaE0T[3 * t + n];
      for (int m = 0; m < 2; ++m) {
        r->nuE0T[t + T * n + 3 * T * m] = g.nuE0T[6 * t + 2 * n + m];
        r->coordV0T[t + T * n + 3 * T * m] = g.coordV0T[6 * t + 2 * n + m];
      }
    }
  }
  *out = r;
  return DGADV_OK;
  });
}

extern "C" void dgadv_grid_free(dgadv_grid *g) {
  if (!g) return;
  std::free(g->V0E); std::free(g->T0E); std::free(g->E0T); std::free(g->E0E);
  std::free(g->areaE); std::free(g->nuE); std::free(g->baryE); std::free(g->areaT); std::free(g->baryT);
  std::free(g->B); std::free(g->areaE0T); std::free(g->nuE0T); std::free(g->coordV0T); std::free(g->detJ0T);
  std::free(g);
}

extern "C" int dgadv_quad_rule_1d(int32_t qOrd, int32_t *R, double *Q, double *W) {
  return guarded(nullptr, [&]() -> int {
  if (!R) return DGADV_EINVAL;
  Rule1D r;
  if (!quad_rule_1d(qOrd, r)) return DGADV_EINVAL;
  *R = (int32_t)r.W.size();
  if (Q && W)
    for (size_t i = 0; i < r.W.size(); ++i) { Q[i] = r.Q[i]; W[i] = r.W[i]; }
  return DGADV_OK;
  });
}

extern "C" int dgadv_quad_rule_2d(int32_t qOrd, int32_t *R, double *Q1, double *Q2, double *W) {
  return guarded(nullptr, [&]() -> int {
  if (!R) return DGADV_EINVAL;
  Rule2D r;
  if (!quad_rule_2d(qOrd, r)) return DGADV_EINVAL;
  *R = (int32_t)r.W.size();
  if (Q1 && Q2 && W)
    for (size_t i = 0; i < r.W.size(); ++i) { Q1[i] = r.Q1[i]; Q2[i] = r.Q2[i]; W[i] = r.W[i]; }
  return DGADV_OK;
  });
}

extern "C" int dgadv_basis_eval(int32_t N, int32_t nPts, const double *X1, const double *X2, double *phiOut,
                                double *gradOut) {
  return guarded(nullptr, [&]() -> int {
  if (N < 1 || N > 15 || nPts < 0 || !X1 || !X2 || !phiOut) return DGADV_EINVAL;
  for (int q = 0; q < nPts; ++q)
    for (int i = 0; i < N; ++i) {
      phiOut[(size_t)i * nPts + q] = phi(i, X1[q], X2[q]);
      if (gradOut) {
        gradOut[(size_t)i * nPts + q] = grad_phi(i, 0, X1[q], X2[q]);
        gradOut[(size_t)N * nPts + (size_t)i * nPts + q] = grad_phi(i, 1, X1[q], X2[q]);
      }
    }
  return DGADV_OK;
  });
}

extern "C" const char *dgadv_status_string(int s) {
  switch (s) {
    case DGADV_OK: return "ok";
    case DGADV_EINVAL: return "invalid argument";
    case DGADV_ECUDA: return "CUDA runtime error";
    case DGADV_ENOMEM: return "out of memory";
    case DGADV_EMESH: return "inconsistent mesh";
    case DGADV_ENONFINITE: return "non-finite value in the state";
    case DGADV_ETIMEOUT: return "bounded device wait timed out";
    case DGADV_EUNSUPPORTED: return "unsupported option";
    case DGADV_EIO: return "output file could not be written";
    case DGADV_ENOCONV: return "iterative solve did not converge";
  }
  return "unknown status";
}
