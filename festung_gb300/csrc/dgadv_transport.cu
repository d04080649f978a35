// The transport problem on the device (transport/*.m, configuration 'rotation' without coupling
// to a shallow-water model): several species on one mesh, each advected as its depth-integrated
// concentration c h with the depth-integrated velocity, only over its active elements, with the
// linear vertex limiter applied to its concentration c.
//
// Per Runge-Kutta stage and species (transport/solveSubStep.m):
//   c h   <- SSP update with the masked advective term of c            (k_tr_stage)
//   c     <- Pi(c h / h)                                               (k_tr_convert)
//   c     <- linear vertex limiter, zero Dirichlet data                (the handle's limiter)
//   c h   <- Pi(c h)                                                   (k_tr_convert)
// and after the step's last stage the species' mask follows from that limiter call's patch
// extremes (transport/postprocessStep.m, core/computeMask.m).  The handle supplies the mesh,
// the depth-integrated velocity (dgadv_set_velocity) and the limiter; its own state serves as the
// limiter's work buffer.
#include <cstring>
#include <string>
#include <vector>

#include "dgadv_handle.h"

namespace dgadv {

struct TransportState {
  int nSpecies = 0;
  double maskTol = 1e-6;
  bool isMask = true;
  std::vector<void *> cH, cH0, conc;
  std::vector<uint8_t *> mask;
  void *hQ = nullptr;   // depth at the volume points, Q x Kp
};

void transport_release(dgadv_handle *h) {
  delete h->trans;   // device buffers belong to h->allocs
  h->trans = nullptr;
}

}  // namespace dgadv

using namespace dgadv;

namespace {

double rk_table_transport(int ord, double omega[3], double cst[3]) {
  omega[0] = omega[1] = omega[2] = 0.0;
  cst[0] = 0.0; cst[1] = 1.0; cst[2] = 0.5;   // core/rungeKuttaExplicit.m:64-78
  if (ord == 2) { omega[1] = 0.5; return 2; }
  if (ord == 3) { omega[1] = 0.75; omega[2] = 1.0 / 3.0; return 3; }
  return 1;
}

int check(dgadv_handle *h) {
  if (!h->trans) { h->err = "dgadv_transport_init was not called"; return DGADV_EINVAL; }
  return DGADV_OK;
}

// Limits the species' concentration in place through the handle's state; on `maskOut` the
// mask from this call's patch extremes.
int limit_species(dgadv_handle *h, int s, double t, bool updateMask) {
  TransportState *st = h->trans;
  const PrecOps &o = ops_of(h);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  DG_CUDA(o.copy(h, h->cn, st->conc[s], bytes));
  DG_CUDA(o.limit(h, t));
  DG_CUDA(o.copy(h, st->conc[s], h->cn, bytes));
  if (updateMask && st->isMask) DG_CUDA(o.tr_mask(h, h->limPass - 1, st->maskTol, st->mask[s]));
  return DGADV_OK;
}

}  // namespace

extern "C" int dgadv_transport_init(dgadv_handle *h, int32_t nSpecies, const double *hDisc, const double *cH0,
                                    double maskTol, int32_t isMask) {
  return guarded(h, [&]() -> int {
  if (!h || nSpecies < 1 || nSpecies > 64 || !hDisc || !cH0 || !(maskTol >= 0.0)) return DGADV_EINVAL;
  const PrecOps &o = ops_of(h);
  if (!o.tr_stage) { h->err = "the transport kernels are built for FP32 and FP64"; return DGADV_EUNSUPPORTED; }
  if (!h->lim || h->limType != DGADV_LIM_LINEAR || h->p < 1 || (h->flags & DGADV_FLAG_IMPLICIT)) {
    h->err = "transport needs an explicit handle with the linear limiter and p >= 1";
    return DGADV_EINVAL;
  }
  if (!h->hasVelocity) { h->err = "dgadv_set_velocity was not called"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  transport_release(h);
  TransportState *st = new (std::nothrow) TransportState();
  if (!st) return DGADV_ENOMEM;
  h->trans = st;
  st->nSpecies = nSpecies;
  st->maskTol = maskTol;
  st->isMask = isMask != 0;
  const size_t K = h->K, Kp = h->Kp, N = h->N, Q = h->Q;
  const size_t bytes = N * Kp * o.realBytes;
  int e;
  // depth at the volume points (internal element order)
  std::vector<double> hq(Q * Kp, 1.0);
  for (size_t k = 0; k < K; ++k) {
    const int ext = h->permv[k];
    for (size_t q = 0; q < Q; ++q) {
      double v = 0.0;
      for (size_t j = 0; j < N; ++j) v += h->tables.phiQ[q * N + j] * hDisc[j * K + ext];
      hq[q * Kp + k] = v;
    }
  }
  if ((e = dev_alloc(h, &st->hQ, Q * Kp * o.realBytes))) return e;
  if ((e = upload_real(h, st->hQ, hq))) return e;
  st->cH.resize(nSpecies); st->cH0.resize(nSpecies); st->conc.resize(nSpecies); st->mask.resize(nSpecies);
  for (int s = 0; s < nSpecies; ++s) {
    if ((e = dev_alloc(h, &st->cH[s], bytes))) return e;
    if ((e = dev_alloc(h, &st->cH0[s], bytes))) return e;
    if ((e = dev_alloc(h, &st->conc[s], bytes))) return e;
    if ((e = dev_alloc(h, (void **)&st->mask[s], Kp))) return e;
    DG_CUDA(cudaMemsetAsync(st->cH[s], 0, bytes, h->stream));
    DG_CUDA(cudaMemsetAsync(st->conc[s], 0, bytes, h->stream));
    DG_CUDA(cudaMemsetAsync(st->mask[s], 1, Kp, h->stream));
    // transport/initializeProblem.m: c = Pi(c h / h), limited at t = 0, c h = Pi(c h), mask
    DG_CUDA(cudaMemcpyAsync(h->stage_ext, cH0 + (size_t)s * K * N, K * N * sizeof(double), cudaMemcpyHostToDevice,
                            h->stream));
    DG_CUDA(o.scatter_in(h, st->cH[s]));
    DG_CUDA(o.tr_convert(h, st->cH[s], st->conc[s], st->hQ, 1));
    if ((e = limit_species(h, s, 0.0, true))) return e;
    DG_CUDA(o.tr_convert(h, st->conc[s], st->cH[s], st->hQ, 0));
  }
  DG_CUDA(cudaStreamSynchronize(h->stream));
  return dgadv_sync(h);
  });
}

extern "C" int dgadv_transport_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau) {
  return guarded(h, [&]() -> int {
  if (!h || nSteps < 0 || !(tau > 0.0)) return DGADV_EINVAL;
  if (int e = check(h)) return e;
  DG_CUDA(cudaSetDevice(h->device));
  TransportState *st = h->trans;
  const PrecOps &o = ops_of(h);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  double omega[3], cst[3];
  const int S = (int)rk_table_transport(h->ordRK, omega, cst);
  for (int n = 0; n < nSteps; ++n) {
    const double t0 = (double)(nStep0 + n) * tau;
    for (int s = 0; s < st->nSpecies; ++s) DG_CUDA(o.copy(h, st->cH0[s], st->cH[s], bytes));
    for (int i = 0; i < S; ++i) {
      // boundary time of the limiter (transport/solveSubStep.m): the next stage's time
      const double tBC = (i + 1 < S) ? t0 + cst[i + 1] * tau : t0 + tau;
      for (int s = 0; s < st->nSpecies; ++s) {
        TrStageArgs a;
        a.conc = st->conc[s]; a.cHin = st->cH[s]; a.cH0 = st->cH0[s]; a.cHout = st->cH[s];
        a.mask = st->mask[s]; a.omega = omega[i]; a.tau = tau;
        DG_CUDA(o.tr_stage(h, a));
        DG_CUDA(o.tr_convert(h, st->cH[s], st->conc[s], st->hQ, 1));
        if (int e = limit_species(h, s, tBC, i == S - 1)) return e;
        DG_CUDA(o.tr_convert(h, st->conc[s], st->cH[s], st->hQ, 0));
      }
    }
  }
  return dgadv_sync(h);
  });
}

extern "C" int dgadv_transport_get(dgadv_handle *h, int32_t species, double *cH, double *conc, uint8_t *mask) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  if (int e = check(h)) return e;
  TransportState *st = h->trans;
  if (species < 0 || species >= st->nSpecies) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const PrecOps &o = ops_of(h);
  const size_t KN = (size_t)h->K * h->N;
  if (cH) {
    DG_CUDA(o.gather_out(h, st->cH[species]));
    DG_CUDA(cudaMemcpyAsync(cH, h->stage_ext, KN * 8, cudaMemcpyDeviceToHost, h->stream));
    DG_CUDA(cudaStreamSynchronize(h->stream));
  }
  if (conc) {
    DG_CUDA(o.gather_out(h, st->conc[species]));
    DG_CUDA(cudaMemcpyAsync(conc, h->stage_ext, KN * 8, cudaMemcpyDeviceToHost, h->stream));
    DG_CUDA(cudaStreamSynchronize(h->stream));
  }
  if (mask) {
    std::vector<uint8_t> m(h->K);
    DG_CUDA(cudaMemcpyAsync(m.data(), st->mask[species], h->K, cudaMemcpyDeviceToHost, h->stream));
    DG_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < h->K; ++k) mask[h->permv[k]] = m[k];
  }
  return dgadv_sync(h);
  });
}
