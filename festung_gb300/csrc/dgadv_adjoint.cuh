// Discrete adjoint of the explicit stage (limiter off): the transpose of
//     c^(s+1) = w_s c^n + (1 - w_s) (c^(s) + tau cDot(c^(s))),
//     cDot = hatM^-1 rhs / detJ,  rhs = (G1 + G2) c - R c + sources
// (advection/solveSubStep.m:62-66,83), stage by stage in reverse.  Given mu = dJ/dc^(s+1):
//     dJ/dc^(s)  = (1 - w_s) mu + A^T ((1 - w_s) tau mu)
//     dJ/dc^n   += w_s mu
// with A^T the transposed volume term (core/assembleMatElemDphiPhiFuncDisc.m:181-202) and the
// transposed upwind flux (core/assembleMatEdgePhiPhiValUpwind.m:261-299).  The transposed flux
// is element-centric like the forward one: an element adds the terms of its own outflow edges
// and gathers, from each neighbour, the terms where that neighbour takes this element's trace
// as its upwind value (its normal velocity < 0 there), so no atomics are needed.
//
// The velocity enters linearly through F (volume factors at the quadrature points) and Vn
// (normal velocities at the edge points), with the upwind choice frozen at the base velocity.
// Each stage adds dJ/dF and dJ/dVn per element into FP64 arrays (aF: 2Q x Kp, aV: 3R x Kp);
// the gradient of a velocity parameter theta_m is then sum aF F_m + aV Vn_m over elements, with
// F_m, Vn_m the factors of velocity mode m.
#pragma once
#include "dgadv_device.cuh"

namespace dgadv {

struct AdjScalars {
  double omega, tau;
  int init;   // accn starts at zero (first reversed stage of a step)
  int last;   // stage 0: its input is c^n itself, so dJ/dc^(0) joins accn
};

template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_adj_stage(const Geo<T> g, const T *muIn, const T *cs, T *__restrict__ muOut, T *__restrict__ accn,
            double *__restrict__ aF, double *__restrict__ aV, const AdjScalars a) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  const Tab<T, P> &tb = tab<T, P>();
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  if (k >= g.K) return;
  const int Kp = g.Kp;
  const T w = T(a.omega), coef = T((1.0 - a.omega) * a.tau);
  // static data before the dependency wait (programmatic dependent launch)
  const int code = g.code[k];
  int nb[3], nk[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    nb[n] = g.nbr[(size_t)n * Kp + k];
    nk[n] = (code >> (2 * n)) & 3;   // the neighbour's local index of the shared edge
  }
  T F[2 * Q], V[3 * R], V2[3][R];
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) F[i] = g.F[(size_t)i * Kp + k];
#pragma unroll
  for (int i = 0; i < 3 * R; ++i) V[i] = g.Vn[(size_t)i * Kp + k];
#pragma unroll
  for (int n = 0; n < 3; ++n)
#pragma unroll
    for (int r = 0; r < R; ++r) V2[n][r] = nb[n] >= 0 ? g.Vn[(size_t)(nk[n] * R + r) * Kp + nb[n]] : T(0);
  pdl_wait();
  // every load of the stage's data up front: the kernel is latency-bound otherwise
  T mu[N], c[N], cn[3][N], mu2[3][N];
  double sF[2 * Q], sV[3 * R];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    mu[i] = muIn[(size_t)i * Kp + k];
    c[i] = cs[(size_t)i * Kp + k];
  }
#pragma unroll
  for (int n = 0; n < 3; ++n)
#pragma unroll
    for (int j = 0; j < N; ++j) {
      cn[n][j] = nb[n] >= 0 ? cs[(size_t)j * Kp + nb[n]] : T(0);
      mu2[n][j] = nb[n] >= 0 ? muIn[(size_t)j * Kp + nb[n]] : T(0);
    }
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) sF[i] = aF[(size_t)i * Kp + k];
#pragma unroll
  for (int i = 0; i < 3 * R; ++i) sV[i] = aV[(size_t)i * Kp + k];
  T mp[N];
#pragma unroll
  for (int i = 0; i < N; ++i) mp[i] = coef * mu[i];   // dJ/dcDot of this stage
  Acc<T> grad[N];
#pragma unroll
  for (int i = 0; i < N; ++i) grad[i] = Acc<T>(T(0));
  // volume term: d/dc of sum_i nu_i sum_q (g1 F1 + g2 F2)_qi c_q, nu = hatM^-1 mp
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    Acc<T> cqa(T(0)), s1a(T(0)), s2a(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) {
      cqa.fma(tb.phiQ[q][j], c[j]);
      s1a.fma(tb.Hg1[q][j], mp[j]);
      s2a.fma(tb.Hg2[q][j], mp[j]);
    }
    const T cq = cqa.get(), s1 = s1a.get(), s2 = s2a.get();
    sF[q] += double(s1 * cq);
    sF[Q + q] += double(s2 * cq);
    const T wq = s1 * F[q] + s2 * F[Q + q];
#pragma unroll
    for (int j = 0; j < N; ++j) grad[j].fma(tb.phiQ[q][j], wq);
  }
  // upwind flux of this element's own edges
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const bool outOk = (code >> (6 + n)) & 1;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T v = V[n * R + r];
      Acc<T> eta(T(0));
#pragma unroll
      for (int j = 0; j < N; ++j) eta.fma(tb.Hphi[n][r][j], mp[j]);
      const T e = eta.get();
      T sens = T(0);
      if (v > T(0) && outOk) {
        Acc<T> tr(T(0));
#pragma unroll
        for (int j = 0; j < N; ++j) tr.fma(tb.phi1D[n][r][j], c[j]);
        sens = -(e * tr.get());
        const T ev = e * v;
#pragma unroll
        for (int j = 0; j < N; ++j) grad[j].fms(tb.phi1D[n][r][j], ev);
      } else if (v < T(0) && nb[n] >= 0) {
        Acc<T> tr(T(0));
#pragma unroll
        for (int j = 0; j < N; ++j) tr.fma(tb.thetaPhi[n][nk[n]][r][j], cn[n][j]);
        sens = -(e * tr.get());
      }
      sV[n * R + r] += double(sens);
    }
  }
  // upwind flux of the neighbours that take this element's trace (their v < 0 on the shared edge)
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    if (nb[n] < 0) continue;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T v2 = V2[n][r];
      if (v2 < T(0)) {
        Acc<T> eta(T(0));
#pragma unroll
        for (int j = 0; j < N; ++j) eta.fma(tb.Hphi[nk[n]][r][j], mu2[n][j]);
        const T ev = coef * eta.get() * v2;
#pragma unroll
        for (int j = 0; j < N; ++j) grad[j].fms(tb.thetaPhi[nk[n]][n][r][j], ev);
      }
    }
  }
  // reverse SSP update and the stores
#pragma unroll
  for (int i = 0; i < N; ++i) {
    const T mo = (T(1) - w) * mu[i] + grad[i].get();
    if (muOut) muOut[(size_t)i * Kp + k] = mo;
    T acc = a.init ? w * mu[i] : accn[(size_t)i * Kp + k] + w * mu[i];
    if (a.last) acc = acc + mo;
    accn[(size_t)i * Kp + k] = acc;
  }
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) aF[(size_t)i * Kp + k] = sF[i];
#pragma unroll
  for (int i = 0; i < 3 * R; ++i) aV[(size_t)i * Kp + k] = sV[i];
}

template <typename T, int P>
static cudaError_t launch_adj_stage(dgadv_handle *h, const AdjStageArgs &s) {
  const Geo<T> g = make_geo<T>(h);
  const int grid = (h->K + kBlock - 1) / kBlock;
  AdjScalars a;
  a.omega = s.omega; a.tau = s.tau; a.init = s.init; a.last = s.last;
  launch_k(h, k_adj_stage<T, P>, grid, (size_t)0, g, (const T *)s.muIn, (const T *)s.cs, (T *)s.muOut,
           (T *)s.accn, h->aF, h->aV, a);
  return cudaGetLastError();
}

template <typename T, int MASK>
static cudaError_t dispatch_adj_stage(dgadv_handle *h, const AdjStageArgs &s) {
  switch (h->p) {
    case 0: if constexpr ((MASK & 1) != 0) return launch_adj_stage<T, 0>(h, s); break;
    case 1: if constexpr ((MASK & 2) != 0) return launch_adj_stage<T, 1>(h, s); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_adj_stage<T, 2>(h, s); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_adj_stage<T, 3>(h, s); break;
  }
  return cudaErrorNotSupported;
}

// The operation table of a unit with the adjoint kernels added.
template <typename T, int MASK>
static PrecOps with_adjoint(PrecOps o) {
  o.adj_stage = dispatch_adj_stage<T, MASK>;
  return o;
}

}  // namespace dgadv
