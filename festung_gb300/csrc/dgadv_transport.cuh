// Kernels of the transport problem (transport/solveSubStep.m, configuration 'rotation' without
// coupling): species advected as depth-integrated concentrations c h, each only over its active
// elements (its mask).
//
// k_tr_stage: the SSP update of c h from the masked advective term of the concentration c with
//   the depth-integrated velocity (the handle's velocity factors).  An inactive element keeps
//   its value.  An active element's outflow counts across an edge to an active element or a
//   boundary edge, its inflow only from an active neighbour (the masked branches of
//   core/assembleMatElemDphiPhiFuncDiscVec.m:115-141 and core/assembleMatEdgePhiPhiValUpwind.m).
//   The reference's transport keeps hatM = I (transport/preprocessProblem.m), so the mass solve
//   is the division by detJ already folded into the factors.
// k_tr_convert: c = Pi(c h / h) or c h = Pi(c h), point values at the volume rule, projected back
//   with hatM = I (core/projectDataQ0T2DataDisc.m).
// k_tr_mask: core/computeMask.m, 'vertex-based': an element is active if at one of its vertices
//   the patch maximum minus the patch minimum of the element means (with the reference's global
//   shift and the zero Dirichlet data of the limiter call) reaches the tolerance.
#pragma once
#include "dgadv_launch.cuh"

namespace dgadv {

struct VolWeights {
  double w[12];
};

template <typename T, int P>
__global__ void __launch_bounds__(kBlock) k_tr_stage(const Geo<T> g, const T *conc, const T *cHin, const T *cH0,
                                                     T *cHout, const uint8_t *__restrict__ mask, double omega,
                                                     double tau) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.K) return;
  const Tab<T, P> &tb = tab<T, P>();
  const size_t Kp = g.Kp;
  T cdot[N];
#pragma unroll
  for (int i = 0; i < N; ++i) cdot[i] = T(0);
  if (mask[k]) {
    T c[N];
#pragma unroll
    for (int i = 0; i < N; ++i) c[i] = conc[i * Kp + k];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      T cq = T(0);
#pragma unroll
      for (int j = 0; j < N; ++j) cq = fma(tb.phiQ[q][j], c[j], cq);
      const T f1 = g.F[q * Kp + k] * cq, f2 = g.F[(Q + q) * Kp + k] * cq;
#pragma unroll
      for (int i = 0; i < N; ++i) cdot[i] = fma(tb.g2[q][i], f2, fma(tb.g1[q][i], f1, cdot[i]));
    }
    const int code = g.code[k];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int nb = g.nbr[n * Kp + k];
      const int np = (code >> (2 * n)) & 3;
      const bool outOk = (code >> (6 + n)) & 1;
      const bool act = nb >= 0 && mask[nb];
      const bool outCounts = nb >= 0 ? act : outOk;
      T cn[N];
#pragma unroll
      for (int j = 0; j < N; ++j) cn[j] = act ? conc[j * Kp + nb] : T(0);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T v = g.Vn[(n * R + r) * Kp + k];
        T tr = T(0);
        if (v > T(0) && outCounts) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr = fma(tb.phi1D[n][r][j], c[j], tr);
        } else if (v < T(0) && act) {
          for (int j = 0; j < N; ++j) tr = fma(tb.thetaPhi[n][np & 3][r][j], cn[j], tr);
        }
        const T fl = v * tr;
#pragma unroll
        for (int i = 0; i < N; ++i) cdot[i] = fma(-tb.phi1D[n][r][i], fl, cdot[i]);
      }
    }
  }
  const T w = T(omega), tt = T(tau);
#pragma unroll
  for (int i = 0; i < N; ++i) cHout[i * Kp + k] = w * cH0[i * Kp + k] + (T(1) - w) * (cHin[i * Kp + k] + tt * cdot[i]);
}

// out = Pi(in / h) (toConc) or Pi(in h): hQ holds h at the volume points (Q x Kp).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock) k_tr_convert(int K, int Kp, const T *__restrict__ in,
                                                       T *__restrict__ out, const T *__restrict__ hQ, int toConc,
                                                       const VolWeights wq) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const Tab<T, P> &tb = tab<T, P>();
  T a[N], s[N];
#pragma unroll
  for (int i = 0; i < N; ++i) { a[i] = in[(size_t)i * Kp + k]; s[i] = T(0); }
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    T v = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) v = fma(tb.phiQ[q][j], a[j], v);
    const T hq = hQ[(size_t)q * Kp + k];
    v = toConc ? v / hq : v * hq;
    const T wv = T(wq.w[q]) * v;
#pragma unroll
    for (int i = 0; i < N; ++i) s[i] = fma(wv, tb.phiQ[q][i], s[i]);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) out[(size_t)i * Kp + k] = s[i];
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_tr_mask(const Geo<T> g, const LimIn<T> li, double tol,
                                                    uint8_t *__restrict__ mask) {
  __shared__ T sh[2];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  const bool active = k < g.K;
  const size_t Kp = g.Kp;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, 1), 1, sh);
  __syncthreads();
  if (!active) return;
  VKeys<T, 1> kv;
  load_vkeys<T, 1>(g, li, vid, kv);
  const int dmask = (g.code[k] >> 9) & 7;
  T valD[3], mn[3], mx[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) valD[n] = ((dmask >> n) & 1) ? T(0) : T(NAN);
  patch_minmax<T, 1>(li, kv, sh, 0, valD, mn, mx);
  const T d = fmax(fmax(mx[0] - mn[0], mx[1] - mn[1]), mx[2] - mn[2]);
  mask[k] = d >= T(tol) ? 1 : 0;
}

template <typename T, int P>
static cudaError_t tr_stage(dgadv_handle *h, const TrStageArgs &a) {
  const Geo<T> g = make_geo<T>(h);
  k_tr_stage<T, P><<<(h->K + 31) / 32, 32, 0, h->stream>>>(
      g, (const T *)a.conc, (const T *)a.cHin, (const T *)a.cH0, (T *)a.cHout, a.mask, a.omega, a.tau);
  return cudaGetLastError();
}
template <typename T, int P>
static cudaError_t tr_convert(dgadv_handle *h, const void *in, void *out, const void *hQ, int toConc) {
  VolWeights wq{};
  for (int q = 0; q < Dims<P>::Q && q < 12; ++q) wq.w[q] = h->tables.vol.W[q];
  k_tr_convert<T, P><<<(h->K + 31) / 32, 32, 0, h->stream>>>(h->K, h->Kp, (const T *)in, (T *)out,
                                                                             (const T *)hQ, toConc, wq);
  return cudaGetLastError();
}
template <typename T>
static cudaError_t tr_mask(dgadv_handle *h, long long pass, double tol, uint8_t *mask) {
  const Geo<T> g = make_geo<T>(h);
  k_tr_mask<T><<<(h->K + kBlock - 1) / kBlock, kBlock, 0, h->stream>>>(g, lim_in_pass<T>(h, pass), tol, mask);
  return cudaGetLastError();
}

template <typename T, int MASK>
static cudaError_t dispatch_tr_stage(dgadv_handle *h, const TrStageArgs &a) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return tr_stage<T, 1>(h, a); break;
    case 2: if constexpr ((MASK & 4) != 0) return tr_stage<T, 2>(h, a); break;
    case 3: if constexpr ((MASK & 8) != 0) return tr_stage<T, 3>(h, a); break;
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK>
static cudaError_t dispatch_tr_convert(dgadv_handle *h, const void *in, void *out, const void *hQ, int toConc) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return tr_convert<T, 1>(h, in, out, hQ, toConc); break;
    case 2: if constexpr ((MASK & 4) != 0) return tr_convert<T, 2>(h, in, out, hQ, toConc); break;
    case 3: if constexpr ((MASK & 8) != 0) return tr_convert<T, 3>(h, in, out, hQ, toConc); break;
  }
  return cudaErrorNotSupported;
}

// The operation table of a unit with the transport kernels added.
template <typename T, int MASK>
static PrecOps with_transport(PrecOps o) {
  o.tr_stage = dispatch_tr_stage<T, MASK>;
  o.tr_convert = dispatch_tr_convert<T, MASK>;
  o.tr_mask = tr_mask<T>;
  return o;
}

}  // namespace dgadv
