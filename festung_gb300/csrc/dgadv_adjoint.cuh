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
// Each stage adds dJ/dF and dJ/dVn per element into 8-byte entries (aF: 2Q x Kp, aV: 3R x Kp;
// FP64, or float pairs on the FP32 path, see SensAcc); the gradient of a velocity parameter
// theta_m is then sum aF F_m + aV Vn_m over elements, with F_m, Vn_m the factors of velocity
// mode m.
#pragma once
#include "dgadv_device.cuh"

namespace dgadv {

struct AdjScalars {
  double omega, tau;
  int init;   // accn starts at zero (first reversed stage of a step)
  int last;   // stage 0: its input is c^n itself, so dJ/dc^(0) joins accn
};

// One entry of the per-element velocity sensitivities aF / aV (8 bytes each).  The FP64 path adds
// in FP64.  The FP32 path keeps the entry as an unevaluated pair hi + lo of floats in the same 8
// bytes and adds with two_sum + fast_two_sum (Knuth; Dekker 1971), about 48 bits: GB300 issues
// FP64 arithmetic at 1/64 of the FP32 rate, and the 2Q + 3R FP64 conversions and adds per element
// were the busiest pipe of the FP32 stage.  k_theta_partial reads the pair as (double)hi + lo.
template <typename T>
struct SensAcc {
  double v;
  __device__ __forceinline__ void load(const double *p) { v = *p; }
  __device__ __forceinline__ void add(T x) { v += double(x); }
  __device__ __forceinline__ void store(double *p) const { *p = v; }
};
template <>
struct SensAcc<float> {
  float hi, lo;
  __device__ __forceinline__ void load(const double *p) {
    const float2 q = *reinterpret_cast<const float2 *>(p);
    hi = q.x;
    lo = q.y;
  }
  __device__ __forceinline__ void add(float x) {
    float s, e;
    df::two_sum(hi, x, s, e);
    df::fast_two_sum(s, e + lo, hi, lo);
  }
  __device__ __forceinline__ void store(double *p) const { *reinterpret_cast<float2 *>(p) = make_float2(hi, lo); }
};

template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_adj_stage(const Geo<T> g, const T *muIn, const T *mpIn, const T *cs, T *__restrict__ muOut,
            T *__restrict__ accn, double *__restrict__ aF, double *__restrict__ aV, const AdjScalars a) {
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
  SensAcc<T> sF[2 * Q], sV[3 * R];
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
      mu2[n][j] = nb[n] >= 0 ? (mpIn ? mpIn[(size_t)j * Kp + nb[n]] : coef * muIn[(size_t)j * Kp + nb[n]]) : T(0);
    }
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) sF[i].load(aF + (size_t)i * Kp + k);
#pragma unroll
  for (int i = 0; i < 3 * R; ++i) sV[i].load(aV + (size_t)i * Kp + k);
  T mp[N];
#pragma unroll
  for (int i = 0; i < N; ++i) mp[i] = mpIn ? mpIn[(size_t)i * Kp + k] : coef * mu[i];   // dJ/dcDot
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
    sF[q].add(s1 * cq);
    sF[Q + q].add(s2 * cq);
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
      sV[n * R + r].add(sens);
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
        const T ev = eta.get() * v2;
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
  for (int i = 0; i < 2 * Q; ++i) sF[i].store(aF + (size_t)i * Kp + k);
#pragma unroll
  for (int i = 0; i < 3 * R; ++i) sV[i].store(aV + (size_t)i * Kp + k);
}

// The same stage with the work of an element split over four warps by role: warp n < 3 takes
// edge n (the outflow terms of the element's own edge n and the terms of the neighbour across it)
// and warp 3 the volume points; the partial gradients meet in shared memory.  Each warp reads its
// tables at one entry at a time (the role is fixed per warp, the edge index a template argument),
// so the table operands stay constant-bank broadcasts.  With one thread per element a
// 32768-triangle mesh gives under two warps per scheduler and the stage waits on its own
// instruction chain; the split gives four times the warps and a quarter of the chain.  A CTA
// covers 32 W elements with W warps per role (DGADV_OPT_ADJ_WARPS).  Sums in a fixed order:
// results are deterministic and do not depend on W.
template <typename T, int P>
struct AdjSplitIn {
  const T *muIn, *mpIn, *cs;
  double *aF, *aV;
  T coef;
  int k, e, Kp;
};

template <typename T, int P, int n>
__device__ __forceinline__ void adj_edge_role(const Geo<T> &g, const AdjSplitIn<T, P> &x, Acc<T> *grad) {
  constexpr int N = Dims<P>::N, R = Dims<P>::R;
  const Tab<T, P> &tb = tab<T, P>();
  const int e = x.e, Kp = x.Kp;
  const int code = g.code[e];
  const int nb = g.nbr[(size_t)n * Kp + e];
  const int nk = (code >> (2 * n)) & 3;   // the neighbour's local index of the shared edge
  const bool outOk = (code >> (6 + n)) & 1;
  T V[R], V2[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    V[r] = g.Vn[(size_t)(n * R + r) * Kp + e];
    V2[r] = nb >= 0 ? g.Vn[(size_t)(nk * R + r) * Kp + nb] : T(0);
  }
  pdl_wait();
  T c[N], mp[N], cn[N], mu2[N];
  SensAcc<T> sV[R];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    c[j] = x.cs[(size_t)j * Kp + e];
    mp[j] = x.mpIn ? x.mpIn[(size_t)j * Kp + e] : x.coef * x.muIn[(size_t)j * Kp + e];
    cn[j] = nb >= 0 ? x.cs[(size_t)j * Kp + nb] : T(0);
    mu2[j] = nb >= 0 ? (x.mpIn ? x.mpIn[(size_t)j * Kp + nb] : x.coef * x.muIn[(size_t)j * Kp + nb]) : T(0);
  }
#pragma unroll
  for (int r = 0; r < R; ++r) sV[r].load(x.aV + (size_t)(n * R + r) * Kp + e);
  // upwind flux of the element's own edge n
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const T v = V[r];
    Acc<T> eta(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) eta.fma(tb.Hphi[n][r][j], mp[j]);
    const T et = eta.get();
    T sens = T(0);
    if (v > T(0) && outOk) {
      Acc<T> tr(T(0));
#pragma unroll
      for (int j = 0; j < N; ++j) tr.fma(tb.phi1D[n][r][j], c[j]);
      sens = -(et * tr.get());
      const T ev = et * v;
#pragma unroll
      for (int j = 0; j < N; ++j) grad[j].fms(tb.phi1D[n][r][j], ev);
    } else if (v < T(0) && nb >= 0) {
      Acc<T> tr(T(0));
#pragma unroll
      for (int j = 0; j < N; ++j) tr.fma(tb.thetaPhi[n][nk][r][j], cn[j]);
      sens = -(et * tr.get());
    }
    sV[r].add(sens);
  }
  // upwind flux of the neighbour across edge n where it takes this element's trace (v < 0 there)
  if (nb >= 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T v2 = V2[r];
      if (v2 < T(0)) {
        Acc<T> eta(T(0));
#pragma unroll
        for (int j = 0; j < N; ++j) eta.fma(tb.Hphi[nk][r][j], mu2[j]);
        const T ev = eta.get() * v2;
#pragma unroll
        for (int j = 0; j < N; ++j) grad[j].fms(tb.thetaPhi[nk][n][r][j], ev);
      }
    }
  }
  if (x.k >= 0) {
#pragma unroll
    for (int r = 0; r < R; ++r) sV[r].store(x.aV + (size_t)(n * R + r) * Kp + x.k);
  }
}

template <typename T, int P>
__device__ __forceinline__ void adj_volume_role(const Geo<T> &g, const AdjSplitIn<T, P> &x, Acc<T> *grad) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q;
  const Tab<T, P> &tb = tab<T, P>();
  const int e = x.e, Kp = x.Kp;
  T F[2 * Q];
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) F[i] = g.F[(size_t)i * Kp + e];
  pdl_wait();
  T c[N], mp[N];
  SensAcc<T> sF[2 * Q];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    c[j] = x.cs[(size_t)j * Kp + e];
    mp[j] = x.mpIn ? x.mpIn[(size_t)j * Kp + e] : x.coef * x.muIn[(size_t)j * Kp + e];
  }
#pragma unroll
  for (int i = 0; i < 2 * Q; ++i) sF[i].load(x.aF + (size_t)i * Kp + e);
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
    sF[q].add(s1 * cq);
    sF[Q + q].add(s2 * cq);
    const T wq = s1 * F[q] + s2 * F[Q + q];
#pragma unroll
    for (int j = 0; j < N; ++j) grad[j].fma(tb.phiQ[q][j], wq);
  }
  if (x.k >= 0) {
#pragma unroll
    for (int i = 0; i < 2 * Q; ++i) sF[i].store(x.aF + (size_t)i * Kp + x.k);
  }
}

// Up to p = 2, 64 registers at most in FP32 (8 / W blocks of 128 W threads per SM): a
// 32768-triangle stage then fits one wave of CTAs with two warps per role.  FP64 holds twice the
// bytes per value: 128 registers at most (4 / W blocks).
template <typename T, int P, int W>
__global__ void __launch_bounds__(128 * W, P <= 2 ? (sizeof(T) == 4 ? 8 / W : (4 / W > 0 ? 4 / W : 1)) : 1)
k_adj_stage_split(const Geo<T> g, const T *muIn, const T *mpIn, const T *cs, T *__restrict__ muOut,
                  T *__restrict__ accn, double *__restrict__ aF, double *__restrict__ aV, const AdjScalars a) {
  constexpr int N = Dims<P>::N;
  constexpr int NL = (N + 3) / 4;   // coefficients each role stores, at most
  __shared__ T part[4][N][32 * W];
  pdl_trigger();
  const int warp = threadIdx.x / 32, role = warp / W;
  const int lane = (warp % W) * 32 + threadIdx.x % 32;   // element of the CTA
  const int k = blockIdx.x * (32 * W) + lane;
  const bool active = k < g.K;
  AdjSplitIn<T, P> x;
  x.muIn = muIn; x.mpIn = mpIn; x.cs = cs; x.aF = aF; x.aV = aV;
  x.coef = T((1.0 - a.omega) * a.tau);
  x.e = active ? k : 0;   // lanes past the end read element 0 and store nothing
  x.k = active ? k : -1;
  x.Kp = g.Kp;
  Acc<T> grad[N];
#pragma unroll
  for (int i = 0; i < N; ++i) grad[i] = Acc<T>(T(0));
  switch (role) {   // uniform per warp
    case 0: adj_edge_role<T, P, 0>(g, x, grad); break;
    case 1: adj_edge_role<T, P, 1>(g, x, grad); break;
    case 2: adj_edge_role<T, P, 2>(g, x, grad); break;
    default: adj_volume_role<T, P>(g, x, grad); break;
  }
  // this role's coefficients of the update, read while the partials meet
  const T w = T(a.omega);
  T muL[NL], acL[NL];
#pragma unroll
  for (int t = 0; t < NL; ++t) {
    const int i = role + 4 * t;
    muL[t] = i < N ? muIn[(size_t)i * x.Kp + x.e] : T(0);
    acL[t] = (i < N && !a.init) ? accn[(size_t)i * x.Kp + x.e] : T(0);
  }
#pragma unroll
  for (int i = 0; i < N; ++i) part[role][i][lane] = grad[i].get();
  __syncthreads();
  if (!active) return;
  // reverse SSP update and the stores: role r stores coefficients r, r + 4, ...
#pragma unroll
  for (int t = 0; t < NL; ++t) {
    const int i = role + 4 * t;
    if (i < N) {
      const T gi = ((part[3][i][lane] + part[0][i][lane]) + part[1][i][lane]) + part[2][i][lane];
      const T mo = (T(1) - w) * muL[t] + gi;
      if (muOut) muOut[(size_t)i * x.Kp + k] = mo;
      T acc = a.init ? w * muL[t] : acL[t] + w * muL[t];
      if (a.last) acc = acc + mo;
      accn[(size_t)i * x.Kp + k] = acc;
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Adjoint of the linear limiter (core/computeVertexBasedLimiter.m:78-106 in the geometry-free form
// of lin_alpha).  With its discrete choices frozen the limiter is rational in its input x:
//   solution limiter (KIND 0):        out = x - DM^-1[:,1:] du(x)             (Dirichlet data)
//   time-derivative limiter (KIND 1): out = x + Q_k du(x)                      (no data)
// du = (0, (1-a) u1, (1-a) u2, u3, ...) for a < 1 (zero otherwise), u = DM x, a = dm / den at
// the first vertex whose factor is the element's, den = dV -/+ tol on the branch taken.  With
// r = M^T lambda (M = -DM^-1[:,1:] or Q_k):
//   dJ/dx = lambda + sum_j r_j d du_j/dx
//         = lambda + (1-a)(r1 DM1 + r2 DM2) + sum_{j>=3} r_j DMj - (r1 u1 + r2 u2) da/dx,
// where da/dx covers x's own mean and vertex value, and da/dm = 1/den goes to the patch element
// holding the extreme (its mean is DM0 . x): recorded here, gathered by k_lim_vjp_gather.  The
// choices are recomputed from the recorded input x (the same keys, shift and comparisons as the
// forward kernels); a tie for the extreme goes to the lowest element index of the caller's order,
// Dirichlet data winning a tie with an element.
//
// Two passes of a stage with the time-derivative limiter share launches:
//   SNEXT (solution limiter): after the dependency wait the kernel also scatters the means of the
//     time-derivative limiter's input `nextX` to the key set of the next pass (`loNext`, which
//     resets the set after that) and stores them in `meanNext`; the grid covers max(K, numV);
//   GIN (time-derivative limiter): each element first adds the solution limiter's extreme terms
//     (the first record set, pSlotT / pSlotW) into its lamIn and writes lamIn back, which is
//     what k_lim_vjp_gather would have done in a launch of its own.
// Records are kept by CSR position (csrPos): the element at position i of patch v writes slot i,
// so a gather reads the slots of its patches directly instead of each patch element's record.
// The key set written by SNEXT was reset by the previous pass's scatter and is read only by the
// next kernel; the set it resets was last read two passes ago.
template <typename T, int P, int KIND, bool GIN, bool SNEXT>
__global__ void __launch_bounds__(kBlock)
k_lim_vjp(const Geo<T> g, const T *x, const T *lamIn, T *__restrict__ lamOut, const LimIn<T> li,
          const StageScalars sc, double scale, const T *__restrict__ meanX, const int *__restrict__ csrPos,
          int *__restrict__ slotT, T *__restrict__ slotW, T *lamInW, const int *__restrict__ pSlotT,
          const T *__restrict__ pSlotW, const T *__restrict__ nextX, const LimOut<T> loNext,
          T *__restrict__ meanNext) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  __shared__ T sh[2];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0}, pos[3] = {0, 0, 0}, dmask = 0;
  if (active) {
    vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k];
    pos[0] = csrPos[k]; pos[1] = csrPos[Kp + k]; pos[2] = csrPos[2 * Kp + k];
    if (KIND == 0) dmask = (g.code[k] >> 9) & 7;
  }
  T data[3] = {T(0), T(0), T(0)};
  if (KIND == 0 && g.cDV0T && active)
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  // static data read before the dependency wait: the patch ranges of the three vertices and, for
  // the time-derivative limiter up to p = 2, the element's packed Taylor mass block (used where
  // the clip is active; loading it here takes a dependent round trip off that path)
  int vp0[3] = {0, 0, 0}, vp1[3] = {0, 0, 0};
  if (active) {
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      vp0[n] = g.vptr[vid[n]];
      vp1[n] = g.vptr[vid[n] + 1];
    }
  }
  constexpr bool kPrefetchMT = KIND == 1 && N <= 6;
  T mtv[kPrefetchMT ? N * (N - 1) : 1];
  if constexpr (kPrefetchMT) {
#pragma unroll
    for (int i = 0; i < N * (N - 1); ++i) mtv[i] = active ? g.MT[(size_t)i * Kp + k] : T(0);
  }
  pdl_wait();
  // blocks past the last element tile (SNEXT grids cover the vertices) use the last tile's
  // instance for the global extremes
  const int tile = min((int)blockIdx.x, (g.K - 1) / kBlock);
  if constexpr (SNEXT) {
    reset_next<T>(g, loNext, k);
    T q0 = T(0);
    if (active) {
      T cc[N];
#pragma unroll
      for (int i = 0; i < N; ++i) cc[i] = nextX[(size_t)i * Kp + k];
      q0 = lin_mean<T, P>(cc);
      meanNext[k] = q0;
    }
    scatter_quantities<T, 1>(g, loNext, &q0, vid, active, tile);
  }
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc, tile), li.nc, sh);
  T xv[N], lam[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    xv[i] = active ? x[(size_t)i * Kp + k] : T(0);
    lam[i] = active ? lamIn[(size_t)i * Kp + k] : T(0);
  }
  if constexpr (GIN) {
    if (active) {
      T acc = T(0);
      bool any = false;
#pragma unroll
      for (int n = 0; n < 3; ++n) {
#pragma unroll 4
        for (int i = vp0[n]; i < vp1[n]; ++i)
          if (pSlotT[i] == k) { acc = acc + pSlotW[i]; any = true; }
      }
      if (any) {
#pragma unroll
        for (int j = 0; j < N; ++j) {
          lam[j] = lam[j] + acc * tb.DM[0][j];
          lamInW[(size_t)j * Kp + k] = lam[j];
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) lam[i] = T(scale) * lam[i];
  VKeys<T, 1> kv;
  load_vkeys<T, 1>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  T u[N];
  lin_u<T, P>(xv, u);
  // the forward's factor (vertex_alpha_1div), with the vertex, branch and raw ratio that set it
  const T third = T(1) / T(3), two3 = T(2) / T(3), tol = T(1.e-8);
  const T hx[3] = {-third, two3, -third}, hy[3] = {-third, -third, two3};
  T v[3], valD[3], mn[3], mx[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    v[n] = (u[0] * T(1) + u[1] * hx[n]) + u[2] * hy[n];
    valD[n] = ((dmask >> n) & 1) ? data[n] : T(NAN);
  }
  patch_minmax<T, 1>(li, kv, sh, 0, valD, mn, mx);
  // the first vertex whose clamped ratio is the smallest (one division, for that vertex)
  RatioWin<T> rw;
  int ns = 0, brW = 0;
  T dmW = T(0), denW = T(1);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T dV = v[n] - u[0], dMin = mn[n] - u[0], dMax = mx[n] - u[0];
    int br = 0;
    T dm = T(0), dn = T(1);
    if (dV < dMin + tol) { dm = dMin; dn = dV - tol; br = 1; }
    if (dV > dMax - tol) { dm = dMax; dn = dV + tol; br = 2; }
    if (br != 0 && rw.offer(dm, dn)) { ns = n; brW = br; dmW = dm; denW = dn; }
  }
  const T rawW = dmW / denW;
  const T alpha = brW != 0 ? fmax(T(0), fmin(T(1), rawW)) : T(1);
  T out[N];
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = lam[i];
  int tgt = -1;
  T w = T(0);
  if (alpha < T(1)) {
    T r[N];
    r[0] = T(0);
#pragma unroll
    for (int j = 1; j < N; ++j) {
      Acc<T> a(T(0));
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (KIND == 0) a.fms(tb.DMinv[i][j], lam[i]);
        else if constexpr (kPrefetchMT) a.fma(mtv[i * (N - 1) + (j - 1)], lam[i]);
        else a.fma(g.MT[(size_t)(i * (N - 1) + (j - 1)) * Kp + k], lam[i]);
      }
      r[j] = a.get();
    }
    T gu[N];   // dJ/du
#pragma unroll
    for (int j = 0; j < N; ++j) gu[j] = (j == 0) ? T(0) : (j <= 2 ? (T(1) - alpha) * r[j] : r[j]);
    const bool isPos = brW == 2;
    const T den = denW, dm = dmW, raw = rawW;
    if (brW != 0 && raw > T(0) && raw < T(1)) {
      const T sa = -(r[1] * u[1] + r[2] * u[2]);                  // dJ / d alpha
      const T q = dm / (den * den);
      gu[0] = gu[0] - sa / den;                                   // d dm / d u0 = -1
      gu[1] = gu[1] - sa * q * hx[ns];
      gu[2] = gu[2] - sa * q * hy[ns];
      // the extreme's source: Dirichlet data, or the patch element with that mean
      const T rawExt = vkey_inv<T>(kv.v[0][isPos ? 1 : 0][ns]);
      const bool fromData = ((dmask >> ns) & 1) && (isPos ? !(data[ns] < rawExt) : !(data[ns] > rawExt));
      if (!fromData) {
        const auto key = kv.v[0][isPos ? 1 : 0][ns];
        int best = -1, bestId = 0x7fffffff;
        const int i0 = ns == 0 ? vp0[0] : (ns == 1 ? vp0[1] : vp0[2]);
        const int i1 = ns == 0 ? vp1[0] : (ns == 1 ? vp1[1] : vp1[2]);
#pragma unroll 4
        for (int i = i0; i < i1; ++i) {   // the means k_mean_lin stored for this pass
          const int k2 = g.vidx[i];
          if (vkey(meanX[k2]) == key && g.permv[k2] < bestId) { best = k2; bestId = g.permv[k2]; }
        }
        tgt = best;
        w = sa / den;                                             // d alpha / d m = 1 / den
      }
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
      Acc<T> a(out[j]);
#pragma unroll
      for (int i = 0; i < N; ++i) a.fma(tb.DM[i][j], gu[i]);
      out[j] = a.get();
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) lamOut[(size_t)i * Kp + k] = out[i];
#pragma unroll
  for (int n = 0; n < 3; ++n)
    if (pos[n] >= 0) slotT[pos[n]] = n == ns ? tgt : -1;
  if (pos[ns] >= 0) slotW[pos[ns]] = w;
}

// k_lim_vjp in two halves, for the sweep on several streams.  The choices depend on the
// recorded input x only, not on lambda: k_lim_choice makes them on the recomputation stream,
// one reversed step ahead, and records per element the factor, the chosen vertex and branch,
// den, dm / den^2 and the element holding the extreme; k_lim_apply applies lambda on the
// reverse stream without the keys, the shifts or the patch walk for the extreme.  Both compute
// k_lim_vjp's expressions in its order, so the gradients are bitwise those of the one-kernel
// form.
template <typename T> struct LimChoice {
  T *alpha, *den, *q;   // per element (Kp)
  int *tgt, *info;      // info: bits 0-1 the vertex, bit 2 limited, bit 3 the clip is active
};

// The record set of a pass's linear-limiter choices (k_lim_choice -> k_lim_apply).
template <typename T>
static LimChoice<T> lim_choice_rec(const dgadv_handle *h, long long pass) {
  const size_t Kp = h->Kp;
  char *b = (char *)h->adjChoice + (size_t)(pass % h->adjKeySets) * Kp * (3 * sizeof(T) + 2 * sizeof(int));
  LimChoice<T> r;
  r.alpha = (T *)b;
  r.den = (T *)(b + Kp * sizeof(T));
  r.q = (T *)(b + 2 * Kp * sizeof(T));
  r.tgt = (int *)(b + 3 * Kp * sizeof(T));
  r.info = (int *)(b + 3 * Kp * sizeof(T) + Kp * sizeof(int));
  return r;
}

template <typename T, int P, int KIND>
__global__ void __launch_bounds__(kBlock)
k_lim_choice(const Geo<T> g, const T *x, const LimIn<T> li, const StageScalars sc,
             const T *__restrict__ meanX, const LimChoice<T> rec) {
  constexpr int N = Dims<P>::N;
  __shared__ T sh[2];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0}, dmask = 0;
  if (active) {
    vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k];
    if (KIND == 0) dmask = (g.code[k] >> 9) & 7;
  }
  T data[3] = {T(0), T(0), T(0)};
  if (KIND == 0 && g.cDV0T && active)
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  int vp0[3] = {0, 0, 0}, vp1[3] = {0, 0, 0};
  if (active) {
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      vp0[n] = g.vptr[vid[n]];
      vp1[n] = g.vptr[vid[n] + 1];
    }
  }
  pdl_wait();
  const int tile = min((int)blockIdx.x, (g.K - 1) / kBlock);
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc, tile), li.nc, sh);
  T xv[N];
#pragma unroll
  for (int i = 0; i < N; ++i) xv[i] = active ? x[(size_t)i * Kp + k] : T(0);
  VKeys<T, 1> kv;
  load_vkeys<T, 1>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  T u[N];
  lin_u<T, P>(xv, u);
  const T third = T(1) / T(3), two3 = T(2) / T(3), tol = T(1.e-8);
  const T hx[3] = {-third, two3, -third}, hy[3] = {-third, -third, two3};
  T v[3], valD[3], mn[3], mx[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    v[n] = (u[0] * T(1) + u[1] * hx[n]) + u[2] * hy[n];
    valD[n] = ((dmask >> n) & 1) ? data[n] : T(NAN);
  }
  patch_minmax<T, 1>(li, kv, sh, 0, valD, mn, mx);
  // the first vertex whose clamped ratio is the smallest (one division, for that vertex)
  RatioWin<T> rw;
  int ns = 0, brW = 0;
  T dmW = T(0), denW = T(1);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T dV = v[n] - u[0], dMin = mn[n] - u[0], dMax = mx[n] - u[0];
    int br = 0;
    T dm = T(0), dn = T(1);
    if (dV < dMin + tol) { dm = dMin; dn = dV - tol; br = 1; }
    if (dV > dMax - tol) { dm = dMax; dn = dV + tol; br = 2; }
    if (br != 0 && rw.offer(dm, dn)) { ns = n; brW = br; dmW = dm; denW = dn; }
  }
  const T rawW = dmW / denW;
  const T alpha = brW != 0 ? fmax(T(0), fmin(T(1), rawW)) : T(1);
  int info = ns, tgt = -1;
  T den = T(1), q = T(0);
  if (alpha < T(1)) {
    info |= 4;
    const bool isPos = brW == 2;
    den = denW;
    const T dm = dmW, raw = rawW;
    if (brW != 0 && raw > T(0) && raw < T(1)) {
      info |= 8;
      q = dm / (den * den);
      const T rawExt = vkey_inv<T>(kv.v[0][isPos ? 1 : 0][ns]);
      const bool fromData = ((dmask >> ns) & 1) && (isPos ? !(data[ns] < rawExt) : !(data[ns] > rawExt));
      if (!fromData) {
        const auto key = kv.v[0][isPos ? 1 : 0][ns];
        int best = -1, bestId = 0x7fffffff;
        const int i0 = ns == 0 ? vp0[0] : (ns == 1 ? vp0[1] : vp0[2]);
        const int i1 = ns == 0 ? vp1[0] : (ns == 1 ? vp1[1] : vp1[2]);
#pragma unroll 4
        for (int i = i0; i < i1; ++i) {
          const int k2 = g.vidx[i];
          if (vkey(meanX[k2]) == key && g.permv[k2] < bestId) { best = k2; bestId = g.permv[k2]; }
        }
        tgt = best;
      }
    }
  }
  rec.alpha[k] = alpha;
  rec.den[k] = den;
  rec.q[k] = q;
  rec.tgt[k] = tgt;
  rec.info[k] = info;
}

template <typename T, int P, int KIND, bool GIN>
__global__ void __launch_bounds__(kBlock)
k_lim_apply(const Geo<T> g, const T *x, const T *lamIn, T *__restrict__ lamOut, const LimChoice<T> rec,
            double scale, const int *__restrict__ csrPos, int *__restrict__ slotT, T *__restrict__ slotW,
            T *lamInW, const int *__restrict__ pSlotT, const T *__restrict__ pSlotW) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  if (k >= g.K) return;
  const int Kp = g.Kp;
  const int pos[3] = {csrPos[k], csrPos[Kp + k], csrPos[2 * Kp + k]};
  int vp0[3] = {0, 0, 0}, vp1[3] = {0, 0, 0};
  if constexpr (GIN) {
    const int vid[3] = {g.V0T[k], g.V0T[Kp + k], g.V0T[2 * Kp + k]};
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      vp0[n] = g.vptr[vid[n]];
      vp1[n] = g.vptr[vid[n] + 1];
    }
  }
  constexpr bool kPrefetchMT = KIND == 1 && N <= 6;
  T mtv[kPrefetchMT ? N * (N - 1) : 1];
  if constexpr (kPrefetchMT) {
#pragma unroll
    for (int i = 0; i < N * (N - 1); ++i) mtv[i] = g.MT[(size_t)i * Kp + k];
  }
  pdl_wait();
  const int info = rec.info[k];
  const int ns = info & 3;
  T lam[N];
#pragma unroll
  for (int i = 0; i < N; ++i) lam[i] = lamIn[(size_t)i * Kp + k];
  if constexpr (GIN) {
    T acc = T(0);
    bool any = false;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
#pragma unroll 4
      for (int i = vp0[n]; i < vp1[n]; ++i)
        if (pSlotT[i] == k) { acc = acc + pSlotW[i]; any = true; }
    }
    if (any) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        lam[j] = lam[j] + acc * tb.DM[0][j];
        lamInW[(size_t)j * Kp + k] = lam[j];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) lam[i] = T(scale) * lam[i];
  T out[N];
#pragma unroll
  for (int i = 0; i < N; ++i) out[i] = lam[i];
  int tgt = -1;
  T w = T(0);
  if (info & 4) {
    const T third = T(1) / T(3), two3 = T(2) / T(3);
    const T hx[3] = {-third, two3, -third}, hy[3] = {-third, -third, two3};
    const T alpha = rec.alpha[k];
    T xv[N], u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) xv[i] = x[(size_t)i * Kp + k];
    lin_u3<T, P>(xv, u);   // rows 0..2 as lin_u computes them
    T r[N];
    r[0] = T(0);
#pragma unroll
    for (int j = 1; j < N; ++j) {
      Acc<T> a(T(0));
#pragma unroll
      for (int i = 0; i < N; ++i) {
        if (KIND == 0) a.fms(tb.DMinv[i][j], lam[i]);
        else if constexpr (kPrefetchMT) a.fma(mtv[i * (N - 1) + (j - 1)], lam[i]);
        else a.fma(g.MT[(size_t)(i * (N - 1) + (j - 1)) * Kp + k], lam[i]);
      }
      r[j] = a.get();
    }
    T gu[N];
#pragma unroll
    for (int j = 0; j < N; ++j) gu[j] = (j == 0) ? T(0) : (j <= 2 ? (T(1) - alpha) * r[j] : r[j]);
    if (info & 8) {
      const T den = rec.den[k], q = rec.q[k];
      const T sa = -(r[1] * u[1] + r[2] * u[2]);
      gu[0] = gu[0] - sa / den;
      gu[1] = gu[1] - sa * q * hx[ns];
      gu[2] = gu[2] - sa * q * hy[ns];
      tgt = rec.tgt[k];
      if (tgt >= 0) w = sa / den;
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
      Acc<T> a(out[j]);
#pragma unroll
      for (int i = 0; i < N; ++i) a.fma(tb.DM[i][j], gu[i]);
      out[j] = a.get();
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) lamOut[(size_t)i * Kp + k] = out[i];
#pragma unroll
  for (int n = 0; n < 3; ++n)
    if (pos[n] >= 0) slotT[pos[n]] = n == ns ? tgt : -1;
  if (pos[ns] >= 0) slotW[pos[ns]] = w;
}

// Gathers the recorded extreme terms: element e adds w DM0 for every element of its vertex
// patches whose limiter factor took its extreme from e at that vertex (CSR order: deterministic).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_lim_vjp_gather(const Geo<T> g, T *lam, const int *slotT, const T *slotW) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  if (k >= g.K) return;
  const int Kp = g.Kp;
  const int vid[3] = {g.V0T[k], g.V0T[Kp + k], g.V0T[2 * Kp + k]};
  int i0[3], i1[3];   // static: read before the dependency wait
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    i0[n] = g.vptr[vid[n]];
    i1[n] = g.vptr[vid[n] + 1];
  }
  pdl_wait();
  T acc = T(0);
  bool any = false;
#pragma unroll
  for (int n = 0; n < 3; ++n) {
#pragma unroll 4
    for (int i = i0[n]; i < i1[n]; ++i) {
      if (slotT[i] == k) { acc = acc + slotW[i]; any = true; }
    }
  }
  if (!any) return;
#pragma unroll
  for (int j = 0; j < N; ++j) lam[(size_t)j * Kp + k] = lam[(size_t)j * Kp + k] + acc * tb.DM[0][j];
}

// ---------------------------------------------------------------------------------------------
// Adjoint of the hierarchical vertex-based limiter
// (core/applySlopeLimiterTaylorHierarchicalVertex.m:124-168), on Taylor coefficients.  With its
// discrete choices frozen the limiter scales each degree d >= 1 of the Taylor coefficients x by
//   A_d = max(alpha_P, ..., alpha_d),   alpha_o = min over the sub-limiters i = 1..o of order o
// and the element's three vertices of the factor of core/computeVertexBasedLimiter.m:78-106,
// and a factor on an unsaturated branch is raw = dm / den with dm = ext - x[i0],
// den = x[i1] pt1_n + x[i2] pt2_n -+ tol (i0, i1, i2 the sub-limiter's derivative and its two
// neighbours, pt the Taylor basis at the vertex), ext the patch extreme of the sub-limiter's
// quantity (another element's x[i0], the element's own vertex value at a Dirichlet vertex above
// order 1, or boundary data).  For lambda = dJ/d(limited):
//   dJ/dx_j   = A_d(j) lambda_j  (+ lambda_0 for the mean)
//   dJ/dalpha_o = S_o = sum over the degrees d whose A_d is alpha_o of sum_j x_j lambda_j
//   dJ/draw   = S_o, spread over x[i0], x[i1], x[i2] and ext as the derivatives of dm / den.
// Terms of an extreme held by another element are recorded (element, its Taylor index, weight)
// by CSR position and order, and gathered by k_lim_vjp_hier_gather.  The limiter's inputs are
// recorded in Taylor form; the map from the modal coefficients is T = S DM (to_taylor), so the
// solution limiter c = T^-1 L(x) gives dJ/dx = L'^T T^-T lambda, and the time-derivative limiter
// T^-1 ((I - Mcorr) L(x) + Mcorr x) gives Mcorr^T mu + L'^T (I - Mcorr)^T mu with mu = T^-T lambda.
// Outputs are modal: dJ/d(modal input) = T^T dJ/dx.
template <typename T, int P> struct HierWin {
  T raw, den, dm;
  int act;       // the factor is raw, on a branch and strictly inside (0, 1)
  int n, s;      // the winning vertex and quantity
  int si;        // the winning sub-limiter of the order (1..order)
  int src;       // extreme: 0 another element (recorded), 1 the element's own vertex value, 2 data
  int tgt;       // element holding the extreme (src 0)
  int vtx;       // the winning vertex (a global vertex id) and its extreme's key
  typename KeyOf<T>::type key;
};

// S (modal-derivative u -> Taylor) blocks: S[d][m][j] = idX^d times deriv_block of A = B^-1.
template <typename T, int P> struct SBlocks {
  T b[P + 1][P + 1][P + 1];
};
template <typename T, int P>
__device__ __forceinline__ void s_blocks(const Affine<T> &af, SBlocks<T, P> &sb) {
  sb.b[0][0][0] = T(1);
  T sc = T(1);
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    sc *= af.idX;
    if (d == 1) {
      T S[2][2]; deriv_block<T, 1>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 1; ++m)
#pragma unroll
        for (int j = 0; j <= 1; ++j) sb.b[1][m][j] = S[m][j] * sc;
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m)
#pragma unroll
        for (int j = 0; j <= 2; ++j) sb.b[2][m][j] = S[m][j] * sc;
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m)
#pragma unroll
        for (int j = 0; j <= 3; ++j) sb.b[3][m][j] = S[m][j] * sc;
    }
  }
}

// y = T^T w = DM^T S^T w (Taylor -> modal adjoint).
template <typename T, int P>
__device__ __forceinline__ void taylor_T_transpose(const SBlocks<T, P> &sb, const T *w, T *y) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T z[N];
  z[0] = w[0];
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    const int off = d * (d + 1) / 2;
#pragma unroll
    for (int j = 0; j <= d; ++j) {
      Acc<T> a(T(0));
#pragma unroll
      for (int m = 0; m <= d; ++m) a.fma(sb.b[d][m][j], w[off + m]);
      z[off + j] = a.get();
    }
  }
#pragma unroll
  for (int c = 0; c < N; ++c) {
    Acc<T> a(T(0));
#pragma unroll
    for (int i = 0; i < N; ++i) a.fma(tb.DM[i][c], z[i]);
    y[c] = a.get();
  }
}

// mu = T^-T lambda = S^-T DM^-T lambda (modal -> Taylor adjoint).
template <typename T, int P>
__device__ __forceinline__ void taylor_Tinv_transpose(const SinvBlocks<T, P> &si, const T *lam, T *mu) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T z[N];
#pragma unroll
  for (int a = 0; a < N; ++a) {
    Acc<T> s(T(0));
#pragma unroll
    for (int i = 0; i < N; ++i) s.fma(tb.DMinv[i][a], lam[i]);
    z[a] = s.get();
  }
  mu[0] = z[0];
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    const int off = d * (d + 1) / 2;
#pragma unroll
    for (int j = 0; j <= d; ++j) {
      Acc<T> s(T(0));
#pragma unroll
      for (int a = 0; a <= d; ++a) s.fma(si.b[d][a][j], z[off + a]);
      mu[off + j] = s.get();
    }
  }
}

// out = Mcorr^T z with Mcorr = diag(1/diag(M_T)) M_T: the stored packed block, or with
// M_T = 2|T| S^-T Gr S^-1 (taylor_mcorr) Mcorr^T z = S^-T Gr S^-1 (z ./ D).
template <typename T, int P>
__device__ __forceinline__ void mcorr_transpose(const Geo<T> &g, int k, const SinvBlocks<T, P> &si, const T *z,
                                                T *out) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  if (g.mtOnTheFly) {
    T w[N], y[N], gy[N];
    w[0] = z[0] / tb.Gr[0][0];
#pragma unroll
    for (int d = 1; d <= P; ++d) {
      const int off = d * (d + 1) / 2;
#pragma unroll
      for (int j = 0; j <= d; ++j) {
        Acc<T> D(T(0));
#pragma unroll
        for (int a = 0; a <= d; ++a) {
          Acc<T> r(T(0));
#pragma unroll
          for (int b = 0; b <= d; ++b) r.fma(tb.Gr[off + a][off + b], si.b[d][b][j]);
          D.fma(si.b[d][a][j], r.get());
        }
        w[off + j] = z[off + j] / D.get();
      }
    }
    y[0] = w[0];
#pragma unroll
    for (int d = 1; d <= P; ++d) {
      const int off = d * (d + 1) / 2;
#pragma unroll
      for (int a = 0; a <= d; ++a) {
        Acc<T> s(T(0));
#pragma unroll
        for (int j = 0; j <= d; ++j) s.fma(si.b[d][a][j], w[off + j]);
        y[off + a] = s.get();
      }
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc<T> s(T(0));
#pragma unroll
      for (int j = 0; j < N; ++j) s.fma(tb.Gr[i][j], y[j]);
      gy[i] = s.get();
    }
    out[0] = gy[0];
#pragma unroll
    for (int d = 1; d <= P; ++d) {
      const int off = d * (d + 1) / 2;
#pragma unroll
      for (int j = 0; j <= d; ++j) {
        Acc<T> s(T(0));
#pragma unroll
        for (int a = 0; a <= d; ++a) s.fma(si.b[d][a][j], gy[off + a]);
        out[off + j] = s.get();
      }
    }
  } else {
    const int Kp = g.Kp;
    T m[N][N];
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
      for (int b = a; b < N; ++b) {
        const T v = g.MT[(size_t)(a * N - a * (a - 1) / 2 + (b - a)) * Kp + k];
        m[a][b] = v;
        m[b][a] = v;
      }
    T w[N];
#pragma unroll
    for (int i = 0; i < N; ++i) w[i] = z[i] / m[i][i];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      Acc<T> s(T(0));
#pragma unroll
      for (int i = 0; i < N; ++i) s.fma(m[i][j], w[i]);
      out[j] = s.get();
    }
  }
}

// Taylor coefficients of the limiter input scattered to the adjoint's vertex keys (one quantity
// per sub-limiter, as the forward's passes), and the quantities stored per element.
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_vjp_scatter_hier(const Geo<T> g, const T *x, const LimOut<T> lo, T *__restrict__ qOut) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k);
  T qv[NQ];
#pragma unroll
  for (int s = 0; s < NQ; ++s) qv[s] = T(0);
  if (active) {
    T cT[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cT[i] = x[(size_t)i * Kp + k];
    centroid_quantities<T, P>(cT, 1, qv);
#pragma unroll
    for (int s = 0; s < NQ; ++s) qOut[(size_t)s * Kp + k] = qv[s];
  }
  scatter_quantities<T, NQ>(g, lo, qv, vid, active);
}

// The records of element k in the slots of its three vertex patches (CSR order, every order o
// at o * nnz + position), summed per Taylor index into acc; false if there are none.
template <typename T, int P>
__device__ __forceinline__ bool hier_records(int k, const int i0[3], const int i1[3], int nnz, const int *slotT,
                                             const T *slotW, T *acc) {
  constexpr int N = Dims<P>::N;
#pragma unroll
  for (int j = 0; j < N; ++j) acc[j] = T(0);
  bool any = false;
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    for (int i = i0[n]; i < i1[n]; ++i)
#pragma unroll
      for (int o = 0; o < P; ++o) {
        const int t = slotT[(size_t)o * nnz + i];
        if (t >= 0 && (t >> 4) == k) {
          const int ti = t & 15;
#pragma unroll
          for (int j = 0; j < N; ++j)
            if (j == ti) acc[j] = acc[j] + slotW[(size_t)o * nnz + i];
          any = true;
        }
      }
  }
  return any;
}

// lamIn of a time-derivative limiter pass with the solution limiter's extreme terms gathered in
// first (gInT != null; the sum is written back, as k_lim_vjp_hier_gather would have written it),
// scaled: lam = scale (lamIn + T^T records).  i0 / i1: the element's three CSR patch ranges.
template <typename T, int P>
__device__ __forceinline__ void hier_lam_in(const Geo<T> &g, int k, const int i0[3], const int i1[3], int nnz,
                                            const int *gInT, const T *gInW, T *lamInW, const SBlocks<T, P> &sb,
                                            const T *lraw, double scale, T *lam) {
  constexpr int N = Dims<P>::N;
  const int Kp = g.Kp;
  T v[N];
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = lraw[i];
  if (gInT) {
    T acc[N];
    if (hier_records<T, P>(k, i0, i1, nnz, gInT, gInW, acc)) {
      T add[N];
      taylor_T_transpose<T, P>(sb, acc, add);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        v[j] = v[j] + add[j];
        lamInW[(size_t)j * Kp + k] = v[j];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) lam[i] = T(scale) * v[i];
}

// The limiter adjoint of one pass (KIND 0 solution limiter, 1 time-derivative limiter).
// slotT / slotW: P records per CSR position (order o at o * nnz + position), element * 16 +
// Taylor index or -1, and the weight.
template <typename T, int P, int KIND>
__global__ void __launch_bounds__(kBlock)
k_lim_vjp_hier(const Geo<T> g, const T *x, const T *lamIn, T *__restrict__ lamOut, const LimIn<T> li,
               const StageScalars sc, double scale, const T *__restrict__ qStore, const int *__restrict__ csrPos,
               int nnz, int *__restrict__ slotT, T *__restrict__ slotW, const int *gInT, const T *gInW,
               T *lamInW) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  __shared__ T sh[2 * NQ];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0}, pos[3] = {-1, -1, -1}, dmask = 0;
  int pr0[3] = {0, 0, 0}, pr1[3] = {0, 0, 0};   // patch ranges of the fused gather (KIND 1)
  T B[4] = {T(1), T(0), T(0), T(1)};
  if (active) {
    vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k];
    pos[0] = csrPos[k]; pos[1] = csrPos[Kp + k]; pos[2] = csrPos[2 * Kp + k];
    dmask = (g.code[k] >> 9) & 7;
    if (KIND == 1 && gInT) {
#pragma unroll
      for (int n = 0; n < 3; ++n) { pr0[n] = g.vptr[vid[n]]; pr1[n] = g.vptr[vid[n] + 1]; }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) B[r] = g.Bm[(size_t)r * Kp + k];
  }
  T data[3] = {T(0), T(0), T(0)};
  if (KIND == 0 && g.cDV0T && active)
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  pdl_wait();
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc), li.nc, sh);
  T xv[N], lraw[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    xv[i] = active ? x[(size_t)i * Kp + k] : T(0);
    lraw[i] = active ? lamIn[(size_t)i * Kp + k] : T(0);
  }
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  const Affine<T> af = affine_from<T>(B[0], B[1], B[2], B[3]);
  SBlocks<T, P> sb;
  s_blocks<T, P>(af, sb);
  T lam[N];
  hier_lam_in<T, P>(g, k, pr0, pr1, nnz, KIND == 1 ? gInT : nullptr, gInW, lamInW, sb, lraw, scale, lam);
  SinvBlocks<T, P> si;
  sinv_blocks<T, P>(af, si);
  T mu[N], lamL[N], mc[N];
  taylor_Tinv_transpose<T, P>(si, lam, mu);
  if (KIND == 1) {
    mcorr_transpose<T, P>(g, k, si, mu, mc);
#pragma unroll
    for (int i = 0; i < N; ++i) lamL[i] = mu[i] - mc[i];
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) lamL[i] = mu[i];
  }
  // the forward's choices (limit_taylor, LT = 1), with the winners recorded
  const T tol = T(1.e-8), nan_ = T(NAN);
  T pt1[3], pt2[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) { pt1[n] = af.ox[n] * af.dX; pt2[n] = af.oy[n] * af.dX; }
  HierWin<T, P> win[P + 1];
  T A[P + 1];
  int winOrd[P + 1];
  T alphaRun = T(0);
  int runOrd = P;
  int s = 0;
#pragma unroll
  for (int ord = P; ord >= 1; --ord) {
    RatioWin<T> rw;   // the order's winner, compared without dividing
    win[ord].act = 0; win[ord].src = 2; win[ord].tgt = -1; win[ord].n = 0; win[ord].s = 0; win[ord].si = 1;
    win[ord].vtx = 0; win[ord].key = 0;
    win[ord].raw = win[ord].den = win[ord].dm = T(0);
#pragma unroll
    for (int i = 1; i <= ord; ++i) {
      const int i0 = mind(ord - i, i - 1), i1 = mind(ord - i + 1, i - 1), i2 = mind(ord - i, i);
      T v[3], valD[3], mn[3], mx[3];
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        v[n] = (xv[i0] * T(1) + xv[i1] * pt1[n]) + xv[i2] * pt2[n];
        valD[n] = ((dmask >> n) & 1) ? (ord > 1 ? v[n] : (KIND == 0 ? data[n] : nan_)) : nan_;
      }
      patch_minmax<T, NQ>(li, kv, sh, s, valD, mn, mx);
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        const T cbar = xv[i0];
        const T dV = v[n] - cbar, dMin = mn[n] - cbar, dMax = mx[n] - cbar;
        T den = T(0), dm = T(0);
        int br = 0;
        if (dV < dMin + tol) { den = dV - tol; dm = dMin; br = 1; }
        if (dV > dMax - tol) { den = dV + tol; dm = dMax; br = 2; }
        if (br != 0 && rw.offer(dm, den)) {   // the first (sub-limiter, vertex) reaching the order's minimum
          HierWin<T, P> &w = win[ord];
          w.den = den; w.dm = dm;
          w.n = n; w.s = s; w.si = i;
          // the extreme's source: the Dirichlet value (which wins a tie) or the patch element
          const bool isPos = br == 2;
          const T rawExt = vkey_inv<T>(kv.v[s][isPos ? 1 : 0][n]);
          const bool hasD = ((dmask >> n) & 1) && !(valD[n] != valD[n]);
          const bool fromD = hasD && (isPos ? !(valD[n] < rawExt) : !(valD[n] > rawExt));
          w.src = fromD ? (ord > 1 ? 1 : 2) : 0;
          w.tgt = -1;
          w.vtx = vid[n];
          w.key = kv.v[s][isPos ? 1 : 0][n];
        }
      }
      ++s;
    }
    // the winner's factor (one division) and the element holding its extreme, found once the
    // winner is known
    T aOrd = T(1);
    {
      HierWin<T, P> &w = win[ord];
      if (rw.cls < 2) {
        const T raw = w.dm / w.den;
        w.raw = raw;
        w.act = raw > T(0) && raw < T(1);
        aOrd = fmax(T(0), fmin(T(1), raw));
      }
      if (w.src == 0 && w.act) {
        const auto key = w.key;
        int best = -1, bestId = 0x7fffffff;
        const int e0 = g.vptr[w.vtx], e1 = g.vptr[w.vtx + 1];
        for (int e = e0; e < e1; ++e) {
          const int k2 = g.vidx[e];
          if (vkey(qStore[(size_t)w.s * Kp + k2]) == key && g.permv[k2] < bestId) { best = k2; bestId = g.permv[k2]; }
        }
        w.tgt = best;
      }
    }
    if (ord == P || aOrd > alphaRun) runOrd = ord;   // the order whose alpha is the running max
    alphaRun = fmax(alphaRun, aOrd);
    A[ord] = alphaRun;
    winOrd[ord] = runOrd;
  }
  // dJ/dx: A_d lambda_j, the mean passed on, then each winning order's factor
  T gx[N];
  gx[0] = lamL[0];
#pragma unroll
  for (int d = 1; d <= P; ++d)
#pragma unroll
    for (int j = d * (d + 1) / 2; j < (d + 1) * (d + 2) / 2; ++j) gx[j] = A[d] * lamL[j];
  if (KIND == 1) {
#pragma unroll
    for (int i = 0; i < N; ++i) gx[i] = gx[i] + mc[i];
  }
  int recT[P + 1];
  T recW[P + 1];
#pragma unroll
  for (int o = 1; o <= P; ++o) { recT[o] = -1; recW[o] = T(0); }
#pragma unroll
  for (int o = 1; o <= P; ++o) {
    Acc<T> so(T(0));
    bool used = false;
#pragma unroll
    for (int d = 1; d <= P; ++d)
      if (winOrd[d] == o) {
        used = true;
#pragma unroll
        for (int j = d * (d + 1) / 2; j < (d + 1) * (d + 2) / 2; ++j) so.fma(xv[j], lamL[j]);
      }
    const HierWin<T, P> &w = win[o];
    if (!used || !w.act) continue;
    const T So = so.get();
    const T q = So / w.den, r = So * w.dm / (w.den * w.den);
    const T p1 = w.n == 0 ? pt1[0] : (w.n == 1 ? pt1[1] : pt1[2]);
    const T p2 = w.n == 0 ? pt2[0] : (w.n == 1 ? pt2[1] : pt2[2]);
    // the winning sub-limiter's DOFs, as compile-time indices (registers, not local memory)
#pragma unroll
    for (int i = 1; i <= o; ++i) {
      if (i != w.si) continue;
      const int i0 = mind(o - i, i - 1), i1 = mind(o - i + 1, i - 1), i2 = mind(o - i, i);
      gx[i0] = gx[i0] - q;
      gx[i1] = gx[i1] - r * p1;
      gx[i2] = gx[i2] - r * p2;
      if (w.src == 1) {                          // ext = the element's own vertex value
        gx[i0] = gx[i0] + q;
        gx[i1] = gx[i1] + q * p1;
        gx[i2] = gx[i2] + q * p2;
      } else if (w.src == 0 && w.tgt >= 0) {     // ext = x[i0] of another element (or this one)
        recT[o] = w.tgt * 16 + i0;
        recW[o] = q;
      }
    }
  }
  T out[N];
  taylor_T_transpose<T, P>(sb, gx, out);
#pragma unroll
  for (int i = 0; i < N; ++i) lamOut[(size_t)i * Kp + k] = out[i];
#pragma unroll
  for (int o = 1; o <= P; ++o)
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (pos[n] >= 0) {
        const bool mine = win[o].n == n && recT[o] >= 0;
        slotT[(size_t)(o - 1) * nnz + pos[n]] = mine ? recT[o] : -1;
        if (mine) slotW[(size_t)(o - 1) * nnz + pos[n]] = recW[o];
      }
}

// ---------------------------------------------------------------------------------------------
// Adjoint of the strict limiter (core/applySlopeLimiterTaylorStrict.m:111-150), on Taylor
// coefficients.  The forward limits the orders ord = P..1 in turn, each on the data the higher
// orders already limited: y^(P+1) = x, and y^(ord) is y^(ord+1) with every DOF of degree >= ord
// scaled by alpha_ord, the minimum over the order's sub-limiters and vertices of the factor of
// core/computeVertexBasedLimiter.m:78-106.  A sub-limiter's vertex values are the degree
// (P - ord + 1) reconstruction from y^(ord+1) about a derivative of order ord - 1, x[i0], which
// no higher order has rescaled (so its patch extremes are those of the hierarchical limiter's
// quantities).  With the choices frozen and lambda = dJ/dy^(1), the orders are reversed,
// ord = 1..P, on ybar = dJ/dy^(ord):
//   S_ord = sum over the DOFs j of degree >= ord of ybar_j y^(ord+1)_j     (dJ/dalpha_ord)
//   ybar_j <- alpha_ord ybar_j on those DOFs
//   and on an unsaturated branch S_ord spread, as the derivatives of dm / den, over x[i0]
//   (dm = ext - x[i0]), the reconstruction's DOFs (den = v_n - x[i0] -+ tol) and the extreme
//   (another element's x[i0], recorded as for the hierarchical limiter, or the element's own
//   vertex value at a Dirichlet vertex above order 1).
// The forward's factor itself (vertex_alpha_1div, minimum over the sub-limiters) is recomputed
// as the forward computes it, so that y^(ord) is bitwise the forward's; the winner's ratio
// dm / den gives the derivative.
template <typename T, int P> struct StrictWin {
  T raw, den, dm;
  int act;       // the factor is raw, on a branch and strictly inside (0, 1)
  int i, n, s;   // sub-limiter, vertex and quantity of the winner
  int src;       // extreme: 0 another element (recorded), 1 the element's own vertex value, 2 data
  int tgt;       // element holding the extreme (src 0)
  int vtx;       // the winning vertex (a global vertex id) and its extreme's key
  typename KeyOf<T>::type key;
};

template <typename T, int P, int KIND>
__global__ void __launch_bounds__(kBlock)
k_lim_vjp_strict(const Geo<T> g, const T *x, const T *lamIn, T *__restrict__ lamOut, const LimIn<T> li,
                 const StageScalars sc, double scale, const T *__restrict__ qStore, const int *__restrict__ csrPos,
                 int nnz, int *__restrict__ slotT, T *__restrict__ slotW, const int *gInT, const T *gInW,
               T *lamInW) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  __shared__ T sh[2 * NQ];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0}, pos[3] = {-1, -1, -1}, dmask = 0;
  int pr0[3] = {0, 0, 0}, pr1[3] = {0, 0, 0};   // patch ranges of the fused gather (KIND 1)
  T B[4] = {T(1), T(0), T(0), T(1)};
  if (active) {
    vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k];
    pos[0] = csrPos[k]; pos[1] = csrPos[Kp + k]; pos[2] = csrPos[2 * Kp + k];
    dmask = (g.code[k] >> 9) & 7;
    if (KIND == 1 && gInT) {
#pragma unroll
      for (int n = 0; n < 3; ++n) { pr0[n] = g.vptr[vid[n]]; pr1[n] = g.vptr[vid[n] + 1]; }
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) B[r] = g.Bm[(size_t)r * Kp + k];
  }
  T data[3] = {T(0), T(0), T(0)};
  if (KIND == 0 && g.cDV0T && active)
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  pdl_wait();
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc), li.nc, sh);
  T xv[N], lraw[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    xv[i] = active ? x[(size_t)i * Kp + k] : T(0);
    lraw[i] = active ? lamIn[(size_t)i * Kp + k] : T(0);
  }
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  const Affine<T> af = affine_from<T>(B[0], B[1], B[2], B[3]);
  SBlocks<T, P> sb;
  s_blocks<T, P>(af, sb);
  T lam[N];
  hier_lam_in<T, P>(g, k, pr0, pr1, nnz, KIND == 1 ? gInT : nullptr, gInW, lamInW, sb, lraw, scale, lam);
  SinvBlocks<T, P> si;
  sinv_blocks<T, P>(af, si);
  T mu[N], lamL[N], mc[N];
  taylor_Tinv_transpose<T, P>(si, lam, mu);
  if (KIND == 1) {
    mcorr_transpose<T, P>(g, k, si, mu, mc);
#pragma unroll
    for (int i = 0; i < N; ++i) lamL[i] = mu[i] - mc[i];
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) lamL[i] = mu[i];
  }
  // the forward's orders (limit_taylor, LT = 2), with the winners recorded
  const T tol = T(1.e-8), nan_ = T(NAN);
  T phi[3][N];
  taylor_vertex_basis<T, P>(af, phi);
  StrictWin<T, P> win[P + 1];
  T alpha[P + 1];
  T y[N];
#pragma unroll
  for (int i = 0; i < N; ++i) y[i] = xv[i];
  int s = 0;
#pragma unroll
  for (int ord = P; ord >= 1; --ord) {
    RatioWin<T> rw;   // the order's winner, compared without dividing
    StrictWin<T, P> &w = win[ord];
    w.act = 0; w.src = 2; w.tgt = -1; w.i = 1; w.n = 0; w.s = 0; w.vtx = 0; w.key = 0;
    w.raw = w.den = w.dm = T(0);
    T aOrd = T(1);
#pragma unroll
    for (int i = 1; i <= ord; ++i) {
      const int ba = ord - i, bb = i - 1, i0 = mind(ba, bb);
      T v[3], valD[3], mn[3], mx[3];
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        T acc = T(0);
#pragma unroll
        for (int a = 0; a <= P - ord + 1; ++a)
#pragma unroll
          for (int b = 0; a + b <= P - ord + 1; ++b) acc = acc + y[mind(ba + a, bb + b)] * phi[n][mind(a, b)];
        v[n] = acc;
        valD[n] = ((dmask >> n) & 1) ? (ord > 1 ? v[n] : (KIND == 0 ? data[n] : nan_)) : nan_;
      }
      patch_minmax<T, NQ>(li, kv, sh, s, valD, mn, mx);
      aOrd = fmin(aOrd, vertex_alpha_1div(y[i0], v, mn, mx));
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        const T cbar = y[i0];
        const T dV = v[n] - cbar, dMin = mn[n] - cbar, dMax = mx[n] - cbar;
        T den = T(0), dm = T(0);
        int br = 0;
        if (dV < dMin + tol) { den = dV - tol; dm = dMin; br = 1; }
        if (dV > dMax - tol) { den = dV + tol; dm = dMax; br = 2; }
        if (br != 0 && rw.offer(dm, den)) {   // the first (sub-limiter, vertex) reaching the order's minimum
          w.den = den; w.dm = dm;
          w.i = i; w.n = n; w.s = s;
          // the extreme's source: the Dirichlet value (which wins a tie) or the patch element
          const bool isPos = br == 2;
          const T rawExt = vkey_inv<T>(kv.v[s][isPos ? 1 : 0][n]);
          const bool hasD = ((dmask >> n) & 1) && !(valD[n] != valD[n]);
          const bool fromD = hasD && (isPos ? !(valD[n] < rawExt) : !(valD[n] > rawExt));
          w.src = fromD ? (ord > 1 ? 1 : 2) : 0;
          w.tgt = -1;
          w.vtx = vid[n];
          w.key = kv.v[s][isPos ? 1 : 0][n];
        }
      }
      ++s;
    }
    if (rw.cls < 2) {
      w.raw = w.dm / w.den;
      w.act = w.raw > T(0) && w.raw < T(1);
    }
    if (w.src == 0 && w.act) {   // the element holding the winner's extreme (lowest original id)
      const auto key = w.key;
      int best = -1, bestId = 0x7fffffff;
      const int e0 = g.vptr[w.vtx], e1 = g.vptr[w.vtx + 1];
      for (int e = e0; e < e1; ++e) {
        const int k2 = g.vidx[e];
        if (vkey(qStore[(size_t)w.s * Kp + k2]) == key && g.permv[k2] < bestId) { best = k2; bestId = g.permv[k2]; }
      }
      w.tgt = best;
    }
    alpha[ord] = aOrd;
#pragma unroll
    for (int j = ord * (ord + 1) / 2; j < N; ++j) y[j] = aOrd * y[j];
  }
  // the orders reversed: gx = dJ/dy^(ord) on entry to order ord, dJ/dx at the end
  T gx[N];
#pragma unroll
  for (int i = 0; i < N; ++i) gx[i] = lamL[i];
  int recT[P + 1];
  T recW[P + 1];
#pragma unroll
  for (int o = 1; o <= P; ++o) { recT[o] = -1; recW[o] = T(0); }
#pragma unroll
  for (int ord = 1; ord <= P; ++ord) {
    const int off = ord * (ord + 1) / 2;
    // y^(ord+1): x rescaled by the orders above ord, in the forward's order
    T yp[N];
#pragma unroll
    for (int j = 0; j < N; ++j) yp[j] = xv[j];
#pragma unroll
    for (int o = P; o > ord; --o)
#pragma unroll
      for (int j = o * (o + 1) / 2; j < N; ++j) yp[j] = alpha[o] * yp[j];
    Acc<T> so(T(0));
#pragma unroll
    for (int j = off; j < N; ++j) so.fma(yp[j], gx[j]);
#pragma unroll
    for (int j = off; j < N; ++j) gx[j] = alpha[ord] * gx[j];
    const StrictWin<T, P> &w = win[ord];
    if (!w.act) continue;
    const T So = so.get();
    const T q = So / w.den, r = So * w.dm / (w.den * w.den);
#pragma unroll
    for (int i = 1; i <= ord; ++i) {
      if (i != w.i) continue;
      const int ba = ord - i, bb = i - 1, i0 = mind(ba, bb);
      // dm = ext - x[i0]; den = (reconstruction at vertex n) - x[i0] -+ tol, whose x[i0] terms cancel
      gx[i0] = gx[i0] - q;
#pragma unroll
      for (int a = 0; a <= P - ord + 1; ++a)
#pragma unroll
        for (int b = 0; a + b <= P - ord + 1; ++b) {
          if (a + b == 0) continue;
          const int m = mind(a, b), j = mind(ba + a, bb + b);
          const T ph = w.n == 0 ? phi[0][m] : (w.n == 1 ? phi[1][m] : phi[2][m]);
          gx[j] = gx[j] - r * ph;
          if (w.src == 1) gx[j] = gx[j] + q * ph;   // ext = the element's own vertex value
        }
      if (w.src == 1) gx[i0] = gx[i0] + q;
      else if (w.src == 0 && w.tgt >= 0) {        // ext = x[i0] of another element (or this one)
        recT[ord] = w.tgt * 16 + i0;
        recW[ord] = q;
      }
    }
  }
  if (KIND == 1) {
#pragma unroll
    for (int i = 0; i < N; ++i) gx[i] = gx[i] + mc[i];
  }
  T out[N];
  taylor_T_transpose<T, P>(sb, gx, out);
#pragma unroll
  for (int i = 0; i < N; ++i) lamOut[(size_t)i * Kp + k] = out[i];
#pragma unroll
  for (int o = 1; o <= P; ++o)
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (pos[n] >= 0) {
        const bool mine = win[o].n == n && recT[o] >= 0;
        slotT[(size_t)(o - 1) * nnz + pos[n]] = mine ? recT[o] : -1;
        if (mine) slotW[(size_t)(o - 1) * nnz + pos[n]] = recW[o];
      }
}

// Gathers the recorded extreme terms: element e adds w T^T e_i for every record (e, i, w) in the
// slots of its vertex patches (CSR order: deterministic).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_lim_vjp_hier_gather(const Geo<T> g, T *lam, int nnz, const int *slotT, const T *slotW) {
  constexpr int N = Dims<P>::N;
  const int k = blockIdx.x * kBlock + threadIdx.x;
  pdl_trigger();
  if (k >= g.K) return;
  const int Kp = g.Kp;
  const int vid[3] = {g.V0T[k], g.V0T[Kp + k], g.V0T[2 * Kp + k]};
  int i0[3], i1[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) { i0[n] = g.vptr[vid[n]]; i1[n] = g.vptr[vid[n] + 1]; }
  T B[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) B[r] = g.Bm[(size_t)r * Kp + k];
  pdl_wait();
  T acc[N];
  if (!hier_records<T, P>(k, i0, i1, nnz, slotT, slotW, acc)) return;
  const Affine<T> af = affine_from<T>(B[0], B[1], B[2], B[3]);
  SBlocks<T, P> sb;
  s_blocks<T, P>(af, sb);
  T add[N];
  taylor_T_transpose<T, P>(sb, acc, add);
#pragma unroll
  for (int j = 0; j < N; ++j) lam[(size_t)j * Kp + k] = lam[(size_t)j * Kp + k] + add[j];
}

// The solution limiter's pass uses the first record set and the means of vjp_scatter; the
// time-derivative limiter's pass the second record set and the means its predecessor scattered.
template <typename T, int P>
static cudaError_t launch_lim_vjp(dgadv_handle *h, const LimVjpArgs &v) {
  const Geo<T> g = make_geo<T>(h);
  const int gridK = (h->K + kBlock - 1) / kBlock;
  StageScalars sc{};
  sc.flag = h->flag;
  for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = v.gco[m];
  if (h->limType != DGADV_LIM_LINEAR) {   // one pass and its gather, P records per position
    int *rT = h->recSlotT[v.kind];
    T *rW = (T *)h->recSlotW[v.kind];
    const T *q = adj_means<T>(h, v.pass);
    const int nnz = 3 * h->K;
    const bool strict = h->limType == DGADV_LIM_STRICT;
    auto kern = strict ? (v.kind == 0 ? k_lim_vjp_strict<T, P, 0> : k_lim_vjp_strict<T, P, 1>)
                       : (v.kind == 0 ? k_lim_vjp_hier<T, P, 0> : k_lim_vjp_hier<T, P, 1>);
    // the time-derivative limiter's pass gathers the solution limiter's extreme terms into its
    // input itself (gatherIn), in place of that pass's gather launch
    const bool gin = v.kind == 1 && v.gatherIn;
    launch_k(h, kern, gridK, (size_t)0, g, (const T *)v.x, (const T *)v.lamIn, (T *)v.lamOut,
             lim_in_adj<T>(h, v.pass), sc, v.scale, q, (const int *)h->csrPos, nnz, rT, rW,
             gin ? (const int *)h->recSlotT[0] : (const int *)nullptr,
             gin ? (const T *)h->recSlotW[0] : (const T *)nullptr, (T *)v.lamIn);
    if (v.gatherOut)
      launch_k(h, k_lim_vjp_hier_gather<T, P>, gridK, (size_t)0, g, (T *)v.lamOut, nnz, (const int *)rT,
               (const T *)rW);
    return cudaGetLastError();
  }
  int *rT = h->recSlotT[v.kind];
  T *rW = (T *)h->recSlotW[v.kind];
  const int *cp = h->csrPos;
  if (v.apply) {   // the choices were recorded by lim_choice
    const LimChoice<T> rec = lim_choice_rec<T>(h, v.pass);
    const T *lamIn = (const T *)v.lamIn;
    T *lamInW = (T *)v.lamIn;
    if (v.kind == 0)
      launch_k(h, k_lim_apply<T, P, 0, false>, gridK, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut, rec,
               v.scale, cp, rT, rW, lamInW, (const int *)nullptr, (const T *)nullptr);
    else if (v.gatherIn)
      launch_k(h, k_lim_apply<T, P, 1, true>, gridK, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut, rec,
               v.scale, cp, rT, rW, lamInW, (const int *)h->recSlotT[0], (const T *)h->recSlotW[0]);
    else
      launch_k(h, k_lim_apply<T, P, 1, false>, gridK, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut, rec,
               v.scale, cp, rT, rW, lamInW, (const int *)nullptr, (const T *)nullptr);
    if (v.gatherOut)
      launch_k(h, k_lim_vjp_gather<T, P>, gridK, (size_t)0, g, (T *)v.lamOut, (const int *)rT, (const T *)rW);
    return cudaGetLastError();
  }
  const T *meanX = adj_means<T>(h, v.pass);
  const LimOut<T> loNext = lim_out_adj<T>(h, v.pass + 1);
  const T *lamIn = (const T *)v.lamIn;
  T *lamInW = (T *)v.lamIn;
  if (v.kind == 0 && v.nextX) {
    const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;
    launch_k(h, k_lim_vjp<T, P, 0, false, true>, grid, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut,
             lim_in_adj<T>(h, v.pass), sc, v.scale, meanX, cp, rT, rW, lamInW, (const int *)nullptr,
             (const T *)nullptr, (const T *)v.nextX, loNext, adj_means<T>(h, v.pass + 1));
  } else if (v.kind == 0) {
    launch_k(h, k_lim_vjp<T, P, 0, false, false>, gridK, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut,
             lim_in_adj<T>(h, v.pass), sc, v.scale, meanX, cp, rT, rW, lamInW, (const int *)nullptr,
             (const T *)nullptr, (const T *)nullptr, loNext, (T *)nullptr);
  } else if (v.gatherIn) {
    launch_k(h, k_lim_vjp<T, P, 1, true, false>, gridK, (size_t)0, g, (const T *)v.x, lamIn, (T *)v.lamOut,
             lim_in_adj<T>(h, v.pass), sc, v.scale, meanX, cp, rT, rW, lamInW, (const int *)h->recSlotT[0],
             (const T *)h->recSlotW[0], (const T *)nullptr, loNext, (T *)nullptr);
  } else {
    return cudaErrorInvalidValue;   // the time-derivative pass follows a solution pass with nextX
  }
  if (v.gatherOut)
    launch_k(h, k_lim_vjp_gather<T, P>, gridK, (size_t)0, g, (T *)v.lamOut, (const int *)rT, (const T *)rW);
  return cudaGetLastError();
}

// The linear limiter's choices of one pass (k_lim_choice), from its keys and means.
template <typename T, int P>
static cudaError_t launch_lim_choice(dgadv_handle *h, const LimVjpArgs &v) {
  const Geo<T> g = make_geo<T>(h);
  const int gridK = (h->K + kBlock - 1) / kBlock;
  StageScalars sc{};
  sc.flag = h->flag;
  for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = v.gco[m];
  const LimChoice<T> rec = lim_choice_rec<T>(h, v.pass);
  if (v.kind == 0)
    launch_k(h, k_lim_choice<T, P, 0>, gridK, (size_t)0, g, (const T *)v.x, lim_in_adj<T>(h, v.pass), sc,
             (const T *)adj_means<T>(h, v.pass), rec);
  else
    launch_k(h, k_lim_choice<T, P, 1>, gridK, (size_t)0, g, (const T *)v.x, lim_in_adj<T>(h, v.pass), sc,
             (const T *)adj_means<T>(h, v.pass), rec);
  return cudaGetLastError();
}

// Means of x scattered to the adjoint's own vertex keys (the limiter's patch extremes).
template <typename T, int P>
static cudaError_t launch_vjp_scatter(dgadv_handle *h, const void *x, long long pass, int kind) {
  const Geo<T> g = make_geo<T>(h);
  const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;
  T *q = adj_means<T>(h, pass);
  if (h->limType != DGADV_LIM_LINEAR)   // the hierarchical and the strict limiter's quantities
    launch_k(h, k_vjp_scatter_hier<T, P>, grid, (size_t)0, g, (const T *)x, lim_out_adj<T>(h, pass), q);
  else
    launch_k(h, k_mean_lin<T, P>, grid, (size_t)0, g, (const T *)x, lim_out_adj<T>(h, pass), q);
  return cudaGetLastError();
}

template <typename T, int P>
static cudaError_t launch_adj_stage(dgadv_handle *h, const AdjStageArgs &s) {
  const Geo<T> g = make_geo<T>(h);
  AdjScalars a;
  a.omega = s.omega; a.tau = s.tau; a.init = s.init; a.last = s.last;
  if (h->adjWarps > 0) {
    // the warp-role split (DGADV_OPT_ADJ_WARPS = W > 0), or one thread per element (0)
    const int W = h->adjWarps, grid = (h->K + 32 * W - 1) / (32 * W);
    auto kern = W == 4 ? k_adj_stage_split<T, P, 4> : (W == 2 ? k_adj_stage_split<T, P, 2> : k_adj_stage_split<T, P, 1>);
    launch_kb(h, kern, grid, 128 * W, (size_t)0, g, (const T *)s.muIn, (const T *)s.mpIn, (const T *)s.cs,
              (T *)s.muOut, (T *)s.accn, h->aF, h->aV, a);
  } else {
    const int grid = (h->K + kBlock - 1) / kBlock;
    launch_k(h, k_adj_stage<T, P>, grid, (size_t)0, g, (const T *)s.muIn, (const T *)s.mpIn, (const T *)s.cs,
             (T *)s.muOut, (T *)s.accn, h->aF, h->aV, a);
  }
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

template <typename T, int MASK>
static cudaError_t dispatch_lim_vjp(dgadv_handle *h, const LimVjpArgs &v) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return launch_lim_vjp<T, 1>(h, v); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_lim_vjp<T, 2>(h, v); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_lim_vjp<T, 3>(h, v); break;
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK>
static cudaError_t dispatch_vjp_scatter(dgadv_handle *h, const void *x, long long pass, int kind) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return launch_vjp_scatter<T, 1>(h, x, pass, kind); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_vjp_scatter<T, 2>(h, x, pass, kind); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_vjp_scatter<T, 3>(h, x, pass, kind); break;
  }
  return cudaErrorNotSupported;
}

template <typename T, int MASK>
static cudaError_t dispatch_lim_choice(dgadv_handle *h, const LimVjpArgs &v) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return launch_lim_choice<T, 1>(h, v); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_lim_choice<T, 2>(h, v); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_lim_choice<T, 3>(h, v); break;
  }
  return cudaErrorNotSupported;
}

// The operation table of a unit with the adjoint kernels added.
template <typename T, int MASK>
static PrecOps with_adjoint(PrecOps o) {
  o.adj_stage = dispatch_adj_stage<T, MASK>;
  o.lim_vjp = dispatch_lim_vjp<T, MASK>;
  o.vjp_scatter = dispatch_vjp_scatter<T, MASK>;
  o.lim_choice = dispatch_lim_choice<T, MASK>;
  return o;
}

}  // namespace dgadv
