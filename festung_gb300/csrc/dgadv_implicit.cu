// Implicit time stepping: the advection_implicit problem on the device.
//
// The reference solves, per stage of a diagonally implicit Runge-Kutta method
// (core/rungeKuttaImplicit.m, advection_implicit/solveSubStep.m),
//     (M + tau a_ii A) x_i = tau a_ii sysV(t_i) + M c^n + sum_{j<i} tau a_ij rhs_j,
//     rhs_i = sysV(t_i) - A x_i,      c^{n+1} = x_S,
// and A x = sysV for a stationary problem, each with a sparse direct solver.  Here the same
// equations are multiplied by M^-1 (block diagonal) and solved matrix-free:
//     (I + tau a_ii M^-1 A) x_i = c^n + tau sum_{j<i} a_ij k_j + tau a_ii s_i,
//     s_i = M^-1 sysV(t_i),   k_i = s_i - M^-1 A x_i,
// by restarted GMRES with classical Gram-Schmidt twice, right-preconditioned by the inverse of
// each element's diagonal block.  The operator kernel is the stage operator's arithmetic
// (volume term, upwind flux, mass solve) with the implicit problem's volume rule of order 2p+1
// (advection_implicit/preprocessProblem.m); handles for it are created with
// DGADV_FLAG_IMPLICIT.  Vectors are the handle's SoA state layout (N x Kp, padding zero);
// inner products accumulate in FP64.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dgadv_handle.h"

namespace dgadv {
namespace {

constexpr int kImplBlock = 128;
constexpr int kElemThreads = 32;      // element kernels: one warp per block spreads a small mesh over every SM
constexpr int kVecThreads = 256;
constexpr int kMaxDotBlocks = 512;
constexpr int kChunk = 8;             // vectors per multi-dot / update launch

template <int P> struct IDims {
  static constexpr int N = (P + 1) * (P + 2) / 2;
  static constexpr int Q = P == 0 ? 1 : (P == 1 ? 4 : (P == 2 ? 7 : 49));   // quadRule2D(2p+1)
  static constexpr int R = P + 1;                                            // quadRule1D(2p+1)
};

template <typename T, int P> struct ImplTab {
  static constexpr int N = IDims<P>::N, Q = IDims<P>::Q, R = IDims<P>::R;
  T phiQ[Q][N];
  T g1[Q][N];
  T g2[Q][N];
  T phi1D[3][R][N];
  T thetaPhi[3][3][R][N];
  T hatMinv[N][N];
};

__constant__ ImplTab<double, 0> c_d0;
__constant__ ImplTab<double, 1> c_d1;
__constant__ ImplTab<double, 2> c_d2;
__constant__ ImplTab<double, 3> c_d3;
__constant__ ImplTab<float, 0> c_f0;
__constant__ ImplTab<float, 1> c_f1;
__constant__ ImplTab<float, 2> c_f2;
__constant__ ImplTab<float, 3> c_f3;

template <typename T, int P> __device__ __forceinline__ const ImplTab<T, P> &itab();
template <> __device__ __forceinline__ const ImplTab<double, 0> &itab<double, 0>() { return c_d0; }
template <> __device__ __forceinline__ const ImplTab<double, 1> &itab<double, 1>() { return c_d1; }
template <> __device__ __forceinline__ const ImplTab<double, 2> &itab<double, 2>() { return c_d2; }
template <> __device__ __forceinline__ const ImplTab<double, 3> &itab<double, 3>() { return c_d3; }
template <> __device__ __forceinline__ const ImplTab<float, 0> &itab<float, 0>() { return c_f0; }
template <> __device__ __forceinline__ const ImplTab<float, 1> &itab<float, 1>() { return c_f1; }
template <> __device__ __forceinline__ const ImplTab<float, 2> &itab<float, 2>() { return c_f2; }
template <> __device__ __forceinline__ const ImplTab<float, 3> &itab<float, 3>() { return c_f3; }

template <typename T, int P> const void *itab_symbol();
template <> const void *itab_symbol<double, 0>() { return (const void *)&c_d0; }
template <> const void *itab_symbol<double, 1>() { return (const void *)&c_d1; }
template <> const void *itab_symbol<double, 2>() { return (const void *)&c_d2; }
template <> const void *itab_symbol<double, 3>() { return (const void *)&c_d3; }
template <> const void *itab_symbol<float, 0>() { return (const void *)&c_f0; }
template <> const void *itab_symbol<float, 1>() { return (const void *)&c_f1; }
template <> const void *itab_symbol<float, 2>() { return (const void *)&c_f2; }
template <> const void *itab_symbol<float, 3>() { return (const void *)&c_f3; }

template <typename T> struct ImplArgs {
  int K, Kp, nTerms;
  const T *F, *Vn, *rhs;
  const int *nbr, *code;
  double gco[4];       // g_m(t) of the source terms
};

// y = ca x + cb cDot(x), cDot = M^-1 (sum_m g_m rhs_m [RHS] + volume(x) - upwind flux(x)).
template <typename T, int P, bool RHS>
__global__ void __launch_bounds__(kImplBlock) k_impl_op(const ImplArgs<T> a, const T *__restrict__ x,
                                                        T *__restrict__ y, double ca, double cb) {
  constexpr int N = IDims<P>::N, Q = IDims<P>::Q, R = IDims<P>::R;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const ImplTab<T, P> &tb = itab<T, P>();
  const size_t Kp = a.Kp;
  T c[N], rhs[N];
#pragma unroll
  for (int i = 0; i < N; ++i) { c[i] = x[i * Kp + k]; rhs[i] = T(0); }
  if (RHS) {
    for (int m = 0; m < a.nTerms; ++m) {
      const T gm = T(a.gco[m]);
#pragma unroll
      for (int i = 0; i < N; ++i) rhs[i] = fma(gm, a.rhs[(m * N + i) * Kp + k], rhs[i]);
    }
  }
#pragma unroll 1
  for (int q = 0; q < Q; ++q) {
    T cq = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) cq = fma(tb.phiQ[q][j], c[j], cq);
    const T f1 = a.F[q * Kp + k] * cq, f2 = a.F[(Q + q) * Kp + k] * cq;
#pragma unroll
    for (int i = 0; i < N; ++i) rhs[i] = fma(tb.g2[q][i], f2, fma(tb.g1[q][i], f1, rhs[i]));
  }
  const int code = a.code[k];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const int nb = a.nbr[n * Kp + k];
    const int np = (code >> (2 * n)) & 3;
    const bool outOk = (code >> (6 + n)) & 1;
    T cn[N];
#pragma unroll
    for (int j = 0; j < N; ++j) cn[j] = nb >= 0 ? x[j * Kp + nb] : T(0);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const T v = a.Vn[(n * R + r) * Kp + k];
      T tr = T(0);
      if (v > T(0) && outOk) {
#pragma unroll
        for (int j = 0; j < N; ++j) tr = fma(tb.phi1D[n][r][j], c[j], tr);
      } else if (v < T(0) && nb >= 0) {
        for (int j = 0; j < N; ++j) tr = fma(tb.thetaPhi[n][np & 3][r][j], cn[j], tr);
      }
      const T fl = v * tr;
#pragma unroll
      for (int i = 0; i < N; ++i) rhs[i] = fma(-tb.phi1D[n][r][i], fl, rhs[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) s = fma(tb.hatMinv[i][j], rhs[j], s);
    y[i * Kp + k] = T(ca) * c[i] + T(cb) * s;
  }
}

// Inverse of each element's diagonal block of y = ca x + cb cDot(x) (volume term and the
// element's own outflow; the neighbours' inflow is off-diagonal), by Gauss-Jordan elimination
// with partial pivoting in FP64.  A block with a vanishing pivot is replaced by the identity.
template <typename T, int P>
__global__ void __launch_bounds__(kImplBlock) k_impl_block(const ImplArgs<T> a, double ca, double cb,
                                                           T *__restrict__ Pinv) {
  constexpr int N = IDims<P>::N, Q = IDims<P>::Q, R = IDims<P>::R;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const ImplTab<T, P> &tb = itab<T, P>();
  const size_t Kp = a.Kp;
  double J[N][N];   // J[i][j]: local part of cDot for c = e_j, before the mass solve
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) J[i][j] = 0.0;
  for (int q = 0; q < Q; ++q) {
    const double f1 = (double)a.F[q * Kp + k], f2 = (double)a.F[(Q + q) * Kp + k];
    for (int j = 0; j < N; ++j) {
      const double pj = (double)tb.phiQ[q][j];
#pragma unroll
      for (int i = 0; i < N; ++i) J[i][j] += ((double)tb.g1[q][i] * f1 + (double)tb.g2[q][i] * f2) * pj;
    }
  }
  const int code = a.code[k];
  for (int n = 0; n < 3; ++n) {
    if (!((code >> (6 + n)) & 1)) continue;
    for (int r = 0; r < R; ++r) {
      const double v = (double)a.Vn[(n * R + r) * Kp + k];
      if (!(v > 0.0)) continue;
      for (int j = 0; j < N; ++j) {
        const double pj = (double)tb.phi1D[n][r][j];
#pragma unroll
        for (int i = 0; i < N; ++i) J[i][j] -= (double)tb.phi1D[n][r][i] * v * pj;
      }
    }
  }
  double A[N][2 * N];
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int l = 0; l < N; ++l) s += (double)tb.hatMinv[i][l] * J[l][j];
      A[i][j] = (i == j ? ca : 0.0) + cb * s;
      A[i][N + j] = i == j ? 1.0 : 0.0;
    }
  }
  bool ok = true;
  for (int col = 0; col < N && ok; ++col) {
    int piv = col;
    for (int r = col + 1; r < N; ++r)
      if (fabs(A[r][col]) > fabs(A[piv][col])) piv = r;
    if (!(fabs(A[piv][col]) > 1e-300)) { ok = false; break; }
    if (piv != col)
      for (int j = 0; j < 2 * N; ++j) { const double t = A[col][j]; A[col][j] = A[piv][j]; A[piv][j] = t; }
    const double inv = 1.0 / A[col][col];
    for (int j = 0; j < 2 * N; ++j) A[col][j] *= inv;
    for (int r = 0; r < N; ++r) {
      if (r == col) continue;
      const double f = A[r][col];
      if (f != 0.0)
        for (int j = 0; j < 2 * N; ++j) A[r][j] -= f * A[col][j];
    }
  }
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) Pinv[(i * N + j) * Kp + k] = T(ok ? A[i][N + j] : (i == j ? 1.0 : 0.0));
}

template <typename T, int P>
__global__ void __launch_bounds__(kImplBlock) k_impl_prec(int K, int Kp, const T *__restrict__ Pinv,
                                                          const T *__restrict__ r, T *__restrict__ z) {
  constexpr int N = IDims<P>::N;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  T rv[N];
#pragma unroll
  for (int j = 0; j < N; ++j) rv[j] = r[(size_t)j * Kp + k];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) s = fma(Pinv[(size_t)(i * N + j) * Kp + k], rv[j], s);
    z[(size_t)i * Kp + k] = s;
  }
}

// ---- vector kernels over n = N Kp values ------------------------------------------------------

__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}

// out[v] = sum of nb partials of vector v (one block per vector, fixed order)
__global__ void __launch_bounds__(kVecThreads) k_dot_final(const double *__restrict__ partial, int nb,
                                                           double *__restrict__ out) {
  __shared__ double sh[kVecThreads / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[blockIdx.x * nb + i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// y = sum_v c_v x_v (host coefficients, up to kChunk vectors; y may alias an input)
template <typename T> struct Comb {
  const T *x[kChunk];
  double c[kChunk];
  int nv;
};
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_comb(T *y, const Comb<T> cb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int v = 0; v < kChunk; ++v)
      if (v < cb.nv) s += cb.c[v] * (double)cb.x[v][i];
    y[i] = T(s);
  }
}

// v = w / sqrt(nrm2[0]) (zero if the norm vanishes)
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_unit(T *__restrict__ v, const T *__restrict__ w,
                                                      const double *__restrict__ nrm2, size_t n) {
  const double s = nrm2[0] > 0.0 ? 1.0 / sqrt(nrm2[0]) : 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = T((double)w[i] * s);
}

// partial[v * gridDim.x + b] = block b's share of <V_v, w> for every v < nv, kChunk vectors per
// pass over w
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_mdot_n(const T *__restrict__ V, size_t ldv, int nv,
                                                        const T *__restrict__ w, size_t n, double *__restrict__ partial) {
  __shared__ double sh[kVecThreads / 32];
  for (int v0 = 0; v0 < nv; v0 += kChunk) {
    const int c = min(kChunk, nv - v0);
    double acc[kChunk];
#pragma unroll
    for (int v = 0; v < kChunk; ++v) acc[v] = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
      const double wi = (double)w[i];
#pragma unroll
      for (int v = 0; v < kChunk; ++v)
        if (v < c) acc[v] += (double)V[(size_t)(v0 + v) * ldv + i] * wi;
    }
    for (int v = 0; v < c; ++v) {
      const double s = block_sum(acc[v], sh);
      if (threadIdx.x == 0) partial[(size_t)(v0 + v) * gridDim.x + blockIdx.x] = s;
    }
  }
}

// y = ay y + sgn sum_{v < nv} coef[v] V_v (coefficients in device memory)
template <typename T>
__global__ void __launch_bounds__(kVecThreads) k_vcomb_n(T *__restrict__ y, double ay, const T *__restrict__ V,
                                                         size_t ldv, int nv, const double *__restrict__ coef,
                                                         double sgn, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double s = ay == 0.0 ? 0.0 : ay * (double)y[i];
    for (int v = 0; v < nv; ++v) s += sgn * coef[v] * (double)V[(size_t)v * ldv + i];
    y[i] = T(s);
  }
}

// The small dense part of GMRES, one thread: Hessenberg column j from the two Gram-Schmidt
// passes and |w|^2, the earlier Givens rotations, a new one, and the residual estimate.
// status: [0] |g_{j+1}|, [1] columns in use, [2] breakdown seen (later columns are ignored).
struct GmresDense {
  double *H, *cs, *sn, *g, *y, *status;   // H: (m + 1) x m, column-major
};
__global__ void k_gmres_start(GmresDense d, const double *__restrict__ nrm2, int m) {
  d.g[0] = sqrt(fmax(nrm2[0], 0.0));
  for (int i = 1; i <= m; ++i) d.g[i] = 0.0;
  d.status[0] = d.g[0];
  d.status[1] = 0.0;
  d.status[2] = 0.0;
}
__global__ void k_gmres_column(GmresDense d, const double *__restrict__ h1, const double *__restrict__ h2,
                               const double *__restrict__ nrm2, int j, int m) {
  if (d.status[2] != 0.0) return;
  double *col = d.H + (size_t)j * (m + 1);
  for (int i = 0; i <= j; ++i) col[i] = h1[i] + h2[i];
  col[j + 1] = sqrt(fmax(nrm2[0], 0.0));
  for (int i = 0; i < j; ++i) {
    const double t0 = d.cs[i] * col[i] + d.sn[i] * col[i + 1];
    col[i + 1] = -d.sn[i] * col[i] + d.cs[i] * col[i + 1];
    col[i] = t0;
  }
  const double r = hypot(col[j], col[j + 1]);
  d.cs[j] = r > 0.0 ? col[j] / r : 1.0;
  d.sn[j] = r > 0.0 ? col[j + 1] / r : 0.0;
  col[j] = r;
  col[j + 1] = 0.0;
  d.g[j + 1] = -d.sn[j] * d.g[j];
  d.g[j] = d.cs[j] * d.g[j];
  d.status[0] = fabs(d.g[j + 1]);
  d.status[1] = (double)(j + 1);
  if (r == 0.0) d.status[2] = 1.0;
}
// y = H^-1 g over the columns in use (upper triangular), zero beyond them.
__global__ void k_gmres_solve(GmresDense d, int m) {
  const int je = (int)d.status[1];
  for (int i = m - 1; i >= je; --i) d.y[i] = 0.0;
  for (int i = je - 1; i >= 0; --i) {
    double s = d.g[i];
    for (int l = i + 1; l < je; ++l) s -= d.H[(size_t)l * (m + 1) + i] * d.y[l];
    const double diag = d.H[(size_t)i * (m + 1) + i];
    d.y[i] = diag != 0.0 ? s / diag : 0.0;
  }
}

double time_factor_of(int fn, double t) { return fn == DGADV_TIME_EXP_NEG ? std::exp(-t) : 1.0; }

// DIRK tables (core/rungeKuttaImplicit.m); returns the number of stages.
int dirk_table(int ord, double a[5][5]) {
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) a[i][j] = 0.0;
  switch (ord) {
    case 1: a[0][0] = 1.0; return 1;
    case 2: {
      const double l = 0.5 * (2.0 - std::sqrt(2.0));
      a[0][0] = l; a[1][0] = 1.0 - l; a[1][1] = l;
      return 2;
    }
    case 3: {
      const double al = 0.4358665215084589994160194511935568425292;
      const double be = 0.5 * (1. + al);
      const double b1 = -0.25 * (6 * al * al - 16 * al + 1);
      const double b2 = 0.25 * (6 * al * al - 20 * al + 5);
      a[0][0] = al; a[1][0] = be - al; a[1][1] = al; a[2][0] = b1; a[2][1] = b2; a[2][2] = al;
      return 3;
    }
    case 4: {
      const double g = 1. / 4.;
      const double t[5][5] = {{g, 0, 0, 0, 0},
                              {1. / 2., g, 0, 0, 0},
                              {17. / 50., -1. / 25., g, 0, 0},
                              {371. / 1360., -137. / 2720., 15. / 544., g, 0},
                              {25. / 24., -49. / 48., 125. / 16., -85. / 12., g}};
      for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) a[i][j] = t[i][j];
      return 5;
    }
  }
  return 0;
}

}  // namespace

// Solver state of a handle: Krylov basis, work vectors, preconditioner, scratch.
struct ImplicitState {
  int m = 0;                      // restart length
  size_t n = 0;                   // N * Kp
  void *V = nullptr;              // (m + 1) x n
  void *w = nullptr, *z = nullptr, *r = nullptr, *x = nullptr, *b = nullptr, *zero = nullptr, *s = nullptr;
  void *kst = nullptr;            // 4 x n stage derivatives
  void *Pinv = nullptr;           // N^2 x Kp
  double pinvA = 0.0, pinvB = 0.0;
  int pinvVersion = -1;           // velocity version the blocks were built for
  double *partial = nullptr;      // kChunk x kMaxDotBlocks
  double *dres = nullptr;         // 3 x (m + 2): h1, h2, |w|^2
  double *dcoef = nullptr;        // m + 1 coefficients
  double *dense = nullptr;        // H ((m + 1) x m), cs, sn, g, y, status
  std::vector<cudaGraphExec_t> arnoldi;   // Arnoldi step j as a CUDA graph, for (graphA, graphB)
  double graphA = 0.0, graphB = 0.0;
  double *hres = nullptr;         // pinned mirror of dres
  bool tablesLoaded = false;
};

void implicit_release(dgadv_handle *h) {
  ImplicitState *st = h->impl;
  if (!st) return;
  for (cudaGraphExec_t g : st->arnoldi)
    if (g) cudaGraphExecDestroy(g);
  if (st->hres) cudaFreeHost(st->hres);
  delete st;   // device buffers belong to h->allocs
  h->impl = nullptr;
}

namespace {

template <typename T, int P>
cudaError_t upload_itab(const RefTables &rt, cudaStream_t stream) {
  using I = IDims<P>;
  static ImplTab<T, P> t;   // host staging (the async copy reads it later on the stream)
  if (rt.Q != I::Q || rt.R != I::R || rt.N != I::N) return cudaErrorInvalidValue;
  for (int q = 0; q < I::Q; ++q)
    for (int i = 0; i < I::N; ++i) {
      t.phiQ[q][i] = T(rt.phiQ[q * I::N + i]);
      t.g1[q][i] = T(rt.gradQ[q * I::N + i]);
      t.g2[q][i] = T(rt.gradQ[I::Q * I::N + q * I::N + i]);
    }
  for (int n = 0; n < 3; ++n)
    for (int r = 0; r < I::R; ++r)
      for (int i = 0; i < I::N; ++i) {
        t.phi1D[n][r][i] = T(rt.phi1D[(n * I::R + r) * I::N + i]);
        for (int np = 0; np < 3; ++np)
          t.thetaPhi[n][np][r][i] = T(rt.thetaPhi[((n * 3 + np) * I::R + r) * I::N + i]);
      }
  for (int i = 0; i < I::N; ++i)
    for (int j = 0; j < I::N; ++j) t.hatMinv[i][j] = T(rt.hatMinv[i * I::N + j]);
  const cudaError_t e = cudaMemcpyToSymbolAsync(itab_symbol<T, P>(), &t, sizeof(t), 0, cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(stream);
}

template <typename T, int P>
struct Solver {
  dgadv_handle *h;
  ImplicitState *st;
  ImplArgs<T> args;
  size_t n;
  int gridK, gridV, nbD;

  explicit Solver(dgadv_handle *hh) : h(hh), st(hh->impl) {
    n = st->n;
    args = ImplArgs<T>{};
    args.K = h->K; args.Kp = h->Kp; args.nTerms = h->nTerms;
    args.F = (const T *)h->F; args.Vn = (const T *)h->Vn; args.rhs = (const T *)h->rhs;
    args.nbr = h->nbr; args.code = h->code;
    gridK = (h->K + kElemThreads - 1) / kElemThreads;
    gridV = (int)std::min<size_t>((n + kVecThreads - 1) / kVecThreads, 4 * 152);
    nbD = (int)std::min<size_t>((n + kVecThreads - 1) / kVecThreads, kMaxDotBlocks);
  }
  T *vec(void *p) const { return (T *)p; }
  T *basis(int j) const { return (T *)st->V + (size_t)j * n; }

  // y = ca x + cb cDot(x; t) (sources if withRhs)
  void op(const T *x, T *y, double ca, double cb, bool withRhs, double t) {
    ImplArgs<T> a = args;
    const bool rhs = withRhs && h->nTerms > 0 && h->rhs;
    for (int m = 0; m < h->nTerms; ++m) a.gco[m] = time_factor_of(h->timeFn[m], t);
    if (rhs) k_impl_op<T, P, true><<<gridK, kElemThreads, 0, h->stream>>>(a, x, y, ca, cb);
    else k_impl_op<T, P, false><<<gridK, kElemThreads, 0, h->stream>>>(a, x, y, ca, cb);
  }
  void prec(const T *r, T *z) {
    k_impl_prec<T, P><<<gridK, kElemThreads, 0, h->stream>>>(h->K, h->Kp, (const T *)st->Pinv, r, z);
  }
  void build_prec(double ca, double cb) {
    if (st->pinvVersion == h->velVersion && st->pinvA == ca && st->pinvB == cb) return;
    k_impl_block<T, P><<<gridK, kElemThreads, 0, h->stream>>>(args, ca, cb, (T *)st->Pinv);
    st->pinvA = ca; st->pinvB = cb; st->pinvVersion = h->velVersion;
  }
  // dres[off + v] = <V_v, w> for v < nv (V: nv vectors of stride n)
  void mdot(const T *V, int nv, const T *w, int off) {
    k_mdot_n<T><<<nbD, kVecThreads, 0, h->stream>>>(V, n, nv, w, n, st->partial);
    k_dot_final<<<nv, kVecThreads, 0, h->stream>>>(st->partial, nbD, st->dres + off);
  }
  // y = ay y + sgn V coef (coef in device memory)
  void vcomb(T *y, double ay, const T *V, int nv, const double *coef, double sgn) {
    if (nv > 0) k_vcomb_n<T><<<gridV, kVecThreads, 0, h->stream>>>(y, ay, V, n, nv, coef, sgn, n);
  }
  void comb(T *y, std::initializer_list<std::pair<const T *, double>> terms) {
    Comb<T> cb{};
    cb.nv = 0;
    for (const auto &t : terms) { cb.x[cb.nv] = t.first; cb.c[cb.nv] = t.second; ++cb.nv; }
    k_comb<T><<<gridV, kVecThreads, 0, h->stream>>>(y, cb, n);
  }
  void comb(T *y, const Comb<T> &cb) { k_comb<T><<<gridV, kVecThreads, 0, h->stream>>>(y, cb, n); }
  double norm2(const T *w) {
    mdot(w, 1, w, 0);
    cudaMemcpyAsync(st->hres, st->dres, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    cudaStreamSynchronize(h->stream);
    return st->hres[0];
  }

  // Arnoldi step j: w = A P^-1 v_j, orthogonalised against v_0..v_j (classical Gram-Schmidt,
  // twice), v_{j+1} = w / |w|, and the dense update of column j.
  void arnoldi_enqueue(int j, double ca, double cb, const GmresDense &d) {
    const int m = st->m;
    T *w = vec(st->w), *z = vec(st->z);
    double *h1 = st->dres, *h2 = st->dres + (m + 1), *nw = st->dres + 2 * (m + 1);
    prec(basis(j), z);
    op(z, w, ca, cb, false, 0.0);
    mdot(basis(0), j + 1, w, 0);
    vcomb(w, 1.0, basis(0), j + 1, h1, -1.0);
    mdot(basis(0), j + 1, w, m + 1);
    vcomb(w, 1.0, basis(0), j + 1, h2, -1.0);
    mdot(w, 1, w, 2 * (m + 1));
    k_unit<T><<<gridV, kVecThreads, 0, h->stream>>>(basis(j + 1), w, nw, n);
    k_gmres_column<<<1, 1, 0, h->stream>>>(d, h1, h2, nw, j, m);
  }
  // The step as a CUDA graph, captured once per j and operator (all its buffers are the
  // handle's own; the operator's coefficients are baked in).
  int arnoldi_step(int j, double ca, double cb, const GmresDense &d) {
    if (h->flags & DGADV_FLAG_NO_GRAPH) {
      arnoldi_enqueue(j, ca, cb, d);
      return DGADV_OK;
    }
    if (st->graphA != ca || st->graphB != cb || (int)st->arnoldi.size() != st->m) {
      for (cudaGraphExec_t g : st->arnoldi)
        if (g) cudaGraphExecDestroy(g);
      st->arnoldi.assign(st->m, nullptr);
      st->graphA = ca;
      st->graphB = cb;
    }
    if (!st->arnoldi[j]) {
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return DGADV_ECUDA;
      arnoldi_enqueue(j, ca, cb, d);
      if (cudaStreamEndCapture(h->stream, &g) != cudaSuccess) return DGADV_ECUDA;
      const cudaError_t e = cudaGraphInstantiate(&st->arnoldi[j], g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return DGADV_ECUDA;
    }
    return cudaGraphLaunch(st->arnoldi[j], h->stream) == cudaSuccess ? DGADV_OK : DGADV_ECUDA;
  }

  // Solves (ca I + cb cDot0) x = b, x holding the initial guess; right block-Jacobi
  // preconditioning.  The Hessenberg column, the Givens rotations and the small triangular
  // solve run on the device; the host reads the residual estimate every kCheck iterations
  // (a few iterations past convergence only improve the iterate).  Returns DGADV_OK or
  // DGADV_ENOCONV; iters accumulates iterations.
  int gmres(const T *b, T *x, double ca, double cb, double tol, int maxIter, int &iters, double &relres) {
    constexpr int kCheck = 4;
    const int m = st->m;
    build_prec(ca, cb);
    T *w = vec(st->w), *z = vec(st->z), *r = vec(st->r);
    const double bnorm = std::sqrt(norm2(b));
    if (bnorm == 0.0) {
      cudaMemsetAsync(x, 0, n * sizeof(T), h->stream);
      relres = 0.0;
      return DGADV_OK;
    }
    GmresDense d;
    d.H = st->dense;
    d.cs = d.H + (size_t)(m + 1) * m;
    d.sn = d.cs + m;
    d.g = d.sn + m;
    d.y = d.g + (m + 1);
    d.status = d.y + m;
    int used = 0;
    for (;;) {
      op(x, w, ca, cb, false, 0.0);
      comb(r, {{b, 1.0}, {w, -1.0}});
      const double beta = std::sqrt(norm2(r));
      relres = beta / bnorm;
      if (relres <= tol) return DGADV_OK;
      if (used >= maxIter) return DGADV_ENOCONV;
      k_unit<T><<<gridV, kVecThreads, 0, h->stream>>>(basis(0), r, st->dres, n);
      k_gmres_start<<<1, 1, 0, h->stream>>>(d, st->dres, m);
      int j = 0;
      while (j < m && used < maxIter) {
        ++used;
        ++iters;
        if (int e = arnoldi_step(j, ca, cb, d)) return e;
        ++j;
        if (j % kCheck == 0 || j == m || used >= maxIter) {
          cudaMemcpyAsync(st->hres, d.status, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
          if (cudaStreamSynchronize(h->stream) != cudaSuccess) return DGADV_ECUDA;
          relres = st->hres[0] / bnorm;
          if (relres <= tol || st->hres[2] != 0.0) break;
        }
      }
      // x += P^-1 V y with y = H^-1 g over the columns in use
      k_gmres_solve<<<1, 1, 0, h->stream>>>(d, m);
      vcomb(r, 0.0, basis(0), j, d.y, 1.0);
      prec(r, z);
      comb(x, {{x, 1.0}, {z, 1.0}});
    }
  }

  int dirk_steps(int nSteps, int nStep0, double tau, int ord, double tol, int maxIter, int &iters,
                 double &worst) {
    double a[5][5];
    const int S = dirk_table(ord, a);
    if (!S) { h->err = "DIRK order must be 1..4"; return DGADV_EINVAL; }
    T *cn = (T *)h->cn, *x = vec(st->x), *rhs = vec(st->b), *s = vec(st->s);
    const T *zero = vec(st->zero);
    worst = 0.0;
    for (int nn = 0; nn < nSteps; ++nn) {
      const double t0 = (double)(nStep0 + nn) * tau;
      cudaMemcpyAsync(x, cn, n * sizeof(T), cudaMemcpyDeviceToDevice, h->stream);
      for (int i = 0; i < S; ++i) {
        double ci = 0.0;
        for (int j = 0; j <= i; ++j) ci += a[i][j];
        const double ti = t0 + ci * tau, gam = tau * a[i][i];
        op(zero, s, 0.0, 1.0, true, ti);                 // s_i = M^-1 sysV(t_i)
        Comb<T> cb{};
        cb.nv = 0;
        cb.x[cb.nv] = cn; cb.c[cb.nv++] = 1.0;
        for (int j = 0; j < i; ++j) { cb.x[cb.nv] = (const T *)st->kst + (size_t)j * n; cb.c[cb.nv++] = tau * a[i][j]; }
        cb.x[cb.nv] = s; cb.c[cb.nv++] = gam;
        comb(rhs, cb);
        double rr = 0.0;
        const int e = gmres(rhs, x, 1.0, -gam, tol, maxIter, iters, rr);
        worst = std::max(worst, rr);
        if (e) return e;
        if (i + 1 < S) op(x, (T *)st->kst + (size_t)i * n, 0.0, 1.0, true, ti);   // k_i
      }
      cudaMemcpyAsync(cn, x, n * sizeof(T), cudaMemcpyDeviceToDevice, h->stream);
    }
    return cudaStreamSynchronize(h->stream) == cudaSuccess ? DGADV_OK : DGADV_ECUDA;
  }

  int stationary(double tol, int maxIter, int &iters, double &res) {
    T *cn = (T *)h->cn, *s = vec(st->s);
    op(vec(st->zero), s, 0.0, 1.0, true, 0.0);         // M^-1 sysV
    const int e = gmres(s, cn, 0.0, -1.0, tol, maxIter, iters, res);   // M^-1 A x = M^-1 sysV
    if (e) return e;
    return cudaStreamSynchronize(h->stream) == cudaSuccess ? DGADV_OK : DGADV_ECUDA;
  }
};

int ensure_state(dgadv_handle *h, int restart) {
  if (h->impl && h->impl->m >= restart) return DGADV_OK;
  if (h->impl) {   // a longer restart: the basis is reallocated, the old buffers stay with the handle
    cudaStreamSynchronize(h->stream);
    implicit_release(h);
  }
  ImplicitState *st = new (std::nothrow) ImplicitState();
  if (!st) return DGADV_ENOMEM;
  h->impl = st;
  const size_t rb = ops_of(h).realBytes;
  st->m = restart;
  st->n = (size_t)h->N * h->Kp;
  const size_t vb = st->n * rb;
  void **bufs[] = {&st->w, &st->z, &st->r, &st->x, &st->b, &st->zero, &st->s};
  int e;
  if ((e = dev_alloc(h, &st->V, (size_t)(restart + 1) * vb))) return e;
  for (void **b : bufs)
    if ((e = dev_alloc(h, b, vb))) return e;
  if ((e = dev_alloc(h, &st->kst, 4 * vb))) return e;
  if ((e = dev_alloc(h, &st->Pinv, (size_t)h->N * h->N * h->Kp * rb))) return e;
  if ((e = dev_alloc(h, (void **)&st->partial, (size_t)(restart + 2) * kMaxDotBlocks * 8))) return e;
  if ((e = dev_alloc(h, (void **)&st->dres, (size_t)3 * (restart + 1) * 8))) return e;
  if ((e = dev_alloc(h, (void **)&st->dcoef, (size_t)(restart + 1) * 8))) return e;
  if ((e = dev_alloc(h, (void **)&st->dense, ((size_t)(restart + 1) * restart + 4 * (size_t)restart + 8) * 8))) return e;
  DG_CUDA(cudaMallocHost((void **)&st->hres, (size_t)3 * (restart + 1) * 8));
  DG_CUDA(cudaMemsetAsync(st->V, 0, (size_t)(restart + 1) * vb, h->stream));
  for (void **b : bufs) DG_CUDA(cudaMemsetAsync(*b, 0, vb, h->stream));
  DG_CUDA(cudaMemsetAsync(st->kst, 0, 4 * vb, h->stream));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  return DGADV_OK;
}

template <typename T, int P>
int load_tables(dgadv_handle *h) {
  if (h->impl->tablesLoaded) return DGADV_OK;
  const cudaError_t e = upload_itab<T, P>(h->tables, h->stream);
  if (e != cudaSuccess) { h->err = std::string("implicit tables: ") + cudaGetErrorString(e); return DGADV_ECUDA; }
  h->impl->tablesLoaded = true;
  return DGADV_OK;
}

int check_handle(dgadv_handle *h) {
  if (!(h->flags & DGADV_FLAG_IMPLICIT)) {
    h->err = "implicit steps need a handle created with DGADV_FLAG_IMPLICIT";
    return DGADV_EINVAL;
  }
  if (h->prec == DGADV_DF32) { h->err = "implicit steps run in FP64 or FP32"; return DGADV_EUNSUPPORTED; }
  if (!h->hasVelocity) { h->err = "no velocity data"; return DGADV_EINVAL; }
  return DGADV_OK;
}

template <typename T, int P>
int run(dgadv_handle *h, int what, int nSteps, int nStep0, double tau, int ord, double tol, int maxIter,
        int32_t *iters, double *res) {
  if (int e = load_tables<T, P>(h)) return e;
  Solver<T, P> s(h);
  int it = 0;
  double rr = 0.0;
  int e = what == 0 ? s.dirk_steps(nSteps, nStep0, tau, ord, tol, maxIter, it, rr) : s.stationary(tol, maxIter, it, rr);
  if (iters) *iters = it;
  if (res) *res = rr;
  if (e == DGADV_ENOCONV) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "GMRES stopped at relative residual %.3e after %d iterations", rr, it);
    h->err = buf;
  } else if (e == DGADV_ECUDA) {
    h->err = std::string("implicit solve: ") + cudaGetErrorString(cudaGetLastError());
  }
  return e;
}

template <typename T>
int run_t(dgadv_handle *h, int what, int nSteps, int nStep0, double tau, int ord, double tol, int maxIter,
          int32_t *iters, double *res) {
  switch (h->p) {
    case 0: return run<T, 0>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
    case 1: return run<T, 1>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
    case 2: return run<T, 2>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
    case 3: return run<T, 3>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
  }
  return DGADV_EUNSUPPORTED;
}

int dispatch(dgadv_handle *h, int what, int nSteps, int nStep0, double tau, int ord, double tol, int maxIter,
             int restart, int32_t *iters, double *res) {
  if (int e = check_handle(h)) return e;
  if (!(tol > 0.0) || maxIter < 1 || restart < 1 || restart > 256) return DGADV_EINVAL;
  if (int e = ensure_state(h, restart)) return e;
  if (h->prec == DGADV_FP64) return run_t<double>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
  return run_t<float>(h, what, nSteps, nStep0, tau, ord, tol, maxIter, iters, res);
}

}  // namespace
}  // namespace dgadv

using namespace dgadv;

extern "C" int dgadv_step_implicit(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau, int32_t ordRK,
                                   const dgadv_krylov *kr, int32_t *iters, double *relres) {
  return guarded(h, [&]() -> int {
  if (!h || nSteps < 0 || !(tau > 0.0) || ordRK < 1 || ordRK > 4) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const dgadv_krylov d = kr ? *kr : dgadv_krylov{1e-12, 2000, 50};
  if (nSteps == 0) return DGADV_OK;
  return dispatch(h, 0, nSteps, nStep0, tau, ordRK, d.tol, d.maxIter, d.restart, iters, relres);
  });
}

extern "C" int dgadv_solve_stationary(dgadv_handle *h, const dgadv_krylov *kr, int32_t *iters, double *relres) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const dgadv_krylov d = kr ? *kr : dgadv_krylov{1e-12, 2000, 50};
  return dispatch(h, 1, 0, 0, 1.0, 1, d.tol, d.maxIter, d.restart, iters, relres);
  });
}
