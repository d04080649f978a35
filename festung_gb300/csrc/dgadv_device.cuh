// Device solver of the explicit DG advection step and its C-ABI entry points.
//
// Per-stage operator (advection/preprocessSubStep.m:56-99 + advection/solveSubStep.m:57-99),
// matrix-free and element-centric:
//   volume  (G1+G2)c |_{k,i} = sum_q c(x_q) [d1 phi_i (B22 u1 - B12 u2) + d2 phi_i (B11 u2 - B21 u1)] W_q
//           (core/assembleMatElemDphiPhiFuncDisc.m:181-202; same rule of order 2p as hatG)
//   flux    (R c)_{k,i} = sum_n |E_kn| sum_r w_r v_knr phi_i(g_n(q_r)) * (v>0 ? c_k : c_k+) traces
//           (core/assembleMatEdgePhiPhiValUpwind.m:261-299: the upwind side is gathered through
//           the neighbour map, so every element writes only its own rows: no atomics)
//   mass    cDot = hatM^-1 rhs / detJ (FP64; the FP32 path uses hatM = I, |hatM - I| < 2e-14)
//   SSP     c^(s) = w_s c^n + (1-w_s)(c^(s-1) + tau cDot)          advection/solveSubStep.m:83
// Limiter: core/applySlopeLimiterTaylor*.m with patch min/max over CSR vertex patches
// (core/computeMinMaxV0TElementPatch.m:66-112) and the Taylor transform in closed form
// (Taylor coefficients = mean and scaled derivatives at the barycentre).
//
// This header holds every kernel, templated on the stored real type T (double, float or the
// double-float df32).  A translation unit that includes it defines the constant tables of its
// T and the tab<T, P>() accessors (DGADV_DEFINE_TABLES) before instantiating kernels, so that
// the kernels of each arithmetic type compile in a unit of their own.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "dgadv_handle.h"
#include "dgadv_kernels.cuh"
#include "dgadv_df32.cuh"

namespace dgadv {

// Constant tables of one (type, degree): defined by the including unit.
template <typename T, int P> __device__ __forceinline__ const Tab<T, P> &tab();
namespace {
template <typename T, int P> const void *tab_symbol();   // host address of the unit's table
}  // namespace

#define DGADV_DEFINE_TABLES(T, NAME)                                                            \
  static __constant__ Tab<T, 0> NAME##0;                                                        \
  static __constant__ Tab<T, 1> NAME##1;                                                        \
  static __constant__ Tab<T, 2> NAME##2;                                                        \
  static __constant__ Tab<T, 3> NAME##3;                                                        \
  template <> __device__ __forceinline__ const Tab<T, 0> &tab<T, 0>() { return NAME##0; }       \
  template <> __device__ __forceinline__ const Tab<T, 1> &tab<T, 1>() { return NAME##1; }       \
  template <> __device__ __forceinline__ const Tab<T, 2> &tab<T, 2>() { return NAME##2; }       \
  template <> __device__ __forceinline__ const Tab<T, 3> &tab<T, 3>() { return NAME##3; }       \
  namespace {                                                                                   \
  template <> [[maybe_unused]] const void *tab_symbol<T, 0>() { return (const void *)&NAME##0; }  \
  template <> [[maybe_unused]] const void *tab_symbol<T, 1>() { return (const void *)&NAME##1; }  \
  template <> [[maybe_unused]] const void *tab_symbol<T, 2>() { return (const void *)&NAME##2; }  \
  template <> [[maybe_unused]] const void *tab_symbol<T, 3>() { return (const void *)&NAME##3; }  \
  }

// ---------------------------------------------------------------------------------------------
// Ordered integer keys: atomicMin/atomicMax on the key order like on the real numbers.
__device__ __forceinline__ unsigned long long okey(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ULL);
}
__device__ __forceinline__ unsigned long long okey(float x) {
  const unsigned int u = __float_as_uint(x);
  return (unsigned long long)((u >> 31) ? ~u : (u | 0x80000000u));
}
template <typename T> __device__ __forceinline__ T okey_inv(unsigned long long k);
template <> __device__ __forceinline__ double okey_inv<double>(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFULL) : ~k;
  return __longlong_as_double((long long)u);
}
template <> __device__ __forceinline__ float okey_inv<float>(unsigned long long k) {
  const unsigned int kk = (unsigned int)k;
  const unsigned int u = (kk >> 31) ? (kk & 0x7FFFFFFFu) : ~kk;
  return __uint_as_float(u);
}
template <typename T> __host__ __device__ constexpr unsigned long long key_max();
template <> __host__ __device__ constexpr unsigned long long key_max<double>() { return ~0ULL; }
template <> __host__ __device__ constexpr unsigned long long key_max<float>() { return 0xFFFFFFFFULL; }

__device__ __forceinline__ bool finite_(double x) { return isfinite(x); }
__device__ __forceinline__ bool finite_(float x) { return isfinite(x); }

// df32: the key of hi in the high half and the key of lo in the low half orders pairs like
// their (hi, lo) lexicographic order, which is the order of the values for normalised pairs;
// the key is exact and invertible.
__device__ __forceinline__ unsigned long long okey(const df32 &x) {
  return (okey(x.hi) << 32) | okey(x.lo);
}
template <> __device__ __forceinline__ df32 okey_inv<df32>(unsigned long long k) {
  return df32(okey_inv<float>(k >> 32), okey_inv<float>(k & 0xFFFFFFFFULL));
}
template <> __host__ __device__ constexpr unsigned long long key_max<df32>() { return ~0ULL; }
__device__ __forceinline__ bool finite_(const df32 &x) { return isfinite(x.hi) && isfinite(x.lo); }

// A stored real in an arithmetic type A: itself, or a double-float's head in FP32 (|lo| is at
// most half an FP32 unit of hi).
template <typename A, typename T> __device__ __forceinline__ A as_arith(const T &x) {
  if constexpr (std::is_same_v<A, T>) return x;
  else return x.hi;
}

// ---------------------------------------------------------------------------------------------
// Sum of products s = s0 + sum a_k b_k.  float / double: the plain multiply-add s += a b.  df32:
// the running sum is an FP32 head, advanced by one exact two_sum per term, and an FP32 tail that
// collects the head's rounding errors and the products' low parts; one two_sum normalises the
// pair at the end.  That is about 13 FP32 instructions per term instead of a double-word
// product plus a double-word addition (about 28), at an error of order n u^2 sum |a_k b_k|.
template <typename T> struct Acc {
  T s;
  Acc() = default;
  __device__ __forceinline__ explicit Acc(const T &s0) : s(s0) {}
  __device__ __forceinline__ void fma(const T &a, const T &b) { s += a * b; }
  __device__ __forceinline__ void fms(const T &a, const T &b) { s -= a * b; }
  __device__ __forceinline__ T get() const { return s; }
};
template <> struct Acc<df32> {
  float hi, lo;
  Acc() = default;
  __device__ __forceinline__ explicit Acc(const df32 &s0) : hi(s0.hi), lo(s0.lo) {}
  __device__ __forceinline__ void fma(const df32 &a, const df32 &b) {
    float p, e, t;
    df::two_prod(a.hi, b.hi, p, e);
    e = fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, e));
    df::two_sum(hi, p, hi, t);
    lo += t + e;
  }
  __device__ __forceinline__ void fms(const df32 &a, const df32 &b) { fma(-a, b); }
  __device__ __forceinline__ df32 get() const {
    float h, l;
    df::two_sum(hi, lo, h, l);
    return df32(h, l);
  }
};

// ---------------------------------------------------------------------------------------------
// Element geometry for the Taylor transform.
template <typename T> struct Affine {
  T B11, B12, B21, B22;   // B(:,m,n): m = coordinate, n = column
  T A11, A12, A21, A22;   // A = B^-1
  T dX, idX;              // dX = 2 / sqrt(detJ)
  T ox[3], oy[3];         // vertex offsets from the barycentre
};

template <typename T> __device__ __forceinline__ Affine<T> load_affine(const Geo<T> &g, int k) {
  Affine<T> a;
  a.B11 = g.Bm[k]; a.B12 = g.Bm[g.Kp + k]; a.B21 = g.Bm[2 * g.Kp + k]; a.B22 = g.Bm[3 * g.Kp + k];
  const T det = a.B11 * a.B22 - a.B12 * a.B21;
  const T idet = T(1) / det;
  a.A11 = a.B22 * idet; a.A12 = -a.B12 * idet; a.A21 = -a.B21 * idet; a.A22 = a.B11 * idet;
  a.dX = T(2) / sqrt(det);
  a.idX = T(1) / a.dX;
  const T bx = -(a.B11 + a.B12) / T(3), by = -(a.B21 + a.B22) / T(3);
  a.ox[0] = bx; a.oy[0] = by;
  a.ox[1] = a.B11 + bx; a.oy[1] = a.B21 + by;
  a.ox[2] = a.B12 + bx; a.oy[2] = a.B22 + by;
  return a;
}

// Coefficients of (a + b z)^(D-m) (c + e z)^m in z^j, for m, j = 0..D.
template <typename T, int D>
__device__ __forceinline__ void deriv_block(T a, T b, T c, T e, T S[D + 1][D + 1]) {
#pragma unroll
  for (int m = 0; m <= D; ++m) {
    T poly[D + 1];
#pragma unroll
    for (int j = 0; j <= D; ++j) poly[j] = (j == 0) ? T(1) : T(0);
#pragma unroll
    for (int r = 0; r < D; ++r) {
      const bool first = r < D - m;
      const T x0 = first ? a : c, x1 = first ? b : e;
#pragma unroll
      for (int j = D; j >= 0; --j) poly[j] = poly[j] * x0 + (j > 0 ? poly[j - 1] * x1 : T(0));
    }
#pragma unroll
    for (int j = 0; j <= D; ++j) S[m][j] = poly[j];
  }
}

// modal c -> Taylor coefficients cT (core/projectDataDisc2DataTaylor.m:56-61 in closed form)
template <typename T, int P>
__device__ __forceinline__ void to_taylor(const T *c, const Affine<T> &af, T *cT) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T u[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) s.fma(tb.DM[i][j], c[j]);
    u[i] = s.get();
  }
  cT[0] = u[0];
  T sc = T(1);
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    sc *= af.idX;
    const int off = d * (d + 1) / 2;
    if (d == 1) {
      T S[2][2]; deriv_block<T, 1>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 1; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 1; ++j) s += S[m][j] * u[off + j]; cT[off + m] = s * sc; }
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 2; ++j) s += S[m][j] * u[off + j]; cT[off + m] = s * sc; }
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 3; ++j) s += S[m][j] * u[off + j]; cT[off + m] = s * sc; }
    }
  }
}

// Taylor coefficients -> modal (core/projectDataTaylor2DataDisc.m:56-61 in closed form)
template <typename T, int P>
__device__ __forceinline__ void from_taylor(const T *cT, const Affine<T> &af, T *c) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T w[N];
  w[0] = cT[0];
  T sc = T(1);
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    sc *= af.dX;
    const int off = d * (d + 1) / 2;
    if (d == 1) {
      T S[2][2]; deriv_block<T, 1>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 1; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 1; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 2; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m) { T s = T(0);
#pragma unroll
        for (int j = 0; j <= 3; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) s.fma(tb.DMinv[i][j], w[j]);
    c[i] = s.get();
  }
}

// Blocks of S^-1 (Taylor coefficients -> reference derivatives at the barycentre) per degree d:
// Si[d][m][j] = dX^d times the coefficient of z^j in (B11 + B21 z)^(d-m) (B12 + B22 z)^m, the
// map from_taylor applies (block 0 is 1).
template <typename T, int P> struct SinvBlocks {
  T b[P + 1][P + 1][P + 1];
};
template <typename T, int P>
__device__ __forceinline__ void sinv_blocks(const Affine<T> &af, SinvBlocks<T, P> &si) {
  si.b[0][0][0] = T(1);
  T sc = T(1);
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    sc *= af.dX;
    if (d == 1) {
      T S[2][2]; deriv_block<T, 1>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 1; ++m)
#pragma unroll
        for (int j = 0; j <= 1; ++j) si.b[1][m][j] = S[m][j] * sc;
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m)
#pragma unroll
        for (int j = 0; j <= 2; ++j) si.b[2][m][j] = S[m][j] * sc;
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m)
#pragma unroll
        for (int j = 0; j <= 3; ++j) si.b[3][m][j] = S[m][j] * sc;
    }
  }
}

// Taylor mass correction without a stored mass block (advection/solveSubStep.m:69-80 with
// Mcorr = diag(1/diag(M_T)) M_T, advection/preprocessProblem.m:107-111).  With u = DM c the
// reference derivatives and S the map u -> Taylor coefficients, an element's Taylor mass block
// is M_T = 2|T| S^-T Gr S^-1 (Gr = DM^-T hatM DM^-1, a constant table).  For a Taylor-space
// difference d given as y = S^-1 d (y_0 = 0), this returns
//     m = Mcorr d = diag(D)^-1 S^-T Gr y,   D_i = (S^-T Gr S^-1)_ii,
// the factor 2|T| cancelling.  S^-1 is block diagonal per degree, so D_i involves only the
// diagonal block of Gr of its degree.
template <typename T, int P>
__device__ __forceinline__ void taylor_mcorr(const SinvBlocks<T, P> &si, const T *y, T *m) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T gy[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 1; j < N; ++j) s.fma(tb.Gr[i][j], y[j]);
    gy[i] = s.get();
  }
  m[0] = gy[0] / tb.Gr[0][0];
#pragma unroll
  for (int d = 1; d <= P; ++d) {
    const int off = d * (d + 1) / 2;
#pragma unroll
    for (int j = 0; j <= d; ++j) {
      Acc<T> t(T(0)), D(T(0));
#pragma unroll
      for (int a = 0; a <= d; ++a) {
        t.fma(si.b[d][a][j], gy[off + a]);
        Acc<T> r(T(0));
#pragma unroll
        for (int b = 0; b <= d; ++b) r.fma(tb.Gr[off + a][off + b], si.b[d][b][j]);
        D.fma(si.b[d][a][j], r.get());
      }
      m[off + j] = t.get() / D.get();
    }
  }
}

// Index of the Taylor DOF with multi-index (a1, a2) (core/mult2ind.m:57-62, 0-based).
__host__ __device__ constexpr int mind(int a1, int a2) { return (a1 + a2) * (a1 + a2 + 1) / 2 + a2; }

template <int P> struct NCQ { static constexpr int value = P * (P + 1) / 2 > 1 ? P * (P + 1) / 2 : 1; };

// Centroid quantities of the sub-limiters (one per computeVertexBasedLimiter call).
template <typename T, int P>
__device__ __forceinline__ void centroid_quantities(const T *cT, int type, T *qv) {
  if (type == 0) {
    qv[0] = cT[0];
  } else {
    int s = 0;
#pragma unroll
    for (int ord = P; ord >= 1; --ord)
#pragma unroll
      for (int i = 1; i <= ord; ++i) { qv[s] = cT[mind(ord - i, i - 1)]; ++s; }
  }
}

// Limiter pass plumbing.  Pass j scatters its centroid quantities into per-vertex min / max
// slots vkeys[j%3] with atomicMin / atomicMax on order-preserving integer keys (each element
// updates its three vertices: the patch of a vertex is exactly the elements that update it,
// core/computeMinMaxV0TElementPatch.m:99-111), and the global extremes (for the reference's
// shift) into slots[j%3].  The producer of pass j resets the slots of pass j+1; three sets keep
// the kernel that consumes pass j and produces pass j+1 clear of both.
template <typename T> struct KeyOf { using type = unsigned int; };
template <> struct KeyOf<double> { using type = unsigned long long; };
template <> struct KeyOf<df32> { using type = unsigned long long; };

__device__ __forceinline__ unsigned int okey32(float x) { return (unsigned int)okey(x); }
__device__ __forceinline__ unsigned int vkey(float x) { return okey32(x); }
__device__ __forceinline__ unsigned long long vkey(double x) { return okey(x); }
__device__ __forceinline__ unsigned long long vkey(const df32 &x) { return okey(x); }
template <typename T> __device__ __forceinline__ T vkey_inv(typename KeyOf<T>::type k) { return okey_inv<T>(k); }
template <typename T> __host__ __device__ constexpr typename KeyOf<T>::type vkey_max() {
  return (typename KeyOf<T>::type)key_max<T>();
}

template <typename T> struct LimOut {
  typename KeyOf<T>::type *vkeys;   // nc x 2 x Vp vertex min / max keys of this pass
  typename KeyOf<T>::type *vreset;  // the next pass's vertex keys, reset here
  unsigned long long *slots;        // nInst x kSlotCopies x 2 x nc encoded global min / max (atomic)
  unsigned long long *reset;        // slots of the next pass, reset by the grid
  int nc, type;
};
template <typename T> struct LimIn {
  const typename KeyOf<T>::type *vkeys;
  const unsigned long long *slots;  // nInst x kSlotCopies x 2 x nc
  int nc, type, shift;
};

// Offset of this block's instance in a slot set (each instance of an ensemble has its own
// global extremes, as each reference problem has).
template <typename T>
__device__ __forceinline__ size_t slot_base(const Geo<T> &g, int nc, int tile = -1) {
  if (tile < 0) tile = blockIdx.x;
  return g.instOf ? (size_t)g.instOf[(tile * (int)blockDim.x) / kBlock] * kSlotCopies * 2 * nc : 0;
}

// Scatter of the element's centroid quantities to its vertices and the block's global extremes.
template <typename T, int NQ>
__device__ __forceinline__ void scatter_quantities(const Geo<T> &g, const LimOut<T> &lo, const T *qv,
                                                   const int vid[3], bool active, int tile = -1) {
  if (tile < 0) tile = blockIdx.x;
  if (active) {
#pragma unroll
    for (int s = 0; s < NQ; ++s) {
      if (s >= lo.nc) break;
      const auto key = vkey(qv[s]);
#pragma unroll
      for (int n = 0; n < 3; ++n) {
        atomicMin(&lo.vkeys[(size_t)(2 * s) * g.Vp + vid[n]], key);
        atomicMax(&lo.vkeys[(size_t)(2 * s + 1) * g.Vp + vid[n]], key);
      }
    }
  }
  // global extremes: warp shuffles, then the block's four warps through shared memory, then one
  // atomic per quantity and block into one of kSlotCopies copies (spreads same-address atomics)
  __shared__ T red[kBlock / 32][2 * NQ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int s = 0; s < NQ; ++s) {
    T mn = (active && s < lo.nc) ? qv[s] : T(INFINITY), mx = (active && s < lo.nc) ? qv[s] : T(-INFINITY);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) { red[warp][2 * s] = mn; red[warp][2 * s + 1] = mx; }
  }
  __syncthreads();
  if (threadIdx.x < lo.nc) {
    const int s = threadIdx.x;
    T mn = red[0][2 * s], mx = red[0][2 * s + 1];
#pragma unroll
    for (int w = 1; w < (int)(blockDim.x / 32); ++w) { mn = fmin(mn, red[w][2 * s]); mx = fmax(mx, red[w][2 * s + 1]); }
    if (mn <= mx) {
      unsigned long long *sl = lo.slots + slot_base(g, lo.nc, tile) + (size_t)(tile % kSlotCopies) * 2 * lo.nc;
      atomicMin(&sl[2 * s], okey(mn));
      atomicMax(&sl[2 * s + 1], okey(mx));
    }
  }
}

// Reset of the next pass's vertex keys (thread t owns vertex t) and global slots (stride over
// the tiles of the mesh: tile / nTiles, by default this block in its grid).
template <typename T>
__device__ __forceinline__ void reset_next(const Geo<T> &g, const LimOut<T> &lo, int t, int tile = -1,
                                           int nTiles = -1) {
  if (tile < 0) tile = blockIdx.x;
  if (nTiles < 0) nTiles = gridDim.x;
  if (t < g.numV)
    for (int s = 0; s < lo.nc; ++s) {
      lo.vreset[(size_t)(2 * s) * g.Vp + t] = vkey_max<T>();
      lo.vreset[(size_t)(2 * s + 1) * g.Vp + t] = 0;
    }
  const int nSlots = (g.instOf ? g.nInst : 1) * kSlotCopies * 2 * lo.nc;
  for (int i = tile * blockDim.x + threadIdx.x; i < nSlots; i += nTiles * blockDim.x)
    lo.reset[i] = (i & 1) ? 0ULL : key_max<T>();
}

// Global extremes of every quantity from the kSlotCopies copies (warp 0), turned into the shift
// values of core/computeMinMaxV0TElementPatch.m:75-78: sh[2s] = |min|+1, sh[2s+1] = |max|+1.
template <typename T>
__device__ __forceinline__ void load_shifts(const unsigned long long *slots, int nc, T *sh) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  for (int s = 0; s < nc; ++s) {
    T mn = okey_inv<T>(slots[(size_t)lane * 2 * nc + 2 * s]);
    T mx = okey_inv<T>(slots[(size_t)lane * 2 * nc + 2 * s + 1]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) { sh[2 * s] = fabs(mn) + T(1); sh[2 * s + 1] = fabs(mx) + T(1); }
  }
}

// alpha of one computeVertexBasedLimiter call (core/computeVertexBasedLimiter.m:78-106): at each
// vertex n on a branch (dV = v_n - cbar below dMin + tol, or above dMax - tol) the clamped ratio
// clamp01(dMin / (dV - tol)) or clamp01(dMax / (dV + tol)), else 1; alpha is their minimum.
// With one division: clamping to [0, 1] is monotone, so the minimum over the vertices of the
// clamped ratios is the clamped smallest ratio.  Each branch's ratio is written
// with a positive denominator, num / den (num >= 0: dMin <= 0 <= dMax, the element's own mean
// being in its patches); the smallest is found by comparing cross products (the first vertex on
// ties) and divided once.  A ratio that ties another to within rounding may be the one divided:
// the factor then differs by at most an ulp.  The limiter's division sits on GB300's FP64 (or
// the double-float) path, where it costs about as much as the rest of the factor.
// A patch extreme that the global shift rounded past the element's own value can leave a
// branch's denominator at or below zero; such a ratio is clamped and divided on its own.
template <typename T>
__device__ __forceinline__ T vertex_alpha_1div(T cbar, const T v[3], const T mn[3], const T mx[3]) {
  const T tol = T(1.e-8);
  T bn = T(0), bd = T(1), extra = T(1);
  bool any = false;
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T dV = v[n] - cbar, dMin = mn[n] - cbar, dMax = mx[n] - cbar;
    bool br = false;
    T num = T(0), den = T(1);
    if (dV < dMin + tol) { num = -dMin; den = tol - dV; br = true; }
    if (dV > dMax - tol) { num = dMax; den = dV + tol; br = true; }
    if (br) {
      if (den > T(0)) {
        if (!any || num * bd < bn * den) { bn = num; bd = den; any = true; }
      } else {
        extra = fmin(extra, fmax(T(0), fmin(T(1), num / den)));
      }
    }
  }
  return fmin(any ? fmax(T(0), fmin(T(1), bn / bd)) : T(1), extra);
}

// The adjoint's side of the same choice: which (sub-limiter, vertex) gives the factor, found
// without dividing.  A branch's ratio dm / den is compared in its positive-denominator form by
// cross products, with a class for the clamped values (0: ratio <= 0, 1: inside (0, 1), 2: >= 1,
// NaN or no branch), so that "clamp(r) < clamp(r_winner)" keeps the first of equal clamped
// factors, as a loop of divisions would; a zero or NaN denominator is divided on its own.
template <typename T> struct RatioWin {
  int cls = 2;
  T pn = T(1), pd = T(1);
  // offers the ratio dm / den of a branch; true if it is now the winner
  __device__ __forceinline__ bool offer(T dm, T den) {
    T n = den < T(0) ? -dm : dm, d = den < T(0) ? -den : den;
    if (!(d > T(0))) {   // zero or NaN denominator: the clamped quotient itself
      n = fmax(T(0), fmin(T(1), dm / den));
      d = T(1);
    }
    const int c = (n != n) ? 2 : (n <= T(0) ? 0 : (n >= d ? 2 : 1));
    const bool less = c < cls || (c == 1 && cls == 1 && n * pd < pn * d);
    if (less) { cls = c; pn = n; pd = d; }
    return less;
  }
};

// ---------------------------------------------------------------------------------------------
// Block staging: the rows of one block's elements (SoA rows, kBlock consecutive elements each)
// are copied global -> shared by the TMA unit (cp.async.bulk, one elected thread) while the
// threads load neighbour and vertex data directly.  The wait on the mbarrier is bounded in time;
// on a timeout the kernel sets bit 1 of the error flag and leaves the element unprocessed.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Ends an mbarrier object's life before its shared memory is put to other use (a kernel that
// runs several tiles per block, with different row layouts, reuses the locations).
__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase 0 of the block's barrier, at most ~2^31 SM cycles (about a second); after a
// timeout it flags the error, gives the copies in flight the same time again, and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, int *flag) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, 0))
    if (clock64() - t0 > (1LL << 31)) {
      atomicOr(flag, 2 | 4);                      // bit 2: a staging copy
      const long long t1 = clock64();
      while (!mbar_try_wait(bar, 0) && clock64() - t1 < (1LL << 31)) {
      }
      return false;
    }
  return true;
}

// Row copies into the staged layout (row index within the T rows / the int rows).
template <typename T>
__device__ __forceinline__ void stage_T(unsigned char *smem, int row, const T *base, int nrows, int Kp, int k0,
                                        uint64_t *bar) {
  for (int r = 0; r < nrows; ++r)
    bulk_g2s(smem + (size_t)(row + r) * blockDim.x * sizeof(T), base + (size_t)r * Kp + k0, blockDim.x * sizeof(T), bar);
}
template <typename T>
__device__ __forceinline__ void stage_I(unsigned char *smem, int nT, int row, const int *base, int nrows, int Kp,
                                        int k0, uint64_t *bar) {
  for (int r = 0; r < nrows; ++r)
    bulk_g2s(smem + (size_t)nT * blockDim.x * sizeof(T) + (size_t)(row + r) * blockDim.x * sizeof(int),
             base + (size_t)r * Kp + k0, blockDim.x * sizeof(int), bar);
}
template <typename T>
__device__ __forceinline__ void stage_expect(uint64_t *bar, int nT, int nI) {
  mbar_expect_tx(bar, nT * blockDim.x * (uint32_t)sizeof(T) + nI * blockDim.x * (uint32_t)sizeof(int));
}

// Programmatic dependent launch: the next kernel in the stream may start its prologue (static
// data only) once every block of this one has started; pdl_wait() blocks until the previous
// kernel has completed and its writes are visible.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// A kernel in such a chain must not declare a buffer that earlier kernels of the chain write as
// `const T *__restrict__`: the compiler may then take its loads for invariant over the whole
// kernel and move them above griddepcontrol.wait.  Outputs that alias no input keep a
// (non-const) __restrict__, which lets input loads move past their stores.

}  // namespace dgadv
#include "dgadv_mma.cuh"
namespace dgadv {

// Device-to-device copy of n 16-byte words as a kernel of the launch chain.  A copy between two
// kernels that use programmatic dependent launch has to be a kernel itself: the second kernel's
// dependency wait covers the kernel launched before it, not a copy-engine transfer queued in
// between, so a cudaMemcpyAsync there is not ordered against the kernel that follows.
static __global__ void k_copy16(const uint4 *src, uint4 *__restrict__ dst, size_t n) {
  pdl_trigger();
  pdl_wait();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

template <typename T> __device__ __forceinline__ const T *srow(const unsigned char *smem, int r) {
  return (const T *)(smem + (size_t)r * blockDim.x * sizeof(T));
}
template <typename T> __device__ __forceinline__ const int *irow(const unsigned char *smem, int nT, int r) {
  return (const int *)(smem + (size_t)nT * blockDim.x * sizeof(T) + (size_t)r * blockDim.x * sizeof(int));
}

template <typename T, int P> struct StageRows {
  static constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R, NMT = Dims<P>::NMT;
  // k_stage_op: c, [c0], F (or the N^2 rows of the element operator), Vn, [B] | code
  __host__ __device__ static constexpr int op(int mode, bool lin, bool eop = false) {
    return N + (mode != 2 ? N : 0) + (eop ? N * N : 2 * Q) + 3 * R + (mode != 0 && !lin ? 4 : 0);
  }
  // k_limit_dot: tbuf, B, c0, cin | code (the packed Taylor mass rows stream from global memory)
  __host__ __device__ static constexpr int limdot() { return N + 4 + 2 * N; }
  // k_limit: tbuf, B | code
  __host__ __device__ static constexpr int lim() { return N + 4; }
  // k_limit_dot_lin: cDot, Q (N x (N-1)) or B (4), c0, cin | code
  __host__ __device__ static constexpr int limdot_lin_rows(bool fly) { return 3 * N + (fly ? 4 : N * (N - 1)); }
  __host__ __device__ static constexpr int limdot_lin() { return limdot_lin_rows(N * (N - 1) < 4); }
  // k_to_taylor: c, B
  __host__ __device__ static constexpr int totaylor() { return N + 4; }
  // rows of eb elements first, then the block's mbarrier (8 bytes, 16 reserved)
  __host__ __device__ static constexpr size_t bar_offset(int nT, int nI, int eb = kBlock) {
    return (size_t)nT * eb * sizeof(T) + (size_t)nI * eb * sizeof(int);
  }
  // + 16 for the mbarrier, + 2 x 6 shift values
  __host__ __device__ static constexpr size_t bytes(int nT, int nI, int eb = kBlock) {
    return bar_offset(nT, nI, eb) + 16 + 12 * sizeof(T);
  }
};

// Prefetch of the three vertices' min / max keys of every sub-limiter quantity.
template <typename T, int NQ> struct VKeys {
  typename KeyOf<T>::type v[NQ][2][3];
};
template <typename T, int NQ>
__device__ __forceinline__ void load_vkeys(const Geo<T> &g, const LimIn<T> &li, const int vid[3], VKeys<T, NQ> &kv) {
#pragma unroll
  for (int s = 0; s < NQ; ++s)
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int n = 0; n < 3; ++n)
        kv.v[s][m][n] = (s < li.nc) ? li.vkeys[(size_t)(2 * s + m) * g.Vp + vid[n]] : 0;
}

// Patch min / max of quantity s at the three vertices (from the prefetched vertex keys), with
// the reference's global shift (min over the patch of (v - sNeg), then + sNeg; a monotone shift
// commutes with min), then combined with the Dirichlet data (NaN = none; fmin / fmax ignore NaN
// like Matlab's min / max).
template <typename T, int NQ>
__device__ __forceinline__ void patch_minmax(const LimIn<T> &li, const VKeys<T, NQ> &kv, const T *sh, int s,
                                             const T valD[3], T mn[3], T mx[3]) {
  T sNeg = T(0), sPos = T(0);
  if (li.shift) { sPos = sh[2 * s]; sNeg = sh[2 * s + 1]; }
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    T a = vkey_inv<T>(kv.v[s][0][n]);
    T c = vkey_inv<T>(kv.v[s][1][n]);
    if (li.shift) { a = (a - sNeg) + sNeg; c = (c + sPos) - sPos; }
    mn[n] = fmin(a, valD[n]);
    mx[n] = fmax(c, valD[n]);
  }
}

// Limit Taylor coefficients in place (linear / hierarchical vertex).  dataV0T: boundary values
// at the three vertices for Dirichlet vertices (NaN means "no data").
// Taylor basis functions of core/phiTaylorPhy.m at the element's vertices, phi[n][j] for the
// first N functions: scaled monomials about the barycentre, mean-free from degree 2 on.  The
// means are the exact triangle moments about the barycentre, E[x^2] = sum_n x_n^2 / 12 and
// E[x^3] = sum_n x_n^3 / 30 (mixed moments likewise), which the reference integrates with
// quadrature rules exact for them.
template <typename T, int P>
__device__ __forceinline__ void taylor_vertex_basis(const Affine<T> &af, T phi[3][Dims<P>::N]) {
  const T d = af.dX;
  T exx = T(0), exy = T(0), eyy = T(0), exxx = T(0), exxy = T(0), exyy = T(0), eyyy = T(0);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T x = af.ox[n], y = af.oy[n];
    exx = exx + x * x; exy = exy + x * y; eyy = eyy + y * y;
    exxx = exxx + x * x * x; exxy = exxy + x * x * y; exyy = exyy + x * y * y; eyyy = eyyy + y * y * y;
  }
  exx = exx / T(12); exy = exy / T(12); eyy = eyy / T(12);
  exxx = exxx / T(30); exxy = exxy / T(30); exyy = exyy / T(30); eyyy = eyyy / T(30);
  const T d2 = d * d, d3 = d2 * d, half = T(1) / T(2), sixth = T(1) / T(6);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T x = af.ox[n], y = af.oy[n];
    phi[n][0] = T(1);
    if (P >= 1) { phi[n][1] = x * d; phi[n][2] = y * d; }
    if (P >= 2) {
      phi[n][3] = half * (x * x - exx) * d2;
      phi[n][4] = (x * y - exy) * d2;
      phi[n][5] = half * (y * y - eyy) * d2;
    }
    if (P >= 3) {
      phi[n][6] = sixth * (x * x * x - exxx) * d3;
      phi[n][7] = half * (x * x * y - exxy) * d3;
      phi[n][8] = half * (x * y * y - exyy) * d3;
      phi[n][9] = sixth * (y * y * y - eyyy) * d3;
    }
  }
}

// LT: the limiter type (0 linear, 1 hierarchical vertex, 2 strict), fixed per kernel so that
// each kernel carries the code of one limiter only.
template <typename T, int P, int NQ, int LT>
__device__ __forceinline__ void limit_taylor(const LimIn<T> &li, const VKeys<T, NQ> &kv, const T *sh,
                                             const Affine<T> &af, int dmask, const T dataV0T[3], T *cT) {
  constexpr int N = Dims<P>::N;
  const T nan_ = T(NAN);
  T pt1[3], pt2[3];   // Taylor basis functions 2 and 3 at the vertices
#pragma unroll
  for (int n = 0; n < 3; ++n) { pt1[n] = af.ox[n] * af.dX; pt2[n] = af.oy[n] * af.dX; }
  if constexpr (LT == 0) {
    T v[3], valD[3], mn[3], mx[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      v[n] = (cT[0] * T(1) + cT[1] * pt1[n]) + cT[2] * pt2[n];
      valD[n] = ((dmask >> n) & 1) ? dataV0T[n] : nan_;
    }
    patch_minmax<T, NQ>(li, kv, sh, 0, valD, mn, mx);
    const T alpha = vertex_alpha_1div(cT[0], v, mn, mx);
    cT[1] *= alpha; cT[2] *= alpha;
    const T keep = (alpha == T(1)) ? T(1) : T(0);
#pragma unroll
    for (int i = 3; i < N; ++i) cT[i] *= keep;
  } else if constexpr (LT == 2) {
    // core/applySlopeLimiterTaylorStrict.m:111-150: for ord = p..1 the reconstructions of
    // degree p - ord + 1 about each derivative of order ord - 1, from the data already limited
    // at the higher orders; every DOF of order >= ord is scaled by the order's factor.  The
    // centroid quantities (derivatives of order ord - 1) are never rescaled by a higher order,
    // so their patch extremes are those of the unlimited data (the same passes as hierarchical).
    T phi[3][N];
    taylor_vertex_basis<T, P>(af, phi);
    int s = 0;
#pragma unroll
    for (int ord = P; ord >= 1; --ord) {
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
            for (int b = 0; a + b <= P - ord + 1; ++b) acc = acc + cT[mind(ba + a, bb + b)] * phi[n][mind(a, b)];
          v[n] = acc;
          valD[n] = ((dmask >> n) & 1) ? (ord > 1 ? v[n] : dataV0T[n]) : nan_;
        }
        patch_minmax<T, NQ>(li, kv, sh, s, valD, mn, mx);
        aOrd = fmin(aOrd, vertex_alpha_1div(cT[i0], v, mn, mx));
        ++s;
      }
#pragma unroll
      for (int i = ord * (ord + 1) / 2; i < N; ++i) cT[i] = aOrd * cT[i];
    }
  } else {
    T orig[N];
#pragma unroll
    for (int i = 0; i < N; ++i) orig[i] = cT[i];
    T alpha = T(0);
    int s = 0;
#pragma unroll
    for (int ord = P; ord >= 1; --ord) {
      T aOrd = T(1);
#pragma unroll
      for (int i = 1; i <= ord; ++i) {
        const int i0 = mind(ord - i, i - 1), i1 = mind(ord - i + 1, i - 1), i2 = mind(ord - i, i);
        T v[3], valD[3], mn[3], mx[3];
#pragma unroll
        for (int n = 0; n < 3; ++n) {
          v[n] = (orig[i0] * T(1) + orig[i1] * pt1[n]) + orig[i2] * pt2[n];
          valD[n] = ((dmask >> n) & 1) ? (ord > 1 ? v[n] : dataV0T[n]) : nan_;
        }
        patch_minmax<T, NQ>(li, kv, sh, s, valD, mn, mx);
        aOrd = fmin(aOrd, vertex_alpha_1div(orig[i0], v, mn, mx));
        ++s;
      }
      alpha = fmax(alpha, aOrd);
#pragma unroll
      for (int i = ord * (ord + 1) / 2; i < (ord + 1) * (ord + 2) / 2; ++i) cT[i] = alpha * orig[i];
    }
  }
}

// Element geometry from staged rows of B.
template <typename T> __device__ __forceinline__ Affine<T> affine_from(T B11, T B12, T B21, T B22) {
  Affine<T> a;
  a.B11 = B11; a.B12 = B12; a.B21 = B21; a.B22 = B22;
  const T det = a.B11 * a.B22 - a.B12 * a.B21;
  const T idet = T(1) / det;
  a.A11 = a.B22 * idet; a.A12 = -a.B12 * idet; a.A21 = -a.B21 * idet; a.A22 = a.B11 * idet;
  a.dX = T(2) / sqrt(det);
  a.idX = T(1) / a.dX;
  const T bx = -(a.B11 + a.B12) / T(3), by = -(a.B21 + a.B22) / T(3);
  a.ox[0] = bx; a.oy[0] = by;
  a.ox[1] = a.B11 + bx; a.oy[1] = a.B21 + by;
  a.ox[2] = a.B12 + bx; a.oy[2] = a.B22 + by;
  return a;
}

// ---------------------------------------------------------------------------------------------
// Linear limiter without element geometry.  The centroid value and the vertex values of the
// linear Taylor reconstruction (core/applySlopeLimiterTaylorLinear.m:108-122) are
//     cbar = u_0,   v_n = u_0 + u_1 (x^_n - c^)_1 + u_2 (x^_n - c^)_2,   u = DM c,
// because grad u(b) . (x_n - b) is invariant under the affine map to the reference element
// (x^_n the reference vertices, c^ = (1/3, 1/3)).  Scaling Taylor degree blocks commutes with
// the block-diagonal map between reference derivatives and Taylor coefficients, so the limited
// coefficients are c - DM^-1 du with du = (0, (1-a) u_1, (1-a) u_2, [a != 1] u_3, ...).
template <typename T, int P>
__device__ __forceinline__ void lin_u(const T *c, T *u) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
#pragma unroll
  for (int i = 0; i < N; ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) s.fma(tb.DM[i][j], c[j]);
    u[i] = s.get();
  }
}
// The first three rows of u = DM c (mean and the linear part), all the linear limiter's
// decision needs; the other rows only matter where the limiter acts (lin_alpha_lazy).
template <typename T, int P>
__device__ __forceinline__ void lin_u3(const T *c, T *u) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
#pragma unroll
  for (int i = 0; i < (N < 3 ? N : 3); ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) s.fma(tb.DM[i][j], c[j]);
    u[i] = s.get();
  }
#pragma unroll
  for (int i = 3; i < N; ++i) u[i] = T(0);
}
template <typename T, int P> __device__ __forceinline__ T lin_mean(const T *c) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  Acc<T> s(T(0));
#pragma unroll
  for (int j = 0; j < N; ++j) s.fma(tb.DM[0][j], c[j]);
  return s.get();
}
// alpha of the linear limiter from u, and the removed part du (returns false if alpha == 1).
template <typename T, int P, int NQ>
__device__ __forceinline__ bool lin_alpha(const LimIn<T> &li, const VKeys<T, NQ> &kv, const T *sh, const T *u,
                                          int dmask, const T dataV0T[3], T *du) {
  constexpr int N = Dims<P>::N;
  const T third = T(1) / T(3), two3 = T(2) / T(3);
  const T hx[3] = {-third, two3, -third}, hy[3] = {-third, -third, two3};
  T v[3], valD[3], mn[3], mx[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    v[n] = (u[0] * T(1) + u[1] * hx[n]) + u[2] * hy[n];
    valD[n] = ((dmask >> n) & 1) ? dataV0T[n] : T(NAN);
  }
  patch_minmax<T, NQ>(li, kv, sh, 0, valD, mn, mx);
  const T alpha = vertex_alpha_1div(u[0], v, mn, mx);
  if (alpha == T(1)) return false;
  du[0] = T(0);
  du[1] = (T(1) - alpha) * u[1];
  du[2] = (T(1) - alpha) * u[2];
#pragma unroll
  for (int i = 3; i < N; ++i) du[i] = u[i];
  return true;
}

// lin_alpha with only u_0, u_1, u_2 given: the rows u_3.. of DM c are computed where the element
// is limited (each row as lin_u computes it, so the results are the same).
template <typename T, int P, int NQ>
__device__ __forceinline__ bool lin_alpha_lazy(const LimIn<T> &li, const VKeys<T, NQ> &kv, const T *sh, T *u,
                                               const T *c, int dmask, const T dataV0T[3], T *du) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  if (!lin_alpha<T, P, NQ>(li, kv, sh, u, dmask, dataV0T, du)) return false;
#pragma unroll
  for (int i = 3; i < N; ++i) {
    Acc<T> s(T(0));
#pragma unroll
    for (int j = 0; j < N; ++j) s.fma(tb.DM[i][j], c[j]);
    u[i] = s.get();
    du[i] = u[i];
  }
  return true;
}

// ---------------------------------------------------------------------------------------------
// Stage operator.  MODE 0: write c^(s);  MODE 1: write Taylor(c^(s)) and scatter its centroid
// quantities;  MODE 2: write Taylor(cDot) and scatter its quantities (time-derivative limiting
// follows).
struct StageScalars {
  double omega, tau;
  double gco[4];        // g_m(t) of the source terms / boundary data
  int *flag;            // bit 0: non-finite value seen; bit 1: a bounded wait timed out
};

// Operator variants of the stage kernel (VAR):
//   kOpPlain    volume term at the quadrature points, upwind flux at the edge points;
//   kOpFp32     (double-float state only) the operator (volume, flux, hatM^-1 = I) in FP32
//               arithmetic; the SSP update, the outputs and the limiter's quantities stay in the
//               stored type;
//   kOpElement  (FP64 or double-float, no source terms) the element operator g.Aop, N x N per element: the
//               volume term and the element's own outflow terms as one product with c, built
//               by k_build_element_operator whenever the velocity changes; only the inflow terms
//               are evaluated at the edge points.  GB300's FP64 rate bounds the FP64 stage: this
//               takes the operator from about 244 FP64 instructions per element to about 100
//               (p = 2).
constexpr int kOpPlain = 0, kOpFp32 = 1, kOpElement = 2;

template <typename T, int P, int MODE, bool RHS, bool LIN, int VAR = kOpPlain>
__device__ __forceinline__ void stage_op_tile(const Geo<T> g, const T *cin, const T *c0, T *out,
           const LimOut<T> lo, const StageScalars sc, const int tile, const int nTiles = -1) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R, NQ = NCQ<P>::value;
  constexpr bool OPF = VAR == kOpFp32, EOP = VAR == kOpElement;
  static_assert(!EOP || ((std::is_same_v<T, double> || std::is_same_v<T, df32>) && !RHS),
                "the element operator is FP64 or double-float without source terms");
  using A = std::conditional_t<OPF, float, T>;
  // with the mass solve (FP64, double-float) and no source terms, hatM^-1 is folded into the
  // test-function tables of the volume and flux terms (Fg1, Fg2, Fphi)
  constexpr bool kFold = sizeof(A) == 8 && !RHS;
  constexpr int NT = StageRows<T, P>::op(MODE, LIN, EOP);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  const Tab<T, P> &tb = tab<T, P>();
  const int t = threadIdx.x, eb = blockDim.x, k0 = tile * eb, k = k0 + t;
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;                   // blocks beyond the elements only reset keys
  constexpr int rC = 0, rC0 = N, rF = (MODE != 2) ? 2 * N : N, rV = rF + (EOP ? N * N : 2 * Q), rB = rV + 3 * R;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {                                 // static rows before the dependency wait
      stage_expect<T>(bar, NT, 1);
      if constexpr (EOP) stage_T(smem, rF, g.Aop, N * N, Kp, k0, bar);
      else stage_T(smem, rF, g.F, 2 * Q, Kp, k0, bar);
      stage_T(smem, rV, g.Vn, 3 * R, Kp, k0, bar);
      if (MODE != 0 && !LIN) stage_T(smem, rB, g.Bm, 4, Kp, k0, bar);
      stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
    }
  }
  const bool active = k < g.K;
  int nb[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) nb[n] = active ? g.nbr[(size_t)n * Kp + k] : -1;
  int vid[3] = {0, 0, 0};
  if (MODE != 0 && active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  if (MODE != 0) reset_next<T>(g, lo, k, nTiles < 0 ? -1 : tile, nTiles);
  if (!staged) return;
  if (t == 0) {                                   // state rows after it
    stage_T(smem, rC, cin, N, Kp, k0, bar);
    if (MODE != 2) stage_T(smem, rC0, c0, N, Kp, k0, bar);
  }
  // neighbour coefficients: outside the block from global memory now, inside from shared later
  A cn[3][N];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const bool outside = nb[n] >= 0 && (nb[n] < k0 || nb[n] >= k0 + eb);
#pragma unroll
    for (int j = 0; j < N; ++j) cn[n][j] = outside ? as_arith<A>(cin[(size_t)j * Kp + nb[n]]) : A(0);
  }
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T qv[NQ];
  bool bad = false;
  if (active && ok) {
    A c[N];
    Acc<A> rhs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) { c[i] = as_arith<A>(srow<T>(smem, rC + i)[t]); rhs[i] = Acc<A>(A(0)); }
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (nb[n] >= k0 && nb[n] < k0 + eb)
#pragma unroll
        for (int j = 0; j < N; ++j) cn[n][j] = as_arith<A>(srow<T>(smem, rC + j)[nb[n] - k0]);
    if (RHS) {
      for (int m = 0; m < g.nTerms; ++m) {
        const A gm = A(sc.gco[m]);
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i].fma(gm, as_arith<A>(g.rhs[((size_t)m * N + i) * Kp + k]));
      }
    }
    if constexpr (EOP) {   // volume term and own outflow: the element operator
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) rhs[i].fma(srow<T>(smem, rF + i * N + j)[t], c[j]);
    } else {
    // volume term (at p = 3, 12 points: unrolled by 3 to keep the body in the instruction cache)
#pragma unroll(P >= 3 ? 3 : Q)
    for (int qq = 0; qq < Q; ++qq) {
      Acc<A> cqa(A(0));
#pragma unroll
      for (int j = 0; j < N; ++j) cqa.fma(as_arith<A>(tb.phiQ[qq][j]), c[j]);
      const A cq = cqa.get();
      const A f1 = as_arith<A>(srow<T>(smem, rF + qq)[t]) * cq;
      const A f2 = as_arith<A>(srow<T>(smem, rF + Q + qq)[t]) * cq;
      const T(&G1)[Q][N] = kFold ? tb.Fg1 : tb.g1;
      const T(&G2)[Q][N] = kFold ? tb.Fg2 : tb.g2;
#pragma unroll
      for (int i = 0; i < N; ++i) { rhs[i].fma(as_arith<A>(G1[qq][i]), f1); rhs[i].fma(as_arith<A>(G2[qq][i]), f2); }
    }
    }
    // upwind edge term (with the element operator: the inflow terms only)
    const int code = irow<T>(smem, NT, 0)[t];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int np = (code >> (2 * n)) & 3;
      const bool outOk = !EOP && ((code >> (6 + n)) & 1);
#pragma unroll
      for (int r2 = 0; r2 < R; ++r2) {
        const A v = as_arith<A>(srow<T>(smem, rV + n * R + r2)[t]);
        if (EOP && !(v < A(0) && nb[n] >= 0)) continue;
        Acc<A> tr(A(0));
        if (v > A(0) && outOk) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(as_arith<A>(tb.phi1D[n][r2][j]), c[j]);
        } else if (v < A(0) && nb[n] >= 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(as_arith<A>(tb.thetaPhi[n][np][r2][j]), cn[n][j]);
        }
        const A fl = v * tr.get();
        const T(&PR)[3][R][N] = kFold ? tb.Fphi : tb.phi1D;
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i].fms(as_arith<A>(PR[n][r2][i]), fl);
      }
    }
    // mass solve
    T cdot[N];
    if constexpr (sizeof(A) == 8 && !kFold) {
      A r[N];
#pragma unroll
      for (int j = 0; j < N; ++j) r[j] = rhs[j].get();
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc<A> s(A(0));
#pragma unroll
        for (int j = 0; j < N; ++j) s.fma(tb.hatMinv[i][j], r[j]);
        cdot[i] = s.get();
      }
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) cdot[i] = T(rhs[i].get());
    }
    if (MODE == 2 && LIN) {
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cdot[i]; bad |= !finite_(cdot[i]); }
      qv[0] = lin_mean<T, P>(cdot);
    } else if (MODE == 2) {
      const Affine<T> af = affine_from<T>(srow<T>(smem, rB)[t], srow<T>(smem, rB + 1)[t],
                                          srow<T>(smem, rB + 2)[t], srow<T>(smem, rB + 3)[t]);
      T cT[N];
      to_taylor<T, P>(cdot, af, cT);
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cT[i]; bad |= !finite_(cT[i]); }
      centroid_quantities<T, P>(cT, lo.type, qv);
    } else {
      const T w = T(sc.omega), tau = T(sc.tau);
      T cnew[N];
#pragma unroll
      for (int i = 0; i < N; ++i)
        cnew[i] = w * srow<T>(smem, rC0 + i)[t] + (T(1) - w) * (srow<T>(smem, rC + i)[t] + tau * cdot[i]);
      if (MODE == 0 || LIN) {
#pragma unroll
        for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cnew[i]; bad |= !finite_(cnew[i]); }
        if (MODE == 1) qv[0] = lin_mean<T, P>(cnew);
      } else {
        const Affine<T> af = affine_from<T>(srow<T>(smem, rB)[t], srow<T>(smem, rB + 1)[t],
                                            srow<T>(smem, rB + 2)[t], srow<T>(smem, rB + 3)[t]);
        T cT[N];
        to_taylor<T, P>(cnew, af, cT);
#pragma unroll
        for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cT[i]; bad |= !finite_(cT[i]); }
        centroid_quantities<T, P>(cT, lo.type, qv);
      }
    }
  }
  if (MODE != 0) scatter_quantities<T, NQ>(g, lo, qv, vid, active && ok, tile);
  if (bad) atomicOr(sc.flag, 1);
}
template <typename T, int P, int MODE, bool RHS, bool LIN, int VAR = kOpPlain>
__global__ void __launch_bounds__(kBlock)
k_stage_op(const Geo<T> g, const T *cin, const T *c0, T *out,
           const LimOut<T> lo, const StageScalars sc) {
  stage_op_tile<T, P, MODE, RHS, LIN, VAR>(g, cin, c0, out, lo, sc, blockIdx.x);
}

// The element operator of every element (kOpElement), from the velocity factors F and Vn:
//   A_ij = sum_q (Fg1_qi F1_q + Fg2_qi F2_q) phiQ_qj  -  sum_(n,r outflow) Fphi_nri v_nr phi1D_nrj,
// the stage operator's volume term and its own outflow terms with hatM^-1 folded in
// (advection/solveSubStep.m:66 with core/assembleMatElemDphiPhiFuncDisc.m:181-202 and the
// element's own trace of core/assembleMatEdgePhiPhiValUpwind.m:261-299).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock) k_build_element_operator(const Geo<T> g, T *__restrict__ aop) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  const Tab<T, P> &tb = tab<T, P>();
  const int k = blockIdx.x * kBlock + threadIdx.x;
  if (k >= g.K) return;
  const int Kp = g.Kp;
  const int code = g.code[k];
  for (int i = 0; i < N; ++i) {
    T w1[Q], w2[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      w1[q] = tb.Fg1[q][i] * g.F[(size_t)q * Kp + k];
      w2[q] = tb.Fg2[q][i] * g.F[(size_t)(Q + q) * Kp + k];
    }
    T wv[3][R];
#pragma unroll
    for (int n = 0; n < 3; ++n)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const T v = g.Vn[(size_t)(n * R + r) * Kp + k];
        wv[n][r] = (v > T(0) && ((code >> (6 + n)) & 1)) ? tb.Fphi[n][r][i] * v : T(0);
      }
    for (int j = 0; j < N; ++j) {
      Acc<T> a(T(0));
#pragma unroll
      for (int q = 0; q < Q; ++q) { a.fma(w1[q], tb.phiQ[q][j]); a.fma(w2[q], tb.phiQ[q][j]); }
#pragma unroll
      for (int n = 0; n < 3; ++n)
#pragma unroll
        for (int r = 0; r < R; ++r) a.fms(wv[n][r], tb.phi1D[n][r][j]);
      aop[(size_t)(i * N + j) * Kp + k] = a.get();
    }
  }
}

// The stage operator with the volume term on the tensor cores (dgadv_mma.cuh): FP32, p >= 2,
// MODE 2 (cDot out, time-derivative limiting follows), no source terms.  The rest of the stage
// (the upwind flux, the output, the scatter of centroid quantities) is stage_op_tile's; the
// flux is computed while the first contraction runs.  Shared memory: the staged rows, then the
// MMA area at the next 1024-byte boundary.
template <int P> struct MmaSmem {
  __host__ __device__ static constexpr size_t rows(bool lin) {
    return StageRows<float, P>::bytes(StageRows<float, P>::op(2, lin), 1);
  }
  __host__ __device__ static constexpr size_t area(bool lin) { return (rows(lin) + 1023) / 1024 * 1024; }
  __host__ __device__ static constexpr size_t bytes(bool lin) { return area(lin) + vmma::kBytes; }
};

template <int P, bool LIN>
__device__ __forceinline__ void stage_op_tile_mma(const Geo<float> g, const float *cin, float *out,
                                                  const LimOut<float> lo, const StageScalars sc, const int tile) {
  using T = float;
  constexpr int MODE = 2;
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R, NQ = NCQ<P>::value;
  static_assert(N <= 16 && 2 * Q <= 32, "one 16-column accumulator per contraction");
  constexpr int NT = StageRows<T, P>::op(MODE, LIN);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  unsigned char *mm = smem + MmaSmem<P>::area(LIN);
  uint64_t *mbar = (uint64_t *)(mm + vmma::oBar);
  uint32_t *tslot = (uint32_t *)(mm + vmma::oTmem);
  const Tab<T, P> &tb = tab<T, P>();
  const int t = threadIdx.x, k0 = tile * kBlock, k = k0 + t;
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  constexpr int rC = 0, rF = N, rV = rF + 2 * Q, rB = rV + 3 * R;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_init(mbar, 1); mbar_fence_init(); }
    if (t < 32) vmma::alloc(tslot);
    vmma::fill_tables<P>(mm);
    vmma::fence_before();
    __syncthreads();
    vmma::fence_after();
    if (t == 0) {
      stage_expect<T>(bar, NT, 1);
      stage_T(smem, rF, g.F, 2 * Q, Kp, k0, bar);
      stage_T(smem, rV, g.Vn, 3 * R, Kp, k0, bar);
      if (!LIN) stage_T(smem, rB, g.Bm, 4, Kp, k0, bar);
      stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
    }
  }
  const bool active = k < g.K;
  int nb[3];
#pragma unroll
  for (int n = 0; n < 3; ++n) nb[n] = active ? g.nbr[(size_t)n * Kp + k] : -1;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k);
  if (!staged) return;
  const uint32_t tbase = *tslot;
  if (t == 0) stage_T(smem, rC, cin, N, Kp, k0, bar);
  T cn[3][N];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const bool outside = nb[n] >= 0 && (nb[n] < k0 || nb[n] >= k0 + kBlock);
#pragma unroll
    for (int j = 0; j < N; ++j) cn[n][j] = outside ? cin[(size_t)j * Kp + nb[n]] : T(0);
  }
  const bool okAll = __syncthreads_and(mbar_wait_bounded(bar, sc.flag) ? 1 : 0) != 0;
  T c[N];
#pragma unroll
  for (int i = 0; i < N; ++i) c[i] = (active && okAll) ? srow<T>(smem, rC + i)[t] : T(0);
  // first contraction: A1 = this block's coefficients (row t), c_q into D1
#pragma unroll
  for (int j = 0; j < 16; ++j) vmma::put_split(mm, vmma::oA1h, vmma::oA1l, vmma::koff(t, j, 16), j < N ? c[j] : 0.f);
  vmma::sync_for_mma();
  const uint32_t mmBase = smem_u32(mm);
  if (t == 0 && okAll)
    vmma::issue(tbase, mmBase + vmma::oA1h, mmBase + vmma::oA1l, mmBase + vmma::oB1h, mmBase + vmma::oB1l, 16, mbar);
  // the upwind flux meanwhile
  Acc<T> rhs[N];
#pragma unroll
  for (int i = 0; i < N; ++i) rhs[i] = Acc<T>(T(0));
  if (active && okAll) {
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (nb[n] >= k0 && nb[n] < k0 + kBlock)
#pragma unroll
        for (int j = 0; j < N; ++j) cn[n][j] = srow<T>(smem, rC + j)[nb[n] - k0];
    const int code = irow<T>(smem, NT, 0)[t];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int np = (code >> (2 * n)) & 3;
      const bool outOk = (code >> (6 + n)) & 1;
#pragma unroll
      for (int r2 = 0; r2 < R; ++r2) {
        const T v = srow<T>(smem, rV + n * R + r2)[t];
        Acc<T> tr(T(0));
        if (v > T(0) && outOk) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(tb.phi1D[n][r2][j], c[j]);
        } else if (v < T(0) && nb[n] >= 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(tb.thetaPhi[n][np][r2][j], cn[n][j]);
        }
        const T fl = v * tr.get();
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i].fms(tb.phi1D[n][r2][i], fl);
      }
    }
  }
  // second contraction: A2 = (F1_q c_q, F2_q c_q), vol_i into D2
  bool okM = okAll;
  if (okAll) okM = vmma::wait_bounded(mbar, 0, sc.flag);
  okM = __syncthreads_and(okM ? 1 : 0) != 0;
  float cq[16];
  if (okM) {
    vmma::fence_after();
    vmma::ld16(tbase + ((uint32_t)(32 * (t >> 5)) << 16), cq);
  }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const bool use = okM && active && q < Q;
    const float f1 = use ? srow<T>(smem, rF + (q < Q ? q : 0))[t] * cq[q] : 0.f;
    const float f2 = use ? srow<T>(smem, rF + Q + (q < Q ? q : 0))[t] * cq[q] : 0.f;
    if (q < Q) {
      vmma::put_split(mm, vmma::oA2h, vmma::oA2l, vmma::koff(t, q, 32), f1);
      vmma::put_split(mm, vmma::oA2h, vmma::oA2l, vmma::koff(t, Q + q, 32), f2);
    }
  }
#pragma unroll
  for (int kk = 2 * Q; kk < 32; ++kk) vmma::put_split(mm, vmma::oA2h, vmma::oA2l, vmma::koff(t, kk, 32), 0.f);
  vmma::sync_for_mma();
  if (t == 0 && okM)
    vmma::issue(tbase + 16, mmBase + vmma::oA2h, mmBase + vmma::oA2l, mmBase + vmma::oB2h, mmBase + vmma::oB2l, 32, mbar);
  bool okV = okM;
  if (okM) okV = vmma::wait_bounded(mbar, 1, sc.flag);
  okV = __syncthreads_and(okV ? 1 : 0) != 0;
  float vol[16];
  if (okV) {
    vmma::fence_after();
    vmma::ld16(tbase + 16 + ((uint32_t)(32 * (t >> 5)) << 16), vol);
  }
  vmma::fence_before();
  __syncthreads();
  if (t < 32) vmma::dealloc(tbase);
  T qv[NQ];
  bool bad = false;
  const bool done = active && okV;
  if (done) {
    T cdot[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cdot[i] = rhs[i].get() + vol[i];
    if (LIN) {
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cdot[i]; bad |= !finite_(cdot[i]); }
      qv[0] = lin_mean<T, P>(cdot);
    } else {
      const Affine<T> af = affine_from<T>(srow<T>(smem, rB)[t], srow<T>(smem, rB + 1)[t],
                                          srow<T>(smem, rB + 2)[t], srow<T>(smem, rB + 3)[t]);
      T cT[N];
      to_taylor<T, P>(cdot, af, cT);
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cT[i]; bad |= !finite_(cT[i]); }
      centroid_quantities<T, P>(cT, lo.type, qv);
    }
  }
  scatter_quantities<T, NQ>(g, lo, qv, vid, done, tile);
  if (bad) atomicOr(sc.flag, 1);
}
template <int P, bool LIN>
__global__ void __launch_bounds__(kBlock)
k_stage_op_mma(const Geo<float> g, const float *cin, float *out, const LimOut<float> lo, const StageScalars sc) {
  stage_op_tile_mma<P, LIN>(g, cin, out, lo, sc, blockIdx.x);
}

// Time-derivative limiting and SSP update (advection/solveSubStep.m:69-83), then the Taylor
// form of the new stage value and the scatter of its centroid quantities for the solution
// limiter.
// Resident blocks per SM asked of k_limit_dot in FP32: six for the hierarchical limiter (80
// registers), five for the strict one, whose larger body would spill at six; no bound for the
// wider types.
template <typename T, int LT> struct LimDotBlocks { static constexpr int value = 1; };
template <> struct LimDotBlocks<float, 1> { static constexpr int value = 6; };
template <> struct LimDotBlocks<float, 2> { static constexpr int value = 5; };
// ... and of k_limit
template <typename T> struct LimBlocks { static constexpr int value = 1; };
template <> struct LimBlocks<float> { static constexpr int value = 5; };

template <typename T, int P, int LT>
__global__ void __launch_bounds__(kBlock, LimDotBlocks<T, LT>::value)
k_limit_dot(const Geo<T> g, const T *cin, const T *c0, const T *tbuf, T *tout,
            const LimIn<T> li, const LimOut<T> lo, const StageScalars sc) {
  // tbuf: Taylor coefficients of cDot (in); tout: those of the new stage value (out; the same
  // buffer in a plain run, the record slot of the stage in a recorded one)
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::limdot();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x) + 16);
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  constexpr int rT = 0, rB = N, rC0 = N + 4, rC = rC0 + N;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {
      stage_expect<T>(bar, NT, 1);
      stage_T(smem, rB, g.Bm, 4, Kp, k0, bar);
      stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
    }
  }
  const bool active = k < g.K;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k);
  if (!staged) return;
  if (t == 0) {
    stage_T(smem, rT, tbuf, N, Kp, k0, bar);
    stage_T(smem, rC0, c0, N, Kp, k0, bar);
    stage_T(smem, rC, cin, N, Kp, k0, bar);
  }
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc), li.nc, sh);
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T qv[NQ];
  bool bad = false;
  if (active && ok) {
    const Affine<T> af = affine_from<T>(srow<T>(smem, rB)[t], srow<T>(smem, rB + 1)[t],
                                        srow<T>(smem, rB + 2)[t], srow<T>(smem, rB + 3)[t]);
    T cT[N], lim[N];
#pragma unroll
    for (int i = 0; i < N; ++i) { cT[i] = srow<T>(smem, rT + i)[t]; lim[i] = cT[i]; }
    const int dmask = (irow<T>(smem, NT, 0)[t] >> 9) & 7;
    const T nan3[3] = {T(NAN), T(NAN), T(NAN)};
    limit_taylor<T, P, NQ, LT>(li, kv, sh, af, dmask, nan3, lim);
    // Taylor mass correction M_corr = diag(1/diag(M_T)) M_T applied to (cT - lim); the packed
    // upper triangle is read once, row by row, and every row i of the product still sums its
    // terms in the order j = 0..N-1
    T d[N];
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = cT[i] - lim[i];
    T cor[N];
    if (g.mtOnTheFly) {
      // Mcorr d from B and the constant Gram table: y = S^-1 d, then taylor_mcorr
      SinvBlocks<T, P> si;
      sinv_blocks<T, P>(af, si);
      T y[N], m[N];
      y[0] = d[0];
#pragma unroll
      for (int dd = 1; dd <= P; ++dd) {
        const int off = dd * (dd + 1) / 2;
#pragma unroll
        for (int a = 0; a <= dd; ++a) {
          Acc<T> sy(T(0));
#pragma unroll
          for (int j = 0; j <= dd; ++j) sy.fma(si.b[dd][a][j], d[off + j]);
          y[off + a] = sy.get();
        }
      }
      taylor_mcorr<T, P>(si, y, m);
#pragma unroll
      for (int i = 0; i < N; ++i) cor[i] = lim[i] + m[i];
    } else {
      T acc[N], dii[N];
#pragma unroll
      for (int i = 0; i < N; ++i) { acc[i] = T(0); dii[i] = T(1); }
#pragma unroll
      for (int a = 0; a < N; ++a)
#pragma unroll
        for (int b = a; b < N; ++b) {
          const int idx = a * N - a * (a - 1) / 2 + (b - a);
          const T m = g.MT[(size_t)idx * Kp + k];
          if (a == b) {
            acc[a] += m * d[a];
            dii[a] = m;
          } else {
            acc[a] += m * d[b];
            acc[b] += m * d[a];
          }
        }
#pragma unroll
      for (int i = 0; i < N; ++i) cor[i] = lim[i] + acc[i] / dii[i];
    }
    T cdot[N];
    from_taylor<T, P>(cor, af, cdot);
    const T w = T(sc.omega), tau = T(sc.tau);
    T cnew[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
      cnew[i] = w * srow<T>(smem, rC0 + i)[t] + (T(1) - w) * (srow<T>(smem, rC + i)[t] + tau * cdot[i]);
    T cT2[N];
    to_taylor<T, P>(cnew, af, cT2);
#pragma unroll
    for (int i = 0; i < N; ++i) { tout[(size_t)i * Kp + k] = cT2[i]; bad |= !finite_(cT2[i]); }
    centroid_quantities<T, P>(cT2, lo.type, qv);
  }
  scatter_quantities<T, NQ>(g, lo, qv, vid, active && ok);
  if (bad) atomicOr(sc.flag, 1);
}

// Solution limiter: limited Taylor coefficients back to the modal basis
// (core/applySlopeLimiterDisc.m:77-86).
template <typename T, int P, int LT>
__global__ void __launch_bounds__(kBlock, LimBlocks<T>::value)
k_limit(const Geo<T> g, const T *tbuf, T *__restrict__ out, const LimIn<T> li,
        const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::lim();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x) + 16);
  pdl_trigger();
  if (k0 >= g.K) { pdl_wait(); return; }
  const int Kp = g.Kp;
  if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
  __syncthreads();
  if (t == 0) {
    stage_expect<T>(bar, NT, 1);
    stage_T(smem, N, g.Bm, 4, Kp, k0, bar);
    stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
  }
  const bool active = k < g.K;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  if (t == 0) stage_T(smem, 0, tbuf, N, Kp, k0, bar);
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc), li.nc, sh);
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  T data[3] = {T(0), T(0), T(0)};
  if (g.cDV0T && active) {
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  }
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  if (!active || !ok) return;
  const Affine<T> af = affine_from<T>(srow<T>(smem, N)[t], srow<T>(smem, N + 1)[t],
                                      srow<T>(smem, N + 2)[t], srow<T>(smem, N + 3)[t]);
  T cT[N];
#pragma unroll
  for (int i = 0; i < N; ++i) cT[i] = srow<T>(smem, i)[t];
  const int dmask = (irow<T>(smem, NT, 0)[t] >> 9) & 7;
  limit_taylor<T, P, NQ, LT>(li, kv, sh, af, dmask, data, cT);
  T c[N];
  from_taylor<T, P>(cT, af, c);
  bool bad = false;
#pragma unroll
  for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = c[i]; bad |= !finite_(c[i]); }
  if (bad) atomicOr(sc.flag, 1);
}

// Modal state -> Taylor form and scatter of its centroid quantities (initial limiting).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_to_taylor(const Geo<T> g, const T *c, T *__restrict__ tbuf, const LimOut<T> lo,
            const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::totaylor();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 0, blockDim.x));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) { stage_expect<T>(bar, NT, 0); stage_T(smem, N, g.Bm, 4, Kp, k0, bar); }
  }
  const bool active = k < g.K;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k);
  if (!staged) return;
  if (t == 0) stage_T(smem, 0, c, N, Kp, k0, bar);
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T qv[NQ];
  if (active && ok) {
    const Affine<T> af = affine_from<T>(srow<T>(smem, N)[t], srow<T>(smem, N + 1)[t],
                                        srow<T>(smem, N + 2)[t], srow<T>(smem, N + 3)[t]);
    T cc[N], cT[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cc[i] = srow<T>(smem, i)[t];
    to_taylor<T, P>(cc, af, cT);
#pragma unroll
    for (int i = 0; i < N; ++i) tbuf[(size_t)i * Kp + k] = cT[i];
    centroid_quantities<T, P>(cT, lo.type, qv);
  }
  scatter_quantities<T, NQ>(g, lo, qv, vid, active && ok);
}

// Time-derivative limiting and SSP update for the linear limiter: cDot += Q_k du with
// Q_k = DM^-1 (S_k^-1 Mcorr_k S_k - I) (advection/solveSubStep.m:69-83), either read as
// precomputed rows or, with g.mtOnTheFly, applied from the element's B and the constant Gram
// table (taylor_mcorr; 4 staged rows instead of N(N-1)); the new stage value is written in the
// modal basis and its mean scattered for the solution limiter.
template <typename T, int P>
__device__ __forceinline__ void limit_dot_lin_tile(const Geo<T> g, const T *cin, const T *c0, const T *tbuf,
                T *out, const LimIn<T> li, const LimOut<T> lo, const StageScalars sc, const int tile,
                const int nTiles = -1) {
  constexpr int N = Dims<P>::N, NQ = 1;
  // staged rows: cDot, then N(N-1) rows of Q_k or the 4 rows of B, then c^n and c^(s-1)
  const bool fly = g.mtOnTheFly != 0;
  const int NT = StageRows<T, P>::limdot_lin_rows(fly);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  const int t = threadIdx.x, k0 = tile * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x) + 16);
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  const int rD = 0, rQ = N, rC0 = NT - 2 * N, rC = rC0 + N;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {
      stage_expect<T>(bar, NT, 1);
      if (fly) stage_T(smem, rQ, g.Bm, 4, Kp, k0, bar);
      else stage_T(smem, rQ, g.MT, N * (N - 1), Kp, k0, bar);
      stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
    }
  }
  const bool active = k < g.K;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k, nTiles < 0 ? -1 : tile, nTiles);
  if (!staged) return;
  if (t == 0) {
    stage_T(smem, rD, (const T *)tbuf, N, Kp, k0, bar);
    stage_T(smem, rC0, c0, N, Kp, k0, bar);
    stage_T(smem, rC, cin, N, Kp, k0, bar);
  }
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc, tile), li.nc, sh);
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T q0 = T(0);
  bool bad = false;
  if (active && ok) {
    T cd[N], u[N], du[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cd[i] = srow<T>(smem, rD + i)[t];
    lin_u3<T, P>(cd, u);
    const int dmask = (irow<T>(smem, NT, 0)[t] >> 9) & 7;
    const T nan3[3] = {T(NAN), T(NAN), T(NAN)};
    if (lin_alpha_lazy<T, P, NQ>(li, kv, sh, u, cd, dmask, nan3, du)) {
      if (fly) {
        const Affine<T> af = affine_from<T>(srow<T>(smem, rQ)[t], srow<T>(smem, rQ + 1)[t],
                                            srow<T>(smem, rQ + 2)[t], srow<T>(smem, rQ + 3)[t]);
        SinvBlocks<T, P> si;
        sinv_blocks<T, P>(af, si);
        T m[N], z[N];
        taylor_mcorr<T, P>(si, du, m);               // Mcorr S du, Taylor coordinates
        z[0] = m[0] - du[0];                         // S^-1 Mcorr S du - du
#pragma unroll
        for (int dd = 1; dd <= P; ++dd) {
          const int off = dd * (dd + 1) / 2;
#pragma unroll
          for (int a = 0; a <= dd; ++a) {
            Acc<T> sz(T(0));
#pragma unroll
            for (int j = 0; j <= dd; ++j) sz.fma(si.b[dd][a][j], m[off + j]);
            z[off + a] = sz.get() - du[off + a];
          }
        }
        const Tab<T, P> &tbl = tab<T, P>();
#pragma unroll
        for (int i = 0; i < N; ++i) {
          Acc<T> s(cd[i]);
#pragma unroll
          for (int j = 0; j < N; ++j) s.fma(tbl.DMinv[i][j], z[j]);
          cd[i] = s.get();
        }
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          Acc<T> s(cd[i]);
#pragma unroll
          for (int j = 1; j < N; ++j) s.fma(srow<T>(smem, rQ + i * (N - 1) + (j - 1))[t], du[j]);
          cd[i] = s.get();
        }
      }
    }
    const T w = T(sc.omega), tau = T(sc.tau);
    T cnew[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
      cnew[i] = w * srow<T>(smem, rC0 + i)[t] + (T(1) - w) * (srow<T>(smem, rC + i)[t] + tau * cd[i]);
#pragma unroll
    for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cnew[i]; bad |= !finite_(cnew[i]); }
    q0 = lin_mean<T, P>(cnew);
  }
  scatter_quantities<T, NQ>(g, lo, &q0, vid, active && ok, tile);
  if (bad) atomicOr(sc.flag, 1);
}
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit_dot_lin(const Geo<T> g, const T *cin, const T *c0, const T *tbuf,
                T *out, const LimIn<T> li, const LimOut<T> lo, const StageScalars sc) {
  limit_dot_lin_tile<T, P>(g, cin, c0, tbuf, out, li, lo, sc, blockIdx.x);
}

// Solution limiter for the linear limiter (core/applySlopeLimiterDisc.m:77-86 without the
// Taylor round trip): c <- c - DM^-1 du.
template <typename T, int P>
__device__ __forceinline__ void limit_lin_tile(const Geo<T> g, const T *cbuf, T *out, const LimIn<T> li,
            const StageScalars sc, const int tile) {
  constexpr int N = Dims<P>::N, NQ = 1;
  const Tab<T, P> &tb = tab<T, P>();
  __shared__ T sh[2];
  const int t = threadIdx.x, k = tile * kBlock + t;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0}, dmask = 0;
  if (active) {
    vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k];
    dmask = (g.code[k] >> 9) & 7;
  }
  T data[3] = {T(0), T(0), T(0)};
  if (g.cDV0T && active) {
    for (int m = 0; m < g.nTerms; ++m) {
      const T gm = T(sc.gco[m]);
#pragma unroll
      for (int n = 0; n < 3; ++n) data[n] += gm * g.cDV0T[((size_t)m * 3 + n) * Kp + k];
    }
  }
  pdl_wait();
  if (li.shift) load_shifts<T>(li.slots + slot_base(g, li.nc, tile), li.nc, sh);
  T c[N];
#pragma unroll
  for (int i = 0; i < N; ++i) c[i] = active ? cbuf[(size_t)i * Kp + k] : T(0);
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  T u[N], du[N];
  lin_u3<T, P>(c, u);
  if (lin_alpha<T, P, NQ>(li, kv, sh, u, dmask, data, du)) {
    // limited: u - du is the linear Taylor polynomial (u_0, alpha u_1, alpha u_2); back in the
    // modal basis that is the first three columns of DM^-1 (3N multiply-adds instead of the
    // rows u_3.. and DM^-1 du, N(N-1) + 3(N-3))
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc<T> s(T(0));
      s.fma(tb.DMinv[i][0], u[0]);
      if constexpr (N > 1) {
        s.fma(tb.DMinv[i][1], u[1] - du[1]);
        s.fma(tb.DMinv[i][2], u[2] - du[2]);
      }
      c[i] = s.get();
    }
  }
  bool bad = false;
#pragma unroll
  for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = c[i]; bad |= !finite_(c[i]); }
  if (bad) atomicOr(sc.flag, 1);
}
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit_lin(const Geo<T> g, const T *cbuf, T *out, const LimIn<T> li,
            const StageScalars sc) {
  limit_lin_tile<T, P>(g, cbuf, out, li, sc, blockIdx.x);
}

// Mean of the modal state scattered to the vertices (initial limiting, linear limiter); with
// meanOut the means are also stored per element (the limiter adjoint looks up extremes there).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_mean_lin(const Geo<T> g, const T *c, const LimOut<T> lo, T *__restrict__ meanOut) {
  constexpr int N = Dims<P>::N;
  const int t = threadIdx.x, k = blockIdx.x * kBlock + t;
  pdl_trigger();
  const bool active = k < g.K;
  const int Kp = g.Kp;
  int vid[3] = {0, 0, 0};
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
  pdl_wait();
  reset_next<T>(g, lo, k);
  T q0 = T(0);
  if (active) {
    T cc[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cc[i] = c[(size_t)i * Kp + k];
    q0 = lin_mean<T, P>(cc);
    if (meanOut) meanOut[k] = q0;
  }
  scatter_quantities<T, 1>(g, lo, &q0, vid, active);
}

// ---------------------------------------------------------------------------------------------
// Stage operator fused with the previous pass's solution limiter (linear limiter, zero
// Dirichlet data).  The input x is the unlimited stage value (limitIn = 1), or, in the first
// stage of a call, the limited state itself (limitIn = 0).  Each element limits
// its own coefficients and those of the three neighbours it gathers for the flux, each with its
// own vertex patches (core/applySlopeLimiterDisc.m:77-86 applied where the value is used instead
// of in a separate pass), then
//   MODE 1: writes the new unlimited stage value (SSP update, advection/solveSubStep.m:83),
//   MODE 2: writes cDot for the time-derivative limiter,
// and scatters the mean of what it wrote for the next limiter pass.  xLout receives the limited
// own input where later kernels need it (the limited c^n, or c^(s-1) for the SSP update).
template <typename T, int P>
__device__ __forceinline__ void lin_limit_inplace(const LimIn<T> &li, const VKeys<T, 1> &kv, const T *sh,
                                                  int dmask, T *c) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T u[N], du[N];
  lin_u3<T, P>(c, u);
  const T zero3[3] = {T(0), T(0), T(0)};
  if (lin_alpha<T, P, 1>(li, kv, sh, u, dmask, zero3, du)) {   // as limit_lin_tile
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc<T> s(T(0));
      s.fma(tb.DMinv[i][0], u[0]);
      if constexpr (N > 1) {
        s.fma(tb.DMinv[i][1], u[1] - du[1]);
        s.fma(tb.DMinv[i][2], u[2] - du[2]);
      }
      c[i] = s.get();
    }
  }
}

template <typename T, int P, int MODE, bool RHS>
__global__ void __launch_bounds__(kBlock)
k_op_fused(const Geo<T> g, const T *x, int limitIn, T *xLout,
           const T *c0L, int firstStage, T *out, const LimIn<T> li,
           const LimOut<T> lo, const StageScalars sc) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  constexpr int NT = StageRows<T, P>::op(MODE, true);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x));
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1, blockDim.x) + 16);
  const Tab<T, P> &tb = tab<T, P>();
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  constexpr int rC = 0, rC0 = N, rF = (MODE != 2) ? 2 * N : N, rV = rF + 2 * Q;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {
      stage_expect<T>(bar, NT - ((MODE == 1 && firstStage) ? N : 0), 1);
      stage_T(smem, rF, g.F, 2 * Q, Kp, k0, bar);
      stage_T(smem, rV, g.Vn, 3 * R, Kp, k0, bar);
      stage_I<T>(smem, NT, 0, g.code, 1, Kp, k0, bar);
    }
  }
  const bool active = k < g.K;
  // static connectivity before the dependency wait: neighbours, their boundary bits and the
  // vertex of each neighbour opposite the shared edge
  int nb[3], nbc[3], v3[3];
  int vid[3] = {0, 0, 0};
  const int myCode = active ? g.code[k] : 0;
  if (active) { vid[0] = g.V0T[k]; vid[1] = g.V0T[Kp + k]; vid[2] = g.V0T[2 * Kp + k]; }
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    nb[n] = active ? g.nbr[(size_t)n * Kp + k] : -1;
    const int np = (myCode >> (2 * n)) & 3;
    nbc[n] = nb[n] >= 0 ? g.code[nb[n]] : 0;
    v3[n] = nb[n] >= 0 ? g.V0T[(size_t)np * Kp + nb[n]] : 0;
  }
  pdl_wait();
  reset_next<T>(g, lo, k);
  if (!staged) return;
  if (t == 0) {
    stage_T(smem, rC, x, N, Kp, k0, bar);
    if (MODE == 1 && !firstStage) stage_T(smem, rC0, c0L, N, Kp, k0, bar);
  }
  // neighbour coefficients: outside the block from global memory now, inside from shared later
  T cn[3][N];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const bool outside = nb[n] >= 0 && (nb[n] < k0 || nb[n] >= k0 + kBlock);
#pragma unroll
    for (int j = 0; j < N; ++j) cn[n][j] = outside ? x[(size_t)j * Kp + nb[n]] : T(0);
  }
  // vertex keys of the own element and of each neighbour (two vertices shared with the edge)
  VKeys<T, 1> kvOwn, kvNb[3];
  load_vkeys<T, 1>(g, li, vid, kvOwn);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const int np = (myCode >> (2 * n)) & 3;
    const typename KeyOf<T>::type k3min = li.vkeys[v3[n]], k3max = li.vkeys[(size_t)g.Vp + v3[n]];
    // neighbour's local vertex np is opposite the shared edge; np+1 is our n+2, np+2 our n+1
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const int mm = (m + 3 - np) % 3;
      const int ours = mm == 1 ? (n + 2) % 3 : (n + 1) % 3;
      kvNb[n].v[0][0][m] = mm == 0 ? k3min : kvOwn.v[0][0][ours];
      kvNb[n].v[0][1][m] = mm == 0 ? k3max : kvOwn.v[0][1][ours];
    }
  }
  if (li.shift && limitIn) load_shifts<T>(li.slots + slot_base(g, li.nc), li.nc, sh);
  __syncthreads();
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T q0 = T(0);
  bool bad = false;
  if (active && ok) {
    T c[N];
    Acc<T> rhs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) { c[i] = srow<T>(smem, rC + i)[t]; rhs[i] = Acc<T>(T(0)); }
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (nb[n] >= k0 && nb[n] < k0 + kBlock)
#pragma unroll
        for (int j = 0; j < N; ++j) cn[n][j] = srow<T>(smem, rC + j)[nb[n] - k0];
    if (limitIn) {
      lin_limit_inplace<T, P>(li, kvOwn, sh, (myCode >> 9) & 7, c);
#pragma unroll
      for (int n = 0; n < 3; ++n)
        if (nb[n] >= 0) lin_limit_inplace<T, P>(li, kvNb[n], sh, (nbc[n] >> 9) & 7, cn[n]);
    }
    if (xLout) {
#pragma unroll
      for (int i = 0; i < N; ++i) xLout[(size_t)i * Kp + k] = c[i];
    }
    if (RHS) {
      for (int m = 0; m < g.nTerms; ++m) {
        const T gm = T(sc.gco[m]);
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i].fma(gm, g.rhs[((size_t)m * N + i) * Kp + k]);
      }
    }
#pragma unroll
    for (int qq = 0; qq < Q; ++qq) {
      Acc<T> cqa(T(0));
#pragma unroll
      for (int j = 0; j < N; ++j) cqa.fma(tb.phiQ[qq][j], c[j]);
      const T cq = cqa.get();
      const T f1 = srow<T>(smem, rF + qq)[t] * cq;
      const T f2 = srow<T>(smem, rF + Q + qq)[t] * cq;
#pragma unroll
      for (int i = 0; i < N; ++i) { rhs[i].fma(tb.g1[qq][i], f1); rhs[i].fma(tb.g2[qq][i], f2); }
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int np = (myCode >> (2 * n)) & 3;
      const bool outOk = (myCode >> (6 + n)) & 1;
#pragma unroll
      for (int r2 = 0; r2 < R; ++r2) {
        const T v = srow<T>(smem, rV + n * R + r2)[t];
        Acc<T> tr(T(0));
        if (v > T(0) && outOk) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(tb.phi1D[n][r2][j], c[j]);
        } else if (v < T(0) && nb[n] >= 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr.fma(tb.thetaPhi[n][np][r2][j], cn[n][j]);
        }
        const T fl = v * tr.get();
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i].fms(tb.phi1D[n][r2][i], fl);
      }
    }
    T cdot[N];
    if (sizeof(T) == 8) {
      T r[N];
#pragma unroll
      for (int j = 0; j < N; ++j) r[j] = rhs[j].get();
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc<T> s(T(0));
#pragma unroll
        for (int j = 0; j < N; ++j) s.fma(tb.hatMinv[i][j], r[j]);
        cdot[i] = s.get();
      }
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) cdot[i] = rhs[i].get();
    }
    if (MODE == 2) {
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cdot[i]; bad |= !finite_(cdot[i]); }
      q0 = lin_mean<T, P>(cdot);
    } else {
      const T w = T(sc.omega), tau = T(sc.tau);
      T cnew[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const T c0v = firstStage ? c[i] : srow<T>(smem, rC0 + i)[t];
        cnew[i] = w * c0v + (T(1) - w) * (c[i] + tau * cdot[i]);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = cnew[i]; bad |= !finite_(cnew[i]); }
      q0 = lin_mean<T, P>(cnew);
    }
  }
  scatter_quantities<T, 1>(g, lo, &q0, vid, active && ok);
  if (bad) atomicOr(sc.flag, 1);
}

// External (caller order, K x N column-major, FP64) <-> internal (SoA, stride Kp, precision T).
template <typename T>
__global__ void k_scatter_in(int K, int Kp, int N, const int *__restrict__ perm,
                             const double *__restrict__ ext, T *__restrict__ c) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const int e = perm[k];
  for (int i = 0; i < N; ++i) c[(size_t)i * Kp + k] = T(ext[(size_t)i * K + e]);
}
template <typename T>
__global__ void k_gather_out(int K, int Kp, int N, const int *__restrict__ perm,
                             const T *__restrict__ c, double *__restrict__ ext) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const int e = perm[k];
  for (int i = 0; i < N; ++i) ext[(size_t)i * K + e] = double(c[(size_t)i * Kp + k]);
}

template <typename T>
__global__ void k_from_f64(size_t n, const double *__restrict__ src, T *__restrict__ dst) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = T(src[i]);
}

}  // namespace dgadv
