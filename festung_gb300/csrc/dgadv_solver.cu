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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/dgadv.h"
#include "dgadv_host.h"
#include "dgadv_kernels.cuh"

namespace dgadv {

// ---------------------------------------------------------------------------------------------
// Constant tables, one instance per (precision, degree).
__constant__ Tab<double, 0> cTd0;
__constant__ Tab<double, 1> cTd1;
__constant__ Tab<double, 2> cTd2;
__constant__ Tab<double, 3> cTd3;
__constant__ Tab<float, 0> cTf0;
__constant__ Tab<float, 1> cTf1;
__constant__ Tab<float, 2> cTf2;
__constant__ Tab<float, 3> cTf3;

template <typename T, int P> __device__ __forceinline__ const Tab<T, P> &tab();
template <> __device__ __forceinline__ const Tab<double, 0> &tab<double, 0>() { return cTd0; }
template <> __device__ __forceinline__ const Tab<double, 1> &tab<double, 1>() { return cTd1; }
template <> __device__ __forceinline__ const Tab<double, 2> &tab<double, 2>() { return cTd2; }
template <> __device__ __forceinline__ const Tab<double, 3> &tab<double, 3>() { return cTd3; }
template <> __device__ __forceinline__ const Tab<float, 0> &tab<float, 0>() { return cTf0; }
template <> __device__ __forceinline__ const Tab<float, 1> &tab<float, 1>() { return cTf1; }
template <> __device__ __forceinline__ const Tab<float, 2> &tab<float, 2>() { return cTf2; }
template <> __device__ __forceinline__ const Tab<float, 3> &tab<float, 3>() { return cTf3; }

constexpr int kBlock = 128;
constexpr int kSlotCopies = 32;   // copies of the global min / max slots (atomics spread over them)

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
    T s = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) s += tb.DM[i][j] * c[j];
    u[i] = s;
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
      for (int m = 0; m <= 1; ++m) { T s = 0;
#pragma unroll
        for (int j = 0; j <= 1; ++j) s += S[m][j] * u[off + j]; cT[off + m] = s * sc; }
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m) { T s = 0;
#pragma unroll
        for (int j = 0; j <= 2; ++j) s += S[m][j] * u[off + j]; cT[off + m] = s * sc; }
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.A11, af.A21, af.A12, af.A22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m) { T s = 0;
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
      for (int m = 0; m <= 1; ++m) { T s = 0;
#pragma unroll
        for (int j = 0; j <= 1; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    } else if (d == 2) {
      T S[3][3]; deriv_block<T, 2>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 2; ++m) { T s = 0;
#pragma unroll
        for (int j = 0; j <= 2; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    } else if (d == 3) {
      T S[4][4]; deriv_block<T, 3>(af.B11, af.B21, af.B12, af.B22, S);
#pragma unroll
      for (int m = 0; m <= 3; ++m) { T s = 0;
#pragma unroll
        for (int j = 0; j <= 3; ++j) s += S[m][j] * cT[off + j]; w[off + m] = s * sc; }
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    T s = 0;
#pragma unroll
    for (int j = 0; j < N; ++j) s += tb.DMinv[i][j] * w[j];
    c[i] = s;
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

__device__ __forceinline__ unsigned int okey32(float x) { return (unsigned int)okey(x); }
__device__ __forceinline__ unsigned int vkey(float x) { return okey32(x); }
__device__ __forceinline__ unsigned long long vkey(double x) { return okey(x); }
template <typename T> __device__ __forceinline__ T vkey_inv(typename KeyOf<T>::type k) { return okey_inv<T>(k); }
template <typename T> __host__ __device__ constexpr typename KeyOf<T>::type vkey_max() {
  return (typename KeyOf<T>::type)key_max<T>();
}

template <typename T> struct LimOut {
  typename KeyOf<T>::type *vkeys;   // nc x 2 x Vp vertex min / max keys of this pass
  typename KeyOf<T>::type *vreset;  // the next pass's vertex keys, reset here
  unsigned long long *slots;        // kSlotCopies x 2 x nc encoded global min / max (atomic)
  unsigned long long *reset;        // slots of the next pass, reset by block 0
  int nc, type;
};
template <typename T> struct LimIn {
  const typename KeyOf<T>::type *vkeys;
  const unsigned long long *slots;  // kSlotCopies x 2 x nc
  int nc, type, shift;
};

// Scatter of the element's centroid quantities to its vertices and the block's global extremes.
template <typename T, int NQ>
__device__ __forceinline__ void scatter_quantities(const Geo<T> &g, const LimOut<T> &lo, const T *qv,
                                                   const int vid[3], bool active) {
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
    for (int w = 1; w < kBlock / 32; ++w) { mn = fmin(mn, red[w][2 * s]); mx = fmax(mx, red[w][2 * s + 1]); }
    if (mn <= mx) {
      unsigned long long *sl = lo.slots + (size_t)(blockIdx.x % kSlotCopies) * 2 * lo.nc;
      atomicMin(&sl[2 * s], okey(mn));
      atomicMax(&sl[2 * s + 1], okey(mx));
    }
  }
}

// Reset of the next pass's vertex keys (thread t owns vertex t) and global slots (block 0).
template <typename T>
__device__ __forceinline__ void reset_next(const Geo<T> &g, const LimOut<T> &lo, int t) {
  if (t < g.numV)
    for (int s = 0; s < lo.nc; ++s) {
      lo.vreset[(size_t)(2 * s) * g.Vp + t] = vkey_max<T>();
      lo.vreset[(size_t)(2 * s + 1) * g.Vp + t] = 0;
    }
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < kSlotCopies * 2 * lo.nc; i += blockDim.x)
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

// alpha of one computeVertexBasedLimiter call (core/computeVertexBasedLimiter.m:78-106)
template <typename T>
__device__ __forceinline__ T vertex_alpha(T cbar, const T v[3], const T mn[3], const T mx[3]) {
  const T tol = T(1.e-8);
  T alpha = T(1);
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const T dV = v[n] - cbar, dMin = mn[n] - cbar, dMax = mx[n] - cbar;
    T a = T(1);
    if (dV < dMin + tol) a = fmax(T(0), fmin(T(1), dMin / (dV - tol)));
    if (dV > dMax - tol) a = fmax(T(0), fmin(T(1), dMax / (dV + tol)));
    alpha = (n == 0) ? a : fmin(alpha, a);
  }
  return alpha;
}

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
      atomicOr(flag, 2);
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
    bulk_g2s(smem + (size_t)(row + r) * kBlock * sizeof(T), base + (size_t)r * Kp + k0, kBlock * sizeof(T), bar);
}
template <typename T>
__device__ __forceinline__ void stage_I(unsigned char *smem, int nT, int row, const int *base, int nrows, int Kp,
                                        int k0, uint64_t *bar) {
  for (int r = 0; r < nrows; ++r)
    bulk_g2s(smem + (size_t)nT * kBlock * sizeof(T) + (size_t)(row + r) * kBlock * sizeof(int),
             base + (size_t)r * Kp + k0, kBlock * sizeof(int), bar);
}
template <typename T>
__device__ __forceinline__ void stage_expect(uint64_t *bar, int nT, int nI) {
  mbar_expect_tx(bar, nT * kBlock * (uint32_t)sizeof(T) + nI * kBlock * (uint32_t)sizeof(int));
}

// Programmatic dependent launch: the next kernel in the stream may start its prologue (static
// data only) once every block of this one has started; pdl_wait() blocks until the previous
// kernel has completed and its writes are visible.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename T> __device__ __forceinline__ const T *srow(const unsigned char *smem, int r) {
  return (const T *)(smem + (size_t)r * kBlock * sizeof(T));
}
template <typename T> __device__ __forceinline__ const int *irow(const unsigned char *smem, int nT, int r) {
  return (const int *)(smem + (size_t)nT * kBlock * sizeof(T) + (size_t)r * kBlock * sizeof(int));
}

template <typename T, int P> struct StageRows {
  static constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R, NMT = Dims<P>::NMT;
  // k_stage_op: c, [c0], F, Vn, [B] | code
  __host__ __device__ static constexpr int op(int mode, bool lin) {
    return N + (mode != 2 ? N : 0) + 2 * Q + 3 * R + (mode != 0 && !lin ? 4 : 0);
  }
  // k_limit_dot: tbuf, B, MT, c0, cin | code
  __host__ __device__ static constexpr int limdot() { return N + 4 + NMT + 2 * N; }
  // k_limit: tbuf, B | code
  __host__ __device__ static constexpr int lim() { return N + 4; }
  // k_limit_dot_lin: cDot, Q (N x (N-1)), c0, cin | code
  __host__ __device__ static constexpr int limdot_lin() { return N + N * (N - 1) + 2 * N; }
  // k_to_taylor: c, B
  __host__ __device__ static constexpr int totaylor() { return N + 4; }
  // rows first, then the block's mbarrier (8 bytes, 16 reserved)
  __host__ __device__ static constexpr size_t bar_offset(int nT, int nI) {
    return (size_t)nT * kBlock * sizeof(T) + (size_t)nI * kBlock * sizeof(int);
  }
  // + 16 for the mbarrier, + 2 x 6 shift values
  __host__ __device__ static constexpr size_t bytes(int nT, int nI) { return bar_offset(nT, nI) + 16 + 12 * sizeof(T); }
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
  T sNeg = 0, sPos = 0;
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
template <typename T, int P, int NQ>
__device__ __forceinline__ void limit_taylor(const LimIn<T> &li, const VKeys<T, NQ> &kv, const T *sh,
                                             const Affine<T> &af, int dmask, const T dataV0T[3], T *cT) {
  constexpr int N = Dims<P>::N;
  const T nan_ = T(NAN);
  T pt1[3], pt2[3];   // Taylor basis functions 2 and 3 at the vertices
#pragma unroll
  for (int n = 0; n < 3; ++n) { pt1[n] = af.ox[n] * af.dX; pt2[n] = af.oy[n] * af.dX; }
  if (li.type == 0) {
    T v[3], valD[3], mn[3], mx[3];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      v[n] = (cT[0] * T(1) + cT[1] * pt1[n]) + cT[2] * pt2[n];
      valD[n] = ((dmask >> n) & 1) ? dataV0T[n] : nan_;
    }
    patch_minmax<T, NQ>(li, kv, sh, 0, valD, mn, mx);
    const T alpha = vertex_alpha(cT[0], v, mn, mx);
    cT[1] *= alpha; cT[2] *= alpha;
    const T keep = (alpha == T(1)) ? T(1) : T(0);
#pragma unroll
    for (int i = 3; i < N; ++i) cT[i] *= keep;
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
        aOrd = fmin(aOrd, vertex_alpha(orig[i0], v, mn, mx));
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
    T s = T(0);
#pragma unroll
    for (int j = 0; j < N; ++j) s += tb.DM[i][j] * c[j];
    u[i] = s;
  }
}
template <typename T, int P> __device__ __forceinline__ T lin_mean(const T *c) {
  constexpr int N = Dims<P>::N;
  const Tab<T, P> &tb = tab<T, P>();
  T s = T(0);
#pragma unroll
  for (int j = 0; j < N; ++j) s += tb.DM[0][j] * c[j];
  return s;
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
  const T alpha = vertex_alpha(u[0], v, mn, mx);
  if (alpha == T(1)) return false;
  du[0] = T(0);
  du[1] = (T(1) - alpha) * u[1];
  du[2] = (T(1) - alpha) * u[2];
#pragma unroll
  for (int i = 3; i < N; ++i) du[i] = u[i];
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

template <typename T, int P, int MODE, bool RHS, bool LIN>
__global__ void __launch_bounds__(kBlock)
k_stage_op(const Geo<T> g, const T *__restrict__ cin, const T *__restrict__ c0, T *__restrict__ out,
           const LimOut<T> lo, const StageScalars sc) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::op(MODE, LIN);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1));
  const Tab<T, P> &tb = tab<T, P>();
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;                   // blocks beyond the elements only reset keys
  constexpr int rC = 0, rC0 = N, rF = (MODE != 2) ? 2 * N : N, rV = rF + 2 * Q, rB = rV + 3 * R;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {                                 // static rows before the dependency wait
      stage_expect<T>(bar, NT, 1);
      stage_T(smem, rF, g.F, 2 * Q, Kp, k0, bar);
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
  if (MODE != 0) reset_next<T>(g, lo, k);
  if (!staged) return;
  if (t == 0) {                                   // state rows after it
    stage_T(smem, rC, cin, N, Kp, k0, bar);
    if (MODE != 2) stage_T(smem, rC0, c0, N, Kp, k0, bar);
  }
  // neighbour coefficients: outside the block from global memory now, inside from shared later
  T cn[3][N];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    const bool outside = nb[n] >= 0 && (nb[n] < k0 || nb[n] >= k0 + kBlock);
#pragma unroll
    for (int j = 0; j < N; ++j) cn[n][j] = outside ? cin[(size_t)j * Kp + nb[n]] : T(0);
  }
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T qv[NQ];
  bool bad = false;
  if (active && ok) {
    T c[N], rhs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) { c[i] = srow<T>(smem, rC + i)[t]; rhs[i] = T(0); }
#pragma unroll
    for (int n = 0; n < 3; ++n)
      if (nb[n] >= k0 && nb[n] < k0 + kBlock)
#pragma unroll
        for (int j = 0; j < N; ++j) cn[n][j] = srow<T>(smem, rC + j)[nb[n] - k0];
    if (RHS) {
      for (int m = 0; m < g.nTerms; ++m) {
        const T gm = T(sc.gco[m]);
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i] += gm * g.rhs[((size_t)m * N + i) * Kp + k];
      }
    }
    // volume term
#pragma unroll
    for (int qq = 0; qq < Q; ++qq) {
      T cq = T(0);
#pragma unroll
      for (int j = 0; j < N; ++j) cq += tb.phiQ[qq][j] * c[j];
      const T f1 = srow<T>(smem, rF + qq)[t] * cq;
      const T f2 = srow<T>(smem, rF + Q + qq)[t] * cq;
#pragma unroll
      for (int i = 0; i < N; ++i) rhs[i] += tb.g1[qq][i] * f1 + tb.g2[qq][i] * f2;
    }
    // upwind edge term
    const int code = irow<T>(smem, NT, 0)[t];
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int np = (code >> (2 * n)) & 3;
      const bool outOk = (code >> (6 + n)) & 1;
#pragma unroll
      for (int r2 = 0; r2 < R; ++r2) {
        const T v = srow<T>(smem, rV + n * R + r2)[t];
        T tr = T(0);
        if (v > T(0) && outOk) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr += tb.phi1D[n][r2][j] * c[j];
        } else if (v < T(0) && nb[n] >= 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr += tb.thetaPhi[n][np][r2][j] * cn[n][j];
        }
        const T fl = v * tr;
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i] -= tb.phi1D[n][r2][i] * fl;
      }
    }
    // mass solve
    T cdot[N];
    if (sizeof(T) == 8) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < N; ++j) s += tb.hatMinv[i][j] * rhs[j];
        cdot[i] = s;
      }
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) cdot[i] = rhs[i];
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
      for (int i = 0; i < N; ++i) cnew[i] = w * srow<T>(smem, rC0 + i)[t] + (T(1) - w) * (c[i] + tau * cdot[i]);
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
  if (MODE != 0) scatter_quantities<T, NQ>(g, lo, qv, vid, active && ok);
  if (bad) atomicOr(sc.flag, 1);
}

// Time-derivative limiting and SSP update (advection/solveSubStep.m:69-83), then the Taylor
// form of the new stage value and the scatter of its centroid quantities for the solution
// limiter.
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit_dot(const Geo<T> g, const T *__restrict__ cin, const T *__restrict__ c0, T *__restrict__ tbuf,
            const LimIn<T> li, const LimOut<T> lo, const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value, NMT = Dims<P>::NMT;
  constexpr int NT = StageRows<T, P>::limdot();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1) + 16);
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  constexpr int rT = 0, rB = N, rM = N + 4, rC0 = N + 4 + NMT, rC = rC0 + N;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {
      stage_expect<T>(bar, NT, 1);
      stage_T(smem, rB, g.Bm, 4, Kp, k0, bar);
      stage_T(smem, rM, g.MT, NMT, Kp, k0, bar);
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
    stage_T(smem, rT, (const T *)tbuf, N, Kp, k0, bar);
    stage_T(smem, rC0, c0, N, Kp, k0, bar);
    stage_T(smem, rC, cin, N, Kp, k0, bar);
  }
  if (li.shift) load_shifts<T>(li.slots, li.nc, sh);
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
    limit_taylor<T, P, NQ>(li, kv, sh, af, dmask, nan3, lim);
    // Taylor mass correction M_corr = diag(1/diag(M_T)) M_T applied to (cT - lim)
    T d[N];
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = cT[i] - lim[i];
    T cor[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T s = T(0), dii = T(1);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const int a = i < j ? i : j, b = i < j ? j : i;
        const int idx = a * N - a * (a - 1) / 2 + (b - a);
        const T m = srow<T>(smem, rM + idx)[t];
        s += m * d[j];
        if (j == i) dii = m;
      }
      cor[i] = lim[i] + s / dii;
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
    for (int i = 0; i < N; ++i) { tbuf[(size_t)i * Kp + k] = cT2[i]; bad |= !finite_(cT2[i]); }
    centroid_quantities<T, P>(cT2, lo.type, qv);
  }
  scatter_quantities<T, NQ>(g, lo, qv, vid, active && ok);
  if (bad) atomicOr(sc.flag, 1);
}

// Solution limiter: limited Taylor coefficients back to the modal basis
// (core/applySlopeLimiterDisc.m:77-86).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit(const Geo<T> g, const T *__restrict__ tbuf, T *__restrict__ out, const LimIn<T> li,
        const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::lim();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1) + 16);
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
  if (li.shift) load_shifts<T>(li.slots, li.nc, sh);
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
  limit_taylor<T, P, NQ>(li, kv, sh, af, dmask, data, cT);
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
k_to_taylor(const Geo<T> g, const T *__restrict__ c, T *__restrict__ tbuf, const LimOut<T> lo,
            const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = NCQ<P>::value;
  constexpr int NT = StageRows<T, P>::totaylor();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 0));
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

// Time-derivative limiting and SSP update for the linear limiter: cDot += Q_k du with the
// precomputed Q_k = DM^-1 (S_k^-1 Mcorr_k S_k - I) (advection/solveSubStep.m:69-83); the new
// stage value is written in the modal basis and its mean scattered for the solution limiter.
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit_dot_lin(const Geo<T> g, const T *__restrict__ cin, const T *__restrict__ c0, const T *__restrict__ tbuf,
                T *__restrict__ out, const LimIn<T> li, const LimOut<T> lo, const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = 1;
  constexpr int NT = StageRows<T, P>::limdot_lin();
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1));
  const int t = threadIdx.x, k0 = blockIdx.x * kBlock, k = k0 + t;
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1) + 16);
  pdl_trigger();
  const int Kp = g.Kp;
  const bool staged = k0 < g.K;
  constexpr int rD = 0, rQ = N, rC0 = N + N * (N - 1), rC = rC0 + N;
  if (staged) {
    if (t == 0) { mbar_init(bar, 1); mbar_fence_init(); }
    __syncthreads();
    if (t == 0) {
      stage_expect<T>(bar, NT, 1);
      stage_T(smem, rQ, g.MT, N * (N - 1), Kp, k0, bar);
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
    stage_T(smem, rD, (const T *)tbuf, N, Kp, k0, bar);
    stage_T(smem, rC0, c0, N, Kp, k0, bar);
    stage_T(smem, rC, cin, N, Kp, k0, bar);
  }
  if (li.shift) load_shifts<T>(li.slots, li.nc, sh);
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
    lin_u<T, P>(cd, u);
    const int dmask = (irow<T>(smem, NT, 0)[t] >> 9) & 7;
    const T nan3[3] = {T(NAN), T(NAN), T(NAN)};
    if (lin_alpha<T, P, NQ>(li, kv, sh, u, dmask, nan3, du)) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T s = T(0);
#pragma unroll
        for (int j = 1; j < N; ++j) s += srow<T>(smem, rQ + i * (N - 1) + (j - 1))[t] * du[j];
        cd[i] += s;
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
  scatter_quantities<T, NQ>(g, lo, &q0, vid, active && ok);
  if (bad) atomicOr(sc.flag, 1);
}

// Solution limiter for the linear limiter (core/applySlopeLimiterDisc.m:77-86 without the
// Taylor round trip): c <- c - DM^-1 du.
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_limit_lin(const Geo<T> g, const T *__restrict__ cbuf, T *__restrict__ out, const LimIn<T> li,
            const StageScalars sc) {
  constexpr int N = Dims<P>::N, NQ = 1;
  const Tab<T, P> &tb = tab<T, P>();
  __shared__ T sh[2];
  const int t = threadIdx.x, k = blockIdx.x * kBlock + t;
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
  if (li.shift) load_shifts<T>(li.slots, li.nc, sh);
  T c[N];
#pragma unroll
  for (int i = 0; i < N; ++i) c[i] = active ? cbuf[(size_t)i * Kp + k] : T(0);
  VKeys<T, NQ> kv;
  load_vkeys<T, NQ>(g, li, vid, kv);
  __syncthreads();
  if (!active) return;
  T u[N], du[N];
  lin_u<T, P>(c, u);
  if (lin_alpha<T, P, NQ>(li, kv, sh, u, dmask, data, du)) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T s = T(0);
#pragma unroll
      for (int j = 1; j < N; ++j) s += tb.DMinv[i][j] * du[j];
      c[i] -= s;
    }
  }
  bool bad = false;
#pragma unroll
  for (int i = 0; i < N; ++i) { out[(size_t)i * Kp + k] = c[i]; bad |= !finite_(c[i]); }
  if (bad) atomicOr(sc.flag, 1);
}

// Mean of the modal state scattered to the vertices (initial limiting, linear limiter).
template <typename T, int P>
__global__ void __launch_bounds__(kBlock)
k_mean_lin(const Geo<T> g, const T *__restrict__ c, const LimOut<T> lo) {
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
  lin_u<T, P>(c, u);
  const T zero3[3] = {T(0), T(0), T(0)};
  if (lin_alpha<T, P, 1>(li, kv, sh, u, dmask, zero3, du)) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T s = T(0);
#pragma unroll
      for (int j = 1; j < N; ++j) s += tb.DMinv[i][j] * du[j];
      c[i] -= s;
    }
  }
}

template <typename T, int P, int MODE, bool RHS>
__global__ void __launch_bounds__(kBlock)
k_op_fused(const Geo<T> g, const T *__restrict__ x, int limitIn, T *__restrict__ xLout,
           const T *__restrict__ c0L, int firstStage, T *__restrict__ out, const LimIn<T> li,
           const LimOut<T> lo, const StageScalars sc) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  constexpr int NT = StageRows<T, P>::op(MODE, true);
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *bar = (uint64_t *)(smem + StageRows<T, P>::bar_offset(NT, 1));
  T *sh = (T *)(smem + StageRows<T, P>::bar_offset(NT, 1) + 16);
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
  if (li.shift && limitIn) load_shifts<T>(li.slots, li.nc, sh);
  __syncthreads();
  const bool ok = mbar_wait_bounded(bar, sc.flag);
  T q0 = T(0);
  bool bad = false;
  if (active && ok) {
    T c[N], rhs[N];
#pragma unroll
    for (int i = 0; i < N; ++i) { c[i] = srow<T>(smem, rC + i)[t]; rhs[i] = T(0); }
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
        for (int i = 0; i < N; ++i) rhs[i] += gm * g.rhs[((size_t)m * N + i) * Kp + k];
      }
    }
#pragma unroll
    for (int qq = 0; qq < Q; ++qq) {
      T cq = T(0);
#pragma unroll
      for (int j = 0; j < N; ++j) cq += tb.phiQ[qq][j] * c[j];
      const T f1 = srow<T>(smem, rF + qq)[t] * cq;
      const T f2 = srow<T>(smem, rF + Q + qq)[t] * cq;
#pragma unroll
      for (int i = 0; i < N; ++i) rhs[i] += tb.g1[qq][i] * f1 + tb.g2[qq][i] * f2;
    }
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const int np = (myCode >> (2 * n)) & 3;
      const bool outOk = (myCode >> (6 + n)) & 1;
#pragma unroll
      for (int r2 = 0; r2 < R; ++r2) {
        const T v = srow<T>(smem, rV + n * R + r2)[t];
        T tr = T(0);
        if (v > T(0) && outOk) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr += tb.phi1D[n][r2][j] * c[j];
        } else if (v < T(0) && nb[n] >= 0) {
#pragma unroll
          for (int j = 0; j < N; ++j) tr += tb.thetaPhi[n][np][r2][j] * cn[n][j];
        }
        const T fl = v * tr;
#pragma unroll
        for (int i = 0; i < N; ++i) rhs[i] -= tb.phi1D[n][r2][i] * fl;
      }
    }
    T cdot[N];
    if (sizeof(T) == 8) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < N; ++j) s += tb.hatMinv[i][j] * rhs[j];
        cdot[i] = s;
      }
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) cdot[i] = rhs[i];
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

}  // namespace dgadv

struct dgadv_handle {
  int device = 0;
  int K = 0, Kp = 0, numV = 0, Vp = 0, p = 0, N = 0, Q = 0, R = 0, ordRK = 1, prec = 0;
  int lim = 0, limType = 0, flags = 0, nc = 0;
  bool limdot = false;
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  // device arrays (element type depends on prec)
  void *F = nullptr, *Vn = nullptr, *Bm = nullptr, *MT = nullptr, *rhs = nullptr, *cDV0T = nullptr;
  int *nbr = nullptr, *code = nullptr, *V0T = nullptr, *vptr = nullptr, *vidx = nullptr, *perm = nullptr;
  void *cn = nullptr, *cA = nullptr, *cB = nullptr, *tbuf = nullptr;
  void *cR = nullptr, *cnL = nullptr, *cLx = nullptr;   // fused path: raw step output, limited c^n / c^(s-1)
  void *vkeys = nullptr;               // 3 passes x nc x 2 x Vp vertex min / max keys
  unsigned long long *gmm = nullptr;   // 3 passes x kSlotCopies x 2 x nc encoded global extremes
  long long limPass = 1;               // limiter passes enqueued so far (selects key / slot set)
  int passesPerStep = 0;
  int *flag = nullptr;
  double *stage_ext = nullptr;         // K x N staging for set/get state
  int nTerms = 0;
  int timeFn[4] = {0, 0, 0, 0};
  bool hasVelocity = false;
  // host copies needed later
  std::vector<double> detJ, areaE0T, Bhost;   // internal order
  std::vector<uint8_t> markNotN;              // internal order, 3 per element
  std::vector<int> permv;                     // internal -> external element id
  dgadv::RefTables tables;
  // CUDA graphs of a chunk of steps, one per phase (limPass mod 3) at the chunk start
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  bool profiling = false;
  std::vector<cudaEvent_t> profEvents;
  std::vector<int> profKinds;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double graphTau[3] = {-1.0, -1.0, -1.0};
  std::string err;
};

namespace dgadv {

static std::mutex g_tab_mutex;
static bool g_tab_loaded[64][2][kMaxP + 1];

template <typename T, int P>
static cudaError_t upload_tables(const RefTables &rt) {
  Tab<T, P> t;
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q, R = Dims<P>::R;
  for (int q = 0; q < Q; ++q)
    for (int i = 0; i < N; ++i) {
      t.phiQ[q][i] = T(rt.phiQ[q * N + i]);
      t.g1[q][i] = T(rt.gradQ[q * N + i]);
      t.g2[q][i] = T(rt.gradQ[Q * N + q * N + i]);
    }
  for (int n = 0; n < 3; ++n)
    for (int r = 0; r < R; ++r)
      for (int i = 0; i < N; ++i) t.phi1D[n][r][i] = T(rt.phi1D[(n * R + r) * N + i]);
  for (int nn = 0; nn < 3; ++nn)
    for (int np = 0; np < 3; ++np)
      for (int r = 0; r < R; ++r)
        for (int i = 0; i < N; ++i) t.thetaPhi[nn][np][r][i] = T(rt.thetaPhi[((nn * 3 + np) * R + r) * N + i]);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      t.hatMinv[i][j] = T(rt.hatMinv[i * N + j]);
      t.DM[i][j] = T(rt.DM[i * N + j]);
      t.DMinv[i][j] = T(rt.DMinv[i * N + j]);
    }
  const void *sym = nullptr;
  if (std::is_same<T, double>::value) {
    if (P == 0) sym = &cTd0; else if (P == 1) sym = &cTd1; else if (P == 2) sym = &cTd2; else sym = &cTd3;
  } else {
    if (P == 0) sym = &cTf0; else if (P == 1) sym = &cTf1; else if (P == 2) sym = &cTf2; else sym = &cTf3;
  }
  return cudaMemcpyToSymbol(sym, &t, sizeof(t));
}

template <typename T>
static Geo<T> make_geo(const dgadv_handle *h) {
  Geo<T> g;
  g.K = h->K; g.Kp = h->Kp; g.numV = h->numV; g.Vp = h->Vp;
  g.F = (const T *)h->F; g.Vn = (const T *)h->Vn; g.nbr = h->nbr; g.code = h->code;
  g.Bm = (const T *)h->Bm; g.MT = (const T *)h->MT; g.V0T = h->V0T; g.vptr = h->vptr; g.vidx = h->vidx;
  g.rhs = (const T *)h->rhs; g.cDV0T = (const T *)h->cDV0T; g.nTerms = h->nTerms;
  for (int i = 0; i < 4; ++i) g.timeFn[i] = h->timeFn[i];
  return g;
}

static double time_factor(int fn, double t) { return fn == DGADV_TIME_EXP_NEG ? std::exp(-t) : 1.0; }

// SSP-RK tables (core/rungeKuttaExplicit.m:64-78)
static int rk_table(int ord, double omega[3], double cstage[3]) {
  if (ord == 1) { omega[0] = 0; cstage[0] = 0; return 1; }
  if (ord == 2) { omega[0] = 0; omega[1] = 0.5; cstage[0] = 0; cstage[1] = 1; return 2; }
  omega[0] = 0; omega[1] = 3.0 / 4.0; omega[2] = 1.0 / 3.0;
  cstage[0] = 0; cstage[1] = 1; cstage[2] = 0.5;
  return 3;
}

template <typename T>
static LimOut<T> lim_out(dgadv_handle *h) {
  using K_ = typename KeyOf<T>::type;
  const int set = (int)(h->limPass % 3), next = (set + 1) % 3;
  const size_t vset = (size_t)2 * h->nc * h->Vp;
  LimOut<T> o;
  o.vkeys = (K_ *)h->vkeys + set * vset;
  o.vreset = (K_ *)h->vkeys + next * vset;
  o.slots = h->gmm + (size_t)set * kSlotCopies * 2 * h->nc;
  o.reset = h->gmm + (size_t)next * kSlotCopies * 2 * h->nc;
  o.nc = h->nc; o.type = h->limType;
  return o;
}
template <typename T>
static LimIn<T> lim_in_pass(const dgadv_handle *h, long long pass) {
  using K_ = typename KeyOf<T>::type;
  const int set = (int)(((pass % 3) + 3) % 3);
  LimIn<T> i;
  i.vkeys = (const K_ *)h->vkeys + (size_t)set * 2 * h->nc * h->Vp;
  i.slots = h->gmm + (size_t)set * kSlotCopies * 2 * h->nc;
  i.nc = h->nc; i.type = h->limType;
  i.shift = (h->flags & DGADV_FLAG_NO_SHIFT) ? 0 : 1;
  return i;
}

template <typename T>
static LimIn<T> lim_in(const LimOut<T> &o, const dgadv_handle *h) {
  LimIn<T> i;
  i.vkeys = o.vkeys; i.slots = o.slots; i.nc = o.nc; i.type = o.type;
  i.shift = (h->flags & DGADV_FLAG_NO_SHIFT) ? 0 : 1;
  return i;
}

// Optional per-kernel timing with CUDA events on the handle's stream (dgadv_profile_kernels).
static void prof_mark(dgadv_handle *h, int kind) {
  if (!h->profiling) return;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, h->stream);
  h->profEvents.push_back(e);
  h->profKinds.push_back(kind);
}

// Kernel launch on the handle's stream, with programmatic dependent launch unless disabled.
template <typename... KArgs, typename... Args>
static void launch_k(const dgadv_handle *h, void (*kern)(KArgs...), int grid, size_t smem, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = (h->flags & DGADV_FLAG_NO_PDL) ? 0 : 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

// Opt-in shared memory sizes of the staged kernels of one (precision, degree).
template <typename T, int P>
static cudaError_t set_smem_attributes() {
  using SR = StageRows<T, P>;
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, size_t b) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b);
  };
  set((const void *)k_stage_op<T, P, 0, true, false>, SR::bytes(SR::op(0, false), 1));
  set((const void *)k_stage_op<T, P, 0, false, false>, SR::bytes(SR::op(0, false), 1));
  set((const void *)k_stage_op<T, P, 1, true, false>, SR::bytes(SR::op(1, false), 1));
  set((const void *)k_stage_op<T, P, 1, false, false>, SR::bytes(SR::op(1, false), 1));
  set((const void *)k_stage_op<T, P, 2, true, false>, SR::bytes(SR::op(2, false), 1));
  set((const void *)k_stage_op<T, P, 2, false, false>, SR::bytes(SR::op(2, false), 1));
  set((const void *)k_stage_op<T, P, 1, true, true>, SR::bytes(SR::op(1, true), 1));
  set((const void *)k_stage_op<T, P, 1, false, true>, SR::bytes(SR::op(1, true), 1));
  set((const void *)k_stage_op<T, P, 2, true, true>, SR::bytes(SR::op(2, true), 1));
  set((const void *)k_stage_op<T, P, 2, false, true>, SR::bytes(SR::op(2, true), 1));
  set((const void *)k_limit_dot_lin<T, P>, SR::bytes(SR::limdot_lin(), 1));
  set((const void *)k_op_fused<T, P, 1, true>, SR::bytes(SR::op(1, true), 1));
  set((const void *)k_op_fused<T, P, 1, false>, SR::bytes(SR::op(1, true), 1));
  set((const void *)k_op_fused<T, P, 2, true>, SR::bytes(SR::op(2, true), 1));
  set((const void *)k_op_fused<T, P, 2, false>, SR::bytes(SR::op(2, true), 1));
  set((const void *)k_limit_dot<T, P>, SR::bytes(SR::limdot(), 1));
  set((const void *)k_limit<T, P>, SR::bytes(SR::lim(), 1));
  set((const void *)k_to_taylor<T, P>, SR::bytes(SR::totaylor(), 0));
  return e;
}

template <typename T, int P>
static cudaError_t launch_step(dgadv_handle *h, double t0, double tau) {
  using SR = StageRows<T, P>;
  const Geo<T> g = make_geo<T>(h);
  const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;   // producers also reset vertex keys
  const int gridK = (h->K + kBlock - 1) / kBlock;
  double omega[3], cst[3];
  const int S = rk_table(h->ordRK, omega, cst);
  T *cn = (T *)h->cn, *cA = (T *)h->cA, *cB = (T *)h->cB, *tb = (T *)h->tbuf;
  const bool rhs = h->nTerms > 0 && h->rhs;
  for (int s = 0; s < S; ++s) {
    T *in = (s == 0) ? cn : (s == 1 ? cA : cB);
    T *out = (s == S - 1) ? (S == 1 ? cA : cn) : (s == 0 ? cA : cB);
    StageScalars sc{};
    sc.omega = omega[s]; sc.tau = tau; sc.flag = h->flag;
    const double ts = t0 + cst[s] * tau;
    for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = time_factor(h->timeFn[m], ts);
    LimOut<T> lo{};
    if (!h->lim) {
      prof_mark(h, 0);
      if (rhs) launch_k(h, k_stage_op<T, P, 0, true, false>, grid, SR::bytes(SR::op(0, false), 1), g, in, cn, out, lo, sc);
      else launch_k(h, k_stage_op<T, P, 0, false, false>, grid, SR::bytes(SR::op(0, false), 1), g, in, cn, out, lo, sc);
      prof_mark(h, -1);
      continue;
    }
    // limiter boundary data at tBC = t(s+1) or t(1) + tau (advection/solveSubStep.m:88)
    const double tBC = (s + 1 < S) ? t0 + cst[s + 1] * tau : t0 + tau;
    StageScalars scBC = sc;
    for (int m = 0; m < h->nTerms; ++m) scBC.gco[m] = time_factor(h->timeFn[m], tBC);
    const bool lin = h->limType == DGADV_LIM_LINEAR;
    const LimOut<T> lo1 = lim_out<T>(h);
    ++h->limPass;
    const int mode = h->limdot ? 2 : 1;
    prof_mark(h, 0);
    if (mode == 2) {
      if (lin) {
        if (rhs) launch_k(h, k_stage_op<T, P, 2, true, true>, grid, SR::bytes(SR::op(2, true), 1), g, in, cn, tb, lo1, sc);
        else launch_k(h, k_stage_op<T, P, 2, false, true>, grid, SR::bytes(SR::op(2, true), 1), g, in, cn, tb, lo1, sc);
      } else {
        if (rhs) launch_k(h, k_stage_op<T, P, 2, true, false>, grid, SR::bytes(SR::op(2, false), 1), g, in, cn, tb, lo1, sc);
        else launch_k(h, k_stage_op<T, P, 2, false, false>, grid, SR::bytes(SR::op(2, false), 1), g, in, cn, tb, lo1, sc);
      }
    } else {
      if (lin) {
        if (rhs) launch_k(h, k_stage_op<T, P, 1, true, true>, grid, SR::bytes(SR::op(1, true), 1), g, in, cn, tb, lo1, sc);
        else launch_k(h, k_stage_op<T, P, 1, false, true>, grid, SR::bytes(SR::op(1, true), 1), g, in, cn, tb, lo1, sc);
      } else {
        if (rhs) launch_k(h, k_stage_op<T, P, 1, true, false>, grid, SR::bytes(SR::op(1, false), 1), g, in, cn, tb, lo1, sc);
        else launch_k(h, k_stage_op<T, P, 1, false, false>, grid, SR::bytes(SR::op(1, false), 1), g, in, cn, tb, lo1, sc);
      }
    }
    prof_mark(h, -1);
    LimOut<T> loS = lo1;
    if (mode == 2) {
      const LimOut<T> lo2 = lim_out<T>(h);
      ++h->limPass;
      prof_mark(h, 1);
      if (lin) launch_k(h, k_limit_dot_lin<T, P>, grid, SR::bytes(SR::limdot_lin(), 1), g, (const T *)in, (const T *)cn, (const T *)tb, tb, lim_in<T>(lo1, h), lo2, sc);
      else launch_k(h, k_limit_dot<T, P>, grid, SR::bytes(SR::limdot(), 1), g, in, cn, tb, lim_in<T>(lo1, h), lo2, sc);
      prof_mark(h, -1);
      loS = lo2;
    }
    prof_mark(h, 2);
    if (lin) launch_k(h, k_limit_lin<T, P>, gridK, (size_t)0, g, (const T *)tb, out, lim_in<T>(loS, h), scBC);
    else launch_k(h, k_limit<T, P>, grid, SR::bytes(SR::lim(), 1), g, (const T *)tb, out, lim_in<T>(loS, h), scBC);
    prof_mark(h, -1);
  }
  if (S == 1)
    cudaMemcpyAsync(cn, cA, (size_t)h->N * h->Kp * sizeof(T), cudaMemcpyDeviceToDevice, h->stream);
  return cudaGetLastError();
}

// Fused path (linear limiter, zero Dirichlet data): per stage the operator kernel limits its
// input on the fly; for p >= 2 the time-derivative limiter follows.  The state between calls
// stays limited in cn; inside a call the step output R is unlimited, and finalize_fused limits
// it back into cn at the end of the call.
static bool use_fused(const dgadv_handle *h) {
  return h->lim && h->limType == DGADV_LIM_LINEAR && !h->cDV0T && (h->flags & DGADV_FLAG_FUSE);
}

template <typename T, int P>
static cudaError_t launch_step_fused(dgadv_handle *h, double t0, double tau, bool firstOfCall) {
  using SR = StageRows<T, P>;
  const Geo<T> g = make_geo<T>(h);
  const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;
  double omega[3], cst[3];
  const int S = rk_table(h->ordRK, omega, cst);
  T *cn = (T *)h->cn, *R = (T *)h->cR, *rA = (T *)h->cA, *rB = (T *)h->cB;
  T *cnL = (T *)h->cnL, *Lx = (T *)h->cLx, *tb = (T *)h->tbuf;
  const bool rhs = h->nTerms > 0 && h->rhs;
  for (int s = 0; s < S; ++s) {
    const T *x = (s == 0) ? (firstOfCall ? cn : R) : (s == 1 ? rA : rB);
    const int limitIn = (firstOfCall && s == 0) ? 0 : 1;
    T *outRaw = (s == S - 1) ? R : (s == 0 ? rA : rB);
    StageScalars sc{};
    sc.omega = omega[s]; sc.tau = tau; sc.flag = h->flag;
    const double ts = t0 + cst[s] * tau;
    for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = time_factor(h->timeFn[m], ts);
    const LimIn<T> li = lim_in_pass<T>(h, h->limPass - 1);
    const LimOut<T> lo1 = lim_out<T>(h);
    ++h->limPass;
    prof_mark(h, 0);
    if (!h->limdot) {
      if (rhs) launch_k(h, k_op_fused<T, P, 1, true>, grid, SR::bytes(SR::op(1, true), 1), g, x, limitIn,
                        s == 0 ? cnL : (T *)nullptr, (const T *)cnL, s == 0 ? 1 : 0, outRaw, li, lo1, sc);
      else launch_k(h, k_op_fused<T, P, 1, false>, grid, SR::bytes(SR::op(1, true), 1), g, x, limitIn,
                    s == 0 ? cnL : (T *)nullptr, (const T *)cnL, s == 0 ? 1 : 0, outRaw, li, lo1, sc);
      prof_mark(h, -1);
      continue;
    }
    T *xL = (s == 0) ? cnL : Lx;
    if (rhs) launch_k(h, k_op_fused<T, P, 2, true>, grid, SR::bytes(SR::op(2, true), 1), g, x, limitIn, xL,
                      (const T *)nullptr, s == 0 ? 1 : 0, tb, li, lo1, sc);
    else launch_k(h, k_op_fused<T, P, 2, false>, grid, SR::bytes(SR::op(2, true), 1), g, x, limitIn, xL,
                  (const T *)nullptr, s == 0 ? 1 : 0, tb, li, lo1, sc);
    prof_mark(h, -1);
    const LimOut<T> lo2 = lim_out<T>(h);
    ++h->limPass;
    prof_mark(h, 1);
    launch_k(h, k_limit_dot_lin<T, P>, grid, SR::bytes(SR::limdot_lin(), 1), g, (const T *)xL, (const T *)cnL,
             (const T *)tb, outRaw, lim_in<T>(lo1, h), lo2, sc);
    prof_mark(h, -1);
  }
  return cudaGetLastError();
}

template <typename T, int P>
static cudaError_t launch_finalize_fused(dgadv_handle *h) {
  const Geo<T> g = make_geo<T>(h);
  const int gridK = (h->K + kBlock - 1) / kBlock;
  StageScalars sc{};
  sc.flag = h->flag;
  prof_mark(h, 2);
  launch_k(h, k_limit_lin<T, P>, gridK, (size_t)0, g, (const T *)h->cR, (T *)h->cn,
           lim_in_pass<T>(h, h->limPass - 1), sc);
  prof_mark(h, -1);
  return cudaGetLastError();
}

template <typename T, int P>
static cudaError_t launch_limit_state(dgadv_handle *h, double t) {
  using SR = StageRows<T, P>;
  const Geo<T> g = make_geo<T>(h);
  const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;   // producers also reset vertex keys
  StageScalars sc{};
  sc.flag = h->flag;
  for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = time_factor(h->timeFn[m], t);
  const LimOut<T> lo = lim_out<T>(h);
  ++h->limPass;
  if (h->limType == DGADV_LIM_LINEAR) {
    const int gridK = (h->K + kBlock - 1) / kBlock;
    launch_k(h, k_mean_lin<T, P>, grid, (size_t)0, g, (const T *)h->cn, lo);
    launch_k(h, k_limit_lin<T, P>, gridK, (size_t)0, g, (const T *)h->cn, (T *)h->cn, lim_in<T>(lo, h), sc);
  } else {
    launch_k(h, k_to_taylor<T, P>, grid, SR::bytes(SR::totaylor(), 0), g, (const T *)h->cn, (T *)h->tbuf, lo, sc);
    launch_k(h, k_limit<T, P>, grid, SR::bytes(SR::lim(), 1), g, (const T *)h->tbuf, (T *)h->cn, lim_in<T>(lo, h), sc);
  }
  return cudaGetLastError();
}

template <typename T>
static cudaError_t dispatch_step(dgadv_handle *h, double t0, double tau) {
  switch (h->p) {
    case 0: return launch_step<T, 0>(h, t0, tau);
    case 1: return launch_step<T, 1>(h, t0, tau);
    case 2: return launch_step<T, 2>(h, t0, tau);
    default: return launch_step<T, 3>(h, t0, tau);
  }
}
template <typename T>
static cudaError_t dispatch_step_fused(dgadv_handle *h, double t0, double tau, bool first) {
  switch (h->p) {
    case 1: return launch_step_fused<T, 1>(h, t0, tau, first);
    case 2: return launch_step_fused<T, 2>(h, t0, tau, first);
    default: return launch_step_fused<T, 3>(h, t0, tau, first);
  }
}
template <typename T>
static cudaError_t dispatch_finalize_fused(dgadv_handle *h) {
  switch (h->p) {
    case 1: return launch_finalize_fused<T, 1>(h);
    case 2: return launch_finalize_fused<T, 2>(h);
    default: return launch_finalize_fused<T, 3>(h);
  }
}

template <typename T>
static cudaError_t dispatch_limit(dgadv_handle *h, double t) {
  switch (h->p) {
    case 1: return launch_limit_state<T, 1>(h, t);
    case 2: return launch_limit_state<T, 2>(h, t);
    default: return launch_limit_state<T, 3>(h, t);
  }
}

}  // namespace dgadv

// ---------------------------------------------------------------------------------------------
// C-ABI
using namespace dgadv;

#define DG_CUDA(call)                                                               \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
      return DGADV_ECUDA;                                                           \
    }                                                                               \
  } while (0)

static int dev_alloc(dgadv_handle *h, void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) { h->err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return DGADV_ENOMEM; }
  h->allocs.push_back(*p);
  return DGADV_OK;
}

static int upload(dgadv_handle *h, void *dst, const void *src, size_t bytes) {
  DG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return DGADV_OK;
}

template <typename T>
static int upload_real(dgadv_handle *h, void *dst, const std::vector<double> &src) {
  if (sizeof(T) == 8) return upload(h, dst, src.data(), src.size() * sizeof(double));
  std::vector<float> tmp(src.size());
  for (size_t i = 0; i < src.size(); ++i) tmp[i] = (float)src[i];
  return upload(h, dst, tmp.data(), tmp.size() * sizeof(float));
}

static uint32_t morton2(uint32_t x, uint32_t y) {
  auto spread = [](uint32_t v) {
    v &= 0xFFFF;
    v = (v | (v << 8)) & 0x00FF00FF;
    v = (v | (v << 4)) & 0x0F0F0F0F;
    v = (v | (v << 2)) & 0x33333333;
    v = (v | (v << 1)) & 0x55555555;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

extern "C" int dgadv_create(const dgadv_mesh *mesh, const dgadv_params *prm, dgadv_handle **out) {
  if (!out) return DGADV_EINVAL;
  *out = nullptr;
  if (!mesh || !prm) return DGADV_EINVAL;
  if (prm->p < 0 || prm->p > 4 || prm->ordRK < 1 || prm->ordRK > 3) return DGADV_EINVAL;
  if (prm->precision != DGADV_FP64 && prm->precision != DGADV_FP32) return DGADV_EINVAL;
  if (prm->isSlopeLim && prm->p < 1) return DGADV_EINVAL;
  if (prm->p > kMaxP) return DGADV_EUNSUPPORTED;
  if (prm->isSlopeLim && prm->typeSlopeLim != DGADV_LIM_LINEAR && prm->typeSlopeLim != DGADV_LIM_HIERARCH_VERT)
    return prm->typeSlopeLim == DGADV_LIM_STRICT ? DGADV_EUNSUPPORTED : DGADV_EINVAL;
  dgadv_handle *h = new (std::nothrow) dgadv_handle();
  if (!h) return DGADV_ENOMEM;
  *out = h;
  h->device = prm->device;
  h->p = prm->p; h->N = N_of_p(prm->p); h->ordRK = prm->ordRK; h->prec = prm->precision;
  h->lim = prm->isSlopeLim ? 1 : 0; h->limType = prm->typeSlopeLim; h->flags = prm->flags;
  h->limdot = h->lim && h->p > 1;
  h->nc = h->lim ? (h->limType == DGADV_LIM_LINEAR ? 1 : h->p * (h->p + 1) / 2) : 1;
  h->passesPerStep = h->lim ? h->ordRK * (h->limdot ? 2 : 1) : 0;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  // static grid data (core/generateGridData.m semantics)
  Grid gr;
  if (!build_grid(mesh->numV, mesh->coordV, mesh->numT, mesh->V0T, gr, h->err)) return DGADV_EMESH;
  if (!build_ref_tables(h->p, h->tables, h->err)) return DGADV_EINVAL;
  const int K = gr.numT, N = h->N;
  h->K = K; h->Kp = (K + kBlock - 1) / kBlock * kBlock;   // whole blocks of rows for the bulk copies h->numV = gr.numV; h->Vp = (gr.numV + 63) / 64 * 64;
  h->Q = h->tables.Q; h->R = h->tables.R;
  const int Kp = h->Kp;
  // element order on the device: Morton order of the barycentres
  std::vector<int> perm(K);
  std::iota(perm.begin(), perm.end(), 0);
  if (!(h->flags & DGADV_FLAG_NO_REORDER)) {
    double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
    for (int t = 0; t < K; ++t) {
      xmin = std::min(xmin, gr.baryT[2 * t]); xmax = std::max(xmax, gr.baryT[2 * t]);
      ymin = std::min(ymin, gr.baryT[2 * t + 1]); ymax = std::max(ymax, gr.baryT[2 * t + 1]);
    }
    const double sx = 65535.0 / std::max(xmax - xmin, 1e-300), sy = 65535.0 / std::max(ymax - ymin, 1e-300);
    std::vector<uint32_t> key(K);
    for (int t = 0; t < K; ++t)
      key[t] = morton2((uint32_t)((gr.baryT[2 * t] - xmin) * sx), (uint32_t)((gr.baryT[2 * t + 1] - ymin) * sy));
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return key[a] < key[b]; });
  }
  std::vector<int> inv(K);
  for (int k = 0; k < K; ++k) inv[perm[k]] = k;
  h->permv = perm;
  // vertex ids renumbered by first appearance in the device element order
  std::vector<int> vnew(gr.numV, -1);
  int nv = 0;
  for (int k = 0; k < K; ++k)
    for (int n = 0; n < 3; ++n) {
      const int v = gr.V0T[3 * (size_t)perm[k] + n];
      if (vnew[v] < 0) vnew[v] = nv++;
    }
  h->numV = nv; h->Vp = (nv + 63) / 64 * 64;
  // boundary markers
  std::vector<uint8_t> bdrD(3 * (size_t)K), bdrN(3 * (size_t)K, 0), idOk(3 * (size_t)K, 1);
  for (int t = 0; t < K; ++t)
    for (int n = 0; n < 3; ++n) {
      const int e = gr.E0T[3 * (size_t)t + n];
      const bool interior = gr.T0E[2 * (size_t)e + 1] >= 0;
      const size_t cm = (size_t)n * K + t;
      if (mesh->markE0TbdrN) bdrN[3 * (size_t)t + n] = mesh->markE0TbdrN[cm] ? 1 : 0;
      if (mesh->markE0TbdrD) bdrD[3 * (size_t)t + n] = mesh->markE0TbdrD[cm] ? 1 : 0;
      else bdrD[3 * (size_t)t + n] = (!interior && !bdrN[3 * (size_t)t + n]) ? 1 : 0;
      if (mesh->idE0T) idOk[3 * (size_t)t + n] = (interior || mesh->idE0T[cm] != 0) ? 1 : 0;
    }
  // markV0TbdrD: vertices of Dirichlet edges (advection/preprocessProblem.m:75-76)
  std::vector<uint8_t> vD(gr.numV, 0);
  for (int t = 0; t < K; ++t)
    for (int n = 0; n < 3; ++n)
      if (bdrD[3 * (size_t)t + n]) {
        const int e = gr.E0T[3 * (size_t)t + n];
        vD[gr.V0E[2 * (size_t)e]] = 1; vD[gr.V0E[2 * (size_t)e + 1]] = 1;
      }
  // per-element device arrays (internal order)
  std::vector<int> nbr(3 * (size_t)Kp, -1), code(Kp, 0), V0T(3 * (size_t)Kp, 0);
  h->detJ.assign(K, 0); h->areaE0T.assign(3 * (size_t)K, 0); h->Bhost.assign(4 * (size_t)K, 0);
  h->markNotN.assign(3 * (size_t)K, 0);
  std::vector<double> Bsoa(4 * (size_t)Kp, 0.0);
  for (int k = 0; k < K; ++k) {
    const int t = perm[k];
    int cd = 0;
    for (int n = 0; n < 3; ++n) {
      const int e = gr.E0T[3 * (size_t)t + n];
      int other = gr.T0E[2 * (size_t)e] == t ? gr.T0E[2 * (size_t)e + 1] : gr.T0E[2 * (size_t)e];
      int np = gr.T0E[2 * (size_t)e] == t ? gr.E0E[2 * (size_t)e + 1] : gr.E0E[2 * (size_t)e];
      if (other < 0) np = 3;
      nbr[(size_t)n * Kp + k] = other >= 0 ? inv[other] : -1;
      cd |= (np & 3) << (2 * n);
      if (idOk[3 * (size_t)t + n]) cd |= 1 << (6 + n);
      if (vD[gr.V0T[3 * (size_t)t + n]]) cd |= 1 << (9 + n);
      V0T[(size_t)n * Kp + k] = vnew[gr.V0T[3 * (size_t)t + n]];
      h->areaE0T[3 * (size_t)k + n] = gr.areaE0T[3 * (size_t)t + n];
      h->markNotN[3 * (size_t)k + n] = bdrN[3 * (size_t)t + n] ? 0 : 1;
    }
    code[k] = cd;
    h->detJ[k] = gr.detJ0T[t];
    for (int i = 0; i < 4; ++i) { Bsoa[(size_t)i * Kp + k] = gr.B[4 * (size_t)t + i]; h->Bhost[4 * (size_t)k + i] = gr.B[4 * (size_t)t + i]; }
  }
  // CSR vertex -> elements (internal ids)
  std::vector<int> vptr(h->numV + 1, 0), vidx(3 * (size_t)K);
  for (int k = 0; k < K; ++k)
    for (int n = 0; n < 3; ++n) vptr[V0T[(size_t)n * Kp + k] + 1]++;
  for (int v = 0; v < h->numV; ++v) vptr[v + 1] += vptr[v];
  {
    std::vector<int> fill(vptr.begin(), vptr.end() - 1);
    for (int k = 0; k < K; ++k)
      for (int n = 0; n < 3; ++n) vidx[fill[V0T[(size_t)n * Kp + k]]++] = k;
  }
  const size_t w = h->prec == DGADV_FP64 ? 8 : 4;
  int st;
  const int Q = h->Q, R = h->R, nc = h->nc;
  if ((st = dev_alloc(h, &h->F, 2 * (size_t)Q * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->Vn, 3 * (size_t)R * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->Bm, 4 * (size_t)Kp * w))) return st;
  if ((st = dev_alloc(h, (void **)&h->nbr, 3 * (size_t)Kp * 4))) return st;
  if ((st = dev_alloc(h, (void **)&h->code, (size_t)Kp * 4))) return st;
  if ((st = dev_alloc(h, (void **)&h->V0T, 3 * (size_t)Kp * 4))) return st;
  if ((st = dev_alloc(h, (void **)&h->vptr, (size_t)(h->numV + 1) * 4))) return st;
  if ((st = dev_alloc(h, (void **)&h->vidx, 3 * (size_t)K * 4))) return st;
  if ((st = dev_alloc(h, (void **)&h->perm, (size_t)K * 4))) return st;
  if ((st = dev_alloc(h, &h->cn, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->cA, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->cB, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->tbuf, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->cR, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->cnL, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->cLx, (size_t)N * Kp * w))) return st;
  if ((st = dev_alloc(h, &h->vkeys, 3 * 2 * (size_t)nc * h->Vp * w))) return st;
  if ((st = dev_alloc(h, (void **)&h->gmm, 3 * kSlotCopies * 2 * (size_t)nc * 8))) return st;
  if ((st = dev_alloc(h, (void **)&h->flag, 16))) return st;
  if ((st = dev_alloc(h, (void **)&h->stage_ext, (size_t)N * K * 8))) return st;
  DG_CUDA(cudaMemset(h->F, 0, 2 * (size_t)Q * Kp * w));
  DG_CUDA(cudaMemset(h->Vn, 0, 3 * (size_t)R * Kp * w));
  DG_CUDA(cudaMemset(h->cn, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->cA, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->cB, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->tbuf, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->cR, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->cnL, 0, (size_t)N * Kp * w));
  DG_CUDA(cudaMemset(h->cLx, 0, (size_t)N * Kp * w));
  {
    // vertex keys of every pass start reset (min = largest key, max = 0)
    std::vector<unsigned char> vk(3 * 2 * (size_t)nc * h->Vp * w, 0);
    for (size_t set = 0; set < 3 * (size_t)nc; ++set)
      std::memset(vk.data() + set * 2 * h->Vp * w, 0xFF, (size_t)h->Vp * w);
    if ((st = upload(h, h->vkeys, vk.data(), vk.size()))) return st;
  }
  {
    // slots of pass 0 start reset; every later pass is reset by the previous producer
    std::vector<unsigned long long> init(3 * kSlotCopies * 2 * (size_t)nc);
    const unsigned long long kmax = h->prec == DGADV_FP64 ? ~0ULL : 0xFFFFFFFFULL;
    for (size_t i = 0; i < init.size(); ++i) init[i] = (i & 1) ? 0ULL : kmax;
    if ((st = upload(h, h->gmm, init.data(), init.size() * 8))) return st;
  }
  DG_CUDA(cudaMemset(h->flag, 0, 16));
  if (h->prec == DGADV_FP64) { if ((st = upload_real<double>(h, h->Bm, Bsoa))) return st; }
  else { if ((st = upload_real<float>(h, h->Bm, Bsoa))) return st; }
  if ((st = upload(h, h->nbr, nbr.data(), nbr.size() * 4))) return st;
  if ((st = upload(h, h->code, code.data(), code.size() * 4))) return st;
  if ((st = upload(h, h->V0T, V0T.data(), V0T.size() * 4))) return st;
  if ((st = upload(h, h->vptr, vptr.data(), vptr.size() * 4))) return st;
  if ((st = upload(h, h->vidx, vidx.data(), vidx.size() * 4))) return st;
  if ((st = upload(h, h->perm, perm.data(), perm.size() * 4))) return st;
  if (h->limdot && h->limType == DGADV_LIM_LINEAR) {
    std::vector<double> qk;
    taylor_correction(gr, h->p, h->tables, qk);
    const int NQk = N * (N - 1);
    std::vector<double> soa((size_t)NQk * Kp, 0.0);
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < NQk; ++i) soa[(size_t)i * Kp + k] = qk[(size_t)perm[k] * NQk + i];
    if ((st = dev_alloc(h, &h->MT, soa.size() * w))) return st;
    if (h->prec == DGADV_FP64) { if ((st = upload_real<double>(h, h->MT, soa))) return st; }
    else { if ((st = upload_real<float>(h, h->MT, soa))) return st; }
  } else if (h->limdot) {
    std::vector<double> mt;
    taylor_mass_packed(gr, h->p, mt);
    const int NMT = N * (N + 1) / 2;
    std::vector<double> soa((size_t)NMT * Kp, 0.0);
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < NMT; ++i) soa[(size_t)i * Kp + k] = mt[(size_t)perm[k] * NMT + i];
    if ((st = dev_alloc(h, &h->MT, soa.size() * w))) return st;
    if (h->prec == DGADV_FP64) { if ((st = upload_real<double>(h, h->MT, soa))) return st; }
    else { if ((st = upload_real<float>(h, h->MT, soa))) return st; }
  }
  // constant tables (once per device, precision and degree)
  {
    std::lock_guard<std::mutex> lk(g_tab_mutex);
    const int pi = h->prec == DGADV_FP64 ? 0 : 1;
    if (h->device < 0 || h->device >= 64) { h->err = "device ordinal out of range"; return DGADV_EINVAL; }
    if (!g_tab_loaded[h->device][pi][h->p]) {
      cudaError_t e = cudaSuccess;
      if (pi == 0) {
        switch (h->p) { case 0: e = upload_tables<double, 0>(h->tables); break; case 1: e = upload_tables<double, 1>(h->tables); break;
                        case 2: e = upload_tables<double, 2>(h->tables); break; default: e = upload_tables<double, 3>(h->tables); }
      } else {
        switch (h->p) { case 0: e = upload_tables<float, 0>(h->tables); break; case 1: e = upload_tables<float, 1>(h->tables); break;
                        case 2: e = upload_tables<float, 2>(h->tables); break; default: e = upload_tables<float, 3>(h->tables); }
      }
      if (e != cudaSuccess) { h->err = std::string("table upload: ") + cudaGetErrorString(e); return DGADV_ECUDA; }
      if (pi == 0) {
        switch (h->p) { case 0: e = set_smem_attributes<double, 0>(); break; case 1: e = set_smem_attributes<double, 1>(); break;
                        case 2: e = set_smem_attributes<double, 2>(); break; default: e = set_smem_attributes<double, 3>(); }
      } else {
        switch (h->p) { case 0: e = set_smem_attributes<float, 0>(); break; case 1: e = set_smem_attributes<float, 1>(); break;
                        case 2: e = set_smem_attributes<float, 2>(); break; default: e = set_smem_attributes<float, 3>(); }
      }
      if (e != cudaSuccess) { h->err = std::string("kernel attributes: ") + cudaGetErrorString(e); return DGADV_ECUDA; }
      g_tab_loaded[h->device][pi][h->p] = true;
    }
  }
  DG_CUDA(cudaDeviceSynchronize());
  return DGADV_OK;
}

extern "C" int dgadv_set_velocity(dgadv_handle *h, const double *u1, const double *u2, const double *vN) {
  if (!h || !u1 || !u2 || !vN) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const int K = h->K, Kp = h->Kp, N = h->N, Q = h->Q, R = h->R;
  const RefTables &t = h->tables;
  std::vector<double> F(2 * (size_t)Q * Kp, 0.0), Vn(3 * (size_t)R * Kp, 0.0);
  for (int k = 0; k < K; ++k) {
    const int e = h->permv[k];
    const double B11 = h->Bhost[4 * (size_t)k], B12 = h->Bhost[4 * (size_t)k + 1];
    const double B21 = h->Bhost[4 * (size_t)k + 2], B22 = h->Bhost[4 * (size_t)k + 3];
    const double dj = h->detJ[k];
    for (int q = 0; q < Q; ++q) {
      double a = 0, b = 0;
      for (int l = 0; l < N; ++l) {
        a += t.phiQ[q * N + l] * u1[(size_t)l * K + e];
        b += t.phiQ[q * N + l] * u2[(size_t)l * K + e];
      }
      F[(size_t)q * Kp + k] = t.vol.W[q] * (B22 * a - B12 * b) / dj;
      F[(size_t)(Q + q) * Kp + k] = t.vol.W[q] * (B11 * b - B21 * a) / dj;
    }
    for (int n = 0; n < 3; ++n)
      for (int r = 0; r < R; ++r) {
        const double v = vN[(size_t)e + (size_t)K * n + (size_t)3 * K * r];
        Vn[(size_t)(n * R + r) * Kp + k] =
            h->markNotN[3 * (size_t)k + n] ? h->areaE0T[3 * (size_t)k + n] * t.edge.W[r] * v / dj : 0.0;
      }
  }
  int st;
  if (h->prec == DGADV_FP64) {
    if ((st = upload_real<double>(h, h->F, F))) return st;
    if ((st = upload_real<double>(h, h->Vn, Vn))) return st;
  } else {
    if ((st = upload_real<float>(h, h->F, F))) return st;
    if ((st = upload_real<float>(h, h->Vn, Vn))) return st;
  }
  h->hasVelocity = true;
  return DGADV_OK;
}

extern "C" int dgadv_set_source_terms(dgadv_handle *h, int32_t nTerms, const int32_t *timeFn,
                                      const double *rhsTerms, const double *cDV0T) {
  if (!h || nTerms < 0 || nTerms > 4) return DGADV_EINVAL;
  if (nTerms > 0 && (!timeFn || !rhsTerms)) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  const int K = h->K, Kp = h->Kp, N = h->N;
  const size_t w = h->prec == DGADV_FP64 ? 8 : 4;
  for (int m = 0; m < nTerms; ++m)
    if (timeFn[m] != DGADV_TIME_CONST && timeFn[m] != DGADV_TIME_EXP_NEG) return DGADV_EINVAL;
  h->nTerms = nTerms;
  for (int m = 0; m < 4; ++m) h->timeFn[m] = m < nTerms ? timeFn[m] : 0;
  for (int i = 0; i < 3; ++i)
    if (h->graph[i]) { cudaGraphExecDestroy(h->graph[i]); h->graph[i] = nullptr; }
  if (nTerms == 0) return DGADV_OK;
  std::vector<double> r((size_t)nTerms * N * Kp, 0.0), d((size_t)nTerms * 3 * Kp, 0.0);
  for (int m = 0; m < nTerms; ++m)
    for (int k = 0; k < K; ++k) {
      const int e = h->permv[k];
      for (int i = 0; i < N; ++i)
        r[((size_t)m * N + i) * Kp + k] = rhsTerms[(size_t)m * K * N + (size_t)i * K + e] / h->detJ[k];
      if (cDV0T)
        for (int n = 0; n < 3; ++n) d[((size_t)m * 3 + n) * Kp + k] = cDV0T[(size_t)m * K * 3 + (size_t)n * K + e];
    }
  int st;
  if (!h->rhs && (st = dev_alloc(h, &h->rhs, 4 * (size_t)N * Kp * w))) return st;
  if (cDV0T && !h->cDV0T && (st = dev_alloc(h, &h->cDV0T, 4 * (size_t)3 * Kp * w))) return st;
  if (h->prec == DGADV_FP64) {
    if ((st = upload_real<double>(h, h->rhs, r))) return st;
    if (cDV0T && (st = upload_real<double>(h, h->cDV0T, d))) return st;
  } else {
    if ((st = upload_real<float>(h, h->rhs, r))) return st;
    if (cDV0T && (st = upload_real<float>(h, h->cDV0T, d))) return st;
  }
  if (!cDV0T && h->cDV0T) DG_CUDA(cudaMemset(h->cDV0T, 0, 4 * (size_t)3 * Kp * w));
  return DGADV_OK;
}

extern "C" int dgadv_set_state(dgadv_handle *h, const double *c) {
  if (!h || !c) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaMemcpyAsync(h->stage_ext, c, (size_t)h->N * h->K * 8, cudaMemcpyHostToDevice, h->stream));
  const int grid = (h->K + 255) / 256;
  if (h->prec == DGADV_FP64)
    k_scatter_in<double><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, h->stage_ext, (double *)h->cn);
  else
    k_scatter_in<float><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, h->stage_ext, (float *)h->cn);
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaStreamSynchronize(h->stream));
  return DGADV_OK;
}

extern "C" int dgadv_sync(dgadv_handle *h) {
  if (!h) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  int flag = 0;
  DG_CUDA(cudaMemcpy(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag & 2) { h->err = "a bounded device wait timed out"; return DGADV_ETIMEOUT; }
  if (flag & 1) { h->err = "non-finite value in the state"; return DGADV_ENONFINITE; }
  return DGADV_OK;
}

extern "C" int dgadv_get_state(dgadv_handle *h, double *c) {
  if (!h || !c) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const int grid = (h->K + 255) / 256;
  if (h->prec == DGADV_FP64)
    k_gather_out<double><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, (const double *)h->cn, h->stage_ext);
  else
    k_gather_out<float><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, (const float *)h->cn, h->stage_ext);
  DG_CUDA(cudaGetLastError());
  DG_CUDA(cudaMemcpyAsync(c, h->stage_ext, (size_t)h->N * h->K * 8, cudaMemcpyDeviceToHost, h->stream));
  return dgadv_sync(h);
}

extern "C" int dgadv_limit_state(dgadv_handle *h, double t) {
  if (!h) return DGADV_EINVAL;
  if (!h->lim) { h->err = "limiter is off for this handle"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  cudaError_t e = h->prec == DGADV_FP64 ? dispatch_limit<double>(h, t) : dispatch_limit<float>(h, t);
  if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  return dgadv_sync(h);
}

static bool time_dependent(const dgadv_handle *h) {
  for (int m = 0; m < h->nTerms; ++m)
    if (h->timeFn[m] != DGADV_TIME_CONST) return true;
  return false;
}

// One time step: fused or separate-pass pipeline.
static cudaError_t one_step(dgadv_handle *h, double t0, double tau, bool firstOfCall) {
  if (use_fused(h))
    return h->prec == DGADV_FP64 ? dispatch_step_fused<double>(h, t0, tau, firstOfCall)
                                 : dispatch_step_fused<float>(h, t0, tau, firstOfCall);
  return h->prec == DGADV_FP64 ? dispatch_step<double>(h, t0, tau) : dispatch_step<float>(h, t0, tau);
}
static cudaError_t end_of_call(dgadv_handle *h) {
  if (!use_fused(h)) return cudaSuccess;
  return h->prec == DGADV_FP64 ? dispatch_finalize_fused<double>(h) : dispatch_finalize_fused<float>(h);
}

extern "C" int dgadv_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau) {
  if (!h || nSteps < 0 || !(tau > 0)) return DGADV_EINVAL;
  if (!h->hasVelocity) { if (h) h->err = "dgadv_set_velocity was not called"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  if (nSteps == 0) return DGADV_OK;
  const bool fused = use_fused(h);
  const bool useGraph = !(h->flags & DGADV_FLAG_NO_GRAPH) && !time_dependent(h);
  int done = 0;
  if (fused) {   // the first step of a call starts from the limited state
    cudaError_t e = one_step(h, (double)nStep0 * tau, tau, true);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
    done = 1;
  }
  if (useGraph) {
    // time-independent data: a captured graph of a chunk of steps, replayed.  The chunk makes a
    // multiple of three limiter passes, so the pass phase is the same before and after it.
    const int chunk = 12;
    while (nSteps - done >= chunk) {
      const int ph = (int)(h->limPass % 3);
      if (!h->graph[ph] || h->graphTau[ph] != tau) {
        if (h->graph[ph]) { cudaGraphExecDestroy(h->graph[ph]); h->graph[ph] = nullptr; }
        const long long saved = h->limPass;
        cudaGraph_t gph;
        DG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int s = 0; s < chunk && e == cudaSuccess; ++s) e = one_step(h, 0.0, tau, false);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &gph);
        h->limPass = saved;
        if (e != cudaSuccess || e2 != cudaSuccess) {
          h->err = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
          return DGADV_ECUDA;
        }
        DG_CUDA(cudaGraphInstantiate(&h->graph[ph], gph, 0));
        cudaGraphDestroy(gph);
        h->graphTau[ph] = tau;
      }
      DG_CUDA(cudaGraphLaunch(h->graph[ph], h->stream));
      h->limPass += (long long)chunk * h->passesPerStep;
      done += chunk;
    }
  }
  for (; done < nSteps; ++done) {
    cudaError_t e = one_step(h, (double)(nStep0 + done) * tau, tau, false);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  }
  cudaError_t e = end_of_call(h);
  if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  return DGADV_OK;
}

extern "C" int dgadv_time_steps(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau, double *ms) {
  if (!h || !ms) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  if (!h->ev0) { DG_CUDA(cudaEventCreate(&h->ev0)); DG_CUDA(cudaEventCreate(&h->ev1)); }
  DG_CUDA(cudaStreamSynchronize(h->stream));
  DG_CUDA(cudaEventRecord(h->ev0, h->stream));
  int st = dgadv_step(h, nSteps, nStep0, tau);
  if (st) return st;
  DG_CUDA(cudaEventRecord(h->ev1, h->stream));
  DG_CUDA(cudaEventSynchronize(h->ev1));
  float f = 0;
  DG_CUDA(cudaEventElapsedTime(&f, h->ev0, h->ev1));
  *ms = f;
  return dgadv_sync(h);
}

extern "C" int dgadv_profile_kernels(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau,
                                     double *msPerLaunch, int32_t *launches) {
  if (!h || !msPerLaunch || !launches || nSteps < 1) return DGADV_EINVAL;
  if (!h->hasVelocity) { h->err = "dgadv_set_velocity was not called"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  h->profiling = true;
  h->profEvents.clear(); h->profKinds.clear();
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < nSteps && e == cudaSuccess; ++s) e = one_step(h, (double)(nStep0 + s) * tau, tau, s == 0);
  if (e == cudaSuccess) e = end_of_call(h);
  h->profiling = false;
  cudaError_t e2 = cudaStreamSynchronize(h->stream);
  for (int k = 0; k < 4; ++k) { msPerLaunch[k] = 0; launches[k] = 0; }
  for (size_t i = 0; i + 1 < h->profEvents.size(); i += 2) {
    float f = 0;
    if (e2 == cudaSuccess) cudaEventElapsedTime(&f, h->profEvents[i], h->profEvents[i + 1]);
    const int kind = h->profKinds[i];
    if (kind >= 0 && kind < 4) { msPerLaunch[kind] += f; launches[kind] += 1; }
  }
  for (cudaEvent_t ev : h->profEvents) cudaEventDestroy(ev);
  h->profEvents.clear(); h->profKinds.clear();
  for (int k = 0; k < 4; ++k)
    if (launches[k]) msPerLaunch[k] /= launches[k];
  if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  if (e2 != cudaSuccess) { h->err = cudaGetErrorString(e2); return DGADV_ECUDA; }
  return dgadv_sync(h);
}

extern "C" int dgadv_kernels_per_step(const dgadv_handle *h, int32_t *count) {
  if (!h || !count) return DGADV_EINVAL;
  int perStage = 1;
  if (use_fused(h)) perStage = h->limdot ? 2 : 1;
  else if (h->lim) perStage = h->limdot ? 3 : 2;
  *count = h->ordRK * perStage;
  return DGADV_OK;
}

extern "C" const char *dgadv_last_error(const dgadv_handle *h) { return h ? h->err.c_str() : "null handle"; }

extern "C" void dgadv_destroy(dgadv_handle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (int i = 0; i < 3; ++i)
    if (h->graph[i]) cudaGraphExecDestroy(h->graph[i]);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (void *p : h->allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// ---------------------------------------------------------------------------------------------
// Linear slope limiter on caller-owned device arrays that allocates nothing on the device.
// It is for callers that cannot call cudaMalloc: code whose device memory all comes from
// another framework's pool or arena (a cudaMalloc behind that pool's back breaks its
// accounting), code that runs under a device-memory budget fixed before it starts, and code
// called from places where a device allocation would synchronise the device.  Its scratch (the
// per-vertex min / max keys and the copies of the global extremes) lives in the fixed array
// below, which every GPU that loads this library keeps until the process exits.
namespace dgadv {

constexpr int kNoAllocMaxVertices = DGADV_NOALLOC_MAX_VERTICES;
static __device__ __align__(256) unsigned long long
    g_noalloc_scratch[2 * kNoAllocMaxVertices + 2 * kSlotCopies];
static unsigned long long *g_noalloc_addr[64];   // device address of the array, per device

// Clears the keys of numV vertices (min = largest key, max = 0) and the extremes' copies.
__global__ void k_na_reset(unsigned long long *s, int numV) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < numV) { s[v] = ~0ULL; s[kNoAllocMaxVertices + v] = 0ULL; }
  if (blockIdx.x == 0 && threadIdx.x < 2 * kSlotCopies)
    s[2 * kNoAllocMaxVertices + threadIdx.x] = (threadIdx.x & 1) ? 0ULL : ~0ULL;
}

// Element means (the centroid values) scattered to the three vertices' keys and to the
// global extremes (core/computeMinMaxV0TElementPatch.m).
template <int P>
__global__ void __launch_bounds__(kBlock)
k_na_scatter(int K, const int *__restrict__ V0T, const double *__restrict__ c, unsigned long long *s) {
  constexpr int N = Dims<P>::N;
  const int k = blockIdx.x * kBlock + threadIdx.x;
  const bool active = k < K;
  Geo<double> g{};
  g.Vp = kNoAllocMaxVertices;
  LimOut<double> lo{};
  lo.vkeys = s; lo.slots = s + 2 * kNoAllocMaxVertices; lo.nc = 1; lo.type = 0;
  int vid[3] = {0, 0, 0};
  double q0 = 0.0;
  if (active) {
    vid[0] = V0T[k]; vid[1] = V0T[K + k]; vid[2] = V0T[2 * K + k];
    double cc[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cc[i] = c[(size_t)i * K + k];
    q0 = lin_mean<double, P>(cc);
  }
  scatter_quantities<double, 1>(g, lo, &q0, vid, active);
}

// The limiter (core/applySlopeLimiterTaylorLinear.m with the vertex-based limiter of
// core/computeVertexBasedLimiter.m): c <- c - DM^-1 du, Dirichlet data where markD is set.
template <int P>
__global__ void __launch_bounds__(kBlock)
k_na_limit(int K, const int *__restrict__ V0T, const uint8_t *__restrict__ markD,
           const double *__restrict__ dataD, const double *cin, double *cout, const unsigned long long *s) {
  constexpr int N = Dims<P>::N;
  const Tab<double, P> &tb = tab<double, P>();
  __shared__ double sh[2];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  const bool active = k < K;
  Geo<double> g{};
  g.Vp = kNoAllocMaxVertices;
  LimIn<double> li{};
  li.vkeys = s; li.slots = s + 2 * kNoAllocMaxVertices; li.nc = 1; li.type = 0; li.shift = 1;
  load_shifts<double>(li.slots, 1, sh);
  __syncthreads();
  if (!active) return;
  const int vid[3] = {V0T[k], V0T[K + k], V0T[2 * K + k]};
  int dmask = 0;
  double data[3] = {0.0, 0.0, 0.0};
  if (markD)
    for (int n = 0; n < 3; ++n) dmask |= (markD[(size_t)n * K + k] ? 1 : 0) << n;
  if (dataD)
    for (int n = 0; n < 3; ++n) data[n] = dataD[(size_t)n * K + k];
  VKeys<double, 1> kv;
  load_vkeys<double, 1>(g, li, vid, kv);
  double c[N], u[N], du[N];
#pragma unroll
  for (int i = 0; i < N; ++i) c[i] = cin[(size_t)i * K + k];
  lin_u<double, P>(c, u);
  if (lin_alpha<double, P, 1>(li, kv, sh, u, dmask, data, du)) {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double t = 0.0;
#pragma unroll
      for (int j = 1; j < N; ++j) t += tb.DMinv[i][j] * du[j];
      c[i] -= t;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) cout[(size_t)i * K + k] = c[i];
}

template <int P>
static cudaError_t na_launch(int K, int numV, const int *V0T, const uint8_t *markD, const double *dataD,
                             const double *cin, double *cout, unsigned long long *s, cudaStream_t st) {
  k_na_reset<<<(numV + 255) / 256, 256, 0, st>>>(s, numV);
  const int grid = (K + kBlock - 1) / kBlock;
  k_na_scatter<P><<<grid, kBlock, 0, st>>>(K, V0T, cin, s);
  k_na_limit<P><<<grid, kBlock, 0, st>>>(K, V0T, markD, dataD, cin, cout, s);
  return cudaGetLastError();
}

}  // namespace dgadv

extern "C" int dgadv_limit_linear_noalloc(int32_t p, int32_t numT, int32_t numV, const int32_t *V0T,
                                          const uint8_t *markV0TbdrD, const double *dataV0T,
                                          const double *cIn, double *cOut, void *stream) {
  if (p < 1 || p > 3 || numT <= 0 || numV <= 0 || !V0T || !cIn || !cOut) return DGADV_EINVAL;
  if (numV > kNoAllocMaxVertices) return DGADV_ENOMEM;   // more vertices than the fixed scratch holds
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DGADV_ECUDA;
  if (dev < 0 || dev >= 64) return DGADV_EINVAL;
  {
    // Set-up on the first call per device (and per degree), with that device current: the
    // scratch array's device address and the FP64 constant tables of degree p.  Both are
    // synchronous runtime calls.
    std::lock_guard<std::mutex> lk(g_tab_mutex);
    if (!g_noalloc_addr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return DGADV_ECUDA;
      g_noalloc_addr[dev] = (unsigned long long *)ptr;
    }
    if (!g_tab_loaded[dev][0][p]) {
      RefTables rt;
      std::string err;
      if (!build_ref_tables(p, rt, err)) return DGADV_EINVAL;
      const cudaError_t e = p == 1 ? upload_tables<double, 1>(rt)
                          : p == 2 ? upload_tables<double, 2>(rt) : upload_tables<double, 3>(rt);
      if (e != cudaSuccess) return DGADV_ECUDA;
      g_tab_loaded[dev][0][p] = true;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long *s = g_noalloc_addr[dev];
  const cudaError_t e = p == 1 ? na_launch<1>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st)
                      : p == 2 ? na_launch<2>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st)
                               : na_launch<3>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st);
  return e == cudaSuccess ? DGADV_OK : DGADV_ECUDA;
}
