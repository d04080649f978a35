// dgadv_limit_linear_noalloc (include/dgadv.h): one linear limiter pass on device arrays owned
// by the caller, with its scratch in a fixed __device__ array instead of an allocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "dgadv_device.cuh"

namespace dgadv {
DGADV_DEFINE_TABLES(double, cTn)
}  // namespace dgadv

#include "dgadv_launch.cuh"

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
static bool g_noalloc_tables[64][kMaxP + 1];      // FP64 tables of this unit uploaded, per device
static std::mutex g_noalloc_mutex;

// Clears the keys of numV vertices (min = largest key, max = 0) and the extremes' copies.
__global__ void k_na_reset(unsigned long long *s, int numV) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v < numV) { s[v] = ~0ULL; s[kNoAllocMaxVertices + v] = 0ULL; }
  if (blockIdx.x == 0 && threadIdx.x < 2 * kSlotCopies)
    s[2 * kNoAllocMaxVertices + threadIdx.x] = (threadIdx.x & 1) ? 0ULL : ~0ULL;
}

// Element means (the centroid values) scattered to the three vertices' keys and to the
// global extremes (core/computeMinMaxV0TElementPatch.m).
// The three vertex ids of element k, and whether all lie in [0, numV) (numV never exceeds the
// scratch array's vertex slots).  Elements with an id outside that range take no part in any
// patch and are not limited: their output is NaN, so that the caller sees the bad input.
__device__ __forceinline__ bool na_vertices(const int *V0T, int K, int numV, int k, int vid[3]) {
  bool ok = true;
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    vid[n] = V0T[(size_t)n * K + k];
    ok &= (unsigned)vid[n] < (unsigned)numV;
  }
  return ok;
}

template <int P>
__global__ void __launch_bounds__(kBlock)
k_na_scatter(int K, int numV, const int *__restrict__ V0T, const double *__restrict__ c, unsigned long long *s) {
  constexpr int N = Dims<P>::N;
  const int k = blockIdx.x * kBlock + threadIdx.x;
  Geo<double> g{};
  g.Vp = kNoAllocMaxVertices;
  LimOut<double> lo{};
  lo.vkeys = s; lo.slots = s + 2 * kNoAllocMaxVertices; lo.nc = 1; lo.type = 0;
  int vid[3] = {0, 0, 0};
  const bool active = k < K && na_vertices(V0T, K, numV, k, vid);
  double q0 = 0.0;
  if (active) {
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
k_na_limit(int K, int numV, const int *__restrict__ V0T, const uint8_t *__restrict__ markD,
           const double *__restrict__ dataD, const double *cin, double *cout, const unsigned long long *s) {
  constexpr int N = Dims<P>::N;
  const Tab<double, P> &tb = tab<double, P>();
  __shared__ double sh[2];
  const int k = blockIdx.x * kBlock + threadIdx.x;
  Geo<double> g{};
  g.Vp = kNoAllocMaxVertices;
  LimIn<double> li{};
  li.vkeys = s; li.slots = s + 2 * kNoAllocMaxVertices; li.nc = 1; li.type = 0; li.shift = 1;
  load_shifts<double>(li.slots, 1, sh);
  __syncthreads();
  if (k >= K) return;
  int vid[3];
  if (!na_vertices(V0T, K, numV, k, vid)) {
#pragma unroll
    for (int i = 0; i < N; ++i) cout[(size_t)i * K + k] = __longlong_as_double(0x7FF8000000000000LL);
    return;
  }
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
  k_na_scatter<P><<<grid, kBlock, 0, st>>>(K, numV, V0T, cin, s);
  k_na_limit<P><<<grid, kBlock, 0, st>>>(K, numV, V0T, markD, dataD, cin, cout, s);
  return cudaGetLastError();
}

}  // namespace dgadv

using namespace dgadv;

extern "C" int dgadv_limit_linear_noalloc(int32_t p, int32_t numT, int32_t numV, const int32_t *V0T,
                                          const uint8_t *markV0TbdrD, const double *dataV0T,
                                          const double *cIn, double *cOut, void *stream) {
  return guarded(nullptr, [&]() -> int {
  if (p < 1 || p > 3 || numT <= 0 || numV <= 0 || !V0T || !cIn || !cOut) return DGADV_EINVAL;
  if (numV > kNoAllocMaxVertices) return DGADV_ENOMEM;   // more vertices than the fixed scratch holds
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return DGADV_ECUDA;
  if (dev < 0 || dev >= 64) return DGADV_EINVAL;
  {
    // Set-up on the first call per device (and per degree), with that device current: the
    // scratch array's device address and the FP64 constant tables of degree p.  Both are
    // synchronous runtime calls.
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return DGADV_ECUDA;
      g_noalloc_addr[dev] = (unsigned long long *)ptr;
    }
    if (!g_noalloc_tables[dev][p]) {
      RefTables rt;
      std::string err;
      if (!build_ref_tables(p, rt, err)) return DGADV_EINVAL;
      const cudaError_t e = p == 1 ? upload_tables<double, 1>(rt)
                          : p == 2 ? upload_tables<double, 2>(rt) : upload_tables<double, 3>(rt);
      if (e != cudaSuccess) return DGADV_ECUDA;
      g_noalloc_tables[dev][p] = true;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long *s = g_noalloc_addr[dev];
  const cudaError_t e = p == 1 ? na_launch<1>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st)
                      : p == 2 ? na_launch<2>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st)
                               : na_launch<3>(numT, numV, V0T, markV0TbdrD, dataV0T, cIn, cOut, s, st);
  return e == cudaSuccess ? DGADV_OK : DGADV_ECUDA;
  });
}
