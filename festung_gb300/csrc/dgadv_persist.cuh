// Persistent time step: one cooperative launch runs every stage of a time step, with grid-wide
// barriers where the separate-kernel pipeline has kernel boundaries.
//
// At meshes of about 10^5 elements every stage kernel is one partial wave: a fair part of its
// time is launch ramp and drain, and a time step is nine dependent kernels (three per stage
// with the linear limiter at p >= 2).  Here the blocks stay resident and walk the element tiles
// of each phase (operator, time-derivative limiter, solution limiter) with the same per-tile
// code as the separate kernels (stage_op_tile, limit_dot_lin_tile, limit_lin_tile); a phase
// ends at a grid barrier.  Results are the separate pipeline's, bit for bit.
//
// The launch is cooperative (all blocks co-resident, or the launch fails), and each barrier
// wait is bounded: after ~2^31 SM cycles a block sets bit 1 of the error flag
// (DGADV_ETIMEOUT at the next sync) and returns instead of waiting on.
#pragma once
#include <cstring>

#include "dgadv_launch.cuh"

namespace dgadv {

// Barrier state: arrivals counted in 32 groups (blockIdx % 32), each counter on its own 128-byte
// line, then one counter over the groups; the last arrival advances the generation that the
// other blocks poll.  Spreading the arrivals keeps same-address atomics to ~gridDim/32 + 32.
constexpr int kBarLine = 32;   // 32 x 4 B = one 128-byte line
struct GridBar {
  unsigned int gen[kBarLine];                // gen[0]: barriers completed
  unsigned int top[kBarLine];                // top[0]: groups complete at the current barrier
  unsigned int group[32][kBarLine];          // group[g][0]: arrivals of group g
};

// Grid-wide barrier over the cooperative grid; false (in every thread of the block) if this
// block gave up waiting.
__device__ __forceinline__ bool grid_sync(GridBar *b, int *flag) {
  __shared__ int okShared;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int *vgen = &b->gen[0];
    const unsigned int g0 = *vgen;
    __threadfence();
    const unsigned int grp = blockIdx.x & 31u;
    const unsigned int grpSize = (gridDim.x - grp + 31u) / 32u;   // blocks b with b % 32 == grp
    const unsigned int nGroups = gridDim.x < 32u ? gridDim.x : 32u;
    if (atomicAdd(&b->group[grp][0], 1u) == grpSize - 1u) {
      atomicExch(&b->group[grp][0], 0u);
      if (atomicAdd(&b->top[0], 1u) == nGroups - 1u) {
        atomicExch(&b->top[0], 0u);
        __threadfence();
        atomicAdd(&b->gen[0], 1u);
      }
    }
    const long long t0 = clock64();
    while (*vgen == g0) {
      __nanosleep(32);
      if (clock64() - t0 > (1LL << 31)) {
        atomicOr(flag, 2 | 8);                   // bit 3: the grid barrier
        ok = 0;
        break;
      }
    }
    __threadfence();
    okShared = ok;
  }
  __syncthreads();
  return okShared != 0;
}

template <typename T> struct PersistArgs {
  Geo<T> g;
  int S;              // stages of the step
  int nTiles;         // tiles of the producer phases (cover max(K, numV): they reset vertex keys)
  int nTilesK;        // tiles of the elements
  T *cn, *cA, *cB, *tb;
  StageScalars sc[3];     // per stage, at t(s)
  StageScalars scBC[3];   // per stage, boundary time of the solution limiter
  LimOut<T> lo1[3], lo2[3];
  LimIn<T> li1[3], li2[3];
  GridBar *bar;
};

// After a tile (and the block barrier that follows it): thread 0 ends the life of the tile's
// mbarrier, which the tile function placed after `nT` staged rows, before the next tile stages
// rows of another layout over that location.  Tiles past the elements staged nothing.
template <typename T, int P>
__device__ __forceinline__ void end_tile_barrier(const Geo<T> &g, int tile, int nT) {
  if (threadIdx.x == 0 && tile * kBlock < g.K) {
    extern __shared__ __align__(128) unsigned char smem[];
    mbar_inval((uint64_t *)(smem + StageRows<T, P>::bar_offset(nT, 1, blockDim.x)));
  }
}

// LIMMODE 0: no limiter; 1: linear limiter at p = 1; 2: linear limiter at p >= 2 (with the
// time-derivative limiter).  Time-independent data without source terms.
template <typename T, int P, int LIMMODE>
__global__ void __launch_bounds__(kBlock) k_step_persistent(const PersistArgs<T> a) {
  using SR = StageRows<T, P>;
#pragma unroll
  for (int s = 0; s < 3; ++s) {
    if (s >= a.S) break;
    T *in = (s == 0) ? a.cn : (s == 1 ? a.cA : a.cB);
    T *out = (s == a.S - 1) ? (a.S == 1 ? a.cA : a.cn) : (s == 0 ? a.cA : a.cB);
    // FP64 with the element operator: its variant, as the separate kernels use it
    const bool elem = std::is_same_v<T, double> && a.g.Aop != nullptr;
    if (LIMMODE == 0) {
      for (int tile = blockIdx.x; tile < a.nTilesK; tile += gridDim.x) {
        if constexpr (std::is_same_v<T, double>)
          if (elem) stage_op_tile<T, P, 0, false, false, kOpElement>(a.g, in, a.cn, out, a.lo1[s], a.sc[s], tile);
        if (!elem) stage_op_tile<T, P, 0, false, false>(a.g, in, a.cn, out, a.lo1[s], a.sc[s], tile);
        __syncthreads();
        end_tile_barrier<T, P>(a.g, tile, SR::op(0, false, elem));
      }
      if (!grid_sync(a.bar, a.sc[s].flag)) return;
      continue;
    }
    // operator: cDot (p >= 2) or the unlimited stage value (p = 1), means scattered
    for (int tile = blockIdx.x; tile < a.nTiles; tile += gridDim.x) {
      if constexpr (std::is_same_v<T, double>)
        if (elem) stage_op_tile<T, P, (LIMMODE == 2 ? 2 : 1), false, true, kOpElement>(a.g, in, a.cn, a.tb, a.lo1[s], a.sc[s], tile);
      if (!elem) stage_op_tile<T, P, (LIMMODE == 2 ? 2 : 1), false, true>(a.g, in, a.cn, a.tb, a.lo1[s], a.sc[s], tile);
      __syncthreads();
      end_tile_barrier<T, P>(a.g, tile, SR::op(LIMMODE == 2 ? 2 : 1, true, elem));
    }
    if (!grid_sync(a.bar, a.sc[s].flag)) return;
    if (LIMMODE == 2) {
      // time-derivative limiter, Taylor mass correction, SSP update, means scattered
      for (int tile = blockIdx.x; tile < a.nTiles; tile += gridDim.x) {
        limit_dot_lin_tile<T, P>(a.g, in, a.cn, a.tb, a.tb, a.li1[s], a.lo2[s], a.sc[s], tile);
        __syncthreads();
        end_tile_barrier<T, P>(a.g, tile, SR::limdot_lin_rows(a.g.mtOnTheFly != 0));
      }
      if (!grid_sync(a.bar, a.sc[s].flag)) return;
    }
    // solution limiter
    for (int tile = blockIdx.x; tile < a.nTilesK; tile += gridDim.x) {
      limit_lin_tile<T, P>(a.g, a.tb, out, LIMMODE == 2 ? a.li2[s] : a.li1[s], a.scBC[s], tile);
      __syncthreads();
    }
    if (!grid_sync(a.bar, a.sc[s].flag)) return;
  }
  if (a.S == 1) {   // first-order steps end in cA
    const size_t n = (size_t)Dims<P>::N * a.g.Kp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
      a.cn[i] = a.cA[i];
  }
}

template <typename T, int P>
static size_t persist_smem() {
  using SR = StageRows<T, P>;
  constexpr bool e = std::is_same_v<T, double>;   // the element operator's rows (FP64)
  size_t b = SR::bytes(SR::op(0, false, e), 1);
  b = std::max(b, SR::bytes(SR::op(1, true, e), 1));
  b = std::max(b, SR::bytes(SR::op(2, true, e), 1));
  b = std::max(b, SR::bytes(SR::limdot_lin(), 1));
  return b;
}

template <typename T, int P>
static void *persist_kernel(const dgadv_handle *h) {
  if (!h->lim) return (void *)k_step_persistent<T, P, 0>;
  return h->limdot ? (void *)k_step_persistent<T, P, 2> : (void *)k_step_persistent<T, P, 1>;
}

// Shared memory opt-in of the persistent kernels of one degree.
template <typename T, int P>
static cudaError_t persist_attributes() {
  const int b = (int)persist_smem<T, P>();
  cudaError_t e = cudaFuncSetAttribute((const void *)k_step_persistent<T, P, 0>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess && P >= 1)
    e = cudaFuncSetAttribute((const void *)k_step_persistent<T, P, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess && P >= 1)
    e = cudaFuncSetAttribute((const void *)k_step_persistent<T, P, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  return e;
}

template <typename T, int P>
static cudaError_t launch_step_persistent(dgadv_handle *h, double t0, double tau) {
  PersistArgs<T> a;
  std::memset((void *)&a, 0, sizeof(a));
  a.g = make_geo<T>(h);
  double omega[3], cst[3];
  a.S = rk_table(h->ordRK, omega, cst);
  a.nTiles = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;
  a.nTilesK = (h->K + kBlock - 1) / kBlock;
  a.cn = (T *)h->cn; a.cA = (T *)h->cA; a.cB = (T *)h->cB; a.tb = (T *)h->tbuf;
  a.bar = (GridBar *)h->gridBar;
  for (int s = 0; s < a.S; ++s) {
    a.sc[s].omega = omega[s]; a.sc[s].tau = tau; a.sc[s].flag = h->flag;
    a.scBC[s] = a.sc[s];
    if (!h->lim) continue;
    a.lo1[s] = lim_out<T>(h);
    a.li1[s] = lim_in<T>(a.lo1[s], h);
    ++h->limPass;
    if (h->limdot) {
      a.lo2[s] = lim_out<T>(h);
      a.li2[s] = lim_in<T>(a.lo2[s], h);
      ++h->limPass;
    }
  }
  const size_t smem = persist_smem<T, P>();
  void *kern = persist_kernel<T, P>(h);
  if (h->persistGrid <= 0) {
    int perSM = 0, dev = 0, nSM = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, (const void *)kern, kBlock, smem);
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nSM, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (perSM < 1) return cudaErrorCooperativeLaunchTooLarge;
    if (h->persistPerSM > 0) perSM = std::min(perSM, h->persistPerSM);
    h->persistGrid = std::min(perSM * nSM, a.nTiles);
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(h->persistGrid);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  prof_mark(h, 0);
  const cudaError_t e = cudaLaunchKernelEx(&cfg, (void (*)(PersistArgs<T>))kern, a);
  prof_mark(h, -1);
  return e;
}

template <typename T, int MASK>
static cudaError_t dispatch_step_persistent(dgadv_handle *h, double t0, double tau) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return launch_step_persistent<T, 1>(h, t0, tau); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_step_persistent<T, 2>(h, t0, tau); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_step_persistent<T, 3>(h, t0, tau); break;
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK>
static cudaError_t dispatch_persist_attributes(int p) {
  switch (p) {
    case 1: if constexpr ((MASK & 2) != 0) return persist_attributes<T, 1>(); break;
    case 2: if constexpr ((MASK & 4) != 0) return persist_attributes<T, 2>(); break;
    case 3: if constexpr ((MASK & 8) != 0) return persist_attributes<T, 3>(); break;
  }
  return cudaSuccess;
}

// The operation table of a unit with the persistent step added.
template <typename T, int MASK>
static PrecOps with_persistent(PrecOps o) {
  o.step_persist = dispatch_step_persistent<T, MASK>;
  o.persist_attributes = dispatch_persist_attributes<T, MASK>;
  return o;
}

}  // namespace dgadv
