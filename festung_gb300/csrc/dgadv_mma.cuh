// The volume term's two contractions on the fifth-generation tensor cores (tcgen05), FP32 path,
// p >= 2, as an opt-in variant of the stage operator (DGADV_OPT_VOLUME_MMA):
//   c_q   = sum_j phi_j(x_q) c_j                     [128 elements x N] x [N x Q]
//   vol_i = sum_q d1phi_i(x_q) F1_q c_q + d2phi_i(x_q) F2_q c_q
//                                                    [128 elements x 2Q] x [2Q x N]
// (core/assembleMatElemDphiPhiFuncDiscVec.m:117-141 framed as GEMMs over the elements of a
// block).  Operands are split into TF32 pairs, x = hi + lo with hi the top 19 bits of x and lo
// the exact rest, and each product is accumulated in FP32 in tensor memory as
// A_hi B_hi + A_hi B_lo + A_lo B_hi, which leaves an error of order 2^-21 |A| |B|, near FP32's.
// Layouts: both operands K-major without swizzle, in core matrices of 8 rows x 16 bytes
// (row r, column k at (r/8) * 32K + (k/4) * 128 + (r%8) * 16 + (k%4) * 4 bytes; leading byte
// offset 128 between K-adjacent core matrices, stride byte offset 32K between row groups).
// One thread issues the MMAs (M = 128, N = 16, K = 8 per instruction) and commits them to an
// mbarrier; thread r of the block reads row r of the accumulator with tcgen05.ld (warp w owns
// tensor-memory lanes 32w..32w+31).  Waits are bounded: after a timeout the block flags bit 1,
// waits the same time again for its MMAs, frees its tensor memory and leaves the tile undone.
#pragma once
#include <cstdint>

namespace dgadv {
namespace vmma {

constexpr int kA1 = 128 * 16 * 4;    // A of the first contraction: 128 x 16 TF32
constexpr int kA2 = 128 * 32 * 4;    // A of the second: 128 x 32
constexpr int kB1 = 16 * 16 * 4;     // B of the first: Q (<= 16) rows x N (<= 16)
constexpr int kB2 = 16 * 32 * 4;     // B of the second: N (<= 16) rows x 2Q (<= 32)
constexpr int oA1h = 0, oA1l = oA1h + kA1, oA2h = oA1l + kA1, oA2l = oA2h + kA2;
constexpr int oB1h = oA2l + kA2, oB1l = oB1h + kB1, oB2h = oB1l + kB1, oB2l = oB2h + kB2;
constexpr int oBar = oB2l + kB2, oTmem = oBar + 8;
constexpr int kBytes = oBar + 16;    // the area, placed at a 1024-byte boundary
constexpr int kCols = 32;            // tensor-memory columns: D1 at 0..15, D2 at 16..31

__host__ __device__ constexpr int koff(int r, int k, int K) {
  return (r / 8) * (K * 32) + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4;
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// x = hi + lo into the two operand copies at byte offset `off`
__device__ __forceinline__ void put_split(unsigned char *m, int oh, int ol, int off, float x) {
  const float h = tf32_hi(x);
  *(float *)(m + oh + off) = h;
  *(float *)(m + ol + off) = x - h;
}

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;     // leading byte offset: K-adjacent core matrices
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;      // stride byte offset: 8-row groups
  d |= (uint64_t)1 << 46;                          // descriptor version of this architecture
  return d;                                        // base offset 0, no swizzle
}

// TF32 x TF32 -> FP32, M = 128, N = 16, both operands K-major
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
               "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}

// D = A_hi B_hi + A_hi B_lo + A_lo B_hi over K columns (K a multiple of 8), then a commit to bar.
__device__ __forceinline__ void issue(uint32_t dtmem, uint32_t aH, uint32_t aL, uint32_t bH, uint32_t bL, int K,
                                      uint64_t *bar) {
  const uint32_t sboA = (uint32_t)K * 32, sboB = (uint32_t)K * 32;
  for (int ks = 0; ks < K / 8; ++ks) {
    const uint32_t o = (uint32_t)ks * 256;
    mma_tf32(dtmem, sdesc(aH + o, sboA), sdesc(bH + o, sboB), ks > 0);
    mma_tf32(dtmem, sdesc(aH + o, sboA), sdesc(bL + o, sboB), 1);
    mma_tf32(dtmem, sdesc(aL + o, sboA), sdesc(bH + o, sboB), 1);
  }
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(bar))
               : "memory");
}

__device__ __forceinline__ void ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                 "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void alloc(uint32_t *dst) {   // warp-wide
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)), "r"(kCols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void dealloc(uint32_t base) {   // warp-wide
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(kCols));
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Block-wide barrier that also orders generic-proxy shared-memory writes before the tensor
// cores' reads and tcgen05 operations across it.
__device__ __forceinline__ void sync_for_mma() {
  proxy_fence();
  fence_before();
  __syncthreads();
  fence_after();
}

// The constant B operands of degree P (tables phiQ, g1, g2 of this unit), split, zero-padded.
template <int P>
__device__ __forceinline__ void fill_tables(unsigned char *m) {
  constexpr int N = Dims<P>::N, Q = Dims<P>::Q;
  const Tab<float, P> &tb = tab<float, P>();
  for (int e = threadIdx.x; e < 16 * 16; e += blockDim.x) {
    const int q = e / 16, j = e % 16;
    put_split(m, oB1h, oB1l, koff(q, j, 16), (q < Q && j < N) ? tb.phiQ[q][j] : 0.f);
  }
  for (int e = threadIdx.x; e < 16 * 32; e += blockDim.x) {
    const int i = e / 32, kk = e % 32;
    float v = 0.f;
    if (i < N && kk < Q) v = tb.g1[kk][i];
    else if (i < N && kk >= Q && kk < 2 * Q) v = tb.g2[kk - Q][i];
    put_split(m, oB2h, oB2l, koff(i, kk, 32), v);
  }
}

// Bounded wait on phase `parity` of the MMA barrier (see the header comment).
__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t parity, int *flag) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1LL << 31)) {
      atomicOr(flag, 2 | 16);                    // bit 4: the tensor cores
      const long long t1 = clock64();
      while (!mbar_try_wait(bar, parity) && clock64() - t1 < (1LL << 31)) {
      }
      return false;
    }
  return true;
}

}  // namespace vmma
}  // namespace dgadv
