// Linked stepping: the stage kernels of several handles (meshes of different degrees, e.g. the
// degree groups of an ensemble) as one launch per stage kernel.  Every block of a launch
// belongs to one handle ("part"): it finds its part in the launch table, then runs that part's
// tile function of its degree on the part's own data, key sets and scalars, exactly as the
// part's own launch would (the same tile functions, tile index and tile count local to the
// part), so results are bitwise those of stepping each handle alone.
//
// Per stage s of a step (parts with fewer RK stages sit out the later ones):
//   k_link_op      every part with s < its stage count: stage operator (MODE 0, 1 or 2)
//   k_link_limdot  the parts with time-derivative limiting (p >= 2, linear limiter)
//   k_link_lim     every limited part: solution limiter
// Included by a precision unit after dgadv_launch.cuh.
#pragma once
#include "dgadv_launch.cuh"

namespace dgadv {

constexpr int kMaxLinked = kMaxLinkedParts;   // parts of one linked launch

template <typename T> struct LinkPart {
  int p, mode;                 // degree; 0 no limiter, 1 limiter at p = 1, 2 limiter with cDot limiting
  int block0, nBlocks;         // this part's blocks in the launch
  Geo<T> g;
  const T *a, *b, *c;          // inputs (per kernel: see launch_linked_step)
  T *out;
  LimIn<T> li;
  LimOut<T> lo;
  StageScalars sc;
};
// Passed as a __grid_constant__ parameter: a block indexes its part in the parameter space
// directly, instead of every thread copying the table to local memory first.
template <typename T> struct LinkArgs {
  int n;
  LinkPart<T> part[kMaxLinked];
};

template <typename T>
__device__ __forceinline__ int link_part(const LinkArgs<T> &a) {
  int i = 0;
#pragma unroll
  for (int j = 1; j < kMaxLinked; ++j)
    if (j < a.n && (int)blockIdx.x >= a.part[j].block0) i = j;
  return i;
}

template <typename T, int MASK>
__global__ void __launch_bounds__(kBlock) k_link_op(const __grid_constant__ LinkArgs<T> a) {
  const int i = link_part(a);
  const LinkPart<T> &q = a.part[i];
  const int tile = blockIdx.x - q.block0;
  // FP64 parts with the element operator run its variant, as their own launches would
  constexpr bool kElem = std::is_same_v<T, double>;
#define DGADV_LINK_OP_VAR(P, VAR)                                                                              \
  {                                                                                                            \
    if (q.mode == 0) stage_op_tile<T, P, 0, false, false, VAR>(q.g, q.a, q.b, q.out, q.lo, q.sc, tile, q.nBlocks); \
    else if (q.mode == 1) stage_op_tile<T, P, 1, false, true, VAR>(q.g, q.a, q.b, q.out, q.lo, q.sc, tile, q.nBlocks); \
    else stage_op_tile<T, P, 2, false, true, VAR>(q.g, q.a, q.b, q.out, q.lo, q.sc, tile, q.nBlocks);         \
    return;                                                                                                    \
  }
#define DGADV_LINK_OP(P)                                          \
  if (q.p == P) {                                                 \
    if constexpr (kElem) if (q.g.Aop) DGADV_LINK_OP_VAR(P, kOpElement) \
    DGADV_LINK_OP_VAR(P, kOpPlain)                                \
  }
  if constexpr ((MASK & 2) != 0) { DGADV_LINK_OP(1) }
  if constexpr ((MASK & 4) != 0) { DGADV_LINK_OP(2) }
  if constexpr ((MASK & 8) != 0) { DGADV_LINK_OP(3) }
#undef DGADV_LINK_OP
#undef DGADV_LINK_OP_VAR
}

template <typename T, int MASK>
__global__ void __launch_bounds__(kBlock) k_link_limdot(const __grid_constant__ LinkArgs<T> a) {
  const int i = link_part(a);
  const LinkPart<T> &q = a.part[i];
  const int tile = blockIdx.x - q.block0;
  if constexpr ((MASK & 4) != 0)
    if (q.p == 2) { limit_dot_lin_tile<T, 2>(q.g, q.a, q.b, q.c, q.out, q.li, q.lo, q.sc, tile, q.nBlocks); return; }
  if constexpr ((MASK & 8) != 0)
    if (q.p == 3) { limit_dot_lin_tile<T, 3>(q.g, q.a, q.b, q.c, q.out, q.li, q.lo, q.sc, tile, q.nBlocks); return; }
}

template <typename T, int MASK>
__global__ void __launch_bounds__(kBlock) k_link_lim(const __grid_constant__ LinkArgs<T> a) {
  const int i = link_part(a);
  const LinkPart<T> &q = a.part[i];
  const int tile = blockIdx.x - q.block0;
  if constexpr ((MASK & 2) != 0)
    if (q.p == 1) { limit_lin_tile<T, 1>(q.g, q.a, q.out, q.li, q.sc, tile); return; }
  if constexpr ((MASK & 4) != 0)
    if (q.p == 2) { limit_lin_tile<T, 2>(q.g, q.a, q.out, q.li, q.sc, tile); return; }
  if constexpr ((MASK & 8) != 0)
    if (q.p == 3) { limit_lin_tile<T, 3>(q.g, q.a, q.out, q.li, q.sc, tile); return; }
}

// Largest dynamic shared memory a linked stage kernel needs over the degrees of MASK.
template <typename T, int MASK>
static size_t link_smem(int kind) {
  size_t b = 0;
  auto upd = [&](auto P_) {
    constexpr int P = decltype(P_)::value;
    using SR = StageRows<T, P>;
    constexpr bool e = std::is_same_v<T, double>;   // the element operator's rows (FP64)
    if (kind == 0) b = std::max({b, SR::bytes(SR::op(0, false, e), 1), SR::bytes(SR::op(1, true, e), 1),
                                 SR::bytes(SR::op(2, true, e), 1)});
    else if (kind == 1) b = std::max(b, SR::bytes(SR::limdot_lin(), 1));
  };
  if constexpr ((MASK & 2) != 0) upd(std::integral_constant<int, 1>());
  if constexpr ((MASK & 4) != 0) upd(std::integral_constant<int, 2>());
  if constexpr ((MASK & 8) != 0) upd(std::integral_constant<int, 3>());
  return b;
}

// One time step of every linked handle hs[0..n) (hs[0] the primary, on whose stream the
// launches go), with one launch per stage kernel.  Preconditions checked by the caller: same
// precision and device, degrees 1..3 within MASK, no limiter or the linear one, no source
// terms, no fused / persistent pipeline, no redirected step input or output.
template <typename T, int MASK>
static cudaError_t launch_linked_step(dgadv_handle **hs, int n, double /*t0: no time-dependent data*/,
                                      double tau) {
  static_assert((MASK & 1) == 0, "linked steps cover degrees 1..3");
  dgadv_handle *h0 = hs[0];
  const size_t smemOp = link_smem<T, MASK>(0), smemLd = link_smem<T, MASK>(1);
  cudaError_t e = cudaFuncSetAttribute((const void *)k_link_op<T, MASK>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemOp);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void *)k_link_limdot<T, MASK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smemLd);
  if (e != cudaSuccess) return e;
  const int eb = h0->opBlock;                           // the operator's elements per block
  int S[kMaxLinked];
  double omega[kMaxLinked][3], cst[kMaxLinked][3];
  int Smax = 0;
  for (int i = 0; i < n; ++i) {
    S[i] = rk_table(hs[i]->ordRK, omega[i], cst[i]);
    Smax = std::max(Smax, S[i]);
  }
  for (int s = 0; s < Smax; ++s) {
    LinkArgs<T> op{}, ld{}, lm{};
    int gOp = 0, gLd = 0, gLm = 0;
    for (int i = 0; i < n; ++i) {
      dgadv_handle *h = hs[i];
      if (s >= S[i]) continue;
      const Geo<T> g = make_geo<T>(h);
      const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;
      const int gridE = (std::max(h->K, h->numV) + eb - 1) / eb;
      const int gridK = (h->K + kBlock - 1) / kBlock;
      T *cA = (T *)h->cA, *cB = (T *)h->cB, *tb = (T *)h->tbuf, *cn = (T *)h->cn;
      const T *in = (s == 0) ? cn : (s == 1 ? cA : cB);
      T *out = (s == S[i] - 1) ? (S[i] == 1 ? cA : cn) : (s == 0 ? cA : cB);
      StageScalars sc{};
      sc.omega = omega[i][s]; sc.tau = tau; sc.flag = h->flag;
      LinkPart<T> &q = op.part[op.n++];
      q.p = h->p; q.g = g; q.block0 = gOp; q.nBlocks = gridE; q.sc = sc;
      q.a = in; q.b = cn;
      gOp += gridE;
      if (!h->lim) {
        q.mode = 0; q.out = out;
        continue;
      }
      const LimOut<T> lo1 = lim_out<T>(h);
      ++h->limPass;
      q.lo = lo1;
      q.mode = h->limdot ? 2 : 1;
      q.out = tb;                                       // cDot (mode 2) or the unlimited c^(s) (mode 1)
      LimOut<T> loS = lo1;
      if (h->limdot) {
        const LimOut<T> lo2 = lim_out<T>(h);
        ++h->limPass;
        LinkPart<T> &r = ld.part[ld.n++];
        r.p = h->p; r.mode = 2; r.g = g; r.block0 = gLd; r.nBlocks = grid; r.sc = sc;
        r.a = in; r.b = cn; r.c = tb; r.out = tb;       // the new unlimited stage value over cDot
        r.li = lim_in<T>(lo1, h); r.lo = lo2;
        gLd += grid;
        loS = lo2;
      }
      StageScalars scBC = sc;                           // no Dirichlet terms (checked by the caller)
      LinkPart<T> &l = lm.part[lm.n++];
      l.p = h->p; l.mode = q.mode; l.g = g; l.block0 = gLm; l.nBlocks = gridK; l.sc = scBC;
      l.a = tb; l.out = out; l.li = lim_in<T>(loS, h);
      gLm += gridK;
    }
    if (op.n) { prof_mark(h0, 0); launch_kb(h0, k_link_op<T, MASK>, gOp, eb, smemOp, op); prof_mark(h0, -1); }
    if (ld.n) { prof_mark(h0, 1); launch_k(h0, k_link_limdot<T, MASK>, gLd, smemLd, ld); prof_mark(h0, -1); }
    if (lm.n) { prof_mark(h0, 2); launch_k(h0, k_link_lim<T, MASK>, gLm, (size_t)0, lm); prof_mark(h0, -1); }
  }
  for (int i = 0; i < n; ++i)
    if (S[i] == 1)                   // a one-stage step wrote cA (its input is c^n itself)
      copy_state(h0, hs[i]->cn, hs[i]->cA, (size_t)hs[i]->N * hs[i]->Kp * sizeof(T));
  return cudaGetLastError();
}

// The linked kernels carry the code of every degree they may meet, and their register count is
// that of the largest: groups without p = 3 (the ensemble workload's degrees 1 and 2) use
// kernels built for p <= 2 only.
template <typename T>
static cudaError_t launch_linked_step_any(dgadv_handle **hs, int n, double t0, double tau) {
  int pmax = 0;
  for (int i = 0; i < n; ++i) pmax = std::max(pmax, hs[i]->p);
  if (pmax <= 2) return launch_linked_step<T, 0x6>(hs, n, t0, tau);
  return launch_linked_step<T, 0xE>(hs, n, t0, tau);
}

template <typename T>
static PrecOps with_linked(PrecOps o) {
  o.step_linked = launch_linked_step_any<T>;
  return o;
}

}  // namespace dgadv
