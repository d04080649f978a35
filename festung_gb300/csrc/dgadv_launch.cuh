// Host-side launch sequences of the stage pipeline, templated on the stored real type.
// Included by each dgadv_prec_*.cu after dgadv_device.cuh.
#pragma once
#include <algorithm>
#include <cmath>
#include <string>

#include "dgadv_device.cuh"

namespace dgadv {

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
  // Gr = DM^-T hatM DM^-1 in FP64, then rounded
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int a = 0; a < N; ++a) {
        double r = 0.0;
        for (int b = 0; b < N; ++b) r += rt.hatM[a * N + b] * rt.DMinv[b * N + j];
        s += rt.DMinv[a * N + i] * r;
      }
      t.Gr[i][j] = T(s);
    }
  // adjoint tables (the forward FP32 path takes hatM^-1 = I; so does its adjoint)
  const bool massSolve = sizeof(T) == 8;
  auto fold = [&](const double *row, int j) {
    if (!massSolve) return row[j];
    double a = 0.0;
    for (int i = 0; i < N; ++i) a += row[i] * rt.hatMinv[i * N + j];
    return a;
  };
  for (int q = 0; q < Q; ++q)
    for (int j = 0; j < N; ++j) {
      t.Hg1[q][j] = T(fold(&rt.gradQ[q * N], j));
      t.Hg2[q][j] = T(fold(&rt.gradQ[Q * N + q * N], j));
    }
  for (int n = 0; n < 3; ++n)
    for (int r = 0; r < R; ++r)
      for (int j = 0; j < N; ++j) t.Hphi[n][r][j] = T(fold(&rt.phi1D[(n * R + r) * N], j));
  // forward tables: hatM^-1 applied from the left, in FP64, then rounded
  auto lfold = [&](const double *row, int i) {
    if (!massSolve) return row[i];
    double a = 0.0;
    for (int j = 0; j < N; ++j) a += rt.hatMinv[i * N + j] * row[j];
    return a;
  };
  for (int q = 0; q < Q; ++q)
    for (int i = 0; i < N; ++i) {
      t.Fg1[q][i] = T(lfold(&rt.gradQ[q * N], i));
      t.Fg2[q][i] = T(lfold(&rt.gradQ[Q * N + q * N], i));
    }
  for (int n = 0; n < 3; ++n)
    for (int r = 0; r < R; ++r)
      for (int i = 0; i < N; ++i) t.Fphi[n][r][i] = T(lfold(&rt.phi1D[(n * R + r) * N], i));
  return cudaMemcpyToSymbol(tab_symbol<T, P>(), &t, sizeof(t));
}

// The element operator (kOpElement) is in use: FP64 or double-float, enabled, built for the
// current velocity and no source terms (with them the mass solve is not folded); a
// double-float handle with the FP32 operator keeps that one.
static bool element_operator_on(const dgadv_handle *h) {
  return h->Aop && h->elemOp && h->aopVersion == h->velVersion && !(h->nTerms > 0 && h->rhs) && !h->opFp32;
}
template <typename T> constexpr bool kHasElementOperator = std::is_same_v<T, double> || std::is_same_v<T, df32>;

template <typename T>
static Geo<T> make_geo(const dgadv_handle *h) {
  Geo<T> g;
  g.K = h->K; g.Kp = h->Kp; g.numV = h->numV; g.Vp = h->Vp;
  g.F = (const T *)h->F; g.Vn = (const T *)h->Vn; g.nbr = h->nbr; g.code = h->code;
  g.Aop = element_operator_on(h) ? (const T *)h->Aop : nullptr;
  g.Bm = (const T *)h->Bm; g.MT = (const T *)h->MT; g.V0T = h->V0T; g.vptr = h->vptr; g.vidx = h->vidx;
  g.rhs = (const T *)h->rhs; g.cDV0T = (const T *)h->cDV0T; g.nTerms = h->nTerms;
  for (int i = 0; i < 4; ++i) g.timeFn[i] = h->timeFn[i];
  g.instOf = h->instOf;
  g.nInst = h->nInst;
  g.mtOnTheFly = h->mtOnTheFly ? 1 : 0;
  g.permv = h->perm;
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
  o.slots = h->gmm + (size_t)set * h->nInst * kSlotCopies * 2 * h->nc;
  o.reset = h->gmm + (size_t)next * h->nInst * kSlotCopies * 2 * h->nc;
  o.nc = h->nc; o.type = h->limType;
  return o;
}
template <typename T>
static LimIn<T> lim_in_pass(const dgadv_handle *h, long long pass) {
  using K_ = typename KeyOf<T>::type;
  const int set = (int)(((pass % 3) + 3) % 3);
  LimIn<T> i;
  i.vkeys = (const K_ *)h->vkeys + (size_t)set * 2 * h->nc * h->Vp;
  i.slots = h->gmm + (size_t)set * h->nInst * kSlotCopies * 2 * h->nc;
  i.nc = h->nc; i.type = h->limType;
  i.shift = (h->flags & DGADV_FLAG_NO_SHIFT) ? 0 : 1;
  return i;
}

// The adjoint's own key sets (the limiter adjoint recomputes the forward's patch extremes), with
// the forward's quantities per pass (one for the linear limiter, p(p+1)/2 for the hierarchical),
// and the element means of a pass's limiter input.
template <typename T>
static T *adj_means(const dgadv_handle *h, long long pass) {
  return (T *)h->adjMeans + (size_t)(pass % h->adjKeySets) * h->nc * h->Kp;
}
template <typename T>
static LimOut<T> lim_out_adj(dgadv_handle *h, long long pass) {
  using K_ = typename KeyOf<T>::type;
  const int set = (int)(pass % h->adjKeySets), next = (set + 1) % h->adjKeySets;
  const size_t vset = (size_t)2 * h->nc * h->Vp;
  LimOut<T> o;
  o.vkeys = (K_ *)h->vkeysA + set * vset;
  o.vreset = (K_ *)h->vkeysA + next * vset;
  o.slots = h->gmmA + (size_t)set * h->nInst * kSlotCopies * 2 * h->nc;
  o.reset = h->gmmA + (size_t)next * h->nInst * kSlotCopies * 2 * h->nc;
  o.nc = h->nc; o.type = h->limType;
  return o;
}
template <typename T>
static LimIn<T> lim_in_adj(const dgadv_handle *h, long long pass) {
  using K_ = typename KeyOf<T>::type;
  const int set = (int)(pass % h->adjKeySets);
  LimIn<T> i;
  i.vkeys = (const K_ *)h->vkeysA + (size_t)set * 2 * h->nc * h->Vp;
  i.slots = h->gmmA + (size_t)set * h->nInst * kSlotCopies * 2 * h->nc;
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

// Kernel launch on the handle's stream, with programmatic dependent launch unless disabled;
// `block` threads per CTA (launch_k: kBlock).
template <typename... KArgs, typename... Args>
static void launch_kb(const dgadv_handle *h, void (*kern)(KArgs...), int grid, int block, size_t smem, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = ((h->flags & DGADV_FLAG_NO_PDL) || h->pdlBreak) ? 0 : 1;
  h->pdlBreak = false;
  cudaLaunchKernelEx(&cfg, kern, args...);
}
template <typename... KArgs, typename... Args>
static void launch_k(const dgadv_handle *h, void (*kern)(KArgs...), int grid, size_t smem, Args... args) {
  launch_kb(h, kern, grid, kBlock, smem, args...);
}

// Copy of a state-sized buffer (a multiple of 16 bytes) in the dependent-launch chain.
static cudaError_t copy_state(dgadv_handle *h, void *dst, const void *src, size_t bytes) {
  const size_t n = bytes / 16;
  const int grid = (int)std::min<size_t>((n + kBlock - 1) / kBlock, 4 * 152);
  launch_k(h, k_copy16, std::max(grid, 1), (size_t)0, (const uint4 *)src, (uint4 *)dst, n);
  return cudaGetLastError();
}

// Opt-in shared memory sizes of the staged kernels of one (precision, degree).
template <typename T, int P, bool FUSED>
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
  if constexpr (kHasElementOperator<T>) {   // the element-operator variants
    set((const void *)k_stage_op<T, P, 0, false, false, kOpElement>, SR::bytes(SR::op(0, false, true), 1));
    set((const void *)k_stage_op<T, P, 1, false, false, kOpElement>, SR::bytes(SR::op(1, false, true), 1));
    set((const void *)k_stage_op<T, P, 2, false, false, kOpElement>, SR::bytes(SR::op(2, false, true), 1));
    set((const void *)k_stage_op<T, P, 1, false, true, kOpElement>, SR::bytes(SR::op(1, true, true), 1));
    set((const void *)k_stage_op<T, P, 2, false, true, kOpElement>, SR::bytes(SR::op(2, true, true), 1));
  }
  if constexpr (std::is_same_v<T, df32>) {   // the FP32-operator variants (DGADV_OPT_OPERATOR_FP32)
    set((const void *)k_stage_op<T, P, 0, true, false, true>, SR::bytes(SR::op(0, false), 1));
    set((const void *)k_stage_op<T, P, 0, false, false, true>, SR::bytes(SR::op(0, false), 1));
    set((const void *)k_stage_op<T, P, 1, true, false, true>, SR::bytes(SR::op(1, false), 1));
    set((const void *)k_stage_op<T, P, 1, false, false, true>, SR::bytes(SR::op(1, false), 1));
    set((const void *)k_stage_op<T, P, 2, true, false, true>, SR::bytes(SR::op(2, false), 1));
    set((const void *)k_stage_op<T, P, 2, false, false, true>, SR::bytes(SR::op(2, false), 1));
    set((const void *)k_stage_op<T, P, 1, true, true, true>, SR::bytes(SR::op(1, true), 1));
    set((const void *)k_stage_op<T, P, 1, false, true, true>, SR::bytes(SR::op(1, true), 1));
    set((const void *)k_stage_op<T, P, 2, true, true, true>, SR::bytes(SR::op(2, true), 1));
    set((const void *)k_stage_op<T, P, 2, false, true, true>, SR::bytes(SR::op(2, true), 1));
  }
  if constexpr (FUSED) {
    set((const void *)k_op_fused<T, P, 1, true>, SR::bytes(SR::op(1, true), 1));
    set((const void *)k_op_fused<T, P, 1, false>, SR::bytes(SR::op(1, true), 1));
    set((const void *)k_op_fused<T, P, 2, true>, SR::bytes(SR::op(2, true), 1));
    set((const void *)k_op_fused<T, P, 2, false>, SR::bytes(SR::op(2, true), 1));
  }
  set((const void *)k_limit_dot<T, P, 1>, SR::bytes(SR::limdot(), 1));
  set((const void *)k_limit_dot<T, P, 2>, SR::bytes(SR::limdot(), 1));
  set((const void *)k_limit<T, P, 1>, SR::bytes(SR::lim(), 1));
  set((const void *)k_limit<T, P, 2>, SR::bytes(SR::lim(), 1));
  set((const void *)k_to_taylor<T, P>, SR::bytes(SR::totaylor(), 0));
  if constexpr (std::is_same_v<T, float> && P >= 2) {
    set((const void *)k_stage_op_mma<P, true>, MmaSmem<P>::bytes(true));
    set((const void *)k_stage_op_mma<P, false>, MmaSmem<P>::bytes(false));
  }
  return e;
}

// The stage operator kernel of a handle: with DGADV_OPT_OPERATOR_FP32 on a double-float handle,
// the variant whose operator arithmetic is FP32 (state, SSP update and limiter in double-float);
// on an FP64 handle without source terms, the element-operator variant once it is built.
template <typename T, int P, int MODE, bool RHS, bool LIN>
static auto stage_kernel(const dgadv_handle *h) -> decltype(&k_stage_op<T, P, MODE, RHS, LIN, kOpPlain>) {
  if constexpr (std::is_same_v<T, df32>)
    if (h->opFp32) return &k_stage_op<T, P, MODE, RHS, LIN, kOpFp32>;
  if constexpr (kHasElementOperator<T> && !RHS)
    if (element_operator_on(h)) return &k_stage_op<T, P, MODE, RHS, LIN, kOpElement>;
  return &k_stage_op<T, P, MODE, RHS, LIN, kOpPlain>;
}
// Its staged rows.
template <typename T, int P>
static int stage_rows(const dgadv_handle *h, int mode, bool lin, bool rhs) {
  return StageRows<T, P>::op(mode, lin, kHasElementOperator<T> && !rhs && element_operator_on(h));
}

template <typename T, int P>
static cudaError_t launch_step(dgadv_handle *h, double t0, double tau) {
  using SR = StageRows<T, P>;
  const Geo<T> g = make_geo<T>(h);
  const int grid = (std::max(h->K, h->numV) + kBlock - 1) / kBlock;   // producers also reset vertex keys
  const int gridK = (h->K + kBlock - 1) / kBlock;
  // the stage operator's elements per block (DGADV_OPT_OP_BLOCK; one thread per element)
  const int eb = h->opBlock, gridOp = (std::max(h->K, h->numV) + eb - 1) / eb;
  double omega[3], cst[3];
  const int S = rk_table(h->ordRK, omega, cst);
  T *cA = (T *)h->cA, *cB = (T *)h->cB, *tb = (T *)h->tbuf;
  // c^n and c^(n+1): cn, unless the caller redirects them (stepSrc / stepDst)
  const T *cn = h->stepSrc ? (const T *)h->stepSrc : (const T *)h->cn;
  T *dst = h->stepDst ? (T *)h->stepDst : (T *)h->cn;
  const int nRun = (h->stepStages > 0 && h->stepStages < S) ? h->stepStages : S;
  const bool rhs = h->nTerms > 0 && h->rhs;
  for (int s = 0; s < nRun; ++s) {
    const T *in = (s == 0) ? cn : (s == 1 ? cA : cB);
    // the last stage may write c^(n+1) over c^n (it reads c^n of its own element only), but not
    // over its input, whose neighbour values it reads: with one stage it goes through cA
    T *out = (s == S - 1) ? ((S == 1 && (const T *)dst == cn) ? cA : dst) : (s == 0 ? cA : cB);
    StageScalars sc{};
    sc.omega = omega[s]; sc.tau = tau; sc.flag = h->flag;
    const double ts = t0 + cst[s] * tau;
    for (int m = 0; m < h->nTerms; ++m) sc.gco[m] = time_factor(h->timeFn[m], ts);
    LimOut<T> lo{};
    if (!h->lim) {
      prof_mark(h, 0);
      if (rhs) launch_kb(h, stage_kernel<T, P, 0, true, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 0, false, true), 1, eb), g, in, cn, out, lo, sc);
      else launch_kb(h, stage_kernel<T, P, 0, false, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 0, false, false), 1, eb), g, in, cn, out, lo, sc);
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
    // buffers of the limiter inputs: tb, or in a recorded run of the adjoint this stage's record
    // slots, written directly (cDot before time-derivative limiting; the unlimited stage value)
    T *cdB = (mode == 2 && h->recCdot[s]) ? (T *)h->recCdot[s] : tb;
    T *yB = h->recY[s] ? (T *)h->recY[s] : tb;
    prof_mark(h, 0);
    bool viaMma = false;
    if constexpr (std::is_same_v<T, float> && P >= 2) {
      if (mode == 2 && h->volumeMma && !rhs) {   // the volume term on the tensor cores
        if (lin) launch_k(h, k_stage_op_mma<P, true>, grid, MmaSmem<P>::bytes(true), g, (const T *)in, cdB, lo1, sc);
        else launch_k(h, k_stage_op_mma<P, false>, grid, MmaSmem<P>::bytes(false), g, (const T *)in, cdB, lo1, sc);
        viaMma = true;
      }
    }
    if (viaMma) {
    } else if (mode == 2) {
      if (lin) {
        if (rhs) launch_kb(h, stage_kernel<T, P, 2, true, true>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 2, true, true), 1, eb), g, in, cn, cdB, lo1, sc);
        else launch_kb(h, stage_kernel<T, P, 2, false, true>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 2, true, false), 1, eb), g, in, cn, cdB, lo1, sc);
      } else {
        if (rhs) launch_kb(h, stage_kernel<T, P, 2, true, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 2, false, true), 1, eb), g, in, cn, cdB, lo1, sc);
        else launch_kb(h, stage_kernel<T, P, 2, false, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 2, false, false), 1, eb), g, in, cn, cdB, lo1, sc);
      }
    } else {
      if (lin) {
        if (rhs) launch_kb(h, stage_kernel<T, P, 1, true, true>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 1, true, true), 1, eb), g, in, cn, yB, lo1, sc);
        else launch_kb(h, stage_kernel<T, P, 1, false, true>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 1, true, false), 1, eb), g, in, cn, yB, lo1, sc);
      } else {
        if (rhs) launch_kb(h, stage_kernel<T, P, 1, true, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 1, false, true), 1, eb), g, in, cn, yB, lo1, sc);
        else launch_kb(h, stage_kernel<T, P, 1, false, false>(h), gridOp, eb, SR::bytes(stage_rows<T, P>(h, 1, false, false), 1, eb), g, in, cn, yB, lo1, sc);
      }
    }
    prof_mark(h, -1);
    LimOut<T> loS = lo1;
    if (mode == 2) {
      const LimOut<T> lo2 = lim_out<T>(h);
      ++h->limPass;
      prof_mark(h, 1);
      if (lin) launch_k(h, k_limit_dot_lin<T, P>, grid, SR::bytes(SR::limdot_lin_rows(h->mtOnTheFly), 1), g, (const T *)in, (const T *)cn, (const T *)cdB, yB, lim_in<T>(lo1, h), lo2, sc);
      else if (h->limType == DGADV_LIM_STRICT)
        launch_k(h, k_limit_dot<T, P, 2>, grid, SR::bytes(SR::limdot(), 1), g, in, cn, (const T *)cdB, yB, lim_in<T>(lo1, h), lo2, sc);
      else
        launch_k(h, k_limit_dot<T, P, 1>, grid, SR::bytes(SR::limdot(), 1), g, in, cn, (const T *)cdB, yB, lim_in<T>(lo1, h), lo2, sc);
      prof_mark(h, -1);
      loS = lo2;
    }
    // the adjoint's recomputation wants the limiter inputs only: c^(n+1) is not written
    if (h->stepRecordsOnly && s == S - 1) break;
    prof_mark(h, 2);
    if (lin) launch_k(h, k_limit_lin<T, P>, gridK, (size_t)0, g, (const T *)yB, out, lim_in<T>(loS, h), scBC);
    else if (h->limType == DGADV_LIM_STRICT)
      launch_k(h, k_limit<T, P, 2>, grid, SR::bytes(SR::lim(), 1), g, (const T *)yB, out, lim_in<T>(loS, h), scBC);
    else
      launch_k(h, k_limit<T, P, 1>, grid, SR::bytes(SR::lim(), 1), g, (const T *)yB, out, lim_in<T>(loS, h), scBC);
    prof_mark(h, -1);
  }
  if (S == 1 && nRun == 1 && (const T *)dst == cn && !h->stepRecordsOnly) return copy_state(h, dst, cA, (size_t)h->N * h->Kp * sizeof(T));
  return cudaGetLastError();
}

// Fused path (linear limiter, zero Dirichlet data): per stage the operator kernel limits its
// input on the fly; for p >= 2 the time-derivative limiter follows.  The state between calls
// stays limited in cn; inside a call the step output R is unlimited, and finalize_fused limits
// it back into cn at the end of the call.

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
    launch_k(h, k_limit_dot_lin<T, P>, grid, SR::bytes(SR::limdot_lin_rows(h->mtOnTheFly), 1), g, (const T *)xL, (const T *)cnL,
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
    launch_k(h, k_mean_lin<T, P>, grid, (size_t)0, g, (const T *)h->cn, lo, (T *)nullptr);
    launch_k(h, k_limit_lin<T, P>, gridK, (size_t)0, g, (const T *)h->cn, (T *)h->cn, lim_in<T>(lo, h), sc);
  } else {
    launch_k(h, k_to_taylor<T, P>, grid, SR::bytes(SR::totaylor(), 0), g, (const T *)h->cn, (T *)h->tbuf, lo, sc);
    if (h->limType == DGADV_LIM_STRICT)
      launch_k(h, k_limit<T, P, 2>, grid, SR::bytes(SR::lim(), 1), g, (const T *)h->tbuf, (T *)h->cn, lim_in<T>(lo, h), sc);
    else
      launch_k(h, k_limit<T, P, 1>, grid, SR::bytes(SR::lim(), 1), g, (const T *)h->tbuf, (T *)h->cn, lim_in<T>(lo, h), sc);
  }
  return cudaGetLastError();
}

// Dispatch on the degree over the degrees a unit instantiates: bit P of MASK set for degree P.
// FUSED = false leaves the opt-in fused kernels out of a unit.
template <typename T, int MASK>
static cudaError_t dispatch_step(dgadv_handle *h, double t0, double tau) {
  switch (h->p) {
    case 0: if constexpr ((MASK & 1) != 0) return launch_step<T, 0>(h, t0, tau); break;
    case 1: if constexpr ((MASK & 2) != 0) return launch_step<T, 1>(h, t0, tau); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_step<T, 2>(h, t0, tau); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_step<T, 3>(h, t0, tau); break;
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK, bool FUSED>
static cudaError_t dispatch_step_fused(dgadv_handle *h, double t0, double tau, bool first) {
  if constexpr (FUSED) {
    switch (h->p) {
      case 1: if constexpr ((MASK & 2) != 0) return launch_step_fused<T, 1>(h, t0, tau, first); break;
      case 2: if constexpr ((MASK & 4) != 0) return launch_step_fused<T, 2>(h, t0, tau, first); break;
      case 3: if constexpr ((MASK & 8) != 0) return launch_step_fused<T, 3>(h, t0, tau, first); break;
    }
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK, bool FUSED>
static cudaError_t dispatch_finalize_fused(dgadv_handle *h) {
  if constexpr (FUSED) {
    switch (h->p) {
      case 1: if constexpr ((MASK & 2) != 0) return launch_finalize_fused<T, 1>(h); break;
      case 2: if constexpr ((MASK & 4) != 0) return launch_finalize_fused<T, 2>(h); break;
      case 3: if constexpr ((MASK & 8) != 0) return launch_finalize_fused<T, 3>(h); break;
    }
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK>
static cudaError_t dispatch_limit(dgadv_handle *h, double t) {
  switch (h->p) {
    case 1: if constexpr ((MASK & 2) != 0) return launch_limit_state<T, 1>(h, t); break;
    case 2: if constexpr ((MASK & 4) != 0) return launch_limit_state<T, 2>(h, t); break;
    case 3: if constexpr ((MASK & 8) != 0) return launch_limit_state<T, 3>(h, t); break;
  }
  return cudaErrorNotSupported;
}

template <typename T>
static cudaError_t scatter_in(dgadv_handle *h, void *dst) {
  const int grid = (h->K + 255) / 256;
  k_scatter_in<T><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, h->stage_ext, (T *)dst);
  return cudaGetLastError();
}
template <typename T>
static cudaError_t gather_out(dgadv_handle *h, const void *src) {
  const int grid = (h->K + 255) / 256;
  k_gather_out<T><<<grid, 256, 0, h->stream>>>(h->K, h->Kp, h->N, h->perm, (const T *)src, h->stage_ext);
  return cudaGetLastError();
}

template <typename T>
static cudaError_t from_f64(dgadv_handle *h, void *dst, const double *src, size_t n) {
  const int grid = (int)std::min<size_t>((n + 255) / 256, 4096);
  if (n == 0) return cudaSuccess;
  k_from_f64<T><<<grid, 256, 0, h->stream>>>(n, src, (T *)dst);
  return cudaGetLastError();
}

template <typename T, int MASK>
static cudaError_t upload_tables_p(int p, const RefTables &rt) {
  switch (p) {
    case 0: if constexpr ((MASK & 1) != 0) return upload_tables<T, 0>(rt); break;
    case 1: if constexpr ((MASK & 2) != 0) return upload_tables<T, 1>(rt); break;
    case 2: if constexpr ((MASK & 4) != 0) return upload_tables<T, 2>(rt); break;
    case 3: if constexpr ((MASK & 8) != 0) return upload_tables<T, 3>(rt); break;
  }
  return cudaErrorNotSupported;
}
template <typename T, int MASK, bool FUSED>
static cudaError_t set_smem_p(int p) {
  switch (p) {
    case 0: if constexpr ((MASK & 1) != 0) return set_smem_attributes<T, 0, FUSED>(); break;
    case 1: if constexpr ((MASK & 2) != 0) return set_smem_attributes<T, 1, FUSED>(); break;
    case 2: if constexpr ((MASK & 4) != 0) return set_smem_attributes<T, 2, FUSED>(); break;
    case 3: if constexpr ((MASK & 8) != 0) return set_smem_attributes<T, 3, FUSED>(); break;
  }
  return cudaErrorNotSupported;
}
template <typename T>
static void to_real(const double *src, size_t n, void *dst) {
  T *d = (T *)dst;
  for (size_t i = 0; i < n; ++i) d[i] = T(src[i]);
}

template <typename T, int MASK>
static cudaError_t dispatch_build_element_operator(dgadv_handle *h) {
  if constexpr (kHasElementOperator<T>) {
    const Geo<T> g = make_geo<T>(h);
    const int grid = (h->K + kBlock - 1) / kBlock;
    switch (h->p) {
      case 0: if constexpr ((MASK & 1) != 0) k_build_element_operator<T, 0><<<grid, kBlock, 0, h->stream>>>(g, (T *)h->Aop); break;
      case 1: if constexpr ((MASK & 2) != 0) k_build_element_operator<T, 1><<<grid, kBlock, 0, h->stream>>>(g, (T *)h->Aop); break;
      case 2: if constexpr ((MASK & 4) != 0) k_build_element_operator<T, 2><<<grid, kBlock, 0, h->stream>>>(g, (T *)h->Aop); break;
      case 3: if constexpr ((MASK & 8) != 0) k_build_element_operator<T, 3><<<grid, kBlock, 0, h->stream>>>(g, (T *)h->Aop); break;
    }
    return cudaGetLastError();
  }
  return cudaErrorNotSupported;
}

template <typename T, int MASK, bool FUSED>
static PrecOps make_ops() {
  PrecOps o;
  o.realBytes = sizeof(T);
  o.keyBytes = sizeof(typename KeyOf<T>::type);
  o.slotKeyMax = key_max<T>();
  o.fused = FUSED;
  o.to_real = to_real<T>;
  o.upload_tables = upload_tables_p<T, MASK>;
  o.set_smem = set_smem_p<T, MASK, FUSED>;
  o.step = dispatch_step<T, MASK>;
  o.step_fused = dispatch_step_fused<T, MASK, FUSED>;
  o.finalize_fused = dispatch_finalize_fused<T, MASK, FUSED>;
  o.limit = dispatch_limit<T, MASK>;
  o.scatter_in = scatter_in<T>;
  o.gather_out = gather_out<T>;
  o.adj_stage = nullptr;
  o.lim_vjp = nullptr;
  o.vjp_scatter = nullptr;
  o.lim_choice = nullptr;
  o.step_persist = nullptr;
  o.step_linked = nullptr;
  o.persist_attributes = nullptr;
  o.copy = copy_state;
  o.from_f64 = from_f64<T>;
  o.build_element_operator = kHasElementOperator<T> ? dispatch_build_element_operator<T, MASK> : nullptr;
  o.tr_stage = nullptr;
  o.tr_convert = nullptr;
  o.tr_mask = nullptr;
  return o;
}

}  // namespace dgadv
