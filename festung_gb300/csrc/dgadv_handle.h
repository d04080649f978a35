// Per-handle state of the device solver and the per-precision operation table.
//
// The kernels of one arithmetic type (FP64, FP32, double-float FP32x2) live in their own
// translation unit (dgadv_prec_*.cu) with their own constant tables; each exports one PrecOps
// table through which the C-ABI (dgadv_solver.cu) enqueues work for a handle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dgadv.h"
#include "dgadv_host.h"

namespace dgadv {
constexpr int kBlock = 128;       // elements per CTA (one thread per element)
constexpr int kSlotCopies = 32;   // copies of the global min / max slots (atomics spread over them)
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

// Work of one arithmetic type, enqueued on the handle's stream.
struct PrecOps {
  size_t realBytes;                    // bytes of one stored real
  size_t keyBytes;                     // bytes of one vertex min / max key
  unsigned long long slotKeyMax;       // reset value of a global-min slot
  bool fused;                          // the opt-in fused kernels are built for this type
  // host FP64 -> stored reals (n values), written to dst (host memory of n * realBytes)
  void (*to_real)(const double *src, size_t n, void *dst);
  cudaError_t (*upload_tables)(int p, const RefTables &rt);   // constant tables of degree p
  cudaError_t (*set_smem)(int p);                             // opt-in shared memory sizes
  cudaError_t (*step)(dgadv_handle *h, double t0, double tau);
  cudaError_t (*step_fused)(dgadv_handle *h, double t0, double tau, bool firstOfCall);
  cudaError_t (*finalize_fused)(dgadv_handle *h);
  cudaError_t (*limit)(dgadv_handle *h, double t);
  cudaError_t (*scatter_in)(dgadv_handle *h);   // stage_ext (caller order, FP64) -> cn
  cudaError_t (*gather_out)(dgadv_handle *h);   // cn -> stage_ext
};

// Fused path (linear limiter, zero Dirichlet data, opted in): per stage the operator kernel
// limits its input on the fly.
inline bool use_fused(const dgadv_handle *h) {
  return h->lim && h->limType == DGADV_LIM_LINEAR && !h->cDV0T && (h->flags & DGADV_FLAG_FUSE);
}

const PrecOps &ops_fp64();
const PrecOps &ops_fp32();
const PrecOps &ops_df32_p01();   // df32 kernels compile per degree (three units in parallel)
const PrecOps &ops_df32_p2();
const PrecOps &ops_df32_p3();

}  // namespace dgadv
