// Per-handle state of the device solver and the per-precision operation table.
//
// The kernels of one arithmetic type (FP64, FP32, double-float FP32x2) live in their own
// translation unit (dgadv_prec_*.cu) with their own constant tables; each exports one PrecOps
// table through which the C-ABI (dgadv_solver.cu) enqueues work for a handle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/dgadv.h"
#include "dgadv_guard.h"
#include "dgadv_host.h"

struct dgadv_handle;
namespace dgadv {
struct OutputQueue;
void output_release(dgadv_handle *h);   // joins the writer thread, frees the output buffers
struct ImplicitState;
void implicit_release(dgadv_handle *h); // frees the implicit solver's host state
struct TransportState;
void transport_release(dgadv_handle *h);
// Rebuilds the FP64 element operator after the velocity factors changed (a no-op for the other
// precisions, implicit handles, or with DGADV_OPT_ELEMENT_OPERATOR = 0).
int refresh_element_operator(dgadv_handle *h);
constexpr int kBlock = 128;       // elements per CTA (one thread per element)
constexpr int kSlotCopies = 32;   // copies of the global min / max slots (atomics spread over them)
constexpr int kGridBarBytes = 8192;   // state of the persistent step's grid barrier
constexpr int kMaxLinkedParts = 4;    // handles in one linked step (a primary and three more)
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
  int nInst = 1;                       // ensembles: instances (each its own limiter extremes)
  int *instOf = nullptr;               // ensembles: instance of each block of kBlock elements
  std::vector<int> instStart;          // first element of each instance (caller order), + K
  void *cn = nullptr, *cA = nullptr, *cB = nullptr, *tbuf = nullptr;
  // one call of the staged step (the adjoint's recomputation): c^n read from stepSrc and c^(n+1)
  // written to stepDst instead of cn, and only the first stepStages stages run (0: all)
  const void *stepSrc = nullptr;
  void *stepDst = nullptr;
  int stepStages = 0;
  bool stepRecordsOnly = false;        // ... and the last stage's solution limiter is left out
  mutable bool pdlBreak = false;       // the next launch waits for its predecessors to complete
  int adjWarps = 2;                    // warps per role of the FP32 adjoint stage (1, 2 or 4)
  int adjStreams = 3;                  // reverse sweep: streams (1; 2 with the recomputation on a
                                       // second; 3 with the advances on a third)
  int adjGraph = -1;                   // reverse sweep as one CUDA graph: 1, 0, or -1 (by limiter)
  bool mtOnTheFly = false;             // Taylor mass correction rebuilt from B (DGADV_OPT_TAYLOR_MASS)
  bool volumeMma = false;              // volume term on the tensor cores (DGADV_OPT_VOLUME_MMA)
  int opBlock = 128;                   // elements per block of the stage operator (DGADV_OPT_OP_BLOCK)
  bool opFp32 = false;                 // double-float handle, FP32 operator (DGADV_OPT_OPERATOR_FP32)
  // FP64: the stage operator's volume term and own outflow terms as one N x N matrix per element
  // (DGADV_OPT_ELEMENT_OPERATOR), built for velocity version aopVersion
  bool elemOp = true;
  void *Aop = nullptr;
  int aopVersion = -1;
  // linked stepping (dgadv_link): this handle steps the handles in `linked` together with itself,
  // one launch per stage kernel; a handle in another's list has that handle as linkedTo
  std::vector<dgadv_handle *> linked;
  dgadv_handle *linkedTo = nullptr;
  std::vector<std::pair<long long, cudaGraphExec_t>> linkGraphs;   // key: phases of every part
  double linkGraphTau = -1.0;
  cudaEvent_t linkEv = nullptr;        // orders this handle's stream with the linked ones
  void *cR = nullptr, *cnL = nullptr, *cLx = nullptr;   // fused path: raw step output, limited c^n / c^(s-1)
  void *vkeys = nullptr;               // 3 passes x nc x 2 x Vp vertex min / max keys
  unsigned long long *gmm = nullptr;   // 3 passes x kSlotCopies x 2 x nc encoded global extremes
  long long limPass = 1;               // limiter passes enqueued so far (selects key / slot set)
  int graphSteps = 12;                 // time steps per captured CUDA graph
  void *gridBar = nullptr;             // grid barrier state of the persistent step (zeroed)
  int persistGrid = 0;                 // blocks of the persistent step (0: not yet sized)
  int persistPerSM = 0;                // resident blocks per SM it may use (0: all that fit)
  int passesPerStep = 0;
  int *flag = nullptr;
  double *stage_ext = nullptr;         // K x N staging for set/get state
  int nTerms = 0;
  int timeFn[4] = {0, 0, 0, 0};
  bool hasVelocity = false;
  // host copies needed later
  std::vector<double> detJ, areaE0T, Bhost;   // internal order
  std::vector<uint8_t> markNotN;              // internal order, 3 per element
  std::vector<double> nuE0T, corner0;         // internal order: 3 x 2 normals, first corner
  std::vector<int> permv;                     // internal -> external element id
  std::vector<double> visCoordV;              // caller's vertices, numV x 2 row-major (output files)
  std::vector<int32_t> visV0T;                // caller's V0T, numT x 3 row-major
  dgadv::OutputQueue *outq = nullptr;         // solution output (dgadv_output), made on first use
  dgadv::ImplicitState *impl = nullptr;       // implicit solver (dgadv_step_implicit), on first use
  dgadv::TransportState *trans = nullptr;     // transported species (dgadv_transport_init)
  int velOrder = 1;                           // order of the velocity projections (2p or 2p+1)
  int velVersion = 0;                         // bumped whenever the velocity factors change
  dgadv::RefTables tables;
  // CUDA graphs of a chunk of steps, one per phase (limPass mod 3) at the chunk start
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  bool profiling = false;
  std::vector<cudaEvent_t> profEvents;
  std::vector<int> profKinds;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double graphTau[3] = {-1.0, -1.0, -1.0};
  // discrete adjoint (dgadv_forward_record / dgadv_backward)
  int nModes = 0;
  double *modeF = nullptr, *modeV = nullptr;   // nModes x 2Q x Kp, nModes x 3R x Kp (FP64)
  void *adjSlots = nullptr;                    // state snapshots, nSlots x N x Kp
  void *adjStages = nullptr;                   // stage states c^(1..S-1) of every step (or null)
  int adjStageSteps = 0;
  int nSlots = 0;
  std::vector<int> slotStep;                   // step index held by each slot (-1: none)
  void *lam = nullptr, *mu1 = nullptr, *mu2 = nullptr, *accn = nullptr, *cx = nullptr;
  void *adjBuf[2] = {nullptr, nullptr};        // lam / accn swap between these every step
  cudaGraphExec_t adjExec = nullptr;           // reverse sweep of the recorded schedule
  int adjExecSteps = 0, adjExecSlots = 0;      // ... and the run it was captured for
  double adjExecTau = 0.0;
  double *aF = nullptr, *aV = nullptr;         // velocity sensitivities, 2Q x Kp and 3R x Kp
  double *thetaPart = nullptr;                 // per-block partial sums of the mode gradient
  // adjoint of the linear limiter: the limiter inputs of every stage, recorded by the forward
  // run (recY: the unlimited stage value; recCdot: cDot before time-derivative limiting)
  void *recY[3] = {nullptr, nullptr, nullptr}, *recCdot[3] = {nullptr, nullptr, nullptr};
  void *adjRecY = nullptr, *adjRecCdot = nullptr;   // per step and stage (stage storage mode)
  void *adjScrY = nullptr, *adjScrCdot = nullptr;   // per stage (recomputing modes)
  // the reverse sweep's recomputation stream, its second buffer set (state, two stage states,
  // S + S limiter records) and the events between the streams
  cudaStream_t adjStreamF = nullptr;
  void *adjSet1 = nullptr;
  size_t adjSet1States = 0;
  cudaEvent_t adjFEv = nullptr;
  std::vector<cudaEvent_t> adjRevEv, adjTapeEv;   // per reversed step: its reverse stages, its recomputation
  // the advances of a three-stream sweep: their stream, their buffer set (two work states, two
  // stage states, S + S limiter records), their own limiter key sets and pass count, and per
  // buffer (physical slot, then the two work states) the event of its last write
  cudaStream_t adjStreamA = nullptr;
  void *adjSetA = nullptr;
  size_t adjSetAStates = 0;
  void *vkeysAdv = nullptr;
  unsigned long long *gmmAdv = nullptr;
  long long limPassAdv = 0;
  std::vector<cudaEvent_t> adjBufEv;
  void *tmpY = nullptr, *tmpD = nullptr;            // dJ/dy and dJ/dcDot of a reversed stage
  // extreme terms of the limiter adjoint, one record set per limiter kind, stored by position in
  // the vertex-patch CSR (vidx): the element at position i of patch v writes there the element
  // holding its extreme at v (or -1) and the term's weight
  int *recSlotT[2] = {nullptr, nullptr};
  void *recSlotW[2] = {nullptr, nullptr};
  int *csrPos = nullptr;                            // 3 x Kp: position of element k in patch V0T[n][k]
  // The adjoint's own vertex keys, global-extreme slots and element means of the limiter inputs,
  // one set per pass modulo adjKeySets = 4S + 1: with several streams the scatters of a
  // reversed step may run on the recomputation stream while the reverse stages of the step
  // before it run
  void *adjMeans = nullptr;                         // adjKeySets x nc x Kp
  void *adjChoice = nullptr;                        // adjKeySets x Kp x (3 reals + 2 ints)
  void *vkeysA = nullptr;                           // adjKeySets x nc x 2 x Vp
  unsigned long long *gmmA = nullptr;               // adjKeySets x nInst x kSlotCopies x 2 x nc
  int adjKeySets = 3;
  long long adjPass = 0, adjPassF = 0;              // passes consumed / scattered so far
  std::vector<int> schedule;                   // checkpointing actions of the recorded run
  size_t schedBackward = 0;                    // first action of the reverse sweep
  int recSteps = 0;
  double recTau = 0.0;
  bool recorded = false;
  bool poisoned = false;               // a stage kernel's bounded wait gave up: no further steps
  std::string err;
};

namespace dgadv {

// One reversed stage of the adjoint sweep (device pointers of the handle's real type).
struct AdjStageArgs {
  const void *muIn;    // dJ/dc^(s+1) (with the limiter: dJ/d of the unlimited stage value)
  const void *mpIn;    // dJ/dcDot if precomputed (time-derivative limiter adjoint), else null
  const void *cs;      // c^(s), the stage input of the forward step
  void *muOut;         // dJ/dc^(s) (may be null when s = 0)
  void *accn;          // dJ/dc^n, accumulated over the stages of the step
  double omega, tau;
  int init, last;
};

// One limiter adjoint pass: lamOut = (d limiter / d x)^T (scale * lamIn).
struct LimVjpArgs {
  int kind;            // 0 solution limiter, 1 time-derivative limiter
  const void *x;       // the limiter's recorded input
  const void *lamIn;
  void *lamOut;
  double scale;
  long long pass;      // adjoint key set (pass mod 3) holding x's patch extremes
  double gco[4];       // time factors of the Dirichlet data (solution limiter)
  const void *nextX;   // solution limiter: the time-derivative limiter's input, whose means this
                       // pass scatters to the key set of pass + 1 (null: none)
  int gatherIn;        // time-derivative limiter: first add the solution limiter's extreme
                       // terms into lamIn (written back), in place of their own gather launch
  int gatherOut;       // launch the gather of this pass's extreme terms into lamOut
  int apply;           // linear limiter: the choices of this pass were made by lim_choice (its
                       // record set, pass mod adjKeySets); only lambda is applied here
};

// One stage of one transported species (dgadv_transport.cu): c h out from c h in, the
// step's c h, the species' concentration and mask.
struct TrStageArgs {
  const void *conc, *cHin, *cH0;
  void *cHout;
  const uint8_t *mask;
  double omega, tau;
};

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
  cudaError_t (*scatter_in)(dgadv_handle *h, void *dst);        // stage_ext (caller order, FP64) -> dst
  cudaError_t (*gather_out)(dgadv_handle *h, const void *src);  // src -> stage_ext
  cudaError_t (*adj_stage)(dgadv_handle *h, const AdjStageArgs &a);   // null: no adjoint kernels
  cudaError_t (*step_persist)(dgadv_handle *h, double t0, double tau); // null: not built
  // one step of hs[0] and the handles linked to it, one launch per stage kernel (null: not built)
  cudaError_t (*step_linked)(dgadv_handle **hs, int n, double t0, double tau);
  cudaError_t (*persist_attributes)(int p);
  cudaError_t (*lim_vjp)(dgadv_handle *h, const LimVjpArgs &a);
  // the limiter input's quantities to the adjoint's key set of `pass` and stored per element
  // (kind 0: solution limiter, 1: time-derivative limiter)
  cudaError_t (*vjp_scatter)(dgadv_handle *h, const void *x, long long pass, int kind);
  // linear limiter: the choices of pass a.pass for input a.x (kind, Dirichlet factors a.gco),
  // recorded for a later lim_vjp with a.apply
  cudaError_t (*lim_choice)(dgadv_handle *h, const LimVjpArgs &a);
  // device copy of a state-sized buffer (bytes a multiple of 16) ordered with dependent launches
  cudaError_t (*copy)(dgadv_handle *h, void *dst, const void *src, size_t bytes);
  // n FP64 values on the device -> stored reals
  cudaError_t (*from_f64)(dgadv_handle *h, void *dst, const double *src, size_t n);
  // the element operator of every element from the velocity factors (null: not built)
  cudaError_t (*build_element_operator)(dgadv_handle *h);
  // transport problem (null: not built for this type)
  cudaError_t (*tr_stage)(dgadv_handle *h, const TrStageArgs &a);
  cudaError_t (*tr_convert)(dgadv_handle *h, const void *in, void *out, const void *hQ, int toConc);
  cudaError_t (*tr_mask)(dgadv_handle *h, long long pass, double tol, uint8_t *mask);
};

// Fused path (linear limiter, zero Dirichlet data, opted in): per stage the operator kernel
// limits its input on the fly.
inline bool use_fused(const dgadv_handle *h) {
  return h->lim && h->limType == DGADV_LIM_LINEAR && !h->cDV0T && (h->flags & DGADV_FLAG_FUSE);
}
// Persistent step (opted in): one cooperative launch per time step, linear limiter or none,
// no source terms.
inline bool use_persistent(const dgadv_handle *h) {
  return (h->flags & DGADV_FLAG_PERSIST) && !(h->flags & DGADV_FLAG_FUSE) && h->p >= 1 &&
         (!h->lim || h->limType == DGADV_LIM_LINEAR) && h->nTerms == 0;
}

const PrecOps &ops_of(const dgadv_handle *h);

// Status return of a failed CUDA call inside a C-ABI function holding `h`.
#define DG_CUDA(call)                                                               \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                  \
      return DGADV_ECUDA;                                                           \
    }                                                                               \
  } while (0)

// Shared host helpers of the C-ABI units (dgadv_solver.cu).
int dev_alloc(dgadv_handle *h, void **p, size_t bytes);
int upload(dgadv_handle *h, void *dst, const void *src, size_t bytes);
int upload_real(dgadv_handle *h, void *dst, const std::vector<double> &src);
// Volume factors F (2Q x Kp) and edge factors Vn (3R x Kp) of one velocity, internal order.
void velocity_factors(const dgadv_handle *h, const double *u1, const double *u2, const double *vN,
                      std::vector<double> &F, std::vector<double> &Vn);

const PrecOps &ops_fp64();
const PrecOps &ops_fp32();
const PrecOps &ops_df32_p01();   // df32 kernels compile per degree (three units in parallel)
const PrecOps &ops_df32_p2();
const PrecOps &ops_df32_p3();

}  // namespace dgadv
