// C-ABI of the discrete adjoint (include/dgadv.h): velocity modes, the recorded forward run with
// binomial checkpointing, and the reverse sweep.
//
// Checkpointing.  Reversing T steps needs the state c^i at the start of every step i, in
// reverse order.  With S snapshot slots (slot 0 holds c^0), the schedule is the binomial one
// of Griewank (1992, "Achieving logarithmic growth of temporal and spatial complexity in reverse
// automatic differentiation"): with s free slots and t steps, let r be the smallest integer with
// beta(s, r) = C(s + r, s) >= t; advance to a split point m = a + max(1, t - beta(s - 1, r)),
// store c^m, reverse [m, b) with s - 1 free slots, then [a, m) with s.  No step is recomputed
// more than r times.  With as many slots as steps every state is stored once; unless the
// record also kept every stage state, each reversed step then recomputes, from c^i, the stages
// its reverse stages read (the first S - 1 stages; with the limiter the whole step, whose
// limiter inputs the limiter adjoint reads).  Checkpoints are read and written in place: no
// state is copied into or out of a slot.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dgadv_handle.h"

using namespace dgadv;

namespace {

enum { A_RESTORE = 0, A_ADVANCE = 1, A_STORE = 2, A_BACKWARD = 3 };

double beta(int s, int r) {   // C(s + r, s), as a double (only compared with step counts)
  double b = 1.0;
  for (int i = 1; i <= s; ++i) b = b * (r + i) / i;
  return b;
}

void push(std::vector<int> &o, int op, int arg) { o.push_back(op); o.push_back(arg); }

// Reverse steps [a, b) given c^a in slot sa; slots top, top+1, ... are free (freeS of them).
void reverse_steps(std::vector<int> &o, int a, int b, int sa, int top, int freeS) {
  const int t = b - a;
  if (t == 1) { push(o, A_RESTORE, sa); push(o, A_BACKWARD, a); return; }
  if (freeS == 0) {
    for (int i = b - 1; i >= a; --i) {
      push(o, A_RESTORE, sa);
      if (i > a) push(o, A_ADVANCE, i - a);
      push(o, A_BACKWARD, i);
    }
    return;
  }
  int r = 1;
  while (beta(freeS, r) < t) ++r;
  const int m = a + (int)std::max(1.0, t - beta(freeS - 1, r));
  push(o, A_RESTORE, sa);
  push(o, A_ADVANCE, m - a);
  push(o, A_STORE, top);
  reverse_steps(o, m, b, top, top + 1, freeS - 1);
  reverse_steps(o, a, m, sa, top, freeS);
}

void make_schedule(int nSteps, int nSlots, std::vector<int> &o) {
  o.clear();
  reverse_steps(o, 0, nSteps, 0, 1, nSlots - 1);
}

// First action of the reverse sweep: the last restore before the first backward step (the
// forward phase runs the actions before it, then carries the state on to the final step).
size_t backward_start(const std::vector<int> &o) {
  size_t f = 0;
  while (f < o.size() && o[f] != A_BACKWARD) f += 2;
  while (f >= 2 && o[f] != A_RESTORE) f -= 2;
  return f;
}

// One entry of aF / aV: FP64, or (pairs) the float pair hi + lo of the FP32 stage kernel.
__device__ __forceinline__ double sens_entry(const double *a, size_t i, int pairs) {
  if (!pairs) return a[i];
  const float2 q = reinterpret_cast<const float2 *>(a)[i];
  return (double)q.x + (double)q.y;
}

// dJ/dtheta_m partial sums in FP64: block b of mode m sums aF F_m + aV Vn_m over its elements.
__global__ void k_theta_partial(int K, int Kp, int nF, int nV, int pairs, const double *__restrict__ aF,
                                const double *__restrict__ aV, const double *__restrict__ modeF,
                                const double *__restrict__ modeV, double *__restrict__ part) {
  __shared__ double red[256];
  const int m = blockIdx.y;
  double s = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x) {
    for (int c = 0; c < nF; ++c)
      s += sens_entry(aF, (size_t)c * Kp + k, pairs) * modeF[((size_t)m * nF + c) * Kp + k];
    for (int c = 0; c < nV; ++c)
      s += sens_entry(aV, (size_t)c * Kp + k, pairs) * modeV[((size_t)m * nV + c) * Kp + k];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(size_t)m * gridDim.x + blockIdx.x] = red[0];
}

constexpr int kThetaBlocks = 304;   // 2 x 152 SMs

// Position of each element in the CSR vertex patches of its three vertices (pos[n][k]: index i
// with vidx[i] == k in patch V0T[n][k]).
__global__ void k_csr_pos(int K, int Kp, const int *__restrict__ V0T, const int *__restrict__ vptr,
                          const int *__restrict__ vidx, int *__restrict__ pos) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  for (int n = 0; n < 3; ++n) {
    const int v = V0T[(size_t)n * Kp + k];
    int at = -1;
    for (int i = vptr[v]; i < vptr[v + 1]; ++i)
      if (vidx[i] == k) at = i;
    pos[(size_t)n * Kp + k] = at;
  }
}

// The cached reverse-sweep graph no longer fits the recorded run.
void drop_sweep(dgadv_handle *h) {
  if (h->adjExec) cudaGraphExecDestroy(h->adjExec);
  h->adjExec = nullptr;
  h->adjExecSteps = h->adjExecSlots = 0;
  h->adjExecTau = 0.0;
}

void dev_release(dgadv_handle *h, void *&p) {
  if (!p) return;
  cudaFree(p);
  h->allocs.erase(std::remove(h->allocs.begin(), h->allocs.end(), p), h->allocs.end());
  p = nullptr;
}

// Buffers a forward step of the schedule writes besides its output: its stage states and its
// limiter records (and, for the sets of the recomputation with two streams, a work state).  Set
// 0 is the handle's own (cn, cA, cB, adjScrY, adjScrCdot).  With two or three streams the
// recomputation alternates between set 0 and set 1 (adjSet1), so that it writes one set while
// the reverse stages read the other.
struct WorkSet {
  void *cn = nullptr, *cA = nullptr, *cB = nullptr, *scrY = nullptr, *scrCdot = nullptr;
};

// Cursor of a schedule run: the step the run stands at, the logical slot holding that state
// (-1: none), and the step each work state holds (-1: none).
struct Cursor {
  int step = 0;
  int slot = -1;
  int cnStep[2] = {0, -1};
};

enum { kRev = 0, kFwd = 1, kAdv = 2 };

// The streams of a schedule run.
// - One stream: every action in order on the handle's stream.
// - Two: the forward steps (advances and recomputation) on adjStreamF, the reverse stages on the
//   handle's stream.
// - Three: the recomputation of the reversed steps on adjStreamF, the advances between
//   checkpoints on adjStreamA, with their own stage states, limiter records and limiter key
//   sets, so that they run while the reverse stages and the recomputation of other steps run.
// A reversed step waits for its recomputation.  A write into a set, a slot or a work state
// first waits for the last reads of it on other streams; a read of a slot or a work state that
// the advance stream wrote waits for that write.  The results are bitwise those of one stream:
// the same kernels read the same data.
//
// Buffers are numbered 0 .. nSlots - 1 (physical slots), then the two work states.  A store
// into a logical slot of the schedule may go to another physical slot: with several streams,
// to the free one whose readers finished first, instead of the one the schedule reuses, which
// the reversed step just issued is often still reading.  A slot is free when no checkpoint that
// is still to be read (a step not yet reversed) sits in it.
struct Lanes {
  int n = 1;
  bool two = false;                    // n >= 2
  cudaStream_t st[3] = {nullptr, nullptr, nullptr};   // kRev, kFwd, kAdv (shared when n < 3)
  bool brk[3] = {false, false, false};   // the stream's next launch follows a cross-stream wait
  WorkSet set[2];                      // the recomputation's sets
  WorkSet aset;                        // the advances' stage states and records (n == 3)
  void *work[2] = {nullptr, nullptr};  // the work states an advance writes when it stores nothing
  int cur = 0;                         // the set the next recomputation writes
  int setReader[2] = {-1, -1};         // reversed step that last read a set (-1: none)
  std::vector<int> phys;               // physical slot of each logical slot
  std::vector<int> revReader, tapeReader;   // per buffer: last reversed step / recomputation reading it
  std::vector<char> advWrote;          // per buffer: written by the advances since the recomputation waited
  int nRev = 0;                        // reversed steps issued
  int frontier = 0;                    // the next step to reverse: checkpoints of later steps are dead
};

int rk_stages(const dgadv_handle *h, double omega[3]) {
  omega[0] = omega[1] = omega[2] = 0.0;
  if (h->ordRK == 2) { omega[1] = 0.5; return 2; }
  if (h->ordRK == 3) { omega[1] = 0.75; omega[2] = 1.0 / 3.0; return 3; }
  return 1;
}

int canon(const Lanes &L, int s) { return L.n == 1 ? kRev : (L.n == 2 && s == kAdv ? kFwd : s); }

// Stream s waits for event e, recorded on stream `from`; nothing when they are one stream.
int wait_event(dgadv_handle *h, Lanes &L, int s, int from, cudaEvent_t e) {
  const int c = canon(L, s);
  if (c == canon(L, from)) return DGADV_OK;
  DG_CUDA(cudaStreamWaitEvent(L.st[c], e, 0));
  L.brk[c] = true;
  return DGADV_OK;
}

// Stream s becomes the launch stream; its first launch after a cross-stream wait goes without
// programmatic dependent launch.
void use_stream(dgadv_handle *h, Lanes &L, int s) {
  const int c = canon(L, s);
  h->stream = L.st[c];
  if (L.brk[c]) h->pdlBreak = true;
  L.brk[c] = false;
}

// One forward step from c^step, read from `src`, written to `dst`, through the stage states and
// limiter records of `ws`; advKeys: with the advance stream's limiter key sets.  With stage
// storage the step's stage states are written straight into its stage slots.  With nStages < S
// only the first nStages stages run: their outputs (cA, cB) are what the reverse stages of the
// unlimited scheme read.  recordsOnly runs every stage but the last solution limiter: the limiter
// inputs are what the limiter adjoint reads.  In both cases c^(step+1) is neither needed nor
// written, and the cursor stays.
int forward_step(dgadv_handle *h, Cursor &w, const WorkSet &ws, const void *src, void *dst, int nStages,
                 bool recordsOnly = false, bool advKeys = false) {
  const PrecOps &o = ops_of(h);
  double omega[3];
  const int S = rk_stages(h, omega);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  const bool partial = nStages < S;
  if (partial && nStages <= 0) return DGADV_OK;   // one stage: its input c^step is all it needs
  void *cA = h->cA, *cB = h->cB;
  h->cA = ws.cA;
  h->cB = ws.cB;
  if (h->adjStages && S > 1) {
    char *sp = (char *)h->adjStages + (size_t)w.step * (S - 1) * bytes;
    h->cA = sp;
    if (S > 2) h->cB = sp + bytes;
  }
  if (h->lim) {   // the limiter inputs of every stage: per step (stage storage) or scratch
    for (int s = 0; s < S; ++s) {
      h->recY[s] = h->adjRecY ? (char *)h->adjRecY + ((size_t)w.step * S + s) * bytes
                              : (char *)ws.scrY + (size_t)s * bytes;
      if (h->limdot)
        h->recCdot[s] = h->adjRecCdot ? (char *)h->adjRecCdot + ((size_t)w.step * S + s) * bytes
                                      : (char *)ws.scrCdot + (size_t)s * bytes;
    }
  }
  const bool swapKeys = advKeys && h->lim;
  if (swapKeys) {
    std::swap(h->vkeys, h->vkeysAdv);
    std::swap(h->gmm, h->gmmAdv);
    std::swap(h->limPass, h->limPassAdv);
  }
  h->stepSrc = src;
  h->stepDst = dst;
  h->stepStages = partial ? nStages : 0;
  h->stepRecordsOnly = recordsOnly;
  const cudaError_t e = o.step(h, w.step * h->recTau, h->recTau);
  if (swapKeys) {
    std::swap(h->vkeys, h->vkeysAdv);
    std::swap(h->gmm, h->gmmAdv);
    std::swap(h->limPass, h->limPassAdv);
  }
  h->cA = cA;
  h->cB = cB;
  h->stepSrc = nullptr;
  h->stepDst = nullptr;
  h->stepStages = 0;
  h->stepRecordsOnly = false;
  for (int s = 0; s < 3; ++s) h->recY[s] = h->recCdot[s] = nullptr;
  DG_CUDA(e);
  if (partial || recordsOnly) return DGADV_OK;
  ++w.step;
  return DGADV_OK;
}

// The physical slot a store into logical slot l writes (see Lanes); `avoid` (the store's source)
// only if nothing else is free.
int store_buffer(const dgadv_handle *h, Lanes &L, int l, int avoid) {
  if (!L.two) return L.phys[l];
  std::vector<char> held(h->nSlots, 0);
  held[0] = 1;   // c^0 stays where the end of the sweep reads it
  for (int k = 0; k < h->nSlots; ++k)
    if (k != l && h->slotStep[k] >= 0 && h->slotStep[k] <= L.frontier) held[L.phys[k]] = 1;
  int best = -1, bestR = 0;
  for (int p = 1; p < h->nSlots; ++p) {
    if (held[p] || p == avoid) continue;
    const int r = std::max(L.revReader[p], L.tapeReader[p]);
    if (best < 0 || r < bestR || (r == bestR && p == L.phys[l])) {
      best = p;
      bestR = r;
    }
  }
  if (best >= 0) L.phys[l] = best;
  return L.phys[l];
}

// The work state an advance that stores nothing writes: the other one than its source, else
// the one whose readers finished first (in place with one work state).
int work_buffer(const dgadv_handle *h, const Lanes &L, int src) {
  const int nS = h->nSlots;
  if (!L.work[1]) return nS;
  if (src >= nS) return nS + (1 - (src - nS));
  const int r0 = std::max(L.revReader[nS], L.tapeReader[nS]);
  const int r1 = std::max(L.revReader[nS + 1], L.tapeReader[nS + 1]);
  return r1 < r0 ? nS + 1 : nS;
}

// The advance stream is about to write buffer b: it waits for b's readers on the other streams.
int before_write(dgadv_handle *h, Lanes &L, int b) {
  int st;
  if (L.revReader[b] >= 0) {
    if ((st = wait_event(h, L, kAdv, kRev, h->adjRevEv[L.revReader[b]]))) return st;
    L.revReader[b] = -1;
  }
  if (L.tapeReader[b] >= 0) {
    if ((st = wait_event(h, L, kAdv, kFwd, h->adjTapeEv[L.tapeReader[b]]))) return st;
    L.tapeReader[b] = -1;
  }
  return DGADV_OK;
}

// ... and has written it.
int after_write(dgadv_handle *h, Lanes &L, int b) {
  if (L.n < 3) return DGADV_OK;
  DG_CUDA(cudaEventRecord(h->adjBufEv[b], L.st[kAdv]));
  L.advWrote[b] = 1;
  return DGADV_OK;
}

// Executes schedule actions [from, to).  Restores cost nothing: a step reads c^i from the slot
// that holds it, and an advance whose next action stores its result writes that result straight
// into the slot.  With stage storage (every step's stage states kept by the recorded run) a
// reversed step reads its stages from there and recomputes nothing; without it, the unlimited
// scheme recomputes only the stages whose inputs its reverse stages read, and the limited scheme
// every stage up to the last limiter inputs.
int run_actions(dgadv_handle *h, size_t from, size_t to, Cursor &w, Lanes &L) {
  const PrecOps &o = ops_of(h);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  const double tau = h->recTau;
  double omega[3];
  const int S = rk_stages(h, omega);
  const double cst[3] = {0.0, 1.0, 0.5};   // stage times (core/rungeKuttaExplicit.m:64-78)
  const int nS = h->nSlots;
  char *stages = (char *)h->adjStages;
  auto stage_ptr = [&](int step, int s) { return stages + ((size_t)step * (S - 1) + (s - 1)) * bytes; };
  auto buf_ptr = [&](int b) -> void * {
    return b < nS ? (void *)((char *)h->adjSlots + (size_t)b * bytes) : L.work[b - nS];
  };
  // the buffer holding c^(w.step): its slot, else a work state
  auto current = [&](int &b) -> int {
    if (w.slot >= 0 && h->slotStep[w.slot] == w.step) { b = L.phys[w.slot]; return DGADV_OK; }
    for (int k = 0; k < 2; ++k)
      if (L.work[k] && w.cnStep[k] == w.step) { b = nS + k; return DGADV_OK; }
    h->err = "checkpoint schedule lost its state";
    return DGADV_EINVAL;
  };
  int st;
  for (size_t a = from; a < to; a += 2) {
    const int op = h->schedule[a], arg = h->schedule[a + 1];
    if (op == A_RESTORE) {
      w.step = h->slotStep[arg];
      w.slot = arg;
    } else if (op == A_ADVANCE) {
      const bool storeNext = a + 2 < to && h->schedule[a + 2] == A_STORE;
      for (int i = 0; i < arg; ++i) {
        int src;
        if ((st = current(src))) return st;
        int target = storeNext && i == arg - 1 ? h->schedule[a + 3] : -1;
        int dst = target >= 0 ? store_buffer(h, L, target, src) : work_buffer(h, L, src);
        if (target >= 0 && dst == src) {   // no other slot free: through a work state, then copied
          target = -1;
          dst = work_buffer(h, L, src);
        }
        if ((st = before_write(h, L, dst))) return st;
        // the advances' stage states and records: their own set, or the set the next
        // recomputation writes
        if (L.n < 3 && L.setReader[L.cur] >= 0) {
          if ((st = wait_event(h, L, kAdv, kRev, h->adjRevEv[L.setReader[L.cur]]))) return st;
          L.setReader[L.cur] = -1;
        }
        use_stream(h, L, kAdv);
        if ((st = forward_step(h, w, L.n == 3 ? L.aset : L.set[L.cur], buf_ptr(src), buf_ptr(dst), S, false, L.n == 3)))
          return st;
        if ((st = after_write(h, L, dst))) return st;
        if (target >= 0) {   // the result already sits in the slot the next action stores to
          h->slotStep[target] = w.step;
          w.slot = target;
        } else {
          w.cnStep[dst - nS] = w.step;
          w.slot = -1;
        }
      }
    } else if (op == A_STORE) {
      if (!(w.slot == arg && h->slotStep[arg] == w.step)) {
        int src;
        if ((st = current(src))) return st;
        const int dst = store_buffer(h, L, arg, src);
        if (dst != src) {
          if ((st = before_write(h, L, dst))) return st;
          use_stream(h, L, kAdv);
          DG_CUDA(o.copy(h, buf_ptr(dst), buf_ptr(src), bytes));
          if ((st = after_write(h, L, dst))) return st;
        }
        h->slotStep[arg] = w.step;
        w.slot = arg;
      }
    } else {   // A_BACKWARD: the stage states of step arg (stored or recomputed), then reversed
      if (w.step != arg) { h->err = "checkpoint schedule out of order"; return DGADV_EINVAL; }
      const void *stageIn[3];
      int cb = -1;              // the buffer of c^arg, when recomputed
      const int used = L.cur;   // the set this step's recomputation writes
      const int ev = L.nRev;    // this reversed step's events
      if (stages) {
        if (w.slot < 0) { h->err = "checkpoint schedule lost its state"; return DGADV_EINVAL; }
        stageIn[0] = buf_ptr(L.phys[w.slot]);
        for (int s = 1; s < S; ++s) stageIn[s] = stage_ptr(arg, s);
      } else {
        if ((st = current(cb))) return st;
        if (L.n == 3 && L.advWrote[cb]) {
          if ((st = wait_event(h, L, kFwd, kAdv, h->adjBufEv[cb]))) return st;
          L.advWrote[cb] = 0;
        }
        if (L.setReader[used] >= 0) {
          if ((st = wait_event(h, L, kFwd, kRev, h->adjRevEv[L.setReader[used]]))) return st;
          L.setReader[used] = -1;
        }
        use_stream(h, L, kFwd);
        // unlimited: the stages the reverse stages read; limited: every stage's limiter inputs
        if ((st = forward_step(h, w, L.set[used], buf_ptr(cb), nullptr, h->lim ? S : S - 1, h->lim != 0))) return st;
        stageIn[0] = buf_ptr(cb);
        stageIn[1] = L.set[used].cA;
        stageIn[2] = L.set[used].cB;
      }
      const WorkSet &ws = L.set[used];
      // the limiter inputs of stage s: recorded per step, or this step's recomputation set
      auto recY = [&](int s) -> const char * {
        return h->adjRecY ? (const char *)h->adjRecY + ((size_t)arg * S + s) * bytes : (const char *)ws.scrY + (size_t)s * bytes;
      };
      auto recCd = [&](int s) -> const char * {
        if (!h->limdot) return nullptr;
        return h->adjRecCdot ? (const char *)h->adjRecCdot + ((size_t)arg * S + s) * bytes
                             : (const char *)ws.scrCdot + (size_t)s * bytes;
      };
      // With the limiter and every stage stored, or with the hierarchical or strict limiter on
      // three streams: the scatters of the limiter inputs' quantities to the adjoint's key sets
      // do not depend on the adjoint variable, so they run on the recomputation stream (after
      // the step's recomputation), in the reverse stages' pass order; their key sets were last
      // read two reversed steps ago.  (Measured with 20 snapshots on three streams: the
      // hierarchical and strict sweeps gain 8-10 %, the linear one, whose choices would move
      // too, loses 15-25 %; with two streams the advances keep that stream the busier one.)
      const bool pre = L.two && h->lim && (stages || (L.n == 3 && h->limType != DGADV_LIM_LINEAR));
      // the linear limiter's choices too (k_lim_choice), leaving the reverse stream k_lim_apply
      const bool preChoice = pre && h->limType == DGADV_LIM_LINEAR && h->adjChoice;
      // time factors of the Dirichlet data at the solution limiter of stage s
      auto gcoBC = [&](int s, double *gco) {
        const double tBC = (s + 1 < S) ? (arg + cst[s + 1]) * tau : (arg + 1) * tau;
        for (int m = 0; m < h->nTerms; ++m) gco[m] = h->timeFn[m] == DGADV_TIME_EXP_NEG ? std::exp(-tBC) : 1.0;
      };
      if (pre) {
        if (L.nRev >= 2 && (st = wait_event(h, L, kFwd, kRev, h->adjRevEv[L.nRev - 2]))) return st;
        use_stream(h, L, kFwd);
        for (int s = S - 1; s >= 0; --s) {
          const long long p0 = h->adjPassF;
          DG_CUDA(o.vjp_scatter(h, recY(s), h->adjPassF++, 0));
          if (h->limdot) DG_CUDA(o.vjp_scatter(h, recCd(s), h->adjPassF++, 1));
          if (preChoice) {
            LimVjpArgs c;
            std::memset(&c, 0, sizeof(c));
            c.kind = 0; c.x = recY(s); c.pass = p0;
            gcoBC(s, c.gco);
            DG_CUDA(o.lim_choice(h, c));
            if (h->limdot) {
              LimVjpArgs d;
              std::memset(&d, 0, sizeof(d));
              d.kind = 1; d.x = recCd(s); d.pass = p0 + 1;
              DG_CUDA(o.lim_choice(h, d));
            }
          }
        }
      }
      if (L.two && (pre || !stages)) {
        DG_CUDA(cudaEventRecord(h->adjTapeEv[ev], L.st[kFwd]));
        if ((st = wait_event(h, L, kRev, kFwd, h->adjTapeEv[ev]))) return st;
      }
      use_stream(h, L, kRev);
      void *mub[3] = {nullptr, h->mu1, h->mu2};
      for (int s = S - 1; s >= 0; --s) {
        const void *muNext = (s == S - 1) ? h->lam : mub[s + 1];
        const void *muY = muNext, *mp = nullptr;
        if (h->lim) {
          // solution limiter, then (p >= 2) the time-derivative limiter, transposed
          const char *Y = recY(s);
          LimVjpArgs v;
          std::memset(&v, 0, sizeof(v));
          gcoBC(s, v.gco);
          const char *Cd = recCd(s);
          if (h->limType != DGADV_LIM_LINEAR) {
            // hierarchical and strict limiter (inputs recorded in Taylor form): per limiter its
            // scatter (unless the recomputation stream made it), its pass and its gather
            if (!pre) DG_CUDA(o.vjp_scatter(h, Y, h->adjPass, 0));
            v.kind = 0; v.x = Y; v.lamIn = muNext; v.lamOut = h->tmpY; v.scale = 1.0; v.pass = h->adjPass++;
            v.gatherOut = h->limdot ? 0 : 1;   // else gathered by the time-derivative limiter's pass
            DG_CUDA(o.lim_vjp(h, v));
            muY = h->tmpY;
            if (h->limdot) {
              if (!pre) DG_CUDA(o.vjp_scatter(h, Cd, h->adjPass, 1));
              LimVjpArgs d;
              std::memset(&d, 0, sizeof(d));
              d.kind = 1; d.x = Cd; d.lamIn = h->tmpY; d.lamOut = h->tmpD; d.scale = (1.0 - omega[s]) * tau;
              d.pass = h->adjPass++;
              d.gatherIn = 1;
              d.gatherOut = 1;
              DG_CUDA(o.lim_vjp(h, d));
              mp = h->tmpD;
            }
          } else {
            // p >= 2: the solution limiter's kernel also scatters the time-derivative limiter's
            // means (unless the recomputation stream made both scatters), and the time-derivative
            // limiter's kernel gathers the solution limiter's extreme terms first (5 launches per
            // stage instead of 7; 4 with the scatters on the recomputation stream)
            if (!pre) DG_CUDA(o.vjp_scatter(h, Y, h->adjPass, 0));
            v.kind = 0; v.x = Y; v.lamIn = muNext; v.lamOut = h->tmpY; v.scale = 1.0; v.pass = h->adjPass++;
            v.nextX = pre ? nullptr : Cd;
            v.gatherOut = Cd ? 0 : 1;
            v.apply = preChoice ? 1 : 0;
            DG_CUDA(o.lim_vjp(h, v));
            muY = h->tmpY;
            if (h->limdot) {
              LimVjpArgs d;
              std::memset(&d, 0, sizeof(d));
              d.kind = 1; d.x = Cd; d.lamIn = h->tmpY; d.lamOut = h->tmpD; d.scale = (1.0 - omega[s]) * tau;
              d.pass = h->adjPass++;
              d.gatherIn = 1;
              d.gatherOut = 1;
              d.apply = preChoice ? 1 : 0;
              DG_CUDA(o.lim_vjp(h, d));
              mp = h->tmpD;
            }
          }
        }
        AdjStageArgs x;
        x.muIn = muY;
        x.mpIn = mp;
        x.cs = stageIn[s];
        x.muOut = s > 0 ? mub[s] : nullptr;
        x.accn = h->accn;
        x.omega = omega[s];
        x.tau = tau;
        x.init = s == S - 1;
        x.last = s == 0;
        DG_CUDA(o.adj_stage(h, x));
      }
      if (L.two) {
        DG_CUDA(cudaEventRecord(h->adjRevEv[ev], L.st[kRev]));
        L.nRev = ev + 1;
        if (!stages) {   // what this step read: its set, and the buffer of c^arg
          L.setReader[used] = ev;
          L.revReader[cb] = ev;
          if (L.n == 3) L.tapeReader[cb] = ev;
          L.cur = 1 - used;
        }
      }
      L.frontier = arg - 1;
      std::swap(h->lam, h->accn);
      w.step = arg + 1;
      w.slot = -1;
    }
  }
  h->stream = L.st[kRev];
  return DGADV_OK;
}

// The lanes of a run: the handle's buffers as set 0 and its state as the one work state; for a
// reverse sweep, with the streams enabled: set 1, the second work state and the recomputation
// stream (forked from the handle's stream), and when it recomputes with three streams, the
// advances' stream, set and work states.
int make_lanes(dgadv_handle *h, Lanes &L, bool sweep) {
  L.st[kRev] = L.st[kFwd] = L.st[kAdv] = h->stream;
  L.set[0].cn = h->cn;
  L.set[0].cA = h->cA;
  L.set[0].cB = h->cB;
  L.set[0].scrY = h->adjScrY;
  L.set[0].scrCdot = h->adjScrCdot;
  L.work[0] = h->cn;
  L.phys.resize(h->nSlots);
  for (int k = 0; k < h->nSlots; ++k) L.phys[k] = k;
  L.revReader.assign(h->nSlots + 2, -1);
  L.tapeReader.assign(h->nSlots + 2, -1);
  L.advWrote.assign(h->nSlots + 2, 0);
  L.frontier = h->recSteps - 1;
  // (the resources come from the recorded run: a run recorded with one stream sweeps with one).
  // A sweep that recomputes alternates two buffer sets; one with every stage stored uses the
  // second stream for the limiter adjoint's scatters only
  const bool recomputes = !h->adjStages && !h->adjRecY;
  const bool two = sweep && h->adjStreams >= 2 && h->adjStreamF && (int)h->adjRevEv.size() >= h->recSteps &&
                   (int)h->adjTapeEv.size() >= h->recSteps && (recomputes ? h->adjSet1 != nullptr : h->lim != 0);
  if (!two) return DGADV_OK;
  L.n = 2;
  L.two = true;
  const PrecOps &o = ops_of(h);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  double omega[3];
  const int S = rk_stages(h, omega);
  if (recomputes) {
    char *b = (char *)h->adjSet1;
    L.set[1].cn = b;
    L.set[1].cA = b + bytes;
    L.set[1].cB = b + 2 * bytes;
    if (h->lim) {
      L.set[1].scrY = b + 3 * bytes;
      L.set[1].scrCdot = b + (3 + (size_t)S) * bytes;
    }
    L.work[1] = L.set[1].cn;
  }
  L.st[kFwd] = L.st[kAdv] = h->adjStreamF;
  if (recomputes && h->adjStreams == 3 && h->adjStreamA && h->adjSetA && (int)h->adjBufEv.size() >= h->nSlots + 2) {
    L.n = 3;
    L.st[kAdv] = h->adjStreamA;
    char *b = (char *)h->adjSetA;
    L.work[0] = b;
    L.work[1] = b + bytes;
    L.aset.cA = b + 2 * bytes;
    L.aset.cB = b + 3 * bytes;
    if (h->lim) {
      L.aset.scrY = b + 4 * bytes;
      L.aset.scrCdot = b + (4 + (size_t)S) * bytes;
    }
  }
  DG_CUDA(cudaEventRecord(h->adjFEv, L.st[kRev]));
  DG_CUDA(cudaStreamWaitEvent(L.st[kFwd], h->adjFEv, 0));
  if (L.n == 3) DG_CUDA(cudaStreamWaitEvent(L.st[kAdv], h->adjFEv, 0));
  L.brk[kFwd] = L.brk[kAdv] = true;
  return DGADV_OK;
}

// Joins the other streams back into the handle's stream.
int join_lanes(dgadv_handle *h, Lanes &L) {
  h->stream = L.st[kRev];
  if (!L.two) return DGADV_OK;
  for (int s = kFwd; s < L.n; ++s) {
    DG_CUDA(cudaEventRecord(h->adjFEv, L.st[s]));
    DG_CUDA(cudaStreamWaitEvent(L.st[kRev], h->adjFEv, 0));
  }
  h->pdlBreak = true;
  return DGADV_OK;
}

int make_events(dgadv_handle *h, std::vector<cudaEvent_t> &v, size_t n) {
  while (v.size() < n) {
    cudaEvent_t e;
    DG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    v.push_back(e);
  }
  return DGADV_OK;
}

// Stream resources of a recorded run: the recomputation stream, the events and, if it
// recomputes, set 1; with three streams also the advances' stream, set, key sets and events.
int lanes_alloc(dgadv_handle *h, int nSteps, int nSlots, bool recomputes) {
  const PrecOps &o = ops_of(h);
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  double omega[3];
  const int S = rk_stages(h, omega);
  const size_t records = h->lim ? 2 * (size_t)S : 0;
  int st;
  if (recomputes && h->adjSet1States != 3 + records) {
    drop_sweep(h);
    dev_release(h, h->adjSet1);
    h->adjSet1States = 0;
    if ((st = dev_alloc(h, &h->adjSet1, (3 + records) * bytes))) return st;
    h->adjSet1States = 3 + records;
  }
  if (!h->adjStreamF) DG_CUDA(cudaStreamCreateWithFlags(&h->adjStreamF, cudaStreamNonBlocking));
  if (!h->adjFEv) DG_CUDA(cudaEventCreateWithFlags(&h->adjFEv, cudaEventDisableTiming));
  if ((st = make_events(h, h->adjRevEv, nSteps))) return st;
  if ((st = make_events(h, h->adjTapeEv, nSteps))) return st;
  if (!recomputes || h->adjStreams < 3) return DGADV_OK;
  if (h->adjSetAStates != 4 + records) {
    drop_sweep(h);
    dev_release(h, h->adjSetA);
    h->adjSetAStates = 0;
    if ((st = dev_alloc(h, &h->adjSetA, (4 + records) * bytes))) return st;
    h->adjSetAStates = 4 + records;
  }
  if (h->lim && !h->vkeysAdv) {
    // the advances' limiter passes: three key and slot sets, all reset (each pass resets the
    // next set, as in the handle's own)
    const size_t kb = o.keyBytes, vk = 3 * 2 * (size_t)h->nc * h->Vp * kb;
    const size_t ns = 3 * (size_t)h->nInst * kSlotCopies * 2 * (size_t)h->nc;
    if ((st = dev_alloc(h, &h->vkeysAdv, vk))) return st;
    if ((st = dev_alloc(h, (void **)&h->gmmAdv, ns * 8))) return st;
    std::vector<unsigned char> keys(vk, 0);
    for (size_t q = 0; q < 3 * (size_t)h->nc; ++q) std::memset(keys.data() + q * 2 * h->Vp * kb, 0xFF, (size_t)h->Vp * kb);
    DG_CUDA(cudaMemcpy(h->vkeysAdv, keys.data(), vk, cudaMemcpyHostToDevice));
    std::vector<unsigned long long> init(ns);
    for (size_t i = 0; i < ns; ++i) init[i] = (i & 1) ? 0ULL : o.slotKeyMax;
    DG_CUDA(cudaMemcpy(h->gmmAdv, init.data(), ns * 8, cudaMemcpyHostToDevice));
    h->limPassAdv = 0;
  }
  if (!h->adjStreamA) DG_CUDA(cudaStreamCreateWithFlags(&h->adjStreamA, cudaStreamNonBlocking));
  return make_events(h, h->adjBufEv, (size_t)nSlots + 2);
}

// The reverse sweep: the schedule's actions from the first reversed step on, c^nSteps in cn.
int reverse_sweep(dgadv_handle *h) {
  Cursor w;
  w.step = h->recSteps;
  Lanes L;
  int st = make_lanes(h, L, true);
  w.cnStep[0] = L.n == 3 ? -1 : h->recSteps;
  if (st == DGADV_OK) st = run_actions(h, h->schedBackward, h->schedule.size(), w, L);
  const int sj = join_lanes(h, L);
  return st ? st : sj;
}

}  // namespace

extern "C" int dgadv_set_velocity_modes(dgadv_handle *h, int32_t nModes, const double *u1Modes,
                                        const double *u2Modes, const double *vNModes) {
  return guarded(h, [&]() -> int {
  if (!h || nModes < 0 || nModes > 1024) return DGADV_EINVAL;
  if (nModes > 0 && (!u1Modes || !u2Modes || !vNModes)) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  void *pF = h->modeF, *pV = h->modeV;
  dev_release(h, pF);
  dev_release(h, pV);
  h->modeF = h->modeV = nullptr;
  h->nModes = 0;
  if (nModes == 0) return DGADV_OK;
  const size_t nF = 2 * (size_t)h->Q * h->Kp, nV = 3 * (size_t)h->R * h->Kp;
  const size_t sU = (size_t)h->K * h->N, sV = (size_t)h->K * 3 * h->R;
  std::vector<double> allF(nF * nModes), allV(nV * nModes), F, Vn;
  for (int m = 0; m < nModes; ++m) {
    velocity_factors(h, u1Modes + m * sU, u2Modes + m * sU, vNModes + m * sV, F, Vn);
    std::copy(F.begin(), F.end(), allF.begin() + m * nF);
    std::copy(Vn.begin(), Vn.end(), allV.begin() + m * nV);
  }
  int st;
  if ((st = dev_alloc(h, (void **)&h->modeF, allF.size() * 8))) return st;
  if ((st = dev_alloc(h, (void **)&h->modeV, allV.size() * 8))) return st;
  if ((st = upload(h, h->modeF, allF.data(), allF.size() * 8))) return st;
  if ((st = upload(h, h->modeV, allV.data(), allV.size() * 8))) return st;
  h->nModes = nModes;
  return DGADV_OK;
  });
}

extern "C" int dgadv_set_velocity_theta(dgadv_handle *h, const double *theta) {
  return guarded(h, [&]() -> int {
  if (!h || !theta) return DGADV_EINVAL;
  if (h->nModes == 0) { h->err = "no velocity modes set"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  const size_t nF = 2 * (size_t)h->Q * h->Kp, nV = 3 * (size_t)h->R * h->Kp;
  std::vector<double> allF(nF * h->nModes), allV(nV * h->nModes);
  DG_CUDA(cudaMemcpy(allF.data(), h->modeF, allF.size() * 8, cudaMemcpyDeviceToHost));
  DG_CUDA(cudaMemcpy(allV.data(), h->modeV, allV.size() * 8, cudaMemcpyDeviceToHost));
  std::vector<double> F(nF, 0.0), Vn(nV, 0.0);
  for (int m = 0; m < h->nModes; ++m) {
    for (size_t i = 0; i < nF; ++i) F[i] += theta[m] * allF[m * nF + i];
    for (size_t i = 0; i < nV; ++i) Vn[i] += theta[m] * allV[m * nV + i];
  }
  int st;
  if ((st = upload_real(h, h->F, F))) return st;
  if ((st = upload_real(h, h->Vn, Vn))) return st;
  h->hasVelocity = true;
  ++h->velVersion;
  h->recorded = false;
  return refresh_element_operator(h);
  });
}

extern "C" int dgadv_forward_record(dgadv_handle *h, int32_t nSteps, double tau, int32_t nSnapshots) {
  return guarded(h, [&]() -> int {
  if (!h || nSteps < 1 || !(tau > 0.0)) return DGADV_EINVAL;
  if (h->poisoned) { h->err = "a bounded wait of a stage kernel timed out earlier: create a new handle"; return DGADV_ETIMEOUT; }
  const PrecOps &o = ops_of(h);
  if (!o.adj_stage) { h->err = "no adjoint kernels for this precision"; return DGADV_EUNSUPPORTED; }
  if (h->flags & DGADV_FLAG_IMPLICIT) { h->err = "the adjoint covers the explicit scheme"; return DGADV_EUNSUPPORTED; }
  DG_CUDA(cudaSetDevice(h->device));
  const int nSlots = (nSnapshots <= 0 || nSnapshots >= nSteps) ? nSteps : nSnapshots;
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  double omega[3];
  const int S = rk_stages(h, omega);
  const int stageSteps = (nSnapshots <= 0 && S > 1) ? nSteps : 0;   // keep every stage state
  int st;
  if (stageSteps != h->adjStageSteps) {
    drop_sweep(h);
    dev_release(h, h->adjStages);
    h->adjStageSteps = 0;
    if (stageSteps) {
      if ((st = dev_alloc(h, &h->adjStages, (size_t)stageSteps * (S - 1) * bytes))) return st;
      h->adjStageSteps = stageSteps;
    }
  }
  if (nSlots != h->nSlots || nSteps != h->adjExecSteps || tau != h->adjExecTau) drop_sweep(h);
  if (nSlots != h->nSlots) {
    dev_release(h, h->adjSlots);
    if ((st = dev_alloc(h, &h->adjSlots, (size_t)nSlots * bytes))) return st;
    h->nSlots = nSlots;
  }
  if (!h->lam) {
    if ((st = dev_alloc(h, &h->lam, bytes))) return st;
    if ((st = dev_alloc(h, &h->mu1, bytes))) return st;
    if ((st = dev_alloc(h, &h->mu2, bytes))) return st;
    if ((st = dev_alloc(h, &h->accn, bytes))) return st;
    h->adjBuf[0] = h->lam;
    h->adjBuf[1] = h->accn;
    if ((st = dev_alloc(h, &h->cx, bytes))) return st;
    if ((st = dev_alloc(h, (void **)&h->aF, 2 * (size_t)h->Q * h->Kp * 8))) return st;
    if ((st = dev_alloc(h, (void **)&h->aV, 3 * (size_t)h->R * h->Kp * 8))) return st;
    if ((st = dev_alloc(h, (void **)&h->thetaPart, (size_t)kThetaBlocks * 1024 * 8))) return st;
    DG_CUDA(cudaMemset(h->mu1, 0, bytes));
    DG_CUDA(cudaMemset(h->mu2, 0, bytes));
  }
  if (h->lim) {
    // limiter adjoint: recorded limiter inputs, its own vertex keys, per-element records
    const size_t kb = o.keyBytes;
    const bool perStep = stageSteps > 0;
    if (!h->tmpY) {
      // per pass nc quantities (1 linear, p(p+1)/2 hierarchical); records: per CSR position one
      // (linear) or one per order (hierarchical)
      const size_t nq = (size_t)h->nc, perPos = h->limType == DGADV_LIM_LINEAR ? 1 : (size_t)h->p;
      if ((st = dev_alloc(h, &h->tmpY, bytes))) return st;
      if ((st = dev_alloc(h, &h->tmpD, bytes))) return st;
      for (int r = 0; r < 2; ++r) {
        if ((st = dev_alloc(h, (void **)&h->recSlotT[r], perPos * 3 * (size_t)h->K * 4))) return st;
        if ((st = dev_alloc(h, &h->recSlotW[r], perPos * 3 * (size_t)h->K * o.realBytes))) return st;
      }
      if ((st = dev_alloc(h, (void **)&h->csrPos, 3 * (size_t)h->Kp * 4))) return st;
      k_csr_pos<<<(h->K + 127) / 128, 128, 0, h->stream>>>(h->K, h->Kp, h->V0T, h->vptr, h->vidx, h->csrPos);
      DG_CUDA(cudaGetLastError());
      // 4S + 1 key sets: a pass's set is written at most two reversed steps (4S passes) ahead
      // of the pass that read it last
      const size_t ks = 4 * (size_t)S + 1;
      h->adjKeySets = (int)ks;
      if ((st = dev_alloc(h, &h->adjMeans, ks * nq * h->Kp * o.realBytes))) return st;
      if (h->limType == DGADV_LIM_LINEAR &&
          (st = dev_alloc(h, &h->adjChoice, ks * h->Kp * (3 * o.realBytes + 2 * sizeof(int)))))
        return st;
      if ((st = dev_alloc(h, &h->vkeysA, ks * 2 * nq * h->Vp * kb))) return st;
      if ((st = dev_alloc(h, (void **)&h->gmmA, ks * (size_t)h->nInst * kSlotCopies * 2 * nq * 8))) return st;
      if ((st = dev_alloc(h, &h->adjScrY, (size_t)S * bytes))) return st;
      if ((st = dev_alloc(h, &h->adjScrCdot, (size_t)S * bytes))) return st;
    }
    dev_release(h, h->adjRecY);
    dev_release(h, h->adjRecCdot);
    if (perStep) {
      if ((st = dev_alloc(h, &h->adjRecY, (size_t)nSteps * S * bytes))) return st;
      if (h->limdot && (st = dev_alloc(h, &h->adjRecCdot, (size_t)nSteps * S * bytes))) return st;
    }
    drop_sweep(h);
  }
  // the other streams of the reverse sweep: recomputation (and its buffer set), advances (with
  // three streams) and, with the limiter, the limiter adjoint's scatters
  if (h->adjStreams >= 2 && (h->lim || (stageSteps == 0 && S > 1)) && (st = lanes_alloc(h, nSteps, nSlots, stageSteps == 0)))
    return st;
  h->slotStep.assign(nSlots, -1);
  make_schedule(nSteps, nSlots, h->schedule);
  h->schedBackward = backward_start(h->schedule);
  h->recSteps = nSteps;
  h->recTau = tau;
  // c^0 is the current state
  DG_CUDA(o.copy(h, h->adjSlots, h->cn, bytes));
  h->slotStep[0] = 0;
  Cursor w;
  w.slot = 0;
  Lanes L;
  if ((st = make_lanes(h, L, false))) return st;
  if ((st = run_actions(h, 0, h->schedBackward, w, L))) { h->stream = L.st[kRev]; return st; }
  // on to c^nSteps in cn; the state reached may sit in a slot only
  if (w.cnStep[0] != w.step && (w.slot < 0 || h->slotStep[w.slot] != w.step)) {
    h->err = "checkpoint schedule lost its state";
    return DGADV_EINVAL;
  }
  while (w.step < nSteps) {
    const void *src = w.cnStep[0] == w.step ? h->cn : (const void *)((char *)h->adjSlots + (size_t)w.slot * bytes);
    if ((st = forward_step(h, w, L.set[0], src, h->cn, S))) return st;
    w.cnStep[0] = w.step;
    w.slot = -1;
  }
  if (w.cnStep[0] != w.step) DG_CUDA(o.copy(h, h->cn, (char *)h->adjSlots + (size_t)w.slot * bytes, bytes));
  h->recorded = true;
  return DGADV_OK;
  });
}

extern "C" int dgadv_backward(dgadv_handle *h, const double *dJdcT, double *dJdc0, double *dJdtheta) {
  return guarded(h, [&]() -> int {
  if (!h || !dJdcT) return DGADV_EINVAL;
  if (!h->recorded) { h->err = "no recorded forward run"; return DGADV_EINVAL; }
  if (h->poisoned) { h->err = "a bounded wait of a stage kernel timed out earlier: create a new handle"; return DGADV_ETIMEOUT; }
  const PrecOps &o = ops_of(h);
  DG_CUDA(cudaSetDevice(h->device));
  const size_t bytes = (size_t)h->N * h->Kp * o.realBytes;
  // every sweep starts from the same buffer order, so that a cached graph stays valid
  h->lam = h->adjBuf[0];
  h->accn = h->adjBuf[1];
  // memsets and copies first, then a plain kernel launch, so that the dependent-launch chain of
  // the sweep starts after work that is complete
  DG_CUDA(cudaMemsetAsync(h->lam, 0, bytes, h->stream));
  DG_CUDA(cudaMemsetAsync(h->aF, 0, 2 * (size_t)h->Q * h->Kp * 8, h->stream));
  DG_CUDA(cudaMemsetAsync(h->aV, 0, 3 * (size_t)h->R * h->Kp * 8, h->stream));
  if (h->lim) {
    // every sweep starts with the limiter adjoint's key sets reset and its pass count at 0
    const size_t kb = o.keyBytes, vq = (size_t)h->Vp * kb;   // one quantity's min (or max) keys
    for (int set = 0; set < h->adjKeySets; ++set)
      for (int q = 0; q < h->nc; ++q) {
        char *base = (char *)h->vkeysA + ((size_t)set * h->nc + q) * 2 * vq;
        DG_CUDA(cudaMemsetAsync(base, 0xFF, vq, h->stream));
        DG_CUDA(cudaMemsetAsync(base + vq, 0, vq, h->stream));
      }
    std::vector<unsigned long long> init((size_t)h->adjKeySets * h->nInst * kSlotCopies * 2 * h->nc);
    for (size_t i = 0; i < init.size(); ++i) init[i] = (i & 1) ? 0ULL : o.slotKeyMax;
    DG_CUDA(cudaMemcpyAsync(h->gmmA, init.data(), init.size() * 8, cudaMemcpyHostToDevice, h->stream));
    DG_CUDA(cudaStreamSynchronize(h->stream));
    h->adjPass = h->adjPassF = 0;
  }
  DG_CUDA(cudaMemcpyAsync(h->stage_ext, dJdcT, (size_t)h->N * h->K * 8, cudaMemcpyHostToDevice, h->stream));
  DG_CUDA(o.scatter_in(h, h->lam));
  // The reverse sweep (about 2S + 1 launches per step) runs as one CUDA graph, captured on the
  // first backward of a run length / step / snapshot count and replayed afterwards.
  int st = DGADV_OK;
  // one CUDA graph for the whole sweep (DGADV_OPT_ADJ_GRAPH; default: without the limiter, whose
  // sweeps of thousands of launches over two streams ran faster launched directly)
  const int ag = h->adjGraph < 0 ? (h->lim ? 0 : 1) : h->adjGraph;
  const bool useGraph = !(h->flags & DGADV_FLAG_NO_GRAPH) && ag == 1;
  if (useGraph && !h->adjExec) {
    cudaGraph_t graph = nullptr;
    DG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    st = reverse_sweep(h);
    const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (st == DGADV_OK && e != cudaSuccess) {
      h->err = std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e);
      st = DGADV_ECUDA;
    }
    if (st == DGADV_OK) {
      const cudaError_t e2 = cudaGraphInstantiate(&h->adjExec, graph, 0);
      if (e2 != cudaSuccess) {
        h->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e2);
        h->adjExec = nullptr;
        st = DGADV_ECUDA;
      } else {
        h->adjExecSteps = h->recSteps;
        h->adjExecSlots = h->nSlots;
        h->adjExecTau = h->recTau;
      }
    }
    if (graph) cudaGraphDestroy(graph);
  } else if (!useGraph) {
    st = reverse_sweep(h);
  }
  if (st == DGADV_OK && useGraph) {
    const cudaError_t e = cudaGraphLaunch(h->adjExec, h->stream);
    if (e != cudaSuccess) { h->err = std::string("cudaGraphLaunch: ") + cudaGetErrorString(e); st = DGADV_ECUDA; }
  }
  // after recSteps swaps the result sits in adjBuf[recSteps % 2]
  h->lam = h->adjBuf[h->recSteps % 2];
  h->accn = h->adjBuf[1 - h->recSteps % 2];
  if (st) return st;
  h->recorded = false;
  if (dJdc0) {
    DG_CUDA(o.gather_out(h, h->lam));
    DG_CUDA(cudaMemcpyAsync(dJdc0, h->stage_ext, (size_t)h->N * h->K * 8, cudaMemcpyDeviceToHost, h->stream));
  }
  if (dJdtheta && h->nModes > 0) {
    const int nF = 2 * h->Q, nV = 3 * h->R;
    const int gx = std::min(kThetaBlocks, (h->K + 255) / 256);
    for (int m0 = 0; m0 < h->nModes; m0 += 1024) {
      const int nm = std::min(1024, h->nModes - m0);
      k_theta_partial<<<dim3(gx, nm), 256, 0, h->stream>>>(h->K, h->Kp, nF, nV, o.realBytes == 4, h->aF, h->aV,
                                                          h->modeF + (size_t)m0 * nF * h->Kp,
                                                          h->modeV + (size_t)m0 * nV * h->Kp, h->thetaPart);
      DG_CUDA(cudaGetLastError());
      std::vector<double> part((size_t)nm * gx);
      DG_CUDA(cudaMemcpyAsync(part.data(), h->thetaPart, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
      DG_CUDA(cudaStreamSynchronize(h->stream));
      for (int m = 0; m < nm; ++m) {
        double s = 0.0;
        for (int b = 0; b < gx; ++b) s += part[(size_t)m * gx + b];
        dJdtheta[m0 + m] = s;
      }
    }
  }
  // leave c^0 as the handle's state
  DG_CUDA(o.copy(h, h->cn, h->adjSlots, bytes));
  return dgadv_sync(h);
  });
}

extern "C" int dgadv_checkpoint_schedule(int32_t nSteps, int32_t nSnapshots, int32_t *actions, int32_t *count,
                                         int32_t *backwardStart) {
  return guarded(nullptr, [&]() -> int {
  if (nSteps < 1 || !count) return DGADV_EINVAL;
  const int nSlots = (nSnapshots <= 0 || nSnapshots >= nSteps) ? nSteps : nSnapshots;
  std::vector<int> o;
  make_schedule(nSteps, nSlots, o);
  const int n = (int)o.size() / 2;
  if (actions) {
    if (*count < n) { *count = n; return DGADV_EINVAL; }
    std::memcpy(actions, o.data(), o.size() * sizeof(int));
  }
  *count = n;
  if (backwardStart) *backwardStart = (int32_t)(backward_start(o) / 2);
  return DGADV_OK;
  });
}
