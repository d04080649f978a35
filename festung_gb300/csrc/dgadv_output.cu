// Solution output of a handle: nodal values on the device, files written by a host thread.
//
// dgadv_output replaces the output path of advection/outputStep.m:53-66 (and the same calls in
// advection/initializeProblem.m:80-86 and advection/postprocessProblem.m:44-55):
// projectDataDisc2DataLagr (core/projectDataDisc2DataLagr.m:43-57) runs as a kernel over the
// state, the K x numP values go to a pinned host buffer by an asynchronous copy on the handle's
// stream, and a writer thread formats the files (core/visualizeDataLagr.m) once that copy has
// landed.  The call returns after enqueueing: later time steps run on the GPU while the files
// are written.  Two pinned buffers rotate; a third output waits until the writer frees one.
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

#include "dgadv_handle.h"
#include "dgadv_vis.h"

namespace dgadv {

constexpr int kMaxN = (kMaxP + 1) * (kMaxP + 2) / 2;

struct LagrTab {
  double phi[6][kMaxN];   // phi_i at node j
};

// dataLagr(e, j) = sum_i c(e, i) phi_i(node j), summed in basis order with separate roundings
// (the reference's dataLagr = dataLagr + dataDisc(:, i) * phi(i, L1, L2)).  ext: K x N FP64 in
// caller order; out: K x numP.
__global__ void k_lagrange(int K, int N, int numP, const double *__restrict__ ext, double *__restrict__ out,
                           const LagrTab t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double c[kMaxN];
#pragma unroll
  for (int i = 0; i < kMaxN; ++i) c[i] = i < N ? ext[(size_t)i * K + e] : 0.0;
  for (int j = 0; j < numP; ++j) {
    double v = 0.0;
#pragma unroll
    for (int i = 0; i < kMaxN; ++i)
      if (i < N) v = __dadd_rn(v, __dmul_rn(c[i], t.phi[j][i]));
    out[(size_t)j * K + e] = v;
  }
}

struct OutputJob {
  int slot, numP, tLvl, types;
  std::string var, base;
};

struct OutputQueue {
  std::mutex m;
  std::condition_variable cv;
  std::deque<OutputJob> jobs;
  int running = 0;              // jobs taken by the writer, not yet finished
  bool stop = false;
  double *host[2] = {nullptr, nullptr};   // pinned K x numP buffers
  cudaEvent_t ev[2] = {nullptr, nullptr};
  bool busy[2] = {false, false};
  double *dev = nullptr;        // device K x 6 values
  int device = 0;
  std::string err;              // first write error since the last dgadv_output_wait
  VisMesh mesh;
  std::thread worker;

  void run() {
    cudaSetDevice(device);
    for (;;) {
      OutputJob job;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return stop || !jobs.empty(); });
        if (jobs.empty()) return;
        job = std::move(jobs.front());
        jobs.pop_front();
        ++running;
      }
      std::string e;
      const cudaError_t ce = cudaEventSynchronize(ev[job.slot]);
      if (ce != cudaSuccess)
        e = std::string("output copy: ") + cudaGetErrorString(ce);
      else
        mesh.write(host[job.slot], job.numP, job.var.c_str(), job.base.c_str(), job.tLvl, job.types, e);
      {
        std::lock_guard<std::mutex> lk(m);
        if (!e.empty() && err.empty()) err = e;
        busy[job.slot] = false;
        --running;
      }
      cv.notify_all();
    }
  }
};

void output_release(dgadv_handle *h) {
  OutputQueue *q = h->outq;
  if (!q) return;
  {
    std::lock_guard<std::mutex> lk(q->m);
    q->stop = true;
  }
  q->cv.notify_all();
  if (q->worker.joinable()) q->worker.join();   // pending jobs are written first
  for (int s = 0; s < 2; ++s) {
    if (q->host[s]) cudaFreeHost(q->host[s]);
    if (q->ev[s]) cudaEventDestroy(q->ev[s]);
  }
  delete q;
  h->outq = nullptr;
}

static int numP_of(int p) { return p == 0 ? 1 : (p == 1 ? 3 : 6); }

// Enqueues gather + Lagrange evaluation into `dst` (device, K x numP) on the handle's stream.
static int enqueue_lagrange(dgadv_handle *h, double *dst) {
  LagrTab t = {};
  double tab[6 * kMaxN];
  const int numP = lagrange_table(h->p, h->N, tab);
  for (int j = 0; j < numP; ++j)
    for (int i = 0; i < h->N; ++i) t.phi[j][i] = tab[j * h->N + i];
  DG_CUDA(ops_of(h).gather_out(h, h->cn));
  const int grid = (h->K + 255) / 256;
  k_lagrange<<<grid, 256, 0, h->stream>>>(h->K, h->N, numP, h->stage_ext, dst, t);
  DG_CUDA(cudaGetLastError());
  return DGADV_OK;
}

static int output_init_buffers(dgadv_handle *h, OutputQueue *q) {
  q->device = h->device;
  if (!q->mesh.init(h->K, (int)(h->visCoordV.size() / 2), h->visCoordV.data(), h->visV0T.data(), h->err))
    return DGADV_EMESH;
  const size_t bytes = (size_t)h->K * numP_of(h->p) * sizeof(double);
  if (int st = dev_alloc(h, (void **)&q->dev, bytes)) return st;
  for (int s = 0; s < 2; ++s) {
    DG_CUDA(cudaMallocHost((void **)&q->host[s], bytes));
    DG_CUDA(cudaEventCreateWithFlags(&q->ev[s], cudaEventDisableTiming));
  }
  return DGADV_OK;
}

// Output state of a handle, made on first use (pinned buffers, events, writer thread).
static int output_init(dgadv_handle *h) {
  if (h->outq) return DGADV_OK;
  OutputQueue *q = new (std::nothrow) OutputQueue();
  if (!q) return DGADV_ENOMEM;
  h->outq = q;
  if (int st = output_init_buffers(h, q)) {
    output_release(h);
    return st;
  }
  q->worker = std::thread([q] { q->run(); });
  return DGADV_OK;
}

}  // namespace dgadv

using namespace dgadv;

extern "C" int dgadv_get_lagrange(dgadv_handle *h, double *dataLagr, int32_t *numP) {
  return guarded(h, [&]() -> int {
  if (!h || !dataLagr) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const int st = output_init(h);
  if (st) return st;
  const int n = numP_of(h->p);
  if (numP) *numP = n;
  // the device buffer may still feed an output copy in flight: stream order keeps them apart
  if (int e = enqueue_lagrange(h, h->outq->dev)) return e;
  DG_CUDA(cudaMemcpyAsync(dataLagr, h->outq->dev, (size_t)h->K * n * sizeof(double), cudaMemcpyDeviceToHost,
                          h->stream));
  return dgadv_sync(h);
  });
}

extern "C" int dgadv_output(dgadv_handle *h, const char *varName, const char *fileName, int32_t tLvl,
                            int32_t fileTypes) {
  return guarded(h, [&]() -> int {
  if (!h || !varName || !fileName || !fileTypes || (fileTypes & ~(DGADV_OUT_VTK | DGADV_OUT_TEC)))
    return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  const int st = output_init(h);
  if (st) return st;
  OutputQueue *q = h->outq;
  int slot;
  {
    std::unique_lock<std::mutex> lk(q->m);
    q->cv.wait(lk, [&] { return !q->busy[0] || !q->busy[1]; });
    slot = q->busy[0] ? 1 : 0;
    q->busy[slot] = true;
  }
  const int n = numP_of(h->p);
  int e = enqueue_lagrange(h, q->dev);
  if (!e) {
    const cudaError_t ce = cudaMemcpyAsync(q->host[slot], q->dev, (size_t)h->K * n * sizeof(double),
                                           cudaMemcpyDeviceToHost, h->stream);
    const cudaError_t ce2 = ce == cudaSuccess ? cudaEventRecord(q->ev[slot], h->stream) : ce;
    if (ce2 != cudaSuccess) { h->err = cudaGetErrorString(ce2); e = DGADV_ECUDA; }
  }
  {
    std::lock_guard<std::mutex> lk(q->m);
    if (e)
      q->busy[slot] = false;
    else
      q->jobs.push_back(OutputJob{slot, n, tLvl, fileTypes, varName, fileName});
  }
  q->cv.notify_all();
  return e;
  });
}

extern "C" int dgadv_output_wait(dgadv_handle *h) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  OutputQueue *q = h->outq;
  if (!q) return DGADV_OK;
  std::unique_lock<std::mutex> lk(q->m);
  q->cv.wait(lk, [&] { return q->jobs.empty() && q->running == 0; });
  if (!q->err.empty()) {
    h->err = q->err;
    q->err.clear();
    return DGADV_EIO;
  }
  return DGADV_OK;
  });
}
