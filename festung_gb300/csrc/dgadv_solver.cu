// C-ABI of the device solver (include/dgadv.h): handle set-up (mesh reordering, static
// per-element data, constant tables), state transfer and the time loop with CUDA graphs.
// The kernels of each arithmetic type are enqueued through that type's PrecOps table
// (dgadv_prec_fp64.cu, dgadv_prec_fp32.cu, dgadv_prec_df32_p*.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "dgadv_handle.h"

namespace dgadv {
// constant tables uploaded, per device, arithmetic type and degree
static std::mutex g_tab_mutex;
static bool g_tab_loaded[64][3][kMaxP + 1];
}  // namespace dgadv

// ---------------------------------------------------------------------------------------------
// C-ABI
using namespace dgadv;


void dgadv::set_error(const dgadv_handle *h, const char *msg) {
  if (h) const_cast<dgadv_handle *>(h)->err = msg;
}

int dgadv::dev_alloc(dgadv_handle *h, void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) { h->err = std::string("cudaMalloc: ") + cudaGetErrorString(e); return DGADV_ENOMEM; }
  h->allocs.push_back(*p);
  return DGADV_OK;
}

int dgadv::upload(dgadv_handle *h, void *dst, const void *src, size_t bytes) {
  DG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return DGADV_OK;
}

namespace dgadv {
const PrecOps &ops_of(const dgadv_handle *h) {
  switch (h->prec) {
    case DGADV_FP64: return ops_fp64();
    case DGADV_FP32: return ops_fp32();
    default: return h->p <= 1 ? ops_df32_p01() : h->p == 2 ? ops_df32_p2() : ops_df32_p3();
  }
}
}  // namespace dgadv
static const PrecOps &ops(const dgadv_handle *h) { return ops_of(h); }

// Host FP64 values converted to the handle's stored reals and copied to the device.
int dgadv::upload_real(dgadv_handle *h, void *dst, const std::vector<double> &src) {
  const PrecOps &o = ops(h);
  std::vector<unsigned char> tmp(src.size() * o.realBytes);
  o.to_real(src.data(), src.size(), tmp.data());
  return upload(h, dst, tmp.data(), tmp.size());
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

// One handle over one mesh, or over the disjoint union of an ensemble's meshes: instStart holds
// the first element of every instance and the total element count (empty: one instance).
static int create_impl(const dgadv_mesh *mesh, const dgadv_params *prm, const std::vector<int> &instStart,
                       dgadv_handle **out) {
  if (!out) return DGADV_EINVAL;
  *out = nullptr;
  if (!mesh || !prm) return DGADV_EINVAL;
  if (prm->p < 0 || prm->p > 4 || prm->ordRK < 1 || prm->ordRK > 3) return DGADV_EINVAL;
  if (prm->precision != DGADV_FP64 && prm->precision != DGADV_FP32 && prm->precision != DGADV_DF32)
    return DGADV_EINVAL;
  if (prm->isSlopeLim && prm->p < 1) return DGADV_EINVAL;
  if (prm->p > kMaxP) return DGADV_EUNSUPPORTED;
  if (prm->isSlopeLim && prm->typeSlopeLim != DGADV_LIM_LINEAR && prm->typeSlopeLim != DGADV_LIM_HIERARCH_VERT &&
      prm->typeSlopeLim != DGADV_LIM_STRICT)
    return DGADV_EINVAL;
  dgadv_handle *h = new (std::nothrow) dgadv_handle();
  if (!h) return DGADV_ENOMEM;
  *out = h;
  h->device = prm->device;
  h->p = prm->p; h->N = N_of_p(prm->p); h->ordRK = prm->ordRK; h->prec = prm->precision;
  h->lim = prm->isSlopeLim ? 1 : 0; h->limType = prm->typeSlopeLim; h->flags = prm->flags;
  h->limdot = h->lim && h->p > 1;
  h->mtOnTheFly = h->prec == DGADV_FP32;   // FP32 kernels are bandwidth-bound, the others are not
  h->adjWarps = h->prec == DGADV_FP32 ? 2 : 0;   // the adjoint stage's warp-role split
  h->nc = h->lim ? (h->limType == DGADV_LIM_LINEAR ? 1 : h->p * (h->p + 1) / 2) : 1;
  h->passesPerStep = h->lim ? h->ordRK * (h->limdot ? 2 : 1) : 0;
  if ((h->flags & DGADV_FLAG_FUSE) && !ops(h).fused) {
    h->err = "the fused limiter pipeline is not built for this precision";
    return DGADV_EUNSUPPORTED;
  }
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  // static grid data (core/generateGridData.m semantics)
  Grid gr;
  if (!build_grid(mesh->numV, mesh->coordV, mesh->numT, mesh->V0T, gr, h->err)) return DGADV_EMESH;
  const bool implicit = (h->flags & DGADV_FLAG_IMPLICIT) != 0;
  if (implicit && h->lim) { h->err = "the implicit problem has no limiter"; return DGADV_EINVAL; }
  if (!build_ref_tables(h->p, h->tables, h->err, implicit ? 2 * h->p + 1 : 0)) return DGADV_EINVAL;
  h->velOrder = implicit ? 2 * h->p + 1 : std::max(2 * h->p, 1);
  h->visCoordV = gr.coordV;
  h->visV0T = gr.V0T;
  const int K = gr.numT, N = h->N;
  h->K = K; h->Kp = (K + kBlock - 1) / kBlock * kBlock;   // whole blocks of rows for the bulk copies
  h->Q = h->tables.Q; h->R = h->tables.R;
  const int Kp = h->Kp;
  // instances: contiguous element ranges, each a whole number of blocks
  h->instStart = instStart.empty() ? std::vector<int>{0, K} : instStart;
  h->nInst = (int)h->instStart.size() - 1;
  if (h->instStart.back() != K) { h->err = "instance ranges do not cover the elements"; return DGADV_EINVAL; }
  for (int i = 0; i < h->nInst; ++i)
    if (h->nInst > 1 && (h->instStart[i + 1] - h->instStart[i]) % kBlock != 0) {
      h->err = "every ensemble instance needs a multiple of 128 elements";
      return DGADV_EINVAL;
    }
  // element order on the device: Morton order of the barycentres within each instance
  std::vector<int> perm(K);
  std::iota(perm.begin(), perm.end(), 0);
  if (!(h->flags & DGADV_FLAG_NO_REORDER)) {
    for (int i = 0; i < h->nInst; ++i) {
      const int t0 = h->instStart[i], t1 = h->instStart[i + 1];
      double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
      for (int t = t0; t < t1; ++t) {
        xmin = std::min(xmin, gr.baryT[2 * t]); xmax = std::max(xmax, gr.baryT[2 * t]);
        ymin = std::min(ymin, gr.baryT[2 * t + 1]); ymax = std::max(ymax, gr.baryT[2 * t + 1]);
      }
      const double sx = 65535.0 / std::max(xmax - xmin, 1e-300), sy = 65535.0 / std::max(ymax - ymin, 1e-300);
      std::vector<uint32_t> key(K);
      for (int t = t0; t < t1; ++t)
        key[t] = morton2((uint32_t)((gr.baryT[2 * t] - xmin) * sx), (uint32_t)((gr.baryT[2 * t + 1] - ymin) * sy));
      std::stable_sort(perm.begin() + t0, perm.begin() + t1, [&](int a, int b) { return key[a] < key[b]; });
    }
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
  h->nuE0T.assign(6 * (size_t)K, 0); h->corner0.assign(2 * (size_t)K, 0);
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
      for (int m = 0; m < 2; ++m) h->nuE0T[6 * (size_t)k + 2 * n + m] = gr.nuE0T[6 * (size_t)t + 2 * n + m];
    }
    h->corner0[2 * (size_t)k] = gr.coordV0T[6 * (size_t)t];
    h->corner0[2 * (size_t)k + 1] = gr.coordV0T[6 * (size_t)t + 1];
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
  const size_t w = ops(h).realBytes, kw = ops(h).keyBytes;
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
  if ((st = dev_alloc(h, &h->vkeys, 3 * 2 * (size_t)nc * h->Vp * kw))) return st;
  if ((st = dev_alloc(h, (void **)&h->gmm, 3 * (size_t)h->nInst * kSlotCopies * 2 * (size_t)nc * 8))) return st;
  if ((st = dev_alloc(h, (void **)&h->flag, 16))) return st;
  if ((st = dev_alloc(h, &h->gridBar, kGridBarBytes))) return st;
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
    std::vector<unsigned char> vk(3 * 2 * (size_t)nc * h->Vp * kw, 0);
    for (size_t set = 0; set < 3 * (size_t)nc; ++set)
      std::memset(vk.data() + set * 2 * h->Vp * kw, 0xFF, (size_t)h->Vp * kw);
    if ((st = upload(h, h->vkeys, vk.data(), vk.size()))) return st;
  }
  {
    // slots of pass 0 start reset; every later pass is reset by the previous producer
    std::vector<unsigned long long> init(3 * (size_t)h->nInst * kSlotCopies * 2 * (size_t)nc);
    const unsigned long long kmax = ops(h).slotKeyMax;
    for (size_t i = 0; i < init.size(); ++i) init[i] = (i & 1) ? 0ULL : kmax;
    if ((st = upload(h, h->gmm, init.data(), init.size() * 8))) return st;
  }
  DG_CUDA(cudaMemset(h->flag, 0, 16));
  DG_CUDA(cudaMemset(h->gridBar, 0, kGridBarBytes));
  if ((st = upload_real(h, h->Bm, Bsoa))) return st;
  if ((st = upload(h, h->nbr, nbr.data(), nbr.size() * 4))) return st;
  if ((st = upload(h, h->code, code.data(), code.size() * 4))) return st;
  if ((st = upload(h, h->V0T, V0T.data(), V0T.size() * 4))) return st;
  if ((st = upload(h, h->vptr, vptr.data(), vptr.size() * 4))) return st;
  if ((st = upload(h, h->vidx, vidx.data(), vidx.size() * 4))) return st;
  if ((st = upload(h, h->perm, perm.data(), perm.size() * 4))) return st;
  if (h->nInst > 1) {
    // instance of every block a kernel may launch (grids cover max(K, numV) elements)
    const int nBlocks = (std::max(Kp, h->Vp) + kBlock - 1) / kBlock + 1;
    std::vector<int> instOf(nBlocks, 0);
    for (int i = 0; i < h->nInst; ++i)
      for (int t = h->instStart[i]; t < h->instStart[i + 1]; t += kBlock) instOf[t / kBlock] = i;
    if ((st = dev_alloc(h, (void **)&h->instOf, instOf.size() * 4))) return st;
    if ((st = upload(h, h->instOf, instOf.data(), instOf.size() * 4))) return st;
  }
  if (h->limdot && h->limType == DGADV_LIM_LINEAR) {
    std::vector<double> qk;
    taylor_correction(gr, h->p, h->tables, qk);
    const int NQk = N * (N - 1);
    std::vector<double> soa((size_t)NQk * Kp, 0.0);
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < NQk; ++i) soa[(size_t)i * Kp + k] = qk[(size_t)perm[k] * NQk + i];
    if ((st = dev_alloc(h, &h->MT, soa.size() * w))) return st;
    if ((st = upload_real(h, h->MT, soa))) return st;
  } else if (h->limdot) {
    std::vector<double> mt;
    taylor_mass_packed(gr, h->p, mt);
    const int NMT = N * (N + 1) / 2;
    std::vector<double> soa((size_t)NMT * Kp, 0.0);
    for (int k = 0; k < K; ++k)
      for (int i = 0; i < NMT; ++i) soa[(size_t)i * Kp + k] = mt[(size_t)perm[k] * NMT + i];
    if ((st = dev_alloc(h, &h->MT, soa.size() * w))) return st;
    if ((st = upload_real(h, h->MT, soa))) return st;
  }
  // constant tables (once per device, precision and degree)
  {
    std::lock_guard<std::mutex> lk(g_tab_mutex);
    const int pi = h->prec;
    if (h->device < 0 || h->device >= 64) { h->err = "device ordinal out of range"; return DGADV_EINVAL; }
    if (!implicit && !g_tab_loaded[h->device][pi][h->p]) {   // implicit handles use their own tables
      cudaError_t e = ops(h).upload_tables(h->p, h->tables);
      if (e != cudaSuccess) { h->err = std::string("table upload: ") + cudaGetErrorString(e); return DGADV_ECUDA; }
      e = ops(h).set_smem(h->p);
      if (e == cudaSuccess && ops(h).persist_attributes) e = ops(h).persist_attributes(h->p);
      if (e != cudaSuccess) { h->err = std::string("kernel attributes: ") + cudaGetErrorString(e); return DGADV_ECUDA; }
      g_tab_loaded[h->device][pi][h->p] = true;
    }
  }
  DG_CUDA(cudaDeviceSynchronize());
  return DGADV_OK;
}

extern "C" int dgadv_create(const dgadv_mesh *mesh, const dgadv_params *prm, dgadv_handle **out) {
  return guarded(nullptr, [&]() -> int {
  return create_impl(mesh, prm, std::vector<int>(), out);
  });
}

extern "C" int dgadv_create_ensemble(const dgadv_mesh *meshes, int32_t nInst, const dgadv_params *prm,
                                     dgadv_handle **out) {
  return guarded(nullptr, [&]() -> int {
  if (!out) return DGADV_EINVAL;
  *out = nullptr;
  if (!meshes || !prm || nInst < 1) return DGADV_EINVAL;
  // the disjoint union of the instance meshes, instances in order
  int nT = 0, nV = 0;
  const bool hasId = meshes[0].idE0T, hasD = meshes[0].markE0TbdrD, hasN = meshes[0].markE0TbdrN;
  for (int i = 0; i < nInst; ++i) {
    const dgadv_mesh &m = meshes[i];
    if (m.numT <= 0 || m.numV <= 0 || !m.coordV || !m.V0T) return DGADV_EINVAL;
    if ((bool)m.idE0T != hasId || (bool)m.markE0TbdrD != hasD || (bool)m.markE0TbdrN != hasN) return DGADV_EINVAL;
    nT += m.numT;
    nV += m.numV;
  }
  std::vector<double> coordV(2 * (size_t)nV);
  std::vector<int32_t> V0T(3 * (size_t)nT), idE0T(hasId ? 3 * (size_t)nT : 0);
  std::vector<uint8_t> mD(hasD ? 3 * (size_t)nT : 0), mN(hasN ? 3 * (size_t)nT : 0);
  std::vector<int> instStart(1, 0);
  int t0 = 0, v0 = 0;
  for (int i = 0; i < nInst; ++i) {
    const dgadv_mesh &m = meshes[i];
    for (int v = 0; v < m.numV; ++v) {
      coordV[v0 + v] = m.coordV[v];
      coordV[(size_t)nV + v0 + v] = m.coordV[(size_t)m.numV + v];
    }
    for (int n = 0; n < 3; ++n)
      for (int t = 0; t < m.numT; ++t) {
        const size_t src = (size_t)n * m.numT + t, dst = (size_t)n * nT + t0 + t;
        V0T[dst] = m.V0T[src] + v0;
        if (hasId) idE0T[dst] = m.idE0T[src];
        if (hasD) mD[dst] = m.markE0TbdrD[src];
        if (hasN) mN[dst] = m.markE0TbdrN[src];
      }
    t0 += m.numT;
    v0 += m.numV;
    instStart.push_back(t0);
  }
  dgadv_mesh u;
  u.numT = nT; u.numV = nV; u.coordV = coordV.data(); u.V0T = V0T.data();
  u.idE0T = hasId ? idE0T.data() : nullptr;
  u.markE0TbdrD = hasD ? mD.data() : nullptr;
  u.markE0TbdrN = hasN ? mN.data() : nullptr;
  return create_impl(&u, prm, instStart, out);
  });
}

void dgadv::velocity_factors(const dgadv_handle *h, const double *u1, const double *u2, const double *vN,
                             std::vector<double> &F, std::vector<double> &Vn) {
  const int K = h->K, Kp = h->Kp, N = h->N, Q = h->Q, R = h->R;
  const RefTables &t = h->tables;
  F.assign(2 * (size_t)Q * Kp, 0.0);
  Vn.assign(3 * (size_t)R * Kp, 0.0);
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
}

extern "C" int dgadv_set_velocity(dgadv_handle *h, const double *u1, const double *u2, const double *vN) {
  return guarded(h, [&]() -> int {
  if (!h || !u1 || !u2 || !vN) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  std::vector<double> F, Vn;
  velocity_factors(h, u1, u2, vN, F, Vn);
  int st;
  if ((st = upload_real(h, h->F, F))) return st;
  if ((st = upload_real(h, h->Vn, Vn))) return st;
  h->hasVelocity = true;
  ++h->velVersion;
  return refresh_element_operator(h);
  });
}

extern "C" int dgadv_set_source_terms(dgadv_handle *h, int32_t nTerms, const int32_t *timeFn,
                                      const double *rhsTerms, const double *cDV0T) {
  return guarded(h, [&]() -> int {
  if (!h || nTerms < 0 || nTerms > 4) return DGADV_EINVAL;
  if (nTerms > 0 && (!timeFn || !rhsTerms)) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  const int K = h->K, Kp = h->Kp, N = h->N;
  const size_t w = ops(h).realBytes;
  for (int m = 0; m < nTerms; ++m)
    if (timeFn[m] != DGADV_TIME_CONST && timeFn[m] != DGADV_TIME_EXP_NEG) return DGADV_EINVAL;
  h->nTerms = nTerms;
  for (int m = 0; m < 4; ++m) h->timeFn[m] = m < nTerms ? timeFn[m] : 0;
  for (int i = 0; i < 3; ++i)
    if (h->graph[i]) { cudaGraphExecDestroy(h->graph[i]); h->graph[i] = nullptr; }
  if (h->adjExec) { cudaGraphExecDestroy(h->adjExec); h->adjExec = nullptr; h->adjExecSteps = 0; }
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
  if ((st = upload_real(h, h->rhs, r))) return st;
  if (cDV0T && (st = upload_real(h, h->cDV0T, d))) return st;
  if (!cDV0T && h->cDV0T) DG_CUDA(cudaMemset(h->cDV0T, 0, 4 * (size_t)3 * Kp * w));
  return DGADV_OK;
  });
}

extern "C" int dgadv_set_state(dgadv_handle *h, const double *c) {
  return guarded(h, [&]() -> int {
  if (!h || !c) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaMemcpyAsync(h->stage_ext, c, (size_t)h->N * h->K * 8, cudaMemcpyHostToDevice, h->stream));
  DG_CUDA(ops(h).scatter_in(h, h->cn));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  return DGADV_OK;
  });
}

extern "C" int dgadv_sync(dgadv_handle *h) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  int flag = 0;
  DG_CUDA(cudaMemcpy(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost));
  for (const dgadv_handle *o : h->linked) {   // the linked step's kernels flag in each part's word
    int f = 0;
    DG_CUDA(cudaMemcpy(&f, o->flag, sizeof(int), cudaMemcpyDeviceToHost));
    flag |= f;
  }
  if (flag & 2) {
    // a block gave up at a barrier: the barrier state is reset for the next launch; a stage
    // kernel that gave up may have left copies or MMAs behind, so the handle takes no more steps
    cudaMemset(h->gridBar, 0, kGridBarBytes);
    if (flag & (4 | 8 | 16)) h->poisoned = true;
    h->err = std::string("a bounded device wait timed out:") + ((flag & 4) ? " staging copy" : "") +
             ((flag & 8) ? " grid barrier" : "") + ((flag & 16) ? " tensor-core MMA" : "");
    return DGADV_ETIMEOUT;
  }
  if (flag & 1) { h->err = "non-finite value in the state"; return DGADV_ENONFINITE; }
  return DGADV_OK;
  });
}

extern "C" int dgadv_get_state(dgadv_handle *h, double *c) {
  return guarded(h, [&]() -> int {
  if (!h || !c) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(ops(h).gather_out(h, h->cn));
  DG_CUDA(cudaMemcpyAsync(c, h->stage_ext, (size_t)h->N * h->K * 8, cudaMemcpyDeviceToHost, h->stream));
  return dgadv_sync(h);
  });
}

extern "C" int dgadv_limit_state(dgadv_handle *h, double t) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  if (!h->lim) { h->err = "limiter is off for this handle"; return DGADV_EINVAL; }
  DG_CUDA(cudaSetDevice(h->device));
  cudaError_t e = ops(h).limit(h, t);
  if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  return dgadv_sync(h);
  });
}

static bool time_dependent(const dgadv_handle *h) {
  for (int m = 0; m < h->nTerms; ++m)
    if (h->timeFn[m] != DGADV_TIME_CONST) return true;
  return false;
}

// The parts of a linked step: h, then the handles linked to it.
static int linked_parts(dgadv_handle *h, dgadv_handle **hs) {
  int n = 0;
  hs[n++] = h;
  for (dgadv_handle *o : h->linked) hs[n++] = o;
  return n;
}

// One time step: fused or separate-pass pipeline, or the linked step of h and its linked handles.
static cudaError_t one_step(dgadv_handle *h, double t0, double tau, bool firstOfCall) {
  if (!h->linked.empty()) {
    dgadv_handle *hs[kMaxLinkedParts];
    const int n = linked_parts(h, hs);
    return ops(h).step_linked(hs, n, t0, tau);
  }
  if (use_persistent(h) && ops(h).step_persist) return ops(h).step_persist(h, t0, tau);
  if (use_fused(h))
    return ops(h).step_fused(h, t0, tau, firstOfCall);
  return ops(h).step(h, t0, tau);
}
static cudaError_t end_of_call(dgadv_handle *h) {
  if (!use_fused(h)) return cudaSuccess;
  return ops(h).finalize_fused(h);
}

// Why a handle cannot take part in a linked step (nullptr: it can).
static const char *link_refusal(const dgadv_handle *h) {
  if (h->flags & DGADV_FLAG_IMPLICIT) return "implicit handles are not linked";
  if (h->p < 1 || h->p > 3) return "linked steps cover degrees 1..3";
  if (h->lim && h->limType != DGADV_LIM_LINEAR) return "linked steps take the linear limiter or none";
  if (h->nTerms > 0 || h->rhs || h->cDV0T) return "linked steps take no source or boundary terms";
  if (h->flags & (DGADV_FLAG_FUSE | DGADV_FLAG_PERSIST)) return "linked steps use the separate-pass pipeline";
  if (h->stepSrc || h->stepDst || h->stepStages) return "a recorded adjoint run is in progress";
  if (!h->hasVelocity) return "dgadv_set_velocity was not called";
  return nullptr;
}

// Linked step of h and its linked handles: the others' work queued before waits for h's
// stream first, and theirs waits for the step afterwards.
static int linked_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau) {
  dgadv_handle *hs[kMaxLinkedParts];
  const int n = linked_parts(h, hs);
  for (int i = 0; i < n; ++i)
    if (const char *why = link_refusal(hs[i])) { h->err = std::string("linked step: ") + why; return DGADV_EUNSUPPORTED; }
  for (int i = 1; i < n; ++i) {
    if (!hs[i]->linkEv) DG_CUDA(cudaEventCreateWithFlags(&hs[i]->linkEv, cudaEventDisableTiming));
    DG_CUDA(cudaEventRecord(hs[i]->linkEv, hs[i]->stream));
    DG_CUDA(cudaStreamWaitEvent(h->stream, hs[i]->linkEv, 0));
  }
  int done = 0;
  if (!(h->flags & DGADV_FLAG_NO_GRAPH)) {
    const int chunk = h->graphSteps;
    if (h->linkGraphTau != tau) {
      for (auto &kv : h->linkGraphs) cudaGraphExecDestroy(kv.second);
      h->linkGraphs.clear();
      h->linkGraphTau = tau;
    }
    while (nSteps - done >= chunk) {
      long long key = 0;
      for (int i = n - 1; i >= 0; --i) key = 3 * key + hs[i]->limPass % 3;
      cudaGraphExec_t ex = nullptr;
      for (auto &kv : h->linkGraphs)
        if (kv.first == key) ex = kv.second;
      if (!ex) {
        long long saved[kMaxLinkedParts];
        for (int i = 0; i < n; ++i) saved[i] = hs[i]->limPass;
        cudaGraph_t gph;
        DG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int s = 0; s < chunk && e == cudaSuccess; ++s) e = ops(h).step_linked(hs, n, 0.0, tau);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &gph);
        for (int i = 0; i < n; ++i) hs[i]->limPass = saved[i];
        if (e != cudaSuccess || e2 != cudaSuccess) {
          h->err = std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
          return DGADV_ECUDA;
        }
        DG_CUDA(cudaGraphInstantiate(&ex, gph, 0));
        cudaGraphDestroy(gph);
        h->linkGraphs.emplace_back(key, ex);
      }
      DG_CUDA(cudaGraphLaunch(ex, h->stream));
      for (int i = 0; i < n; ++i) hs[i]->limPass += (long long)chunk * hs[i]->passesPerStep;
      done += chunk;
    }
  }
  for (; done < nSteps; ++done) {
    cudaError_t e = ops(h).step_linked(hs, n, (double)(nStep0 + done) * tau, tau);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
  }
  if (!h->linkEv) DG_CUDA(cudaEventCreateWithFlags(&h->linkEv, cudaEventDisableTiming));
  DG_CUDA(cudaEventRecord(h->linkEv, h->stream));
  for (int i = 1; i < n; ++i) DG_CUDA(cudaStreamWaitEvent(hs[i]->stream, h->linkEv, 0));
  return DGADV_OK;
}

extern "C" int dgadv_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau) {
  return guarded(h, [&]() -> int {
  if (!h || nSteps < 0 || !(tau > 0)) return DGADV_EINVAL;
  if (h->flags & DGADV_FLAG_IMPLICIT) {
    h->err = "explicit steps need a handle without DGADV_FLAG_IMPLICIT";
    return DGADV_EUNSUPPORTED;
  }
  if (!h->hasVelocity) { if (h) h->err = "dgadv_set_velocity was not called"; return DGADV_EINVAL; }
  if (h->linkedTo) { h->err = "this handle is stepped by the handle it is linked to"; return DGADV_EUNSUPPORTED; }
  if (h->poisoned) {
    h->err = "a bounded wait of a stage kernel timed out earlier: the state is undefined, create a new handle";
    return DGADV_ETIMEOUT;
  }
  DG_CUDA(cudaSetDevice(h->device));
  if (nSteps == 0) return DGADV_OK;
  if (!h->linked.empty()) return linked_step(h, nSteps, nStep0, tau);
  const bool fused = use_fused(h);
  const bool useGraph = !(h->flags & DGADV_FLAG_NO_GRAPH) && !time_dependent(h);
  int done = 0;
  if (fused) {   // the first step of a call starts from the limited state
    cudaError_t e = one_step(h, (double)nStep0 * tau, tau, true);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); return DGADV_ECUDA; }
    done = 1;
  }
  if (useGraph) {
    // time-independent data: a captured graph of a chunk of steps, replayed.  Graphs are kept per
    // limiter-pass phase (pass count mod 3) at the chunk start, the key / slot set they use.
    const int chunk = h->graphSteps;
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
  });
}

static void drop_graphs(dgadv_handle *h) {
  for (int i = 0; i < 3; ++i)
    if (h->graph[i]) { cudaGraphExecDestroy(h->graph[i]); h->graph[i] = nullptr; }
  if (h->adjExec) { cudaGraphExecDestroy(h->adjExec); h->adjExec = nullptr; h->adjExecSteps = 0; }
  for (auto &kv : h->linkGraphs) cudaGraphExecDestroy(kv.second);
  h->linkGraphs.clear();
  if (h->linkedTo) drop_graphs(h->linkedTo);   // the linked step's graphs hold this handle's launches
}

int dgadv::refresh_element_operator(dgadv_handle *h) {
  const PrecOps &o = ops(h);
  if (!o.build_element_operator || !h->elemOp || !h->hasVelocity || (h->flags & DGADV_FLAG_IMPLICIT))
    return DGADV_OK;
  if (!h->Aop) {
    int st;
    if ((st = dev_alloc(h, &h->Aop, (size_t)h->N * h->N * h->Kp * o.realBytes))) return st;
    DG_CUDA(cudaMemset(h->Aop, 0, (size_t)h->N * h->N * h->Kp * o.realBytes));
  }
  DG_CUDA(o.build_element_operator(h));
  // captured steps keep their kernels: they are recaptured once the operator comes into use
  if (h->aopVersion < 0) drop_graphs(h);
  h->aopVersion = h->velVersion;
  return DGADV_OK;
}

// Removes `o` from its primary's linked handles.
static void unlink_one(dgadv_handle *o) {
  dgadv_handle *h = o->linkedTo;
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  for (size_t i = 0; i < h->linked.size(); ++i)
    if (h->linked[i] == o) { h->linked.erase(h->linked.begin() + i); break; }
  o->linkedTo = nullptr;
}

extern "C" int dgadv_link(dgadv_handle *h, dgadv_handle *other) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  if (!other) {   // unlink every handle linked to h
    while (!h->linked.empty()) unlink_one(h->linked.back());
    return DGADV_OK;
  }
  if (other == h || other->device != h->device || other->prec != h->prec) {
    h->err = "link: another handle of the same device and precision is needed";
    return DGADV_EINVAL;
  }
  if (!ops(h).step_linked) { h->err = "link: no linked step for this precision"; return DGADV_EUNSUPPORTED; }
  if (h->linkedTo || other->linkedTo || !other->linked.empty()) {
    h->err = "link: a handle is linked into one primary at most, and a primary is linked into none";
    return DGADV_EINVAL;
  }
  if ((int)h->linked.size() + 1 >= kMaxLinkedParts) { h->err = "link: too many linked handles"; return DGADV_EINVAL; }
  for (const dgadv_handle *x : {(const dgadv_handle *)h, (const dgadv_handle *)other})
    if (const char *why = link_refusal(x)) { h->err = std::string("link: ") + why; return DGADV_EUNSUPPORTED; }
  DG_CUDA(cudaStreamSynchronize(other->stream));
  h->linked.push_back(other);
  other->linkedTo = h;
  drop_graphs(h);
  return DGADV_OK;
  });
}

extern "C" int dgadv_set_option(dgadv_handle *h, int32_t option, int32_t value) {
  return guarded(h, [&]() -> int {
  if (!h) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  DG_CUDA(cudaStreamSynchronize(h->stream));
  if (option == DGADV_OPT_GRAPH_STEPS) {
    if (value < 1 || value > 256) return DGADV_EINVAL;
    h->graphSteps = value;
  } else if (option == DGADV_OPT_PERSIST_BLOCKS) {
    if (value < 0 || value > 64) return DGADV_EINVAL;
    h->persistPerSM = value;
    h->persistGrid = 0;
  } else if (option == DGADV_OPT_ADJ_WARPS) {
    if (value != 0 && value != 1 && value != 2 && value != 4) return DGADV_EINVAL;
    h->adjWarps = value;
  } else if (option == DGADV_OPT_ELEMENT_OPERATOR) {
    if (value != 0 && value != 1) return DGADV_EINVAL;
    if (value && !ops(h).build_element_operator) {
      h->err = "the element operator is built for FP64 and double-float";
      return DGADV_EUNSUPPORTED;
    }
    h->elemOp = value == 1;
    if (h->elemOp) {
      h->aopVersion = -1;
      int st;
      if ((st = refresh_element_operator(h))) return st;
    }
  } else if (option == DGADV_OPT_ADJ_GRAPH) {
    if (value != -1 && value != 0 && value != 1) return DGADV_EINVAL;
    h->adjGraph = value;
  } else if (option == DGADV_OPT_ADJ_STREAMS) {
    if (value < 1 || value > 3) return DGADV_EINVAL;
    h->adjStreams = value;
  } else if (option == DGADV_OPT_TAYLOR_MASS) {
    if (value != 0 && value != 1) return DGADV_EINVAL;
    h->mtOnTheFly = value == 1;
  } else if (option == DGADV_OPT_OPERATOR_FP32) {
    if (value != 0 && value != 1) return DGADV_EINVAL;
    if (value && h->prec != DGADV_DF32) { h->err = "the FP32 operator is an option of double-float handles"; return DGADV_EUNSUPPORTED; }
    h->opFp32 = value == 1;
  } else if (option == DGADV_OPT_OP_BLOCK) {
    if (value != 64 && value != 128) return DGADV_EINVAL;
    h->opBlock = value;
  } else if (option == DGADV_OPT_VOLUME_MMA) {
    if (value != 0 && value != 1) return DGADV_EINVAL;
    if (value && (h->prec != DGADV_FP32 || h->p < 2)) {
      h->err = "the tensor-core volume term is built for FP32 at p >= 2";
      return DGADV_EUNSUPPORTED;
    }
    h->volumeMma = value == 1;
  } else if (option == DGADV_OPT_FLAGS) {
    const int runtime = DGADV_FLAG_NO_GRAPH | DGADV_FLAG_NO_PDL | DGADV_FLAG_FUSE | DGADV_FLAG_PERSIST;
    if (value & ~runtime) { h->err = "only NO_GRAPH, NO_PDL, FUSE and PERSIST change after creation"; return DGADV_EINVAL; }
    if ((value & DGADV_FLAG_PERSIST) && !ops(h).step_persist) { h->err = "no persistent step for this precision"; return DGADV_EUNSUPPORTED; }
    if ((value & DGADV_FLAG_FUSE) && !ops(h).fused) { h->err = "no fused pipeline for this precision"; return DGADV_EUNSUPPORTED; }
    h->flags = (h->flags & ~runtime) | value;
  } else {
    return DGADV_EINVAL;
  }
  drop_graphs(h);
  return DGADV_OK;
  });
}

extern "C" int dgadv_get_option(const dgadv_handle *h, int32_t option, int32_t *value) {
  return guarded(h, [&]() -> int {
  if (!h || !value) return DGADV_EINVAL;
  if (option == DGADV_OPT_GRAPH_STEPS) *value = h->graphSteps;
  else if (option == DGADV_OPT_FLAGS) *value = h->flags;
  else if (option == DGADV_OPT_PERSIST_BLOCKS) *value = h->persistPerSM;
  else if (option == DGADV_OPT_ADJ_WARPS) *value = h->adjWarps;
  else if (option == DGADV_OPT_ADJ_STREAMS) *value = h->adjStreams;
  else if (option == DGADV_OPT_ADJ_GRAPH) *value = h->adjGraph < 0 ? (h->lim ? 0 : 1) : h->adjGraph;
  else if (option == DGADV_OPT_ELEMENT_OPERATOR) *value = (h->elemOp && ops(h).build_element_operator) ? 1 : 0;
  else if (option == DGADV_OPT_TAYLOR_MASS) *value = h->mtOnTheFly ? 1 : 0;
  else if (option == DGADV_OPT_VOLUME_MMA) *value = h->volumeMma ? 1 : 0;
  else if (option == DGADV_OPT_OP_BLOCK) *value = h->opBlock;
  else if (option == DGADV_OPT_OPERATOR_FP32) *value = h->opFp32 ? 1 : 0;
  else return DGADV_EINVAL;
  return DGADV_OK;
  });
}

// Self-test of the bounded device wait: one block waits on a device flag that nothing sets,
// gives up after limitCycles SM cycles, and records the timeout in the handle's error flag.
__global__ void k_wait_selftest(const int *never, int *flag, long long limitCycles) {
  if (threadIdx.x != 0) return;
  const volatile int *v = never;
  const long long t0 = clock64();
  while (*v == 0)
    if (clock64() - t0 > limitCycles) {
      atomicOr(flag, 2);
      return;
    }
}

extern "C" int dgadv_selftest_wait(dgadv_handle *h, double seconds) {
  return guarded(h, [&]() -> int {
  if (!h || !(seconds > 0.0) || seconds > 2.0) return DGADV_EINVAL;
  DG_CUDA(cudaSetDevice(h->device));
  int khz = 0;
  DG_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, h->device));
  const long long limit = (long long)(seconds * khz * 1e3);
  int *never = (int *)h->stage_ext;   // any device word that stays 0 for the test
  DG_CUDA(cudaMemsetAsync(never, 0, sizeof(int), h->stream));
  k_wait_selftest<<<1, 32, 0, h->stream>>>(never, h->flag, limit);
  DG_CUDA(cudaGetLastError());
  const int st = dgadv_sync(h);
  // the handle stays usable: clear the recorded error
  DG_CUDA(cudaMemset(h->flag, 0, 16));
  return st;
  });
}

extern "C" int dgadv_time_steps(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau, double *ms) {
  return guarded(h, [&]() -> int {
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
  });
}

extern "C" int dgadv_profile_kernels(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau,
                                     double *msPerLaunch, int32_t *launches) {
  return guarded(h, [&]() -> int {
  if (!h || !msPerLaunch || !launches || nSteps < 1) return DGADV_EINVAL;
  if (!h->hasVelocity) { h->err = "dgadv_set_velocity was not called"; return DGADV_EINVAL; }
  if (h->flags & DGADV_FLAG_IMPLICIT) { h->err = "explicit steps need a handle without DGADV_FLAG_IMPLICIT"; return DGADV_EUNSUPPORTED; }
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
  });
}

extern "C" int dgadv_kernels_per_step(const dgadv_handle *h, int32_t *count) {
  return guarded(h, [&]() -> int {
  if (!h || !count) return DGADV_EINVAL;
  if (use_persistent(h) && ops_of(h).step_persist) { *count = 1; return DGADV_OK; }
  if (!h->linked.empty()) {   // per stage: the operator, the cDot limiter if any part has it, the limiter
    std::vector<const dgadv_handle *> hs{h};
    for (const dgadv_handle *o : h->linked) hs.push_back(o);
    int c = 0;
    for (int s = 0; s < 3; ++s) {
      bool op = false, ld = false, lm = false;
      for (const dgadv_handle *x : hs)
        if (s < x->ordRK) { op = true; ld |= x->limdot; lm |= x->lim != 0; }
      c += (int)op + (int)ld + (int)lm;
    }
    *count = c;
    return DGADV_OK;
  }
  int perStage = 1;
  if (use_fused(h)) perStage = h->limdot ? 2 : 1;
  else if (h->lim) perStage = h->limdot ? 3 : 2;
  *count = h->ordRK * perStage;
  return DGADV_OK;
  });
}

extern "C" const char *dgadv_last_error(const dgadv_handle *h) { return h ? h->err.c_str() : "null handle"; }

extern "C" void dgadv_destroy(dgadv_handle *h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  unlink_one(h);
  while (!h->linked.empty()) unlink_one(h->linked.back());
  if (h->linkEv) cudaEventDestroy(h->linkEv);
  try {
    output_release(h);   // joins the writer thread
  } catch (...) {
  }
  implicit_release(h);
  transport_release(h);
  for (int i = 0; i < 3; ++i)
    if (h->graph[i]) cudaGraphExecDestroy(h->graph[i]);
  if (h->adjExec) cudaGraphExecDestroy(h->adjExec);
  if (h->adjStreamF) {
    cudaStreamSynchronize(h->adjStreamF);
    cudaStreamDestroy(h->adjStreamF);
  }
  if (h->adjStreamA) {
    cudaStreamSynchronize(h->adjStreamA);
    cudaStreamDestroy(h->adjStreamA);
  }
  if (h->adjFEv) cudaEventDestroy(h->adjFEv);
  for (cudaEvent_t e : h->adjRevEv) cudaEventDestroy(e);
  for (cudaEvent_t e : h->adjTapeEv) cudaEventDestroy(e);
  for (cudaEvent_t e : h->adjBufEv) cudaEventDestroy(e);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (void *p : h->allocs) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}
