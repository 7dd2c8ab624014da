// hc_batch.h -- the batch handle of include/hc.h's batched path, shared by the
// forward driver (hc_batch.cu) and the batched adjoint (hc_batch_adjoint.cu).
#pragma once

#include "hc_host.h"

#include <vector>

struct hc_batch {
  hc_config cfg{};
  bool fp32 = false;
  bool scalar = false;  // scalar advection instances ({u, v, q}: 3 of the 4 state planes of a slab)
  int nv = 4;
  size_t rsz = 8;
  int ninst = 0;
  std::vector<int> ni, nj, bc;
  std::vector<std::vector<double>> href;  // 4 per instance
  double gamma = 1.4, Rgas = 287.058, minf = 1e-4;
  unsigned fixes = 0;  // HC_FIX_* corrections (hc_batch_set_corrections)
  int adj_tapes = -1;  // adjoint stage tapes (hc_batch_set_adjoint_tapes); -1 auto
  cudaStream_t own = nullptr, stream = nullptr;
  int sms = 152;
  hc_schedule sched{HC_TILE_8x32, 2, HC_ORDER_LARGEST_FIRST, 0.f};
  std::vector<long long> cell_off, fi_off, fj_off, node_off, gref_off;
  size_t ncell = 0, nfi = 0, nfj = 0, nnode = 0, ngref = 0;
  double *nodes = nullptr, *cx = nullptr, *cy = nullptr, *xm = nullptr, *vol64 = nullptr, *fi64 = nullptr,
         *fj64 = nullptr;
  void *fi = nullptr, *fj = nullptr, *vol = nullptr, *gref = nullptr;
  void* q[3] = {nullptr, nullptr, nullptr};
  void* res[3] = {nullptr, nullptr, nullptr};
  double* staging = nullptr;
  hc::StepInfo* info = nullptr;
  hc::BatchInst* inst_d = nullptr;
  // FP32 Euler batches: per-instance tensor maps of the three state pools and of the i-face
  // records ([4][ninst], device memory) for the TMA-staged 8x32 tile; null where a mesh's rows
  // are not a multiple of 16 bytes
  CUtensorMap* tma_maps = nullptr;
  int* order_d = nullptr;
  int nwork = 0, nwork_cap = 0;
  std::vector<hc::BatchInst> inst_h;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_steps = 0;
  long long launches = 0;
  // the forward sweep recorded by hc_batch_adjoint_record for hc_batch_adjoint_reverse
  // (owned here, released by the reverse sweep, the next record or destroy)
  void* adj_tape = nullptr;
  void (*adj_tape_free)(void*) = nullptr;
  void drop_adj_tape() {
    if (adj_tape && adj_tape_free) adj_tape_free(adj_tape);
    adj_tape = nullptr;
  }

  size_t icells(int k) const { return size_t(ni[k]) * nj[k]; }
};

namespace hc {

template <class R> cudaError_t launch_batch_update0(const BatchArgs<R>& b, int tile, int grid, double cfl,
                                                    R alpha00, R beta0, cudaStream_t s) {
  if (tile == HC_TILE_4x32) batch_update0_kernel<4, 32, R><<<grid, 128, 0, s>>>(b, cfl, alpha00, beta0);
  else if (tile == HC_TILE_16x16) batch_update0_kernel<16, 16, R><<<grid, 256, 0, s>>>(b, cfl, alpha00, beta0);
  else batch_update0_kernel<8, 32, R><<<grid, 256, 0, s>>>(b, cfl, alpha00, beta0);
  return cudaGetLastError();
}

template <class R> BatchArgs<R> batch_args(hc_batch* b) {
  BatchArgs<R> a{};
  a.inst = b->inst_d;
  a.order = b->order_d;
  a.nwork = b->nwork;
  a.gas = with_fixes(make_gas<R>(b->gamma, b->Rgas, b->minf), b->fixes);
  a.limiter = b->cfg.limiter;
  a.basis = b->cfg.basis;
  a.q0 = (const R*)b->q[0];
  a.fi = (const R*)b->fi; a.fj = (const R*)b->fj; a.vol = (const R*)b->vol;
  a.gref = (const R*)b->gref;
  a.cfl = R(b->cfg.cfl);
  a.info = b->info;
  return a;
}

// maxrate and resnorm2 of every instance's StepInfo (strided)
inline int zero_step_words(hc_batch* b) {
  HC_CUDA(cudaMemset2DAsync(&b->info[0].maxrate, sizeof(StepInfo), 0, sizeof(unsigned long long), b->ninst,
                            b->stream));
  HC_CUDA(cudaMemset2DAsync(&b->info[0].resnorm2, sizeof(StepInfo), 0, sizeof(double), b->ninst, b->stream));
  return HC_OK;
}

}  // namespace hc
