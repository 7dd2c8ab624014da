// hc_ctx.h -- the context of the C ABI (one mesh, its state and buffers),
// shared by the translation units of the single-mesh path.
#pragma once

#include "hc_host.h"
#include "hc_oned.cuh"

#include <vector>

struct hc_ctx {
  hc_config cfg{};
  int nv = 4;           // conserved variables of the law (Euler 4, scalar advection 3)
  bool scalar = false;  // HC_LAW_SCALAR
  bool oned = false;    // one-dimensional mesh (hc_mesh_upload_1d): ni cells, nj = 1, nv = 3
  std::vector<double> hx;  // its node coordinates
  bool fp32 = false;
  size_t rsz = 8;
  int ni = 0, nj = 0;
  int bc[4] = {-1, -1, -1, -1};
  bool have_mesh = false, have_bcs = false, have_state = false, geom_dirty = true;
  double gamma = 1.4, Rgas = 287.058, minf = 1e-4;
  double lref = 1., sdt = 1.7976931348623157e308;  // species lref and dt (AUSM+up scaling)
  int vscale = 0, pscale = 0;                       // AUSM+up LowMachScaling pair
  unsigned fixes = 0;                               // HC_FIX_* corrections (hc_set_corrections)
  int adj_tapes = -1;                               // adjoint stage tapes (hc_set_adjoint_tapes); -1 auto
  int stall_copy = 0;                               // test hook (hc_inject_stalled_copy)
  int staged_loads = 1;                             // TMA-staged FP32 tile loads (hc_set_staged_loads)
  // the forward sweep recorded by hc_adjoint_record for hc_adjoint_reverse (owned here,
  // released by the reverse sweep, the next record, a mesh upload or destroy)
  void* adj_tape = nullptr;
  void (*adj_tape_free)(void*) = nullptr;
  void drop_adj_tape() {
    if (adj_tape && adj_tape_free) adj_tape_free(adj_tape);
    adj_tape = nullptr;
  }
  void* dual_src = nullptr;                         // dual time: earlier levels' terms (4 planes, R)
  double dual_g0 = 1.0, dual_b0dt = 0.0;            // dual time: gamma_0 and beta_0 / dt
  double smooth_alpha = 0.0;                        // 1D residual smoothing factor (0: off)
  void* smooth_buf = nullptr;                       // its sweep buffers (2 x 3 planes, R)
  cudaStream_t own = nullptr, stream = nullptr;
  int tile = hc::TILE_8x32;
  // device buffers
  double* nodes = nullptr;
  double* cx = nullptr;
  double* cy = nullptr;
  double* xm = nullptr;
  double* fi64 = nullptr;
  double* fj64 = nullptr;
  double* vol64 = nullptr;
  void* fi = nullptr;   // face records in R (aliases fi64 for FP64)
  void* fj = nullptr;
  bool df = false;      // HC_FP64_DF: stages compute in double-float
  void* fic = nullptr;  // face records as double-float (HC_FP64_DF)
  void* fjc = nullptr;
  void* vol = nullptr;
  void* q[3] = {nullptr, nullptr, nullptr};
  void* res[4] = {nullptr, nullptr, nullptr, nullptr};
  void* gref[4] = {nullptr, nullptr, nullptr, nullptr};
  double* staging = nullptr;  // FP64 staging for FP32 transfers (4 planes)
  hc::StepInfo* info = nullptr;
  std::vector<double> href[4];
  long long launches = 0;

  size_t ncell() const { return size_t(ni) * nj; }
  int nface(int side) const { return side < 2 ? nj : ni; }
};

namespace hc {

// geometry built and state present (builds the geometry on first use)
int ctx_ensure_ready(hc_ctx* c);

template <class R> StageArgs<R> base_args(hc_ctx* c) {
  StageArgs<R> a{};
  a.ni = c->ni; a.nj = c->nj;
  for (int k = 0; k < 4; ++k) a.bc[k] = c->bc[k];
  a.gas = with_fixes(make_gas<R>(c->gamma, c->Rgas, c->minf, c->lref, c->sdt, c->vscale, c->pscale), c->fixes);
  a.limiter = c->cfg.limiter;
  a.basis = c->cfg.basis;
  a.dual_src = (const R*)c->dual_src;
  a.dual_g0 = R(c->dual_g0);
  a.dual_b0dt = R(c->dual_b0dt);
  a.fi = (const R*)c->fi; a.fj = (const R*)c->fj; a.vol = (const R*)c->vol;
  a.fic = c->fic; a.fjc = c->fjc;
  for (int k = 0; k < 4; ++k) a.gref[k] = (const R*)c->gref[k];
  a.q0 = (const R*)c->q[0];
  a.info = c->info;
  a.cfl = R(c->cfg.cfl);
  a.stall_copy = c->stall_copy;
  a.plain_loads = c->staged_loads ? 0 : 1;
  return a;
}

}  // namespace hc
