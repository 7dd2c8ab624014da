// hc_batch.cu -- batched path of include/hc.h: many uneven meshes advanced by
// one persistent launch per RK stage over a shared work list of tiles, with
// CUDA-graph capture and a schedule autotuner.
#include "hc_batch.h"
#include "hc_tma.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

using namespace hc;

namespace {

template <class R> __global__ void batch_d2r(const double* a, R* b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = R(a[k]);
}
template <class R> __global__ void batch_r2d(const R* a, double* b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = double(a[k]);
}


void free_all(hc_batch* b) {
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->graph_exec = nullptr; b->graph = nullptr;
  void* ptrs[] = {b->nodes, b->cx, b->cy, b->xm, b->vol64, b->fi64, b->fj64, b->gref, b->q[0], b->q[1], b->q[2],
                  b->res[0], b->res[1], b->res[2], b->staging, b->info, b->inst_d, b->order_d, b->tma_maps};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->fp32) {
    if (b->fi) cudaFree(b->fi);
    if (b->fj) cudaFree(b->fj);
    if (b->vol) cudaFree(b->vol);
  }
}

// Build the work list of the current schedule: tiles of every instance,
// instance-major, instances in natural or largest-first order.
int build_worklist(hc_batch* b) {
  int ti, tj;
  tile_dims(b->sched.tile, &ti, &tj);
  b->inst_h.resize(b->ninst);
  std::vector<int> perm(b->ninst);
  std::iota(perm.begin(), perm.end(), 0);
  if (b->sched.order == HC_ORDER_LARGEST_FIRST)
    std::stable_sort(perm.begin(), perm.end(), [&](int x, int y) { return b->icells(x) > b->icells(y); });
  std::vector<int> order;
  for (int k = 0; k < b->ninst; ++k) {
    BatchInst& in = b->inst_h[k];
    in.ni = b->ni[k]; in.nj = b->nj[k];
    for (int s = 0; s < 4; ++s) { in.bc[s] = b->bc[4 * k + s]; in.gref[s] = b->gref_off[4 * k + s]; }
    in.tiles_i = (in.ni + ti - 1) / ti;
    in.tiles_j = (in.nj + tj - 1) / tj;
    in.cell = b->cell_off[k]; in.fi = b->fi_off[k]; in.fj = b->fj_off[k];
    if (in.tiles_i * in.tiles_j > 0xffff) return fail(HC_ERR_UNSUPPORTED, "instance has more than 65535 tiles");
  }
  for (int k : perm) {
    const int nt = b->inst_h[k].tiles_i * b->inst_h[k].tiles_j;
    for (int t = 0; t < nt; ++t) order.push_back((k << 16) | t);
  }
  b->nwork = int(order.size());
  if (b->nwork > b->nwork_cap) {
    if (b->order_d) cudaFree(b->order_d);
    b->order_d = nullptr;
    HC_CUDA(cudaMalloc(&b->order_d, order.size() * sizeof(int)));
    b->nwork_cap = b->nwork;
  }
  HC_CUDA(cudaMemcpyAsync(b->order_d, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  HC_CUDA(cudaMemcpyAsync(b->inst_d, b->inst_h.data(), b->inst_h.size() * sizeof(BatchInst), cudaMemcpyHostToDevice,
                          b->stream));
  HC_CUDA(cudaStreamSynchronize(b->stream));
  return HC_OK;
}



// Tensor maps of an FP32 Euler batch (hc_tma.h): per instance, the three state pools' slices
// (4 planes of ni x nj) and its i-face records; none when any instance's rows are not a
// multiple of 16 bytes or a slice is not 16-byte aligned (the batch then keeps plain loads).
int build_tma_maps(hc_batch* b) {
  if (!b->fp32 || b->scalar) return HC_OK;
  const int n = b->ninst;
  std::vector<CUtensorMap> maps(size_t(4) * n);
  for (int k = 0; k < n; ++k) {
    StageArgs<float> a{};
    a.ni = b->ni[k];
    a.nj = b->nj[k];
    a.fi = (const float*)b->fi + (long long)FREC * b->fi_off[k];
    for (int buf = 0; buf < 3; ++buf) {
      a.q = (const float*)b->q[buf] + 4 * b->cell_off[k];
      CUtensorMap tfi;
      if (!stage_tma_maps(a, &maps[size_t(buf) * n + k], &tfi)) return HC_OK;
      if (buf == 0) maps[size_t(3) * n + k] = tfi;
    }
  }
  HC_CUDA(cudaMalloc((void**)&b->tma_maps, maps.size() * sizeof(CUtensorMap)));
  HC_CUDA(cudaMemcpy(b->tma_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
  return HC_OK;
}

// the maps of stage input pool q (one of b->q[0..2]) and of the records, or nulls
template <class R> void tma_args(hc_batch* b, BatchArgs<R>& a) {
  a.tmaps_q = a.tmaps_fi = nullptr;
  if constexpr (std::is_same<R, float>::value) {
    if (!b->tma_maps || b->sched.tile != HC_TILE_8x32) return;
    for (int buf = 0; buf < 3; ++buf)
      if (a.q == (const R*)b->q[buf]) {
        a.tmaps_q = b->tma_maps + size_t(buf) * b->ninst;
        a.tmaps_fi = b->tma_maps + size_t(3) * b->ninst;
      }
  }
}

template <class R> int persistent_step(hc_batch* b) {
  const RKTab tab = rk_table(b->cfg.rk);
  const int nst = tab.nst;
  const bool global = b->cfg.dt_mode == HC_DT_GLOBAL;
  const BatchFn<R> euler_fn = batch_fn<R>(b->cfg.flux);
  auto fn = [b, euler_fn](const BatchArgs<R>& a, int tile, int grid, cudaStream_t st) -> cudaError_t {
    return b->scalar ? launch_scalar_batch_stage<R>(a, b->cfg.flux, tile, grid, st) : euler_fn(a, tile, grid, st);
  };
  const int grid = std::max(1, std::min(b->nwork, b->sms * std::max(1, b->sched.ctas_per_sm)));
  if (int st = zero_step_words(b)) return st;
  auto out_of = [&](int s) -> R* { return (R*)((s == nst - 1) ? b->q[0] : b->q[1 + (s % 2)]); };
  for (int s = 0; s < nst; ++s) {
    BatchArgs<R> a = batch_args<R>(b);
    a.q = (s == 0) ? (const R*)b->q[0] : out_of(s - 1);
    tma_args(b, a);
    a.stage = s;
    a.beta = R(tab.beta[s]);
    for (int k = 0; k <= s; ++k) a.alpha[k] = R(tab.alpha[s][k]);
    for (int k = 0; k < s; ++k) a.res_prev[k] = (const R*)b->res[k];
    a.res_out = (s < nst - 1) ? (R*)b->res[s] : nullptr;
    if (global && s == 0) {
      a.mode = MODE_RES_MAXRATE;
      a.res_out = (R*)b->res[0];
      HC_CUDA(fn(a, b->sched.tile, grid, b->stream));
      a.q_out = out_of(0);
      if (b->scalar)
        HC_CUDA(launch_scalar_batch_update0<R>(a, b->sched.tile, grid, b->cfg.cfl, R(tab.alpha[0][0]),
                                               R(tab.beta[0]), b->stream));
      else
        HC_CUDA(launch_batch_update0<R>(a, b->sched.tile, grid, b->cfg.cfl, R(tab.alpha[0][0]), R(tab.beta[0]),
                                        b->stream));
      b->launches += 2;
    } else {
      a.mode = global ? MODE_FUSED_GLOBAL : MODE_FUSED_LOCAL;
      a.q_out = out_of(s);
      HC_CUDA(fn(a, b->sched.tile, grid, b->stream));
      b->launches += 1;
    }
  }
  return HC_OK;
}

// The same step as plain launches, instance by instance (the comparison path).
template <class R> int per_instance_step(hc_batch* b) {
  const RKTab tab = rk_table(b->cfg.rk);
  const int nst = tab.nst;
  const bool global = b->cfg.dt_mode == HC_DT_GLOBAL;
  const StageFn<R> euler_fn = stage_fn<R>(b->cfg.flux);
  auto fn = [b, euler_fn](const StageArgs<R>& a, int tile, cudaStream_t st) -> cudaError_t {
    return b->scalar ? launch_scalar_stage<R>(a, b->cfg.flux, tile, st) : euler_fn(a, tile, st);
  };
  if (int st = zero_step_words(b)) return st;
  for (int k = 0; k < b->ninst; ++k) {
    const long long c4 = 4 * b->cell_off[k], c5 = 5 * b->cell_off[k];
    auto qp = [&](int i) { return (R*)b->q[i] + c4; };
    auto rp = [&](int i) { return (R*)b->res[i] + c5; };
    auto out_of = [&](int s) -> R* { return (s == nst - 1) ? qp(0) : qp(1 + (s % 2)); };
    StageArgs<R> base{};
    base.ni = b->ni[k]; base.nj = b->nj[k];
    for (int s = 0; s < 4; ++s) {
      base.bc[s] = b->bc[4 * k + s];
      base.gref[s] = (const R*)b->gref + b->gref_off[4 * k + s];
    }
    base.gas = with_fixes(make_gas<R>(b->gamma, b->Rgas, b->minf), b->fixes);
    base.limiter = b->cfg.limiter;
    base.basis = b->cfg.basis;
    base.fi = (const R*)b->fi + (long long)FREC * b->fi_off[k];
    base.fj = (const R*)b->fj + (long long)FREC * b->fj_off[k];
    base.vol = (const R*)b->vol + b->cell_off[k];
    base.q0 = qp(0);
    base.info = b->info + k;
    base.cfl = R(b->cfg.cfl);
    for (int s = 0; s < nst; ++s) {
      StageArgs<R> a = base;
      a.q = (s == 0) ? qp(0) : out_of(s - 1);
      a.stage = s;
      a.beta = R(tab.beta[s]);
      for (int m = 0; m <= s; ++m) a.alpha[m] = R(tab.alpha[s][m]);
      for (int m = 0; m < s; ++m) a.res_prev[m] = rp(m);
      a.res_out = (s < nst - 1) ? rp(s) : nullptr;
      a.norm_stage0 = (s == 0);
      if (global && s == 0) {
        a.mode = MODE_RES_MAXRATE;
        a.res_out = rp(0);
        HC_CUDA(fn(a, b->sched.tile, b->stream));
        const size_t n = b->icells(k);
        const unsigned grid = unsigned(std::min<size_t>((n + 255) / 256, size_t(b->sms) * 16));
        if (b->scalar)
          HC_CUDA(launch_scalar_update0<R>(base.ni, base.nj, qp(0), rp(0), base.vol, R(tab.alpha[0][0]),
                                           R(tab.beta[0]), b->cfg.cfl, base.info, out_of(0), 1, b->stream));
        else
          update0_kernel<R><<<grid, 256, 0, b->stream>>>(base.ni, base.nj, base.gas, qp(0), rp(0), base.vol,
                                                         R(tab.alpha[0][0]), R(tab.beta[0]), b->cfg.cfl, base.info,
                                                         out_of(0), 1, b->cfg.basis, 0.0);
        HC_CUDA(cudaGetLastError());
        b->launches += 2;
      } else {
        a.mode = global ? MODE_FUSED_GLOBAL : MODE_FUSED_LOCAL;
        a.q_out = out_of(s);
        HC_CUDA(fn(a, b->sched.tile, b->stream));
        b->launches += 1;
      }
    }
  }
  return HC_OK;
}

int run_steps(hc_batch* b, int nsteps, int mode) {
  for (int s = 0; s < nsteps; ++s) {
    int st;
    if (mode == HC_BATCH_PER_INSTANCE) st = b->fp32 ? per_instance_step<float>(b) : per_instance_step<double>(b);
    else st = b->fp32 ? persistent_step<float>(b) : persistent_step<double>(b);
    if (st != HC_OK) return st;
  }
  return HC_OK;
}

int check_b(hc_batch* b) { return b ? HC_OK : fail(HC_ERR_ARG, "null batch"); }

}  // namespace

extern "C" {

int hc_batch_create(const hc_config* cfg, int ninst, const int* ni, const int* nj, const double* const* nodes,
                    const int* bc, const double* const* ref, double gamma, double gas_constant, double minf,
                    hc_batch** out) {
  if (!cfg || !out || !ni || !nj || !nodes || !bc) return fail(HC_ERR_ARG, "null argument");
  if (ninst < 1 || ninst > 32767) return fail(HC_ERR_ARG, "instance count must be in [1, 32767]");
  if (cfg->flux < 0 || cfg->flux >= FLUX_COUNT || cfg->limiter < 0 || cfg->limiter >= LIM_COUNT ||
      cfg->rk < HC_RK_SSP11 || cfg->rk > HC_RK_SSP34 || (cfg->precision != HC_FP64 && cfg->precision != HC_FP32) ||
      (cfg->dt_mode != HC_DT_GLOBAL && cfg->dt_mode != HC_DT_LOCAL) || !(cfg->cfl > 0) ||
      (cfg->basis != HC_BASIS_PRIMITIVE && cfg->basis != HC_BASIS_CONSERVED))
    return fail(HC_ERR_ARG, "invalid configuration");
  const bool scalar = cfg->law == HC_LAW_SCALAR;
  if (cfg->law != HC_LAW_EULER && !scalar) return fail(HC_ERR_ARG, "unknown conservation law");
  if (scalar && cfg->flux != HC_FLUX_RUSANOV && cfg->flux != HC_FLUX_CENTRAL)
    return fail(HC_ERR_UNSUPPORTED, "the scalar advection law takes the Rusanov or central flux");
  if (scalar && cfg->basis != HC_BASIS_PRIMITIVE)
    return fail(HC_ERR_UNSUPPORTED, "the scalar advection law has one basis (its conserved set)");
  if (!(gamma > 1.0) || !(gas_constant > 0.0) || !(minf > 0.0)) return fail(HC_ERR_ARG, "invalid species");
  for (int k = 0; k < ninst; ++k) {
    if (ni[k] < 3 || nj[k] < 3 || !nodes[k]) return fail(HC_ERR_ARG, "instance " + std::to_string(k) + ": bad mesh");
    const int* t = bc + 4 * k;
    for (int s = 0; s < 4; ++s)
      if (t[s] < HC_BC_PERIODIC || t[s] > HC_BC_WALL) return fail(HC_ERR_ARG, "unknown bc type");
    if (scalar)
      for (int s = 0; s < 4; ++s)
        if (t[s] == HC_BC_WALL || t[s] == HC_BC_ENTROPY)
          return fail(HC_ERR_UNSUPPORTED, "scalar advection boundaries are periodic, fixed or Riemann");
    if ((t[0] == HC_BC_PERIODIC) != (t[1] == HC_BC_PERIODIC) || (t[2] == HC_BC_PERIODIC) != (t[3] == HC_BC_PERIODIC))
      return fail(HC_ERR_ARG, "periodic sides must come in pairs");
    for (int s = 0; s < 4; ++s)
      if (t[s] != HC_BC_PERIODIC && t[s] != HC_BC_WALL && (!ref || !ref[4 * k + s]))
        return fail(HC_ERR_ARG, "instance " + std::to_string(k) + " side " + std::to_string(s) + " needs reference values");
  }
  hc_batch* b = new hc_batch();
  b->cfg = *cfg;
  b->scalar = scalar;
  b->nv = scalar ? 3 : 4;
  b->fp32 = cfg->precision == HC_FP32;
  b->rsz = b->fp32 ? 4 : 8;
  b->ninst = ninst;
  b->ni.assign(ni, ni + ninst);
  b->nj.assign(nj, nj + ninst);
  b->bc.assign(bc, bc + 4 * ninst);
  b->gamma = gamma; b->Rgas = gas_constant; b->minf = minf;
  auto bail = [&](int code) { free_all(b); if (b->own) cudaStreamDestroy(b->own); delete b; return code; };
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(HC_ERR_CUDA, "no CUDA device"));
  b->stream = b->own;
  cudaError_t pe = scalar ? (b->fp32 ? prepare_scalar_stage<float>() : prepare_scalar_stage<double>())
                          : (b->fp32 ? prepare<float>(cfg->flux) : prepare<double>(cfg->flux));
  if (pe != cudaSuccess) return bail(fail(HC_ERR_CUDA, cudaGetErrorString(pe)));
  // offsets
  size_t maxcell = 0;
  for (int k = 0; k < ninst; ++k) {
    b->cell_off.push_back(b->ncell); b->ncell += b->icells(k);
    b->fi_off.push_back(b->nfi); b->nfi += size_t(ni[k] + 1) * nj[k];
    b->fj_off.push_back(b->nfj); b->nfj += size_t(ni[k]) * (nj[k] + 1);
    b->node_off.push_back(b->nnode); b->nnode += size_t(ni[k] + 1) * (nj[k] + 1) * 2;
    maxcell = std::max(maxcell, b->icells(k));
    for (int s = 0; s < 4; ++s) {
      b->gref_off.push_back(b->ngref);
      b->ngref += size_t(4) * (s < 2 ? nj[k] : ni[k]);
    }
  }
  auto A = [&](void** p, size_t bytes) { return cudaMalloc(p, std::max<size_t>(bytes, 16)); };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = A((void**)&b->nodes, b->nnode * 8);
  if (e == cudaSuccess) e = A((void**)&b->cx, b->ncell * 8);
  if (e == cudaSuccess) e = A((void**)&b->cy, b->ncell * 8);
  if (e == cudaSuccess) e = A((void**)&b->xm, 3 * b->ncell * 8);
  if (e == cudaSuccess) e = A((void**)&b->vol64, b->ncell * 8);
  if (e == cudaSuccess) e = A((void**)&b->fi64, FREC * b->nfi * 8);
  if (e == cudaSuccess) e = A((void**)&b->fj64, FREC * b->nfj * 8);
  if (e == cudaSuccess) e = A(&b->gref, b->ngref * b->rsz);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = A(&b->q[k], 4 * b->ncell * b->rsz);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = A(&b->res[k], 5 * b->ncell * b->rsz);
  if (e == cudaSuccess) e = A((void**)&b->staging, 4 * maxcell * 8);
  if (e == cudaSuccess) e = A((void**)&b->info, ninst * sizeof(StepInfo));
  if (e == cudaSuccess) e = A((void**)&b->inst_d, ninst * sizeof(BatchInst));
  if (e == cudaSuccess) e = cudaMemsetAsync(b->info, 0, ninst * sizeof(StepInfo), b->stream);
  if (e == cudaSuccess && b->fp32) {
    e = A(&b->fi, FREC * b->nfi * 4);
    if (e == cudaSuccess) e = A(&b->fj, FREC * b->nfj * 4);
    if (e == cudaSuccess) e = A(&b->vol, b->ncell * 4);
  } else if (e == cudaSuccess) {
    b->fi = b->fi64; b->fj = b->fj64; b->vol = b->vol64;
  }
  if (e != cudaSuccess) return bail(fail(HC_ERR_CUDA, std::string("batch allocation: ") + cudaGetErrorString(e)));
  // meshes, geometry, reference states
  std::vector<double> gref_h(b->ngref, 0.0);
  for (int k = 0; k < ninst && e == cudaSuccess; ++k) {
    const size_t nn = size_t(ni[k] + 1) * (nj[k] + 1) * 2;
    e = cudaMemcpyAsync(b->nodes + b->node_off[k], nodes[k], nn * 8, cudaMemcpyHostToDevice, b->stream);
    const GeomBuffers g{b->nodes + b->node_off[k], b->cx + b->cell_off[k], b->cy + b->cell_off[k],
                        b->xm + 3 * b->cell_off[k], b->vol64 + b->cell_off[k], b->fi64 + FREC * b->fi_off[k],
                        b->fj64 + FREC * b->fj_off[k]};
    // the xm pool is laid out per instance as 3 planes of its own cell count
    b->launches += enqueue_geometry(g, ni[k], nj[k], bc + 4 * k, b->stream);
    for (int s = 0; s < 4; ++s) {
      const int t = bc[4 * k + s];
      if (t == HC_BC_PERIODIC || t == HC_BC_WALL || !ref || !ref[4 * k + s]) continue;
      const size_t m = size_t(b->nv) * (s < 2 ? nj[k] : ni[k]);  // nv planes in the first nv of the slot's 4
      std::copy(ref[4 * k + s], ref[4 * k + s] + m, gref_h.begin() + b->gref_off[4 * k + s]);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);  // nodes[k] may be reused by the caller
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && b->fp32) {
    batch_d2r<float><<<1024, 256, 0, b->stream>>>(b->fi64, (float*)b->fi, FREC * b->nfi);
    batch_d2r<float><<<1024, 256, 0, b->stream>>>(b->fj64, (float*)b->fj, FREC * b->nfj);
    batch_d2r<float><<<1024, 256, 0, b->stream>>>(b->vol64, (float*)b->vol, b->ncell);
    b->launches += 3;
    std::vector<float> gf(gref_h.begin(), gref_h.end());
    e = cudaMemcpyAsync(b->gref, gf.data(), gf.size() * 4, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  } else if (e == cudaSuccess) {
    e = cudaMemcpyAsync(b->gref, gref_h.data(), gref_h.size() * 8, cudaMemcpyHostToDevice, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  }
  if (e != cudaSuccess) return bail(fail(HC_ERR_CUDA, std::string("batch set-up: ") + cudaGetErrorString(e)));
  if (int st = build_worklist(b)) return bail(st);
  if (int st = build_tma_maps(b)) return bail(st);
  *out = b;
  return HC_OK;
}

int hc_batch_destroy(hc_batch* b) {
  if (!b) return HC_OK;
  cudaStreamSynchronize(b->stream);
  b->drop_adj_tape();
  free_all(b);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return HC_OK;
}

int hc_batch_set_stream(hc_batch* b, void* stream) {
  if (int st = check_b(b)) return st;
  HC_CUDA(cudaStreamSynchronize(b->stream));
  b->stream = (cudaStream_t)stream;
  return HC_OK;
}

int hc_batch_state_upload(hc_batch* b, int k, const double* prim) {
  if (int st = check_b(b)) return st;
  if (k < 0 || k >= b->ninst || !prim) return fail(HC_ERR_ARG, "bad instance or null state");
  const size_t m = size_t(b->nv) * b->icells(k);
  if (b->fp32) {
    HC_CUDA(cudaMemcpyAsync(b->staging, prim, m * 8, cudaMemcpyHostToDevice, b->stream));
    batch_d2r<float><<<512, 256, 0, b->stream>>>(b->staging, (float*)b->q[0] + 4 * b->cell_off[k], m);
    HC_CUDA(cudaGetLastError());
    b->launches += 1;
  } else {
    HC_CUDA(cudaMemcpyAsync((double*)b->q[0] + 4 * b->cell_off[k], prim, m * 8, cudaMemcpyHostToDevice, b->stream));
  }
  HC_CUDA(cudaStreamSynchronize(b->stream));
  return HC_OK;
}

int hc_batch_state_upload_device(hc_batch* b, int k, const double* prim_device) {
  if (int st = check_b(b)) return st;
  if (k < 0 || k >= b->ninst || !prim_device) return fail(HC_ERR_ARG, "bad instance or null state");
  const size_t m = size_t(b->nv) * b->icells(k);
  if (b->fp32) {
    batch_d2r<float><<<512, 256, 0, b->stream>>>(prim_device, (float*)b->q[0] + 4 * b->cell_off[k], m);
    HC_CUDA(cudaGetLastError());
    b->launches += 1;
  } else {
    HC_CUDA(cudaMemcpyAsync((double*)b->q[0] + 4 * b->cell_off[k], prim_device, m * 8, cudaMemcpyDeviceToDevice,
                            b->stream));
  }
  return HC_OK;
}

int hc_batch_state_download(hc_batch* b, int k, double* prim) {
  if (int st = check_b(b)) return st;
  if (k < 0 || k >= b->ninst || !prim) return fail(HC_ERR_ARG, "bad instance or null output");
  const size_t m = size_t(b->nv) * b->icells(k);
  if (b->fp32) {
    batch_r2d<float><<<512, 256, 0, b->stream>>>((const float*)b->q[0] + 4 * b->cell_off[k], b->staging, m);
    HC_CUDA(cudaGetLastError());
    b->launches += 1;
    HC_CUDA(cudaMemcpyAsync(prim, b->staging, m * 8, cudaMemcpyDeviceToHost, b->stream));
  } else {
    HC_CUDA(cudaMemcpyAsync(prim, (const double*)b->q[0] + 4 * b->cell_off[k], m * 8, cudaMemcpyDeviceToHost, b->stream));
  }
  HC_CUDA(cudaStreamSynchronize(b->stream));
  return HC_OK;
}

int hc_batch_set_corrections(hc_batch* b, unsigned mask) {
  if (int st = check_b(b)) return st;
  if (mask & ~unsigned(HC_FIX_ALL)) return fail(HC_ERR_ARG, "unknown correction bits");
  b->fixes = mask;
  // a captured graph holds the old launch arguments
  if (b->graph_exec) { cudaGraphExecDestroy(b->graph_exec); b->graph_exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  return HC_OK;
}

int hc_batch_set_adjoint_tapes(hc_batch* b, int ntapes) {
  if (int st = check_b(b)) return st;
  if (ntapes < -1) return fail(HC_ERR_ARG, "stage tapes: -1 (one per snapshot and one more) or a count >= 0");
  b->adj_tapes = ntapes;
  return HC_OK;
}

int hc_batch_set_schedule(hc_batch* b, const hc_schedule* s) {
  if (int st = check_b(b)) return st;
  if (!s || s->tile < HC_TILE_8x32 || s->tile > HC_TILE_16x16 || s->ctas_per_sm < 1 || s->ctas_per_sm > 64 ||
      (s->order != HC_ORDER_NATURAL && s->order != HC_ORDER_LARGEST_FIRST))
    return fail(HC_ERR_ARG, "invalid schedule");
  b->sched = *s;
  if (b->graph_exec) { cudaGraphExecDestroy(b->graph_exec); b->graph_exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  return build_worklist(b);
}

int hc_batch_get_schedule(hc_batch* b, hc_schedule* s) {
  if (int st = check_b(b)) return st;
  if (!s) return fail(HC_ERR_ARG, "null output");
  *s = b->sched;
  return HC_OK;
}

int hc_batch_step_async(hc_batch* b, int nsteps, int mode) {
  if (int st = check_b(b)) return st;
  if (nsteps < 0 || (mode != HC_BATCH_PERSISTENT && mode != HC_BATCH_PER_INSTANCE))
    return fail(HC_ERR_ARG, "bad step count or mode");
  HC_CUDA(cudaMemset2DAsync(&b->info[0].status, sizeof(StepInfo), 0, 2 * sizeof(int), b->ninst, b->stream));
  return run_steps(b, nsteps, mode);
}

int hc_batch_graph_capture(hc_batch* b, int nsteps) {
  if (int st = check_b(b)) return st;
  if (nsteps < 1) return fail(HC_ERR_ARG, "need at least one step");
  if (b->stream == nullptr) return fail(HC_ERR_ARG, "graph capture needs a non-default stream");
  if (b->graph_exec) { cudaGraphExecDestroy(b->graph_exec); b->graph_exec = nullptr; }
  if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
  const long long before = b->launches;
  HC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int st = run_steps(b, nsteps, HC_BATCH_PERSISTENT);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st != HC_OK) { if (g) cudaGraphDestroy(g); return st; }
  HC_CUDA(e);
  b->graph = g;
  HC_CUDA(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
  b->graph_steps = int(b->launches - before);  // launches per replay
  b->launches = before;
  return HC_OK;
}

int hc_batch_graph_launch(hc_batch* b) {
  if (int st = check_b(b)) return st;
  if (!b->graph_exec) return fail(HC_ERR_ARG, "no captured graph");
  HC_CUDA(cudaMemset2DAsync(&b->info[0].status, sizeof(StepInfo), 0, 2 * sizeof(int), b->ninst, b->stream));
  HC_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
  b->launches += b->graph_steps;
  return HC_OK;
}

int hc_batch_sync(hc_batch* b, hc_step_stats* stats) {
  if (int st = check_b(b)) return st;
  std::vector<StepInfo> info(b->ninst);
  HC_CUDA(cudaMemcpyAsync(info.data(), b->info, b->ninst * sizeof(StepInfo), cudaMemcpyDeviceToHost, b->stream));
  HC_CUDA(cudaStreamSynchronize(b->stream));
  int bad = -1;
  for (int k = 0; k < b->ninst; ++k) {
    if (stats) {
      stats[k].dt = info[k].dt;
      stats[k].t = info[k].t;
      stats[k].resnorm = std::sqrt(info[k].resnorm2);
      stats[k].status = info[k].status == ST_OK ? HC_OK : HC_ERR_NONPHYSICAL;
      stats[k].bad_cell = info[k].bad_cell;
      stats[k].kernel_launches = b->launches;
    }
    if (info[k].status != ST_OK && bad < 0) bad = k;
  }
  if (bad >= 0)
    return fail(HC_ERR_NONPHYSICAL, "instance " + std::to_string(bad) + ": non-physical state at cell " +
                                        std::to_string(info[bad].bad_cell));
  return HC_OK;
}

long long hc_batch_kernel_launches(hc_batch* b) { return b ? b->launches : 0; }

int hc_batch_autotune(hc_batch* b, int steps, hc_schedule* best) {
  if (int st = check_b(b)) return st;
  if (steps < 1) return fail(HC_ERR_ARG, "need at least one step per trial");
  // keep the states and per-instance step info; every trial starts from them
  void* save_q = nullptr;
  StepInfo* save_info = nullptr;
  HC_CUDA(cudaMalloc(&save_q, 4 * b->ncell * b->rsz));
  HC_CUDA(cudaMalloc(&save_info, b->ninst * sizeof(StepInfo)));
  HC_CUDA(cudaMemcpyAsync(save_q, b->q[0], 4 * b->ncell * b->rsz, cudaMemcpyDeviceToDevice, b->stream));
  HC_CUDA(cudaMemcpyAsync(save_info, b->info, b->ninst * sizeof(StepInfo), cudaMemcpyDeviceToDevice, b->stream));
  cudaEvent_t e0, e1;
  HC_CUDA(cudaEventCreate(&e0));
  HC_CUDA(cudaEventCreate(&e1));
  const hc_schedule keep = b->sched;
  hc_schedule top = keep;
  top.ms_per_step = 1e30f;
  int rc = HC_OK;
  const int tiles[3] = {HC_TILE_8x32, HC_TILE_4x32, HC_TILE_16x16};
  const int ctas[3] = {1, 2, 4};
  const int orders[2] = {HC_ORDER_NATURAL, HC_ORDER_LARGEST_FIRST};
  const long long launches0 = b->launches;
  for (int t : tiles)
    for (int c : ctas)
      for (int o : orders) {
        hc_schedule s{t, c, o, 0.f};
        if ((rc = hc_batch_set_schedule(b, &s)) != HC_OK) goto done;
        if ((rc = run_steps(b, 1, HC_BATCH_PERSISTENT)) != HC_OK) goto done;  // warm-up
        cudaEventRecord(e0, b->stream);
        if ((rc = run_steps(b, steps, HC_BATCH_PERSISTENT)) != HC_OK) goto done;
        cudaEventRecord(e1, b->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = fail(HC_ERR_CUDA, "autotune timing"); goto done; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        s.ms_per_step = ms / steps;
        if (s.ms_per_step < top.ms_per_step) top = s;
        cudaMemcpyAsync(b->q[0], save_q, 4 * b->ncell * b->rsz, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(b->info, save_info, b->ninst * sizeof(StepInfo), cudaMemcpyDeviceToDevice, b->stream);
      }
done:
  b->launches = launches0;
  cudaMemcpyAsync(b->q[0], save_q, 4 * b->ncell * b->rsz, cudaMemcpyDeviceToDevice, b->stream);
  cudaMemcpyAsync(b->info, save_info, b->ninst * sizeof(StepInfo), cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  cudaFree(save_q);
  cudaFree(save_info);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != HC_OK) {
    hc_batch_set_schedule(b, &keep);
    return rc;
  }
  rc = hc_batch_set_schedule(b, &top);
  if (best) *best = top;
  return rc;
}

}  // extern "C"
