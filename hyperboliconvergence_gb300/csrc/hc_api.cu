// hc_api.cu -- the C ABI of include/hc.h: contexts, mesh/state transfer and
// the explicit RK time loop over the fused stage kernels.
#include "hc_host.h"
#include "hc_geometry.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace hc;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace hc {

void set_last_error(const std::string& msg) { g_last_error = msg; }

int enqueue_geometry(const GeomBuffers& b, int ni, int nj, const int bc[4], cudaStream_t s) {
  const size_t n = size_t(ni) * nj;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  const int B = 256;
  geom_cells_kernel<<<unsigned((n + B - 1) / B), B, 0, s>>>(b.nodes, ni, nj, b.vol, b.cx, b.cy);
  GeomArgs g{};
  g.nodes = b.nodes; g.ni = ni; g.nj = nj;
  for (int k = 0; k < 4; ++k) g.bc[k] = bc[k];
  g.cx = b.cx; g.cy = b.cy; g.fi = b.fi; g.fj = b.fj; g.xm = b.xm;
  geom_faces1_kernel<<<(nfi + B - 1) / B, B, 0, s>>>(g, 0);
  geom_faces1_kernel<<<(nfj + B - 1) / B, B, 0, s>>>(g, 1);
  geom_xm_kernel<<<unsigned((n + B - 1) / B), B, 0, s>>>(g);
  geom_faces2_kernel<<<(nfi + B - 1) / B, B, 0, s>>>(g, 0);
  geom_faces2_kernel<<<(nfj + B - 1) / B, B, 0, s>>>(g, 1);
  return 6;
}

}  // namespace hc

#include "hc_ctx.h"

namespace {

void free_buffers(hc_ctx* c) {
  void* ptrs[] = {c->nodes, c->cx, c->cy, c->xm, c->fi64, c->fj64, c->vol64, c->q[0], c->q[1], c->q[2],
                  c->res[0], c->res[1], c->res[2], c->res[3], c->gref[0], c->gref[1], c->gref[2], c->gref[3],
                  c->staging, c->info, c->smooth_buf};
  c->smooth_buf = nullptr;
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->fp32) {
    if (c->fi) cudaFree(c->fi);
    if (c->fj) cudaFree(c->fj);
    if (c->vol) cudaFree(c->vol);
  }
  if (c->fic) cudaFree(c->fic);
  if (c->fjc) cudaFree(c->fjc);
  c->nodes = c->cx = c->cy = c->xm = c->fi64 = c->fj64 = c->vol64 = c->staging = nullptr;
  c->fi = c->fj = c->vol = c->fic = c->fjc = nullptr;
  for (int k = 0; k < 3; ++k) c->q[k] = nullptr;
  for (int k = 0; k < 4; ++k) c->res[k] = c->gref[k] = nullptr;
  c->info = nullptr;
}

int check_ctx(hc_ctx* c) {
  if (!c) return fail(HC_ERR_ARG, "null context");
  return HC_OK;
}

// Derive cells, faces and least-squares weights on the device (runs once per mesh/bc set).
int build_geometry_1d(hc_ctx* c) {
  const int nc = c->ni;
  std::vector<double> rec, vol;
  oned_geometry(c->hx.data(), nc, c->bc, rec, vol);
  HC_CUDA(cudaMemcpyAsync(c->fi64, rec.data(), rec.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  HC_CUDA(cudaMemcpyAsync(c->vol64, vol.data(), vol.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->fp32) {
    convert_kernel<float><<<256, 256, 0, c->stream>>>(c->fi64, (float*)c->fi, rec.size());
    convert_kernel<float><<<256, 256, 0, c->stream>>>(c->vol64, (float*)c->vol, vol.size());
    c->launches += 2;
    HC_CUDA(cudaGetLastError());
  }
  for (int s = 0; s < 2; ++s) {
    if (c->bc[s] == HC_BC_PERIODIC || c->bc[s] == HC_BC_WALL || c->href[s].empty()) continue;
    if (c->fp32) {
      const float tmp[3] = {float(c->href[s][0]), float(c->href[s][1]), float(c->href[s][2])};
      HC_CUDA(cudaMemcpyAsync(c->gref[s], tmp, sizeof(tmp), cudaMemcpyHostToDevice, c->stream));
    } else {
      HC_CUDA(cudaMemcpyAsync(c->gref[s], c->href[s].data(), 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));  // the host vectors go out of scope
  c->geom_dirty = false;
  return HC_OK;
}

int build_geometry(hc_ctx* c) {
  if (!c->have_mesh || !c->have_bcs) return fail(HC_ERR_ARG, "mesh and boundary conditions must be set first");
  if (c->oned) return build_geometry_1d(c);
  const int ni = c->ni, nj = c->nj;
  const size_t n = c->ncell();
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);
  const GeomBuffers gb{c->nodes, c->cx, c->cy, c->xm, c->vol64, c->fi64, c->fj64};
  enqueue_geometry(gb, ni, nj, c->bc, c->stream);
  c->launches += 6;
  if (c->fp32) {
    convert_kernel<float><<<1024, 256, 0, c->stream>>>(c->fi64, (float*)c->fi, size_t(FREC) * nfi);
    convert_kernel<float><<<1024, 256, 0, c->stream>>>(c->fj64, (float*)c->fj, size_t(FREC) * nfj);
    convert_kernel<float><<<1024, 256, 0, c->stream>>>(c->vol64, (float*)c->vol, n);
    c->launches += 3;
  }
  if (c->df) {
    convert_kernel<df64><<<1024, 256, 0, c->stream>>>(c->fi64, (df64*)c->fic, size_t(FREC) * nfi);
    convert_kernel<df64><<<1024, 256, 0, c->stream>>>(c->fj64, (df64*)c->fjc, size_t(FREC) * nfj);
    c->launches += 2;
  }
  HC_CUDA(cudaGetLastError());
  // ghost reference planes in the context precision
  for (int s = 0; s < 4; ++s) {
    if (c->bc[s] == HC_BC_PERIODIC || c->bc[s] == HC_BC_WALL || c->href[s].empty()) continue;
    const size_t m = size_t(c->nv) * c->nface(s);
    if (c->fp32) {
      std::vector<float> tmp(m);
      for (size_t k = 0; k < m; ++k) tmp[k] = float(c->href[s][k]);
      HC_CUDA(cudaMemcpyAsync(c->gref[s], tmp.data(), m * sizeof(float), cudaMemcpyHostToDevice, c->stream));
      HC_CUDA(cudaStreamSynchronize(c->stream));
    } else {
      HC_CUDA(cudaMemcpyAsync(c->gref[s], c->href[s].data(), m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    }
  }
  c->geom_dirty = false;
  return HC_OK;
}

int ensure_ready(hc_ctx* c) {
  if (c->geom_dirty) {
    const int st = build_geometry(c);
    if (st != HC_OK) return st;
  }
  if (!c->have_state) return fail(HC_ERR_ARG, "state not uploaded");
  return HC_OK;
}

}  // namespace

int hc::ctx_ensure_ready(hc_ctx* c) { return ensure_ready(c); }

namespace {

template <class R> Stage1DArgs<R> args_1d(hc_ctx* c) {
  Stage1DArgs<R> a{};
  a.nc = c->ni;
  a.bc[0] = c->bc[0]; a.bc[1] = c->bc[1];
  a.gas = with_fixes(make_gas<R>(c->gamma, c->Rgas, c->minf, c->lref, c->sdt, c->vscale, c->pscale), c->fixes);
  a.limiter = c->cfg.limiter;
  a.rec = (const R*)c->fi;
  a.vol = (const R*)c->vol;
  a.gref[0] = (const R*)c->gref[0]; a.gref[1] = (const R*)c->gref[1];
  a.q0 = (const R*)c->q[0];
  a.info = c->info;
  a.cfl = R(c->cfg.cfl);
  return a;
}

template <class R> int run_residual_1d(hc_ctx* c) {
  Stage1DArgs<R> a = args_1d<R>(c);
  a.q = (const R*)c->q[0];
  a.res_out = (R*)c->res[0];
  a.mode = MODE_RESIDUAL;
  HC_CUDA(launch_stage1d<R>(a, c->cfg.flux, c->stream));
  c->launches += 1;
  return HC_OK;
}

// one RK step of the 1D path with residual smoothing (SteadyTimeControls'
// use_residual_smoothing): per stage the residual alone, its three flux planes smoothed
// in place by centralImplicitSmoothing with alpha = smoothing_factor (ends 'p' on a
// periodic line, 'a' otherwise), then the stage update from the smoothed residuals
template <class R> int run_step_1d_smoothed(hc_ctx* c) {
  const RKTab tab = rk_table(c->cfg.rk);
  const int nst = tab.nst;
  const bool global = c->cfg.dt_mode == HC_DT_GLOBAL;
  const long long n = c->ni;
  if (!c->smooth_buf) HC_CUDA(cudaMalloc(&c->smooth_buf, 6 * size_t(n) * sizeof(R)));
  R* wrk = (R*)c->smooth_buf;
  R* tmp = wrk + 3 * n;
  const int ends = c->bc[0] == HC_BC_PERIODIC ? 'p' : 'a';
  HC_CUDA(cudaMemsetAsync(&c->info->maxrate, 0, sizeof(unsigned long long), c->stream));
  HC_CUDA(cudaMemsetAsync(&c->info->resnorm2, 0, sizeof(double), c->stream));
  auto out_of = [&](int s) -> R* { return (R*)((s == nst - 1) ? c->q[0] : c->q[1 + (s % 2)]); };
  for (int s = 0; s < nst; ++s) {
    Stage1DArgs<R> a = args_1d<R>(c);
    a.q = (s == 0) ? (const R*)c->q[0] : out_of(s - 1);
    a.stage = s;
    a.res_out = (R*)c->res[s];
    a.norm_stage0 = (s == 0);
    a.mode = (s == 0) ? MODE_RES_MAXRATE : MODE_RESIDUAL;  // stage 0: max rate and the norm
    HC_CUDA(launch_stage1d<R>(a, c->cfg.flux, c->stream));
    HC_CUDA(launch_smooth_1d<R>(0, (const R*)c->res[s], (R*)c->res[s], wrk, tmp, n, 3, n, c->smooth_alpha, ends,
                                c->stream));
    Update1DArgs<R> u{};
    u.nc = c->ni;
    u.gas = a.gas;
    u.q0 = (const R*)c->q[0];
    for (int k = 0; k <= s; ++k) { u.res[k] = (const R*)c->res[k]; u.alpha[k] = R(tab.alpha[s][k]); }
    u.stage = s;
    u.beta = R(tab.beta[s]);
    u.global = global ? 1 : 0;
    u.cfl = c->cfg.cfl;
    u.info = c->info;
    u.vol = (const R*)c->vol;
    u.q_out = out_of(s);
    const unsigned grid = unsigned(std::min<size_t>((c->ncell() + 255) / 256, 152 * 16));
    update_stage_1d_kernel<R><<<grid, 256, 0, c->stream>>>(u);
    HC_CUDA(cudaGetLastError());
    c->launches += 3;
  }
  return HC_OK;
}

// one RK step of the 1D path (the same stage loop as run_step)
template <class R> int run_step_1d(hc_ctx* c) {
  if (c->smooth_alpha > 0.0) return run_step_1d_smoothed<R>(c);
  const RKTab tab = rk_table(c->cfg.rk);
  const int nst = tab.nst;
  const bool global = c->cfg.dt_mode == HC_DT_GLOBAL;
  HC_CUDA(cudaMemsetAsync(&c->info->maxrate, 0, sizeof(unsigned long long), c->stream));
  HC_CUDA(cudaMemsetAsync(&c->info->resnorm2, 0, sizeof(double), c->stream));
  auto out_of = [&](int s) -> R* { return (R*)((s == nst - 1) ? c->q[0] : c->q[1 + (s % 2)]); };
  for (int s = 0; s < nst; ++s) {
    Stage1DArgs<R> a = args_1d<R>(c);
    a.q = (s == 0) ? (const R*)c->q[0] : out_of(s - 1);
    a.stage = s;
    a.beta = R(tab.beta[s]);
    for (int k = 0; k <= s; ++k) a.alpha[k] = R(tab.alpha[s][k]);
    for (int k = 0; k < s; ++k) a.res_prev[k] = (const R*)c->res[k];
    a.res_out = (s < nst - 1) ? (R*)c->res[s] : nullptr;
    a.norm_stage0 = (s == 0);
    if (global && s == 0) {
      a.mode = MODE_RES_MAXRATE;
      a.res_out = (R*)c->res[0];
      HC_CUDA(launch_stage1d<R>(a, c->cfg.flux, c->stream));
      const unsigned grid = unsigned(std::min<size_t>((c->ncell() + 255) / 256, 152 * 16));
      update0_1d_kernel<R><<<grid, 256, 0, c->stream>>>(c->ni, a.gas, (const R*)c->q[0], (const R*)c->res[0],
                                                         (const R*)c->vol, R(tab.alpha[0][0]), R(tab.beta[0]),
                                                         c->cfg.cfl, c->info, out_of(0));
      HC_CUDA(cudaGetLastError());
      c->launches += 2;
    } else {
      a.mode = global ? MODE_FUSED_GLOBAL : MODE_FUSED_LOCAL;
      a.q_out = out_of(s);
      HC_CUDA(launch_stage1d<R>(a, c->cfg.flux, c->stream));
      c->launches += 1;
    }
  }
  return HC_OK;
}

template <class R> int run_residual(hc_ctx* c) {
  if (c->oned) return run_residual_1d<R>(c);
  StageArgs<R> a = base_args<R>(c);
  a.q = (const R*)c->q[0];
  a.res_out = (R*)c->res[0];
  a.mode = MODE_RESIDUAL;
  if (c->scalar) HC_CUDA(launch_scalar_stage<R>(a, c->cfg.flux, c->tile, c->stream));
  else HC_CUDA(stage_fn<R>(c->cfg.flux)(a, c->tile, c->stream));
  c->launches += 1;
  return HC_OK;
}

// One RK step: the stage loop of integrate() (timestepping/rungeKutta.h:97-164).
template <class R> int run_step(hc_ctx* c) {
  if (c->oned) return run_step_1d<R>(c);
  const RKTab tab = rk_table(c->cfg.rk);
  const int nst = tab.nst;
  const bool global = c->cfg.dt_mode == HC_DT_GLOBAL;
  const StageFn<R> euler_fn = stage_fn<R>(c->cfg.flux);
  auto fn = [c, euler_fn](const StageArgs<R>& a, int tile, cudaStream_t s) -> cudaError_t {
    return c->scalar ? launch_scalar_stage<R>(a, c->cfg.flux, tile, s) : euler_fn(a, tile, s);
  };
  HC_CUDA(cudaMemsetAsync(&c->info->maxrate, 0, sizeof(unsigned long long), c->stream));
  HC_CUDA(cudaMemsetAsync(&c->info->resnorm2, 0, sizeof(double), c->stream));
  auto out_of = [&](int s) -> R* { return (R*)((s == nst - 1) ? c->q[0] : c->q[1 + (s % 2)]); };
  for (int s = 0; s < nst; ++s) {
    StageArgs<R> a = base_args<R>(c);
    a.q = (s == 0) ? (const R*)c->q[0] : out_of(s - 1);
    a.stage = s;
    a.beta = R(tab.beta[s]);
    for (int k = 0; k <= s; ++k) a.alpha[k] = R(tab.alpha[s][k]);
    for (int k = 0; k < s; ++k) a.res_prev[k] = (const R*)c->res[k];
    a.res_out = (s < nst - 1) ? (R*)c->res[s] : nullptr;
    a.norm_stage0 = (s == 0);
    if (global && s == 0) {
      a.mode = MODE_RES_MAXRATE;
      a.res_out = (R*)c->res[0];
      HC_CUDA(fn(a, c->tile, c->stream));
      const size_t n = c->ncell();
      const int B = 256;
      const unsigned grid = unsigned(std::min<size_t>((n + B - 1) / B, 152 * 16));
      if (c->scalar) {
        HC_CUDA(launch_scalar_update0<R>(c->ni, c->nj, (const R*)c->q[0], (const R*)c->res[0], (const R*)c->vol,
                                         R(tab.alpha[0][0]), R(tab.beta[0]), c->cfg.cfl, c->info, out_of(0), 1,
                                         c->stream));
      } else {
        update0_kernel<R><<<grid, B, 0, c->stream>>>(c->ni, c->nj, a.gas, (const R*)c->q[0], (const R*)c->res[0],
                                                     (const R*)c->vol, R(tab.alpha[0][0]), R(tab.beta[0]),
                                                     c->cfg.cfl, c->info, out_of(0), 1, c->cfg.basis,
                                                     c->dual_src ? c->dual_b0dt : 0.0);
      }
      HC_CUDA(cudaGetLastError());
      c->launches += 2;
    } else {
      a.mode = global ? MODE_FUSED_GLOBAL : MODE_FUSED_LOCAL;
      a.q_out = out_of(s);
      HC_CUDA(fn(a, c->tile, c->stream));
      c->launches += 1;
    }
  }
  return HC_OK;
}

int read_stats(hc_ctx* c, hc_step_stats* st) {
  StepInfo info{};
  HC_CUDA(cudaMemcpyAsync(&info, c->info, sizeof(StepInfo), cudaMemcpyDeviceToHost, c->stream));
  HC_CUDA(cudaStreamSynchronize(c->stream));
  if (st) {
    if (c->cfg.dt_mode == HC_DT_LOCAL) {
      // smallest local timestep of the last step: cfl / max(lambda/V)
      double rate;
      std::memcpy(&rate, &info.maxrate, sizeof(double));
      st->dt = c->cfg.cfl / std::fmax(rate, 2.2250738585072014e-308);
    } else {
      st->dt = info.dt;
    }
    st->t = info.t;
    st->resnorm = std::sqrt(info.resnorm2);
    st->status = info.status == ST_OK ? HC_OK : info.status == ST_TIMEOUT ? HC_ERR_TIMEOUT : HC_ERR_NONPHYSICAL;
    st->bad_cell = info.bad_cell;
    st->kernel_launches = c->launches;
  }
  if (info.status == ST_TIMEOUT) return fail(HC_ERR_TIMEOUT, "a staged tile load did not complete in its bounded wait");
  if (info.status != ST_OK)
    return fail(HC_ERR_NONPHYSICAL, "non-physical state at cell " + std::to_string(info.bad_cell));
  return HC_OK;
}

template <class R> __global__ void d2r_kernel(const double* a, R* b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = R(a[k]);
}
template <class R> __global__ void r2d_kernel(const R* a, double* b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = double(a[k]);
}

}  // namespace

namespace {
template <class R>
int run_signatures(hc_ctx* c, unsigned long long* sig_i, unsigned long long* sig_j, double* arg_i, double* arg_j) {
  const size_t nfi = size_t(c->ni + 1) * c->nj, nfj = size_t(c->ni) * (c->nj + 1);
  const bool args = arg_i && arg_j;
  unsigned long long* d = nullptr;
  double* da = nullptr;
  HC_CUDA(cudaMalloc(&d, (nfi + nfj) * sizeof(unsigned long long)));
  struct Free { void* p; ~Free() { if (p) cudaFree(p); } } guard{d};
  if (args) HC_CUDA(cudaMalloc(&da, 16 * (nfi + nfj) * sizeof(double)));
  Free guard_a{da};
  HC_CUDA(cudaMemsetAsync(d, 0, (nfi + nfj) * sizeof(unsigned long long), c->stream));
  if (args) HC_CUDA(cudaMemsetAsync(da, 0, 16 * (nfi + nfj) * sizeof(double), c->stream));
  StageArgs<R> a = base_args<R>(c);
  a.q = (const R*)c->q[0];
  a.mode = MODE_RESIDUAL;
  a.res_out = nullptr;
  a.sig_i = d;
  a.sig_j = d + nfi;
  a.arg_i = da;
  a.arg_j = da ? da + 16 * nfi : nullptr;
  if constexpr (std::is_same<R, double>::value) {
    if (c->df) HC_CUDA((launch_sig_stage<double, true>(a, c->cfg.flux, c->stream)));
    else HC_CUDA((launch_sig_stage<double, false>(a, c->cfg.flux, c->stream)));
  } else {
    HC_CUDA((launch_sig_stage<float, false>(a, c->cfg.flux, c->stream)));
  }
  c->launches += 1;
  HC_CUDA(cudaMemcpyAsync(sig_i, d, nfi * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  HC_CUDA(cudaMemcpyAsync(sig_j, d + nfi, nfj * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
  if (args) {
    HC_CUDA(cudaMemcpyAsync(arg_i, da, 16 * nfi * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaMemcpyAsync(arg_j, da + 16 * nfi, 16 * nfj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));
  return HC_OK;
}
}  // namespace

// ---------------------------------------------------------------- dual time
// ODE::Implicit::MultiStep tables (ode.h:12-82): (b_0 u_{n+1} + b_1 u_n + b_2 u_{n-1})/dt =
// g_0 R(u_{n+1}) + g_1 R(u_n)
struct MultiStepTab { double beta[3], gamma[2]; };
inline MultiStepTab multistep(int scheme) {
  if (scheme == HC_BDF2) return {{1.5, -2.0, 0.5}, {1.0, 0.0}};
  if (scheme == HC_TRAPEZIUM) return {{1.0, -1.0, 0.0}, {0.5, 0.5}};
  return {{1.0, -1.0, 0.0}, {1.0, 0.0}};
}

template <class R>
__global__ void cons_set_kernel(size_t n, Gas<R> g, const R* __restrict__ q, R* __restrict__ Q, int basis) {
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
    R qk[4], qc[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) qk[v] = q[v * n + c];
    basis_to_cons(g, qk, qc, basis != 0);
#pragma unroll
    for (int v = 0; v < 4; ++v) Q[v * n + c] = qc[v];
  }
}

// the earlier levels' terms of the dual-time residual, per cell:
// src = g_1 R(u_n) - V (b_1 Q_n + b_2 Q_{n-1}) / dt
template <class R>
__global__ void dual_source_kernel(size_t n, const R* __restrict__ vol, const R* __restrict__ Qn,
                                   const R* __restrict__ Qnm1, const R* __restrict__ Rn, R b1dt, R b2dt, R g1,
                                   R* __restrict__ src) {
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
    const R V = vol[c];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const R lev = b1dt * Qn[v * n + c] + b2dt * Qnm1[v * n + c];
      src[v * n + c] = (Rn ? g1 * Rn[v * n + c] : R(0)) - V * lev;
    }
  }
}

template <class R> int dual_time_run(hc_ctx* c, const hc_dual_time_controls* ctl, hc_dual_time_stats* out) {
  const size_t n = c->ncell();
  const MultiStepTab ms = multistep(ctl->scheme);
  const unsigned grid = unsigned(std::min<size_t>((n + 255) / 256, 152 * 16));
  const Gas<R> g =
      with_fixes(make_gas<R>(c->gamma, c->Rgas, c->minf, c->lref, c->sdt, c->vscale, c->pscale), c->fixes);
  R* buf = nullptr;
  const bool trap = ms.gamma[1] != 0.0;
  HC_CUDA(cudaMalloc(&buf, (3 * 4 + (trap ? 5 : 0)) * n * sizeof(R)));
  struct Reset {
    hc_ctx* c; void* p;
    ~Reset() { c->dual_src = nullptr; c->dual_g0 = 1.0; c->dual_b0dt = 0.0; cudaFree(p); }
  } reset{c, buf};
  R* Qn = buf;
  R* Qnm1 = buf + 4 * n;
  R* src = buf + 8 * n;
  R* Rn = trap ? buf + 12 * n : nullptr;
  // physical timestep: given, or cfl_outer / max(lambda/V) of the initial state (dualTime.ipp:54-56)
  double dt = ctl->dt;
  if (!(dt > 0.0)) {
    HC_CUDA(cudaMemsetAsync(&c->info->maxrate, 0, sizeof(unsigned long long), c->stream));
    StageArgs<R> a = base_args<R>(c);
    a.q = (const R*)c->q[0];
    a.res_out = (R*)c->res[0];
    a.mode = MODE_RES_MAXRATE;
    HC_CUDA(stage_fn<R>(c->cfg.flux)(a, c->tile, c->stream));
    c->launches += 1;
    unsigned long long bits = 0;
    HC_CUDA(cudaMemcpyAsync(&bits, &c->info->maxrate, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    double rate;
    std::memcpy(&rate, &bits, sizeof(rate));
    dt = ctl->cfl_outer / std::fmax(rate, 2.2250738585072014e-308);
  }
  cons_set_kernel<R><<<grid, 256, 0, c->stream>>>(n, g, (const R*)c->q[0], Qn, c->cfg.basis);
  HC_CUDA(cudaGetLastError());
  HC_CUDA(cudaMemcpyAsync(Qnm1, Qn, 4 * n * sizeof(R), cudaMemcpyDeviceToDevice, c->stream));
  c->launches += 1;
  hc_dual_time_stats st{};
  st.dt = dt;
  HC_CUDA(cudaMemsetAsync(&c->info->status, 0, 2 * sizeof(int), c->stream));
  for (int k = 0; k < ctl->outer_steps; ++k) {
    if (trap) {
      if (int e = run_residual<R>(c)) return e;
      HC_CUDA(cudaMemcpyAsync(Rn, c->res[0], 4 * n * sizeof(R), cudaMemcpyDeviceToDevice, c->stream));
    }
    dual_source_kernel<R><<<grid, 256, 0, c->stream>>>(n, (const R*)c->vol, Qn, Qnm1, Rn, R(ms.beta[1] / dt),
                                                        R(ms.beta[2] / dt), R(ms.gamma[1]), src);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
    c->dual_src = src;
    c->dual_g0 = ms.gamma[0];
    c->dual_b0dt = ms.beta[0] / dt;
    // pseudo-time iterations (dualTime.ipp:49-98): RK steps of the dual-time residual
    double res0 = 0.0, res = 0.0;
    int m = 0;
    while (m < ctl->inner_max) {
      const int chunk = (m == 0) ? 1 : std::min(ctl->check_every, ctl->inner_max - m);
      for (int j = 0; j < chunk; ++j)
        if (int e = run_step<R>(c)) return e;
      m += chunk;
      hc_step_stats s{};
      if (int e = read_stats(c, &s)) return e;
      res = s.resnorm;
      if (m == 1) res0 = res;
      if (ctl->inner_drop > 0.0 && res <= ctl->inner_drop * res0) break;
    }
    c->dual_src = nullptr;
    c->dual_g0 = 1.0;
    c->dual_b0dt = 0.0;
    // next level: u_{n-1} <- u_n, u_n <- u_{n+1}
    std::swap(Qn, Qnm1);
    cons_set_kernel<R><<<grid, 256, 0, c->stream>>>(n, g, (const R*)c->q[0], Qn, c->cfg.basis);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
    st.outer_steps += 1;
    st.inner_steps += m;
    st.last_inner = m;
    st.res0_last = res0;
    st.res_last = res;
    st.t += dt;
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));
  if (out) *out = st;
  return HC_OK;
}

extern "C" {

const char* hc_last_error_string(void) { return g_last_error.c_str(); }
const char* hc_version(void) { return "hyperboliconvergence_gb300 0.1 sm_103a"; }

int hc_context_create(const hc_config* cfg, hc_ctx** out) {
  if (!cfg || !out) return fail(HC_ERR_ARG, "null argument");
  if (cfg->flux < 0 || cfg->flux >= FLUX_COUNT) return fail(HC_ERR_ARG, "unknown flux");
  if (cfg->limiter < 0 || cfg->limiter >= LIM_COUNT) return fail(HC_ERR_ARG, "unknown limiter");
  if (cfg->rk < HC_RK_SSP11 || cfg->rk > HC_RK_SSP34) return fail(HC_ERR_ARG, "unknown RK table");
  if (cfg->precision != HC_FP64 && cfg->precision != HC_FP32 && cfg->precision != HC_FP64_DF)
    return fail(HC_ERR_ARG, "unknown precision");
  if (cfg->dt_mode != HC_DT_GLOBAL && cfg->dt_mode != HC_DT_LOCAL) return fail(HC_ERR_ARG, "unknown dt mode");
  if (!(cfg->cfl > 0)) return fail(HC_ERR_ARG, "cfl must be positive");
  if (cfg->law != HC_LAW_EULER && cfg->law != HC_LAW_SCALAR) return fail(HC_ERR_ARG, "unknown law");
  if (cfg->basis != HC_BASIS_PRIMITIVE && cfg->basis != HC_BASIS_CONSERVED) return fail(HC_ERR_ARG, "unknown basis");
  if (cfg->law == HC_LAW_SCALAR) {
    if (cfg->basis != HC_BASIS_PRIMITIVE)
      return fail(HC_ERR_UNSUPPORTED, "the scalar advection law has one basis (pass HC_BASIS_PRIMITIVE)");
    if (cfg->flux != HC_FLUX_RUSANOV && cfg->flux != HC_FLUX_CENTRAL)
      return fail(HC_ERR_UNSUPPORTED, "the scalar advection law uses the Rusanov or central flux");
    if (cfg->precision == HC_FP64_DF) return fail(HC_ERR_UNSUPPORTED, "the scalar advection law runs in FP64 or FP32");
  }
  hc_ctx* c = new hc_ctx();
  c->cfg = *cfg;
  c->scalar = cfg->law == HC_LAW_SCALAR;
  c->nv = c->scalar ? 3 : 4;
  c->fp32 = cfg->precision == HC_FP32;
  c->df = cfg->precision == HC_FP64_DF;
  // measured on the 512 x 1024 O-grid (Roe, van Albada): FP64 16x16 cells on 128 threads
  // 2.9% faster than on 256 and 4.4% faster than 8x32 (four CTAs per SM instead of two
  // overlap one another's load and barrier phases; the 544 faces fill whole warps), FP32
  // 8x32 (3.6% faster than 16x16)
  c->tile = c->fp32 ? TILE_8x32 : TILE_16x16_H;
  c->rsz = c->fp32 ? sizeof(float) : sizeof(double);
  cudaError_t e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    if (c->scalar) e = c->fp32 ? prepare_scalar_stage<float>() : prepare_scalar_stage<double>();
    else e = c->fp32 ? prepare<float>(cfg->flux) : prepare<double>(cfg->flux);
  }
  if (e == cudaSuccess) e = cudaMalloc(&c->info, sizeof(StepInfo));
  if (e == cudaSuccess) e = cudaMemset(c->info, 0, sizeof(StepInfo));
  if (e != cudaSuccess) {
    if (c->own) cudaStreamDestroy(c->own);
    if (c->info) cudaFree(c->info);
    delete c;
    return fail(HC_ERR_CUDA, std::string("context creation: ") + cudaGetErrorString(e));
  }
  c->stream = c->own;
  *out = c;
  return HC_OK;
}

int hc_context_destroy(hc_ctx* c) {
  if (!c) return HC_OK;
  cudaStreamSynchronize(c->stream);
  c->drop_adj_tape();
  free_buffers(c);
  if (c->own) cudaStreamDestroy(c->own);
  delete c;
  return HC_OK;
}

int hc_set_stream(hc_ctx* c, void* stream) {
  if (int st = check_ctx(c)) return st;
  HC_CUDA(cudaStreamSynchronize(c->stream));
  c->stream = (cudaStream_t)stream;
  return HC_OK;
}

int hc_get_stream(hc_ctx* c, void** stream) {
  if (int st = check_ctx(c)) return st;
  if (!stream) return fail(HC_ERR_ARG, "null output");
  *stream = (void*)c->stream;
  return HC_OK;
}

int hc_mesh_upload(hc_ctx* c, int ni, int nj, const double* nodes_xy) {
  if (int st = check_ctx(c)) return st;
  if (!nodes_xy) return fail(HC_ERR_ARG, "null nodes");
  if (ni < 3 || nj < 3) return fail(HC_ERR_ARG, "mesh needs at least 3 cells in each direction");
  if (size_t(ni + 1) * size_t(nj + 1) > (size_t(1) << 28)) return fail(HC_ERR_ARG, "mesh too large");
  HC_CUDA(cudaStreamSynchronize(c->stream));
  c->drop_adj_tape();
  free_buffers(c);
  c->oned = false;
  c->nv = c->scalar ? 3 : 4;
  c->hx.clear();
  c->ni = ni; c->nj = nj;
  const size_t n = c->ncell();
  const size_t nfi = size_t(ni + 1) * nj, nfj = size_t(ni) * (nj + 1);
  const size_t nn = size_t(ni + 1) * (nj + 1) * 2;
  HC_CUDA(cudaMalloc(&c->info, sizeof(StepInfo)));
  HC_CUDA(cudaMemsetAsync(c->info, 0, sizeof(StepInfo), c->stream));
  HC_CUDA(cudaMalloc(&c->nodes, nn * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->cx, n * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->cy, n * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->xm, 3 * n * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->vol64, n * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->fi64, FREC * nfi * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->fj64, FREC * nfj * sizeof(double)));
  if (c->fp32) {
    HC_CUDA(cudaMalloc(&c->fi, FREC * nfi * sizeof(float)));
    HC_CUDA(cudaMalloc(&c->fj, FREC * nfj * sizeof(float)));
    HC_CUDA(cudaMalloc(&c->vol, n * sizeof(float)));
    HC_CUDA(cudaMalloc(&c->staging, 5 * n * sizeof(double)));
  } else {
    c->fi = c->fi64; c->fj = c->fj64; c->vol = c->vol64;
  }
  if (c->df) {
    HC_CUDA(cudaMalloc(&c->fic, FREC * nfi * sizeof(df64)));
    HC_CUDA(cudaMalloc(&c->fjc, FREC * nfj * sizeof(df64)));
  }
  for (int k = 0; k < 3; ++k) HC_CUDA(cudaMalloc(&c->q[k], 4 * n * c->rsz));
  for (int k = 0; k < 4; ++k) HC_CUDA(cudaMalloc(&c->res[k], 5 * n * c->rsz));
  for (int s = 0; s < 4; ++s) HC_CUDA(cudaMalloc(&c->gref[s], 4 * size_t(c->nface(s)) * c->rsz));
  HC_CUDA(cudaMemcpyAsync(c->nodes, nodes_xy, nn * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  HC_CUDA(cudaStreamSynchronize(c->stream));
  c->have_mesh = true;
  c->have_state = false;
  c->geom_dirty = true;
  for (int s = 0; s < 4; ++s)
    if (!c->href[s].empty() && c->href[s].size() != size_t(4) * c->nface(s)) c->href[s].clear();
  return HC_OK;
}

int hc_mesh_upload_1d(hc_ctx* c, int nc, const double* nodes_x) {
  if (int st = check_ctx(c)) return st;
  if (!nodes_x) return fail(HC_ERR_ARG, "null nodes");
  if (nc < 3 || nc > (1 << 28)) return fail(HC_ERR_ARG, "a 1D mesh needs 3 to 2^28 cells");
  if (c->scalar) return fail(HC_ERR_UNSUPPORTED, "the 1D path covers the Euler law");
  if (c->df || c->cfg.basis != HC_BASIS_PRIMITIVE)
    return fail(HC_ERR_UNSUPPORTED, "the 1D path runs in FP64 or FP32 in the primitive basis");
  for (int i = 0; i < nc; ++i)
    if (!(nodes_x[i + 1] > nodes_x[i])) return fail(HC_ERR_ARG, "1D nodes must increase");
  HC_CUDA(cudaStreamSynchronize(c->stream));
  c->drop_adj_tape();
  free_buffers(c);
  c->oned = true;
  c->nv = 3;
  c->ni = nc; c->nj = 1;
  c->hx.assign(nodes_x, nodes_x + nc + 1);
  const size_t n = size_t(nc), nf = size_t(nc) + 1;
  HC_CUDA(cudaMalloc(&c->info, sizeof(StepInfo)));
  HC_CUDA(cudaMemsetAsync(c->info, 0, sizeof(StepInfo), c->stream));
  HC_CUDA(cudaMalloc(&c->vol64, n * sizeof(double)));
  HC_CUDA(cudaMalloc(&c->fi64, F1REC * nf * sizeof(double)));
  if (c->fp32) {
    HC_CUDA(cudaMalloc(&c->fi, F1REC * nf * sizeof(float)));
    HC_CUDA(cudaMalloc(&c->vol, n * sizeof(float)));
    HC_CUDA(cudaMalloc(&c->staging, 4 * n * sizeof(double)));
  } else {
    c->fi = c->fi64; c->vol = c->vol64;
  }
  for (int k = 0; k < 3; ++k) HC_CUDA(cudaMalloc(&c->q[k], 3 * n * c->rsz));
  for (int k = 0; k < 4; ++k) HC_CUDA(cudaMalloc(&c->res[k], 4 * n * c->rsz));
  for (int s = 0; s < 2; ++s) HC_CUDA(cudaMalloc(&c->gref[s], 3 * c->rsz));
  c->have_mesh = true;
  c->have_bcs = false;
  c->have_state = false;
  c->geom_dirty = true;
  for (int s = 0; s < 4; ++s) c->href[s].clear();
  return HC_OK;
}

int hc_set_species(hc_ctx* c, double gamma, double gas_constant, double minf) {
  if (int st = check_ctx(c)) return st;
  if (!(gamma > 1.0) || !(gas_constant > 0.0) || !(minf > 0.0)) return fail(HC_ERR_ARG, "invalid species");
  c->gamma = gamma; c->Rgas = gas_constant; c->minf = minf;
  return HC_OK;
}

int hc_set_low_mach(hc_ctx* c, int velocity_scaling, int pressure_scaling, double lref, double dt) {
  if (int st = check_ctx(c)) return st;
  auto ok = [](int k) { return k >= HC_SCALING_CONVECTIVE && k <= HC_SCALING_ADAPTIVE; };
  if (!ok(velocity_scaling) || !ok(pressure_scaling)) return fail(HC_ERR_ARG, "unknown low-Mach scaling");
  if (!(lref > 0.0) || !(dt > 0.0) || !std::isfinite(lref) || !std::isfinite(dt))
    return fail(HC_ERR_ARG, "lref and dt must be positive and finite");
  c->vscale = velocity_scaling; c->pscale = pressure_scaling; c->lref = lref; c->sdt = dt;
  return HC_OK;
}

int hc_set_time(hc_ctx* c, double t) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_mesh || !c->info) return fail(HC_ERR_ARG, "upload the mesh before setting the time");
  if (!std::isfinite(t)) return fail(HC_ERR_ARG, "the time must be finite");
  HC_CUDA(cudaMemcpyAsync(&c->info->t, &t, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  HC_CUDA(cudaStreamSynchronize(c->stream));  // t is a host local
  return HC_OK;
}

int hc_set_corrections(hc_ctx* c, unsigned mask) {
  if (int st = check_ctx(c)) return st;
  if (mask & ~unsigned(HC_FIX_ALL)) return fail(HC_ERR_ARG, "unknown correction bits");
  c->fixes = mask;
  return HC_OK;
}

int hc_set_staged_loads(hc_ctx* c, int on) {
  if (int st = check_ctx(c)) return st;
  c->staged_loads = on ? 1 : 0;
  return HC_OK;
}

int hc_inject_stalled_copy(hc_ctx* c, int on) {
  if (int st = check_ctx(c)) return st;
  c->stall_copy = on ? 1 : 0;
  return HC_OK;
}

int hc_set_adjoint_tapes(hc_ctx* c, int ntapes) {
  if (int st = check_ctx(c)) return st;
  if (ntapes < -1) return fail(HC_ERR_ARG, "stage tapes: -1 (one per snapshot and one more) or a count >= 0");
  c->adj_tapes = ntapes;
  return HC_OK;
}

int hc_set_tile(hc_ctx* c, int tile) {
  if (int st = check_ctx(c)) return st;
  if (tile < HC_TILE_8x32 || tile > HC_TILE_16x16_H) return fail(HC_ERR_ARG, "unknown tile shape");
  c->tile = tile;
  return HC_OK;
}

int hc_set_bcs(hc_ctx* c, const int bc_type[4], const double* const ref[4]) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_mesh) return fail(HC_ERR_ARG, "upload the mesh before the boundary conditions");
  if (!bc_type) return fail(HC_ERR_ARG, "null bc types");
  if (c->oned) {  // sides 0 (left) and 1 (right); 2 and 3 do not exist
    for (int s = 0; s < 2; ++s)
      if (bc_type[s] < HC_BC_PERIODIC || bc_type[s] > HC_BC_WALL) return fail(HC_ERR_ARG, "unknown bc type");
    if ((bc_type[0] == HC_BC_PERIODIC) != (bc_type[1] == HC_BC_PERIODIC))
      return fail(HC_ERR_ARG, "periodic sides must come in pairs (0,1)");
    for (int s = 0; s < 4; ++s) {
      c->bc[s] = s < 2 ? bc_type[s] : HC_BC_PERIODIC;
      c->href[s].clear();
      if (s < 2 && bc_type[s] != HC_BC_PERIODIC && bc_type[s] != HC_BC_WALL) {
        if (!ref || !ref[s]) return fail(HC_ERR_ARG, "side " + std::to_string(s) + " needs reference values");
        c->href[s].assign(ref[s], ref[s] + 3);
      }
    }
    c->have_bcs = true;
    c->geom_dirty = true;
    return HC_OK;
  }
  for (int s = 0; s < 4; ++s) {
    if (bc_type[s] < HC_BC_PERIODIC || bc_type[s] > HC_BC_WALL) return fail(HC_ERR_ARG, "unknown bc type");
    if (c->scalar && (bc_type[s] == HC_BC_ENTROPY || bc_type[s] == HC_BC_WALL))
      return fail(HC_ERR_UNSUPPORTED, "the scalar advection law has periodic, fixed and Riemann boundaries");
  }
  if ((bc_type[0] == HC_BC_PERIODIC) != (bc_type[1] == HC_BC_PERIODIC) ||
      (bc_type[2] == HC_BC_PERIODIC) != (bc_type[3] == HC_BC_PERIODIC))
    return fail(HC_ERR_ARG, "periodic sides must come in pairs (0,1) and (2,3)");
  for (int s = 0; s < 4; ++s) {
    c->bc[s] = bc_type[s];
    c->href[s].clear();
    const bool needs = bc_type[s] != HC_BC_PERIODIC && bc_type[s] != HC_BC_WALL;
    if (needs) {
      if (!ref || !ref[s]) return fail(HC_ERR_ARG, "side " + std::to_string(s) + " needs reference values");
      c->href[s].assign(ref[s], ref[s] + size_t(c->nv) * c->nface(s));
    }
  }
  c->have_bcs = true;
  c->geom_dirty = true;
  return HC_OK;
}

int hc_state_upload(hc_ctx* c, const double* prim) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_mesh) return fail(HC_ERR_ARG, "upload the mesh first");
  if (!prim) return fail(HC_ERR_ARG, "null state");
  const size_t m = size_t(c->nv) * c->ncell();
  if (c->fp32) {
    HC_CUDA(cudaMemcpyAsync(c->staging, prim, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    d2r_kernel<float><<<1024, 256, 0, c->stream>>>(c->staging, (float*)c->q[0], m);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
  } else {
    HC_CUDA(cudaMemcpyAsync(c->q[0], prim, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));
  c->have_state = true;
  return HC_OK;
}

int hc_state_download(hc_ctx* c, double* prim) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_state) return fail(HC_ERR_ARG, "no state");
  if (!prim) return fail(HC_ERR_ARG, "null output");
  const size_t m = size_t(c->nv) * c->ncell();
  if (c->fp32) {
    r2d_kernel<float><<<1024, 256, 0, c->stream>>>((const float*)c->q[0], c->staging, m);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
    HC_CUDA(cudaMemcpyAsync(prim, c->staging, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  } else {
    HC_CUDA(cudaMemcpyAsync(prim, c->q[0], m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));
  return HC_OK;
}

int hc_state_upload_device(hc_ctx* c, const void* prim) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_mesh || !prim) return fail(HC_ERR_ARG, "mesh and a state pointer are required");
  HC_CUDA(cudaMemcpyAsync(c->q[0], prim, size_t(c->nv) * c->ncell() * c->rsz, cudaMemcpyDeviceToDevice, c->stream));
  c->have_state = true;
  return HC_OK;
}

int hc_state_download_device(hc_ctx* c, void* prim) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_state || !prim) return fail(HC_ERR_ARG, "no state or null output");
  HC_CUDA(cudaMemcpyAsync(prim, c->q[0], size_t(c->nv) * c->ncell() * c->rsz, cudaMemcpyDeviceToDevice, c->stream));
  return HC_OK;
}

int hc_residual(hc_ctx* c, double* out5) {
  if (int st = check_ctx(c)) return st;
  if (int st = ensure_ready(c)) return st;
  if (!out5) return fail(HC_ERR_ARG, "null output");
  const int st = c->fp32 ? run_residual<float>(c) : run_residual<double>(c);
  if (st != HC_OK) return st;
  const size_t m = size_t(c->nv + 1) * c->ncell();
  if (c->fp32) {
    r2d_kernel<float><<<1024, 256, 0, c->stream>>>((const float*)c->res[0], c->staging, m);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
    HC_CUDA(cudaMemcpyAsync(out5, c->staging, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  } else {
    HC_CUDA(cudaMemcpyAsync(out5, c->res[0], m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  HC_CUDA(cudaStreamSynchronize(c->stream));
  return HC_OK;
}

int hc_face_signatures(hc_ctx* c, unsigned long long* sig_i, unsigned long long* sig_j, double* arg_i,
                       double* arg_j) {
  if (int st = check_ctx(c)) return st;
  if (!sig_i || !sig_j) return fail(HC_ERR_ARG, "null output");
  if (c->scalar || c->oned) return fail(HC_ERR_UNSUPPORTED, "branch signatures cover the 2D Euler path");
  if (int st = ensure_ready(c)) return st;
  return c->fp32 ? run_signatures<float>(c, sig_i, sig_j, arg_i, arg_j)
                  : run_signatures<double>(c, sig_i, sig_j, arg_i, arg_j);
}

int hc_dual_time_run(hc_ctx* c, const hc_dual_time_controls* ctl, hc_dual_time_stats* stats) {
  if (int st = check_ctx(c)) return st;
  if (!ctl || ctl->outer_steps < 0 || ctl->inner_max < 1 || ctl->check_every < 1 || ctl->inner_drop < 0.0 ||
      (ctl->scheme != HC_BDF1 && ctl->scheme != HC_BDF2 && ctl->scheme != HC_TRAPEZIUM) ||
      (!(ctl->dt > 0.0) && !(ctl->cfl_outer > 0.0)))
    return fail(HC_ERR_ARG, "invalid dual-time controls");
  if (c->scalar || c->oned) return fail(HC_ERR_UNSUPPORTED, "dual time covers the 2D Euler path");
  if (int st = ensure_ready(c)) return st;
  return c->fp32 ? dual_time_run<float>(c, ctl, stats) : dual_time_run<double>(c, ctl, stats);
}

int hc_step_async(hc_ctx* c, int nsteps) {
  if (int st = check_ctx(c)) return st;
  if (nsteps < 0) return fail(HC_ERR_ARG, "negative step count");
  if (int st = ensure_ready(c)) return st;
  // clear the device status of earlier calls (status and bad_cell are adjacent ints)
  HC_CUDA(cudaMemsetAsync(&c->info->status, 0, 2 * sizeof(int), c->stream));
  for (int k = 0; k < nsteps; ++k) {
    const int st = c->fp32 ? run_step<float>(c) : run_step<double>(c);
    if (st != HC_OK) return st;
  }
  return HC_OK;
}

int hc_step_host(hc_ctx* c, int nsteps, const double* state_in, double* state_out, hc_step_stats* stats) {
  if (int st = check_ctx(c)) return st;
  if (!c->have_mesh) return fail(HC_ERR_ARG, "upload the mesh first");
  if (!state_in || !state_out) return fail(HC_ERR_ARG, "null state");
  const size_t m = size_t(c->nv) * c->ncell();
  // upload, steps and download in stream order; read_stats waits once for all of them
  if (c->fp32) {
    HC_CUDA(cudaMemcpyAsync(c->staging, state_in, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    d2r_kernel<float><<<1024, 256, 0, c->stream>>>(c->staging, (float*)c->q[0], m);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
  } else {
    HC_CUDA(cudaMemcpyAsync(c->q[0], state_in, m * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  c->have_state = true;
  if (int st = hc_step_async(c, nsteps)) return st;
  if (c->fp32) {
    r2d_kernel<float><<<1024, 256, 0, c->stream>>>((const float*)c->q[0], c->staging, m);
    HC_CUDA(cudaGetLastError());
    c->launches += 1;
    HC_CUDA(cudaMemcpyAsync(state_out, c->staging, m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  } else {
    HC_CUDA(cudaMemcpyAsync(state_out, c->q[0], m * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  }
  return read_stats(c, stats);
}

int hc_sync(hc_ctx* c, hc_step_stats* stats) {
  if (int st = check_ctx(c)) return st;
  return read_stats(c, stats);
}

int hc_step(hc_ctx* c, int nsteps, hc_step_stats* stats) {
  const int st = hc_step_async(c, nsteps);
  if (st != HC_OK) return st;
  return hc_sync(c, stats);
}

// Steady driver: the convergence loop SteadyTimeControls describes (controls.h:31-48)
int hc_steady_run(hc_ctx* c, const hc_steady_controls* ctl, double* history, long long history_len,
                  hc_steady_stats* out) {
  if (int st = check_ctx(c)) return st;
  if (!ctl || ctl->max_steps < 1 || ctl->check_every < 1 || !(ctl->residual_drop > 0.0))
    return fail(HC_ERR_ARG, "invalid steady controls");
  if (ctl->use_residual_smoothing) {
    if (!c->oned) return fail(HC_ERR_UNSUPPORTED, "residual smoothing exists only in the reference's 1D path");
    if (!(ctl->smoothing_factor >= 1.0) || !std::isfinite(ctl->smoothing_factor))
      return fail(HC_ERR_ARG, "the smoothing factor must be finite and at least 1");
    if (c->df) return fail(HC_ERR_UNSUPPORTED, "residual smoothing runs in FP64 or FP32");
  }
  // the smoothed stage loop for the duration of the run
  struct Smooth {
    hc_ctx* c;
    ~Smooth() { c->smooth_alpha = 0.0; }
  } smooth_scope{c};
  c->smooth_alpha = ctl->use_residual_smoothing ? ctl->smoothing_factor : 0.0;
  hc_steady_stats res{};
  auto record = [&](double r) {
    if (history && res.history_len < history_len) history[res.history_len] = r;
    if (history && res.history_len < history_len) ++res.history_len;
  };
  hc_step_stats s{};
  int st = hc_step(c, 1, &s);
  if (st == HC_OK) {
    res.res0 = res.res = s.resnorm;
    res.steps = 1;
    record(s.resnorm);
    res.converged = !(res.res0 > 0.0);
    while (!res.converged && res.steps < ctl->max_steps) {
      const int n = int(std::min<long long>(ctl->check_every, ctl->max_steps - res.steps));
      st = hc_step(c, n, &s);
      if (st != HC_OK) break;
      res.steps += n;
      res.res = s.resnorm;
      record(s.resnorm);
      res.converged = res.res <= ctl->residual_drop * res.res0;
    }
  }
  if (out) *out = res;
  return st;
}

// Residual smoothing of the legacy 1D path on device planes (hc_smooth.cu)
int hc_smooth_1d(hc_ctx* c, int kind, const double* r0_device, double* r1_device, long long n, int nplanes,
                 double alpha, int ends) {
  if (int st = check_ctx(c)) return st;
  if ((kind != HC_SMOOTH_IMPLICIT && kind != HC_SMOOTH_EXPLICIT) || !r0_device || !r1_device || n < 2 ||
      nplanes < 1 || !(alpha > 0.0) || !std::isfinite(alpha))
    return fail(HC_ERR_ARG, "invalid smoothing arguments");
  const size_t total = size_t(n) * nplanes;
  double* scratch = nullptr;
  if (kind == HC_SMOOTH_IMPLICIT) {
    // each plane's CTA reads r0 only before its last barrier and writes r1 after it,
    // so in-place smoothing is safe; the sweeps need two lines of scratch
    HC_CUDA(cudaMallocAsync((void**)&scratch, 2 * total * sizeof(double), c->stream));
    const cudaError_t e = launch_smooth_1d<double>(kind, r0_device, r1_device, scratch, scratch + total, n, nplanes,
                                                   n, alpha, ends, c->stream);
    cudaFreeAsync(scratch, c->stream);
    HC_CUDA(e);
    c->launches += 1;
    return HC_OK;
  }
  // explicit: every value reads its neighbours (and, on a periodic line, both ends),
  // which other threads and blocks would overwrite when r1 overlaps r0; smooth a
  // stream-ordered copy of r0 then
  const double* src = r0_device;
  const uintptr_t a0 = uintptr_t(r0_device), a1 = uintptr_t(r1_device), bytes = total * sizeof(double);
  if (a0 < a1 + bytes && a1 < a0 + bytes) {
    HC_CUDA(cudaMallocAsync((void**)&scratch, bytes, c->stream));
    const cudaError_t ec = cudaMemcpyAsync(scratch, r0_device, bytes, cudaMemcpyDeviceToDevice, c->stream);
    if (ec != cudaSuccess) {
      cudaFreeAsync(scratch, c->stream);
      HC_CUDA(ec);
    }
    src = scratch;
  }
  const cudaError_t e = launch_smooth_1d<double>(kind, src, r1_device, nullptr, nullptr, n, nplanes, n, alpha, ends,
                                                 c->stream);
  if (scratch) cudaFreeAsync(scratch, c->stream);
  HC_CUDA(e);
  c->launches += 1;
  return HC_OK;
}

// make_cylinder_mesh (mesh/generate/twoD.h:139-179) with geometric radial stretching
int hc_mesh_cylinder_nodes(int nr, int nth, double rc, double rb, double stretch, double* nodes) {
  if (nr < 1 || nth < 1 || !nodes || !(rb > rc) || !(stretch > 0)) return fail(HC_ERR_ARG, "invalid cylinder mesh");
  const double dr = (rb - rc) / nr;
  const double dth = (2. * M_PI) / nth;
  const double dr0 = (stretch == 1.0) ? dr : (rb - rc) * (stretch - 1.) / (std::pow(stretch, nr) - 1.);
  for (int i = 0; i <= nr; ++i) {
    const double r = (stretch == 1.0) ? rc + i * dr : rc + dr0 * (std::pow(stretch, i) - 1.) / (stretch - 1.);
    for (int j = 0; j <= nth; ++j) {
      const double th = j * dth;
      nodes[(size_t(i) * (nth + 1) + j) * 2 + 0] = r * cos(th);
      nodes[(size_t(i) * (nth + 1) + j) * 2 + 1] = r * sin(th);
    }
  }
  return HC_OK;
}

// make_linspace_mesh (mesh/generate/twoD.h:15-40)
int hc_mesh_linspace_nodes(int nx, int ny, double lox, double hix, double loy, double hiy, double* nodes) {
  if (nx < 1 || ny < 1 || !nodes) return fail(HC_ERR_ARG, "invalid linspace mesh");
  const double dx = (hix - lox) / nx, dy = (hiy - loy) / ny;
  for (int i = 0; i <= nx; ++i)
    for (int j = 0; j <= ny; ++j) {
      nodes[(size_t(i) * (ny + 1) + j) * 2 + 0] = lox + i * dx;
      nodes[(size_t(i) * (ny + 1) + j) * 2 + 1] = loy + j * dy;
    }
  return HC_OK;
}

}  // extern "C"
