// hc_adjoint_driver.cuh -- discrete adjoint of the RK time loop of one context with
// binomial checkpointing (Griewank & Walther, "Algorithm 799: revolve", ACM TOMS
// 26(1), 2000: with s snapshots and t forward repetitions, C(s+t, s) steps can
// be reversed), templated on the context's storage type R (double or float);
// per-step max rates, timesteps and the objective stay in FP64.  The timestep of
// every step is frozen at the value of the forward run (the max-rate history is
// recorded and replayed), so the gradient is that of the objective at fixed
// timesteps.
//
// Objectives: time-averaged wall force (drag) over steps 1..N, or a weighted
// L2 distance of the final state to a target.  Supported: Euler law (HC_FP64,
// HC_FP64_DF and HC_FP32 contexts; Roe or Rusanov flux reversed by hand, SLAU,
// AUSM+up and RoeUnprecWS by tangents (not double-float); periodic / fixed /
// inviscid-wall boundaries and, by tangents, Riemann / entropy far fields (not
// double-float)) and the scalar advection law (HC_FP64 and HC_FP32;
// Rusanov or central flux; periodic / fixed / Riemann boundaries; the L2 objective); limiters
// NoLimit1/2/3, van Albada, MinMod, van Leer; global timestep.  hc_adjoint.cu instantiates R = double and the C ABI,
// hc_adjoint_f32.cu R = float.
#pragma once

#include "hc_adjoint_kernels.cuh"
#include "hc_ctx.h"
#include "hc_scalar.cuh"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

namespace hc {
namespace adj {

// residual_adjoint's flux parameter for the fluxes reversed by tangents (the context's flux)
constexpr int FLUX_BY_TANGENT = -1;

// buffers and recomputation timing shared by the single-mesh and batched drivers
struct AdjCommon {
  std::vector<void*> allocs;
  std::vector<cudaEvent_t> adv_events;  // (start, end) pairs around checkpoint recomputation

  template <class T> int alloc(T** p, size_t count) {
    HC_CUDA(cudaMalloc((void**)p, std::max<size_t>(count, 1) * sizeof(T)));
    allocs.push_back(*p);
    return HC_OK;
  }
  ~AdjCommon() {
    for (void* p : allocs) cudaFree(p);
    for (cudaEvent_t e : adv_events) cudaEventDestroy(e);
  }
  // time of the recorded recomputation segments (call after the stream is idle)
  double recompute_ms() const {
    double t = 0;
    for (size_t k = 0; k + 1 < adv_events.size(); k += 2) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, adv_events[k], adv_events[k + 1]) == cudaSuccess) t += ms;
    }
    return t;
  }
};

// A stage tape: the start state and the stage states (sq[0..nst-1]) of one step, kept from
// the advance (or the forward sweep) that computed the step last before its reversal, so
// that the reversal needs no replay of the step.  Buffers move between sq and the tapes by
// pointer exchange, never by copy.
template <class R> struct StageTape {
  R* q[4] = {nullptr, nullptr, nullptr, nullptr};
  int step = -1;  // -1: free
};

template <class R> struct Adj : AdjCommon {
  hc_ctx* c = nullptr;
  int nst = 4;
  RKTab tab{};
  size_t n = 0;
  int nfi = 0, nfj = 0;
  R* sq[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};  // stage states; sq[nst] = step output
  R* rbar[4] = {nullptr, nullptr, nullptr, nullptr};
  R* qm = nullptr;
  R* qmbar = nullptr;
  R* ai = nullptr;
  R* aj = nullptr;
  R* lam = nullptr;
  R* qbs = nullptr;
  R* q0bar = nullptr;
  R* refbar[4] = {nullptr, nullptr, nullptr, nullptr};
  R* base = nullptr;
  R* snaps = nullptr;
  R* qnext = nullptr;  // the start state of the step reversed last (the output of the one reversed next)
  int nsnap = 0;
  std::vector<StageTape<R>> tapes;
  long long replays = 0;
  double* rates = nullptr;   // device, one max-rate per step
  R* wall = nullptr;    // per wall face partial forces
  double* jacc = nullptr;    // device accumulator of the objective
  R* target = nullptr;
  std::vector<double> hrates;
  hc_objective obj{};
  int nsteps = 0;
  int nv = 4;  // state variables: 4 Euler, 3 scalar advection
  long long fwd_steps = 0, adj_steps = 0, launches = 0;
  size_t state_values() const { return size_t(nv) * n; }  // one stored state
  cudaStream_t s() const { return c->stream; }
};

template <class R> AdjArgs<R> adj_args(Adj<R>& A) {
  hc_ctx* c = A.c;
  AdjArgs<R> a{};
  a.ni = c->ni; a.nj = c->nj;
  for (int k = 0; k < 4; ++k) a.bc[k] = c->bc[k];
  a.gas = with_fixes(make_gas<R>(c->gamma, c->Rgas, c->minf), c->fixes);
  a.limiter = c->cfg.limiter;
  a.fi = (const R*)c->fi; a.fj = (const R*)c->fj;
  for (int k = 0; k < 4; ++k) { a.gref[k] = (const R*)c->gref[k]; a.refbar[k] = A.refbar[k]; }
  a.qm = A.qm; a.qmbar = A.qmbar; a.ai = A.ai; a.aj = A.aj;
  return a;
}

inline unsigned blocks(size_t n) { return unsigned((n + 255) / 256); }
// the face-adjoint kernel holds ~180 registers a thread: small blocks let more
// warps share an SM than one 256-thread block would
constexpr int kFaceThreads = 64;
inline unsigned face_blocks(size_t n) { return unsigned((n + kFaceThreads - 1) / kFaceThreads); }

// one forward step from sq[0] to sq[nst]; record (rec=true) or replay the max rate of step
// `step`; nstages < nst runs only the first nstages stages (sq[1..nstages])
template <class R> int forward_step(Adj<R>& A, int step, bool rec, int nstages = -1) {
  hc_ctx* c = A.c;
  const StageFn<R> euler_fn = stage_fn<R>(c->cfg.flux);
  auto fn = [c, euler_fn](const StageArgs<R>& a, int tile, cudaStream_t st) -> cudaError_t {
    return c->scalar ? launch_scalar_stage<R>(a, c->cfg.flux, tile, st) : euler_fn(a, tile, st);
  };
  const int ns = nstages < 0 ? A.nst : nstages;
  for (int s = 0; s < ns; ++s) {
    StageArgs<R> a = base_args<R>(c);
    a.q = A.sq[s];
    a.q0 = A.sq[0];
    a.stage = s;
    a.beta = R(A.tab.beta[s]);
    for (int k = 0; k <= s; ++k) a.alpha[k] = R(A.tab.alpha[s][k]);
    for (int k = 0; k < s; ++k) a.res_prev[k] = (const R*)c->res[k];
    a.res_out = (s < A.nst - 1) ? (R*)c->res[s] : nullptr;
    a.norm_stage0 = 0;
    if (s == 0) {
      a.res_out = (R*)c->res[0];
      if (rec) {
        HC_CUDA(cudaMemsetAsync(&c->info->maxrate, 0, sizeof(unsigned long long), A.s()));
        a.mode = MODE_RES_MAXRATE;
        HC_CUDA(fn(a, c->tile, A.s()));
        HC_CUDA(cudaMemcpyAsync(A.rates + step, &c->info->maxrate, sizeof(double), cudaMemcpyDeviceToDevice, A.s()));
      } else {
        HC_CUDA(cudaMemcpyAsync(&c->info->maxrate, A.rates + step, sizeof(double), cudaMemcpyDeviceToDevice, A.s()));
        a.mode = MODE_RESIDUAL;
        HC_CUDA(fn(a, c->tile, A.s()));
      }
      if (c->scalar)
        scalar_update0_kernel<R><<<std::min<unsigned>(blocks(A.n), 152 * 16), 256, 0, A.s()>>>(
            c->ni, c->nj, A.sq[0], (const R*)c->res[0], (const R*)c->vol, R(A.tab.alpha[0][0]), R(A.tab.beta[0]),
            c->cfg.cfl, c->info, A.sq[1], 0);
      else
        update0_kernel<R><<<std::min<unsigned>(blocks(A.n), 152 * 16), 256, 0, A.s()>>>(
            c->ni, c->nj, a.gas, A.sq[0], (const R*)c->res[0], (const R*)c->vol, R(A.tab.alpha[0][0]),
            R(A.tab.beta[0]), c->cfg.cfl, c->info, A.sq[1], 0, c->cfg.basis, 0.0);
      HC_CUDA(cudaGetLastError());
      A.launches += 2;
    } else {
      a.mode = MODE_FUSED_GLOBAL;
      a.q_out = A.sq[s + 1];
      HC_CUDA(fn(a, c->tile, A.s()));
      A.launches += 1;
    }
  }
  A.fwd_steps += 1;
  return HC_OK;
}

// sq[nst] -> sq[0] (the step output becomes the next step's start)
template <class AD> void swap_out(AD& A) { std::swap(A.sq[0], A.sq[A.nst]); }

// ---- stage tapes (shared by the single-mesh and batched drivers)
template <class AD> int tape_of(const AD& A, int step) {
  for (size_t k = 0; k < A.tapes.size(); ++k)
    if (A.tapes[k].step == step) return int(k);
  return -1;
}
// after forward_step(A, step) and before swap_out: keep sq[0..nst-1] (q_step and its stage
// states) in a free tape, if there is one
template <class AD> void keep_stages(AD& A, int step) {
  const int k = tape_of(A, -1);
  if (k < 0) return;
  for (int j = 0; j < A.nst; ++j) std::swap(A.sq[j], A.tapes[k].q[j]);
  A.tapes[k].step = step;
}
// sq[0..nst-1] = q_step and its stage states: from the step's tape (released), or replayed
// from q_step in sq[0]
template <class AD> int stage_states(AD& A, int step) {
  const int k = tape_of(A, step);
  if (k < 0) {
    A.replays += 1;
    return forward_step(A, step, false, A.nst - 1);
  }
  for (int j = 0; j < A.nst; ++j) std::swap(A.sq[j], A.tapes[k].q[j]);
  A.tapes[k].step = -1;
  return HC_OK;
}
// ntapes < 0: snapshots + 1 tapes (none replayed), as many of them as fit in half the
// free device memory
template <class AD> int alloc_tapes(AD& A, int ntapes, int snapshots) {
  if (ntapes < 0) {
    size_t free_b = 0, total_b = 0;
    HC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t per = size_t(A.nst) * A.state_values() * sizeof(*A.sq[0]);
    ntapes = int(std::min<size_t>(size_t(snapshots) + 1, free_b / 2 / std::max<size_t>(per, 1)));
  }
  ntapes = std::min(ntapes, A.nsteps);
  A.tapes.assign(size_t(std::max(ntapes, 0)), {});
  for (auto& t : A.tapes)
    for (int j = 0; j < A.nst; ++j)
      if (int st = A.alloc(&t.q[j], A.state_values())) return st;
  return HC_OK;
}

// acc[0] += sum of v[0..m) by one 256-thread block in a fixed order (deterministic)
template <class R> __device__ __forceinline__ void block_sum_into(const R* __restrict__ v, int m, double* acc) {
  __shared__ double part[256];
  double s = 0;
  for (int k = threadIdx.x; k < m; k += 256) s += double(v[k]);
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) acc[0] += part[0];
}
template <class R> __global__ void sum_into_kernel(const R* __restrict__ v, int m, double* __restrict__ acc) {
  block_sum_into(v, m, acc);
}

// J += scale * wall force of the state q (drag objective)
template <class R> int add_drag(Adj<R>& A, const R* q, double scale) {
  AdjArgs<R> a = adj_args(A);
  a.q = q;
  a.obj_scale = R(scale);
  a.obj_dirx = R(A.obj.dir[0]);
  a.obj_diry = R(A.obj.dir[1]);
  adj_qm_kernel<R><<<blocks(A.n), 256, 0, A.s()>>>(a, A.qm);
  A.launches += 1;
  for (int side = 0; side < 4; ++side) {
    if (A.c->bc[side] != HC_BC_WALL) continue;
    const int m = A.c->nface(side);
    wall_force_kernel<R><<<blocks(m), 256, 0, A.s()>>>(a, A.qm, side, A.wall);
    sum_into_kernel<R><<<1, 256, 0, A.s()>>>(A.wall, m, A.jacc);
    A.launches += 2;
  }
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

// cell c of the L2 objective: part[c] = sum_v w_v (q - t)^2, or (mode_grad) its
// gradient 2 w_v (q - t) into lam
template <class R>
__device__ __forceinline__ void l2_cell(const R* q, const R* t, size_t n, double w0, double w1, double w2, double w3,
                                        R* part, int mode_grad, R* lam, size_t c, int nv = 4) {
  if (c >= n) return;
  const double w[4] = {w0, w1, w2, w3};
  double s = 0;
  for (int v = 0; v < nv; ++v) {
    const double d = double(q[v * n + c]) - double(t[v * n + c]);
    s += w[v] * d * d;
    if (mode_grad) lam[v * n + c] = R(2.0 * w[v] * d);
  }
  if (part) part[c] = R(s);
}
template <class R>
__global__ void l2_kernel(const R* q, const R* t, size_t n, double w0, double w1, double w2, double w3, R* part,
                          int mode_grad, R* lam, int nv = 4) {
  l2_cell(q, t, n, w0, w1, w2, w3, part, mode_grad, lam, blockIdx.x * size_t(blockDim.x) + threadIdx.x, nv);
}

// scalar-law residual adjoint: qbar_out = (dRes/dq at q)^T rbar (+ qbar_add)
template <class R, int FK>
int residual_adjoint_scalar(Adj<R>& A, const R* q, const R* rbar, const R* qbar_add, R* qbar_out) {
  AdjArgs<R> a = adj_args(A);
  a.q = q;
  a.rbar = rbar;
  a.qbar = qbar_out;
  a.qbar_add = qbar_add;
  adj_qm_kernel<R, 3><<<blocks(A.n), 256, 0, A.s()>>>(a, A.qm);
  adj_face_scalar_kernel<R, FK><<<blocks(A.nfi), 256, 0, A.s()>>>(a, 0);
  adj_face_scalar_kernel<R, FK><<<blocks(A.nfj), 256, 0, A.s()>>>(a, 1);
  adj_qmbar_kernel<R, 3><<<blocks(A.n), 256, 0, A.s()>>>(a);
  adj_gather_kernel<R, 3><<<blocks(A.n), 256, 0, A.s()>>>(a);
  A.launches += 5;
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

template <class R> int res_adj_scalar(Adj<R>& A, const R* q, const R* rbar, const R* add, R* out) {
  if (A.c->cfg.flux == HC_FLUX_CENTRAL) return residual_adjoint_scalar<R, FLUX_CENTRAL>(A, q, rbar, add, out);
  return residual_adjoint_scalar<R, FLUX_RUSANOV>(A, q, rbar, add, out);
}

// Euler face pass (pass 1) of the stage state a.q with residual adjoint a.rbar: both
// directions in one launch
template <class R> int euler_faces(Adj<R>& A, const AdjArgs<R>& a) {
  const int nbi = int(face_blocks(A.nfi));
  const unsigned nb = face_blocks(A.nfi) + face_blocks(A.nfj);
  const int flux = A.c->cfg.flux;
  if (flux_by_tangent(flux)) {
    HC_CUDA(launch_adj_face_tangent<R>(flux, a, nbi, nb, kFaceThreads, A.s()));
  } else if (flux == HC_FLUX_ROE) {
    if constexpr (std::is_same<R, double>::value) {
      if (A.c->df) adj_face_kernel<double, FLUX_ROE, df64><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
      else adj_face_kernel<double, FLUX_ROE><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
    } else {
      adj_face_kernel<R, FLUX_ROE><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
    }
  } else {
    if constexpr (std::is_same<R, double>::value) {
      if (A.c->df) adj_face_kernel<double, FLUX_RUSANOV, df64><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
      else adj_face_kernel<double, FLUX_RUSANOV><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
    } else {
      adj_face_kernel<R, FLUX_RUSANOV><<<nb, kFaceThreads, 0, A.s()>>>(a, nbi);
    }
  }
  A.launches += 1;
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

// the arguments of the drag objective's adjoint (J scaled by scale)
template <class R> void drag_args(Adj<R>& A, AdjArgs<R>& a, double scale) {
  a.obj_scale = R(scale);
  a.obj_dirx = R(A.obj.dir[0]);
  a.obj_diry = R(A.obj.dir[1]);
}

template <class R> double step_dt(const Adj<R>& A, int step) {
  const double rate = std::fmax(DBL_MIN, A.hrates[step]);
  return A.c->cfg.cfl / rate;
}

// lam holds the adjoint of q_{step+1}; sq[0] holds q_step.  On return lam holds
// the adjoint of q_step (objective terms of q_step included).
// Euler: per stage s (last first) three launches -- faces of stage s, its qmetric
// adjoint, and the fused cell pass (gather of stage s, update reverse of stage s-1,
// qmetric of stage s-1's state; at s = 0 the gather with the update adjoints of q_step
// and the drag objective into lam) -- after one cell pass that reverses the last
// stage's update.
template <class R> int adjoint_step(Adj<R>& A, int step) {
  // the step's stage states from its tape, or a replay of its stages but the last (its
  // output q_{step+1} is the start state of the step reversed before this one, kept in qnext)
  if (int st = stage_states(A, step)) return st;
  const size_t bytes4 = A.state_values() * sizeof(R);
  // q_{step+1} into sq[nst] by exchange with qnext; qnext takes q_step (sq[0]) the same way
  // when the step is done
  std::swap(A.sq[A.nst], A.qnext);
  const double dt = step_dt(A, step);
  const Gas<R> g = with_fixes(make_gas<R>(A.c->gamma, A.c->Rgas, A.c->minf), A.c->fixes);
  if (A.c->scalar) {
    for (int k = 0; k < A.nst; ++k) HC_CUDA(cudaMemsetAsync(A.rbar[k], 0, bytes4, A.s()));
    HC_CUDA(cudaMemsetAsync(A.q0bar, 0, bytes4, A.s()));
    for (int s = A.nst - 1; s >= 0; --s) {
      const R* qbar_out = (s == A.nst - 1) ? A.lam : A.qbs;
      R al[4] = {R(0), R(0), R(0), R(0)};
      for (int k = 0; k <= s; ++k) al[k] = R(A.tab.alpha[s][k]);
      adj_update_lin_kernel<R, 3><<<blocks(A.n), 256, 0, A.s()>>>(
          int(A.n), (const R*)A.c->vol, qbar_out, A.q0bar, A.rbar[0], A.rbar[1], A.rbar[2], A.rbar[3], al[0],
          al[1], al[2], al[3], s, R(A.tab.beta[s] * dt));
      A.launches += 1;
      HC_CUDA(cudaGetLastError());
      if (int st = res_adj_scalar<R>(A, A.sq[s], A.rbar[s], s == 0 ? A.q0bar : nullptr, A.qbs)) return st;
    }
    HC_CUDA(cudaMemcpyAsync(A.lam, A.qbs, bytes4, cudaMemcpyDeviceToDevice, A.s()));
    std::swap(A.qnext, A.sq[0]);
    A.adj_steps += 1;
    return HC_OK;
  }
  AdjArgs<R> a = adj_args(A);
  drag_args(A, a, A.obj.scale / A.nsteps);
  const unsigned cb = blocks(A.n);
  // update reverse of stage s with the state adjoint qb of its output
  auto update = [&](AdjCellArgs<R>& u, int s) {
    u.update = 1;
    u.g = g;
    u.q_out = A.sq[s + 1];
    u.q0 = A.sq[0];
    u.vol = (const R*)A.c->vol;
    u.q0bar = A.q0bar;
    for (int k = 0; k < 4; ++k) {
      u.rbar[k] = A.rbar[k];
      u.alpha[k] = k <= s ? R(A.tab.alpha[s][k]) : R(0);
    }
    u.stage = s;
    u.dts = R(A.tab.beta[s] * dt);
  };
  {
    AdjCellArgs<R> u{};
    u.qbar_in = A.lam;
    update(u, A.nst - 1);
    u.first = 1;  // q0bar and every rbar_k written, not accumulated: no zeroing
    u.qm_q = A.sq[A.nst - 1];
    adj_cell_kernel<R><<<cb, 256, 0, A.s()>>>(a, u);
    A.launches += 1;
  }
  for (int s = A.nst - 1; s >= 0; --s) {
    a.q = A.sq[s];
    a.rbar = A.rbar[s];
    a.qbar_add = s == 0 ? A.q0bar : nullptr;
    if (int st = euler_faces(A, a)) return st;
    adj_qmbar_kernel<R><<<cb, 256, 0, A.s()>>>(a);
    AdjCellArgs<R> u{};
    u.gather = 1;
    if (s > 0) {
      update(u, s - 1);
      u.qm_q = A.sq[s - 1];
    } else {
      u.qbar_out = A.lam;
      u.drag = A.obj.kind == HC_OBJ_DRAG && step >= 1;
    }
    adj_cell_kernel<R><<<cb, 256, 0, A.s()>>>(a, u);
    A.launches += 2;
    HC_CUDA(cudaGetLastError());
  }
  std::swap(A.qnext, A.sq[0]);
  A.adj_steps += 1;
  return HC_OK;
}

// ---- binomial checkpointing
// Reversing n steps whose start state is restorable, with s free snapshot slots,
// costs T(n, s) recomputed forward steps under the best schedule:
//   T(1, s) = 0,  T(n, 0) = n(n-1)/2 (every state re-advanced from the start),
//   T(n, s) = min_k [k + T(n-k, s-1) + T(k, s)]
// (advance k steps and store, reverse the right part with one slot fewer, then
// the left part with the slot freed).  The first forward sweep passes every
// state, so it stores the checkpoints of the schedule's first descent (the
// right-most path) as it goes; for that path the advance is free:
//   F(n, s) = min_k [F(n-k, s-1) + T(k, s)],  F(n, 0) = T(n, 0).
// Both tables and their minimising splits are computed by dynamic programming
// (O(n^2 s)); beyond kDpLimit operations the split falls back to the binomial
// rule k = n - C(s-1+t, s-1), t the smallest with C(s+t, s) >= n.
constexpr double kDpLimit = 4e8;

inline double binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

inline int binomial_split(int n, int s) {
  int t = 1;
  while (binom(s + t, s) < n) ++t;
  const int k = n - int(binom(s - 1 + t, s - 1));
  return std::max(1, std::min(k, n - 1));
}

struct Schedule {
  int N = 0, S = 0;
  bool dp = false;
  std::vector<long long> T, F;
  std::vector<int> kT, kF;
  size_t at(int n, int s) const { return size_t(s) * (N + 1) + n; }
  void build(int n_max, int s_max) {
    N = n_max; S = s_max;
    dp = double(N) * N * (S + 1) <= kDpLimit;
    if (!dp) return;
    const size_t m = size_t(N + 1) * (S + 1);
    T.assign(m, 0); F.assign(m, 0); kT.assign(m, 1); kF.assign(m, 1);
    for (int n = 0; n <= N; ++n) T[at(n, 0)] = F[at(n, 0)] = (long long)n * (n - 1) / 2;
    for (int s = 1; s <= S; ++s)
      for (int n = 2; n <= N; ++n) {
        long long bt = -1, bf = -1;
        int kt = 1, kf = 1;
        for (int k = 1; k < n; ++k) {
          const long long right_t = T[at(n - k, s - 1)], right_f = F[at(n - k, s - 1)], left = T[at(k, s)];
          const long long ct = k + right_t + left, cf = right_f + left;
          if (bt < 0 || ct < bt) { bt = ct; kt = k; }
          if (bf < 0 || cf < bf) { bf = cf; kf = k; }
        }
        T[at(n, s)] = bt; kT[at(n, s)] = kt;
        F[at(n, s)] = bf; kF[at(n, s)] = kf;
      }
  }
  int split(int n, int s, bool first) const {
    if (!dp) return binomial_split(n, s);
    return first ? kF[at(n, s)] : kT[at(n, s)];
  }
};

// The checkpointing below is written once for both drivers (Adj, and the batched
// BAdj of hc_batch_adjoint.cu): AD supplies sq, base, snaps, state_values(), s(),
// adv_events, and the overloads forward_step(AD&, step, record) and
// adjoint_step(AD&, step), found by argument-dependent lookup.
template <class AD> auto slot_ptr(AD& A, int slot) {
  return slot < 0 ? A.base : A.snaps + size_t(slot) * A.state_values();
}

template <class AD> int restore(AD& A, int slot) {
  HC_CUDA(cudaMemcpyAsync(A.sq[0], slot_ptr(A, slot), A.state_values() * sizeof(*A.sq[0]), cudaMemcpyDeviceToDevice,
                          A.s()));
  return HC_OK;
}
template <class AD> int store(AD& A, int slot) {
  HC_CUDA(cudaMemcpyAsync(slot_ptr(A, slot), A.sq[0], A.state_values() * sizeof(*A.sq[0]), cudaMemcpyDeviceToDevice,
                          A.s()));
  return HC_OK;
}
template <class AD> int advance(AD& A, int from, int to) {
  if (to <= from) return HC_OK;
  cudaEvent_t ev[2];
  HC_CUDA(cudaEventCreate(&ev[0]));
  A.adv_events.push_back(ev[0]);
  HC_CUDA(cudaEventCreate(&ev[1]));
  A.adv_events.push_back(ev[1]);
  HC_CUDA(cudaEventRecord(ev[0], A.s()));
  for (int k = from; k < to; ++k) {
    if (int st = forward_step(A, k, false)) return st;
    if (k == to - 1) keep_stages(A, k);  // the step reversed next after the right part
    swap_out(A);
  }
  HC_CUDA(cudaEventRecord(ev[1], A.s()));
  return HC_OK;
}

// The first descent of the schedule for n steps and s slots: (position, slot)
// pairs, slots taken from the back of `stack` as reverse() takes them.
inline std::vector<std::pair<int, int>> first_descent(const Schedule& sc, int n, int s, std::vector<int> stack) {
  std::vector<std::pair<int, int>> out;
  int a = 0;
  while (n - a > 1 && !stack.empty()) {
    const int k = sc.split(n - a, int(stack.size()), true);
    out.push_back({a + k, stack.back()});
    stack.pop_back();
    a += k;
  }
  return out;
}

// reverse steps [a, b) whose start state is in `slot`, with the free slots on
// `stack`; `first`: the split points of this call's right-most path were stored
// by the forward sweep
template <class AD>
int reverse(AD& A, const Schedule& sc, int a, int b, int slot, std::vector<int>& stack, bool first) {
  const int n = b - a;
  const int sfree = int(stack.size());
  if (n <= 0) return HC_OK;
  if (n == 1) {
    if (tape_of(A, a) < 0)
      if (int st = restore(A, slot)) return st;
    return adjoint_step(A, a);
  }
  if (sfree == 0) {
    // every step re-advanced from a; each advance keeps the stages of its last step, the
    // next one reversed (a step with a tape first releases it, then advances for the next)
    for (int i = b - 1; i >= a; --i) {
      if (tape_of(A, i) >= 0) {
        if (int st = adjoint_step(A, i)) return st;
        if (i == a) break;
        if (int st = restore(A, slot)) return st;
        if (int st = advance(A, a, i)) return st;
      } else {
        if (int st = restore(A, slot)) return st;
        if (int st = advance(A, a, i)) return st;
        if (int st = adjoint_step(A, i)) return st;
      }
    }
    return HC_OK;
  }
  const int k = sc.split(n, sfree, first);
  const int mid = stack.back();
  stack.pop_back();
  if (!first) {
    if (int st = restore(A, slot)) return st;
    if (int st = advance(A, a, a + k)) return st;
    if (int st = store(A, mid)) return st;
  }
  if (int st = reverse(A, sc, a + k, b, mid, stack, first)) return st;
  stack.push_back(mid);
  return reverse(A, sc, a, a + k, slot, stack, false);
}

inline int check_support(hc_ctx* c, const hc_objective* obj) {
  if (c->oned) return fail(HC_ERR_UNSUPPORTED, "the adjoint covers the 2D path");
  if (c->scalar) {
    if (c->df) return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint runs in FP64 or FP32");
    if (c->cfg.flux != HC_FLUX_RUSANOV && c->cfg.flux != HC_FLUX_CENTRAL)
      return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint supports the Rusanov and central fluxes");
    if (obj->kind != HC_OBJ_L2) return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint takes the L2 objective");
    for (int s = 0; s < 4; ++s)
      if (c->bc[s] != HC_BC_PERIODIC && c->bc[s] != HC_BC_FIXED && c->bc[s] != HC_BC_RIEMANN)
        return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint supports periodic, fixed and Riemann boundaries");
  }
  if (c->cfg.basis != HC_BASIS_PRIMITIVE) return fail(HC_ERR_UNSUPPORTED, "the adjoint uses the primitive basis");
  if (!c->scalar && c->cfg.flux != HC_FLUX_ROE && c->cfg.flux != HC_FLUX_RUSANOV && !flux_by_tangent(c->cfg.flux))
    return fail(HC_ERR_UNSUPPORTED, "the Euler adjoint supports the Roe, Rusanov, SLAU, AUSM+up and RoeUnprecWS fluxes");
  if (c->df && c->cfg.flux != HC_FLUX_ROE && c->cfg.flux != HC_FLUX_RUSANOV)
    return fail(HC_ERR_UNSUPPORTED, "the double-float adjoint supports the Roe and Rusanov fluxes");
  const int l = c->cfg.limiter;
  if (!(l == HC_LIM_NOLIMIT1 || l == HC_LIM_NOLIMIT2 || l == HC_LIM_NOLIMIT3 || l == HC_LIM_VANALBADA ||
        l == HC_LIM_MINMOD || l == HC_LIM_VANLEER))
    return fail(HC_ERR_UNSUPPORTED, "limiter not differentiated by the adjoint");
  if (c->cfg.dt_mode != HC_DT_GLOBAL) return fail(HC_ERR_UNSUPPORTED, "the adjoint uses the global timestep");
  for (int s = 0; s < 4; ++s)
    if (c->df && (c->bc[s] == HC_BC_RIEMANN || c->bc[s] == HC_BC_ENTROPY))
      return fail(HC_ERR_UNSUPPORTED, "the double-float adjoint supports periodic, fixed and wall boundaries");
  return HC_OK;
}

template <class R> int setup(Adj<R>& A, hc_ctx* c, int nsteps, int nsnap, const hc_objective* obj) {
  if (!c || !obj || nsteps < 1 || nsnap < 0) return fail(HC_ERR_ARG, "bad adjoint arguments");
  if (obj->kind != HC_OBJ_DRAG && obj->kind != HC_OBJ_L2) return fail(HC_ERR_ARG, "unknown objective");
  if (int st = ctx_ensure_ready(c)) return st;
  if (int st = check_support(c, obj)) return st;
  A.c = c;
  A.nv = c->scalar ? 3 : 4;
  A.tab = rk_table(c->cfg.rk);
  A.nst = A.tab.nst;
  A.n = c->ncell();
  A.nfi = (c->ni + 1) * c->nj;
  A.nfj = c->ni * (c->nj + 1);
  A.obj = *obj;
  A.nsteps = nsteps;
  A.nsnap = nsnap;
  const size_t n4 = A.state_values();
  for (int k = 0; k <= A.nst; ++k) if (int st = A.alloc(&A.sq[k], n4)) return st;
  for (int k = 0; k < 4; ++k) if (int st = A.alloc(&A.rbar[k], n4)) return st;
  if (int st = A.alloc(&A.qm, 2 * n4)) return st;
  if (int st = A.alloc(&A.qmbar, 2 * n4)) return st;
  if (int st = A.alloc(&A.ai, size_t(4 * A.nv) * A.nfi)) return st;
  if (int st = A.alloc(&A.aj, size_t(4 * A.nv) * A.nfj)) return st;
  if (int st = A.alloc(&A.lam, n4)) return st;
  if (int st = A.alloc(&A.qbs, n4)) return st;
  if (int st = A.alloc(&A.q0bar, n4)) return st;
  for (int s = 0; s < 4; ++s) {
    if (int st = A.alloc(&A.refbar[s], size_t(A.nv) * c->nface(s))) return st;
    HC_CUDA(cudaMemsetAsync(A.refbar[s], 0, size_t(A.nv) * c->nface(s) * sizeof(R), A.s()));
  }
  if (int st = A.alloc(&A.base, n4)) return st;
  if (int st = A.alloc(&A.qnext, n4)) return st;
  if (nsnap > 0) if (int st = A.alloc(&A.snaps, size_t(nsnap) * n4)) return st;
  if (int st = A.alloc(&A.rates, size_t(nsteps))) return st;
  if (int st = A.alloc(&A.wall, size_t(std::max(c->ni, c->nj)))) return st;
  if (int st = A.alloc(&A.jacc, 1)) return st;
  HC_CUDA(cudaMemsetAsync(A.jacc, 0, sizeof(double), A.s()));
  if (obj->kind == HC_OBJ_L2) {
    if (!obj->target) return fail(HC_ERR_ARG, "the L2 objective needs a target state");
    if (int st = A.alloc(&A.target, n4)) return st;
    double* t64 = nullptr;
    if (int st = A.alloc(&t64, n4)) return st;
    HC_CUDA(cudaMemcpyAsync(t64, obj->target, n4 * sizeof(double),
                            obj->target_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, A.s()));
    convert_kernel<R><<<1024, 256, 0, A.s()>>>(t64, A.target, n4);
    HC_CUDA(cudaGetLastError());
  }
  HC_CUDA(cudaMemcpyAsync(A.base, c->q[0], n4 * sizeof(R), cudaMemcpyDeviceToDevice, A.s()));
  return HC_OK;
}

// The steps whose stages the forward sweep keeps: the last step and each one before a
// stored position (the first steps reversed after the parts to their right), the latest
// ones when there are fewer tapes than that.
inline std::vector<char> sweep_keeps(int nsteps, const std::vector<std::pair<int, int>>& stores, int ntapes) {
  std::vector<char> keep(size_t(nsteps), 0);
  std::vector<int> cand;
  for (const auto& p : stores) cand.push_back(p.first - 1);
  cand.push_back(nsteps - 1);
  std::sort(cand.begin(), cand.end());
  for (int k = int(cand.size()) - 1, left = ntapes; k >= 0 && left > 0; --k, --left) keep[size_t(cand[k])] = 1;
  return keep;
}

// forward pass from the base state: J and (rates == nullptr) the max-rate
// history; the states at the positions of `stores` go to their snapshot slots
template <class R>
int forward_pass(Adj<R>& A, const double* rates_in, const std::vector<std::pair<int, int>>& stores = {}) {
  if (rates_in) HC_CUDA(cudaMemcpyAsync(A.rates, rates_in, A.nsteps * sizeof(double), cudaMemcpyHostToDevice, A.s()));
  if (int st = restore(A, -1)) return st;
  const std::vector<char> keep = sweep_keeps(A.nsteps, stores, int(A.tapes.size()));
  size_t next = 0;
  for (int k = 0; k < A.nsteps; ++k) {
    if (int st = forward_step(A, k, rates_in == nullptr)) return st;
    if (keep[size_t(k)]) keep_stages(A, k);
    swap_out(A);
    while (next < stores.size() && stores[next].first == k + 1) {
      if (int st = store(A, stores[next].second)) return st;
      ++next;
    }
    if (A.obj.kind == HC_OBJ_DRAG)
      if (int st = add_drag(A, A.sq[0], A.obj.scale / A.nsteps)) return st;
  }
  if (A.obj.kind == HC_OBJ_L2) {
    l2_kernel<R><<<blocks(A.n), 256, 0, A.s()>>>(A.sq[0], A.target, A.n, A.obj.weight[0], A.obj.weight[1],
                                                  A.obj.weight[2], A.obj.weight[3], A.qbs, 0, nullptr, A.nv);
    sum_into_kernel<R><<<1, 256, 0, A.s()>>>(A.qbs, int(A.n), A.jacc);
    A.launches += 2;
  }
  A.hrates.resize(A.nsteps);
  HC_CUDA(cudaMemcpyAsync(A.hrates.data(), A.rates, A.nsteps * sizeof(double), cudaMemcpyDeviceToHost, A.s()));
  HC_CUDA(cudaStreamSynchronize(A.s()));
  return HC_OK;
}

template <class R> int finish_stats(Adj<R>& A, double* J, double* rates_out, hc_adjoint_stats* stats) {
  double j = 0;
  HC_CUDA(cudaMemcpyAsync(&j, A.jacc, sizeof(double), cudaMemcpyDeviceToHost, A.s()));
  HC_CUDA(cudaStreamSynchronize(A.s()));
  if (J) *J = j;
  if (rates_out) std::memcpy(rates_out, A.hrates.data(), A.nsteps * sizeof(double));
  A.c->launches += A.launches;
  if (stats) {
    stats->J = j;
    stats->forward_steps = A.fwd_steps;
    stats->adjoint_steps = A.adj_steps;
    stats->kernel_launches = A.launches;
    stats->replays = A.replays;
    stats->stage_tapes = (long long)A.tapes.size();
  }
  return HC_OK;
}


// the wall pressure force of the context's current state along dir: the momentum flux
// through every inviscid-wall face, the interior state moved to the face with its LSQ
// gradient as the stage kernels' wall flux does (inviscidWall.ipp:33-72)
template <class R> int wall_force(hc_ctx* c, const double dir[2], double* out) {
  if (!c || !dir || !out) return fail(HC_ERR_ARG, "null argument");
  if (int st = ctx_ensure_ready(c)) return st;
  if (c->oned || c->scalar) return fail(HC_ERR_UNSUPPORTED, "the wall force is defined on the 2D Euler path");
  if (c->cfg.basis != HC_BASIS_PRIMITIVE) return fail(HC_ERR_UNSUPPORTED, "the wall force takes the primitive basis");
  Adj<R> A;
  A.c = c;
  A.nv = 4;
  A.n = c->ncell();
  if (int st = A.alloc(&A.qm, 2 * A.state_values())) return st;
  if (int st = A.alloc(&A.wall, size_t(std::max(c->ni, c->nj)))) return st;
  if (int st = A.alloc(&A.jacc, 1)) return st;
  HC_CUDA(cudaMemsetAsync(A.jacc, 0, sizeof(double), A.s()));
  AdjArgs<R> a = adj_args(A);
  a.q = (const R*)c->q[0];
  a.obj_scale = R(1);
  a.obj_dirx = R(dir[0]);
  a.obj_diry = R(dir[1]);
  adj_qm_kernel<R><<<blocks(A.n), 256, 0, A.s()>>>(a, A.qm);
  int launches = 1;
  for (int side = 0; side < 4; ++side) {
    if (c->bc[side] != HC_BC_WALL) continue;
    const int m = c->nface(side);
    wall_force_kernel<R><<<blocks(m), 256, 0, A.s()>>>(a, A.qm, side, A.wall);
    sum_into_kernel<R><<<1, 256, 0, A.s()>>>(A.wall, m, A.jacc);
    launches += 2;
  }
  HC_CUDA(cudaGetLastError());
  HC_CUDA(cudaMemcpyAsync(out, A.jacc, sizeof(double), cudaMemcpyDeviceToHost, A.s()));
  HC_CUDA(cudaStreamSynchronize(A.s()));
  c->launches += launches;
  return HC_OK;
}

template <class R>
int objective_forward(hc_ctx* c, int nsteps, const hc_objective* obj, const double* rates_in, double* rates_out,
                      double* J) {
  Adj<R> A;
  if (int st = setup(A, c, nsteps, 0, obj)) return st;
  if (int st = forward_pass(A, rates_in)) return st;
  return finish_stats(A, J, rates_out, nullptr);
}

// A recorded forward sweep: the adjoint buffers with the checkpoints of the schedule's
// first descent, the schedule and its free snapshot slots, kept in the context between
// hc_adjoint_record and hc_adjoint_reverse.
struct TapeBase {
  virtual ~TapeBase() = default;
};
template <class R> struct Tape : TapeBase {
  Adj<R> A;
  Schedule sched;
  std::vector<int> stack;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~Tape() override {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};
inline void free_tape(void* p) { delete static_cast<TapeBase*>(p); }

template <class R> __global__ void to_double_kernel(const R* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = double(a[k]);
}

// forward half: J, the rates, and the tape kept in the context
template <class R>
int adjoint_record(hc_ctx* c, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                   double* rates_out, double* J) {
  if (c) c->drop_adj_tape();
  std::unique_ptr<Tape<R>> T(new Tape<R>());
  Adj<R>& A = T->A;
  if (int st = setup(A, c, nsteps, snapshots, obj)) return st;
  if (int st = alloc_tapes(A, c->adj_tapes, snapshots)) return st;
  HC_CUDA(cudaEventCreate(&T->e0));
  HC_CUDA(cudaEventCreate(&T->e1));
  for (int k = snapshots - 1; k >= 0; --k) T->stack.push_back(k);
  T->sched.build(nsteps, snapshots);
  const std::vector<std::pair<int, int>> stores = first_descent(T->sched, nsteps, snapshots, T->stack);
  cudaEventRecord(T->e0, A.s());
  if (int st = forward_pass(A, rates_in, stores)) return st;
  cudaEventRecord(T->e1, A.s());
  double j = 0;
  HC_CUDA(cudaMemcpyAsync(&j, A.jacc, sizeof(double), cudaMemcpyDeviceToHost, A.s()));
  HC_CUDA(cudaStreamSynchronize(A.s()));
  if (J) *J = j;
  if (rates_out) std::memcpy(rates_out, A.hrates.data(), A.nsteps * sizeof(double));
  c->adj_tape = T.release();
  c->adj_tape_free = free_tape;
  return HC_OK;
}

// reverse half: consumes the tape; q0_bar / ref_bar to host memory or, with on_device, to
// FP64 device memory
template <class R>
int adjoint_reverse(hc_ctx* c, double* q0_bar, double* ref_bar, bool on_device, hc_adjoint_stats* stats) {
  if (!c) return fail(HC_ERR_ARG, "null context");
  Tape<R>* T = c->adj_tape ? dynamic_cast<Tape<R>*>(static_cast<TapeBase*>(c->adj_tape)) : nullptr;
  if (!T) return fail(HC_ERR_ARG, "no recorded forward sweep of this context's precision to reverse");
  std::unique_ptr<Tape<R>> own(T);
  c->adj_tape = nullptr;
  Adj<R>& A = T->A;
  const int nsteps = A.nsteps;
  cudaEvent_t e2, er;
  HC_CUDA(cudaEventCreate(&e2));
  HC_CUDA(cudaEventCreate(&er));
  HC_CUDA(cudaEventRecord(er, A.s()));
  HC_CUDA(cudaMemcpyAsync(A.qnext, A.sq[0], A.state_values() * sizeof(R), cudaMemcpyDeviceToDevice, A.s()));
  // adjoint of the final state
  if (A.obj.kind == HC_OBJ_DRAG) {
    AdjArgs<R> a = adj_args(A);
    drag_args(A, a, A.obj.scale / A.nsteps);
    AdjCellArgs<R> u{};
    u.drag = 1;
    u.qbar_out = A.lam;
    adj_cell_kernel<R><<<blocks(A.n), 256, 0, A.s()>>>(a, u);
    HC_CUDA(cudaGetLastError());
    A.launches += 1;
  } else {
    l2_kernel<R><<<blocks(A.n), 256, 0, A.s()>>>(A.sq[0], A.target, A.n, A.obj.weight[0], A.obj.weight[1],
                                                  A.obj.weight[2], A.obj.weight[3], nullptr, 1, A.lam, A.nv);
    A.launches += 1;
  }
  if (int st = reverse(A, T->sched, 0, nsteps, -1, T->stack, true)) return st;
  cudaEventRecord(e2, A.s());
  auto fetch = [&](double* dst, const R* src, size_t m) -> int {
    if constexpr (std::is_same<R, double>::value) {
      HC_CUDA(cudaMemcpyAsync(dst, src, m * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, A.s()));
    } else if (on_device) {
      to_double_kernel<R><<<512, 256, 0, A.s()>>>(src, dst, m);
      HC_CUDA(cudaGetLastError());
      A.launches += 1;
    } else {
      std::vector<R> tmp(m);
      HC_CUDA(cudaMemcpyAsync(tmp.data(), src, m * sizeof(R), cudaMemcpyDeviceToHost, A.s()));
      HC_CUDA(cudaStreamSynchronize(A.s()));
      for (size_t k = 0; k < m; ++k) dst[k] = double(tmp[k]);
    }
    return HC_OK;
  };
  if (q0_bar) if (int st = fetch(q0_bar, A.lam, A.state_values())) return st;
  if (ref_bar) {
    size_t off = 0;
    for (int s = 0; s < 4; ++s) {
      const size_t m = size_t(A.nv) * c->nface(s);
      if (int st = fetch(ref_bar + off, A.refbar[s], m)) return st;
      off += m;
    }
  }
  // the tape's buffers are freed when this returns: after the stream's work on them
  HC_CUDA(cudaStreamSynchronize(A.s()));
  float ms_f = 0, ms_t = 0, ms_r = 0;
  cudaEventElapsedTime(&ms_f, T->e0, T->e1);
  cudaEventElapsedTime(&ms_t, T->e0, e2);
  cudaEventElapsedTime(&ms_r, er, e2);
  cudaEventDestroy(e2);
  cudaEventDestroy(er);
  if (int st = finish_stats(A, nullptr, nullptr, stats)) return st;
  if (stats) {
    stats->ms_forward = ms_f;
    stats->ms_total = ms_t;
    stats->ms_recompute = A.recompute_ms();
    stats->ms_reverse = ms_r;
  }
  return HC_OK;
}

template <class R>
int adjoint_gradient(hc_ctx* c, int nsteps, int snapshots, const hc_objective* obj, const double* rates_in,
                     double* q0_bar, double* ref_bar, double* rates_out, hc_adjoint_stats* stats) {
  if (int st = adjoint_record<R>(c, nsteps, snapshots, obj, rates_in, rates_out, nullptr)) return st;
  return adjoint_reverse<R>(c, q0_bar, ref_bar, false, stats);
}


}  // namespace adj
}  // namespace hc
