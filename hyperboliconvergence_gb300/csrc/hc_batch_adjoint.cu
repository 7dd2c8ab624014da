// hc_batch_adjoint.cu -- discrete adjoint of every instance of a batch at once.
//
// The instances share the RK table, the step count and the checkpoint schedule, so
// the single-mesh driver's sequence of operations (forward steps, stores, restores,
// reversed steps) is the same for all of them; only the data differ.  Here each
// operation covers the whole batch: forward, replayed and recomputed steps are the
// batch's persistent stage launches (one per RK stage over the tiles of every
// instance), and each reverse pass is one launch over the blocks of every instance
// (AdjBatchArgs, hc_adjoint_kernels.cuh).  A reversed step of the batch therefore
// costs the launches of one instance's step, and checkpoint copies move the pooled
// states of all instances in one copy.  Timesteps stay per instance (each its own
// global dt), frozen at the forward run's values; J and the rates are FP64.
//
// Objective: the weighted L2 distance of each instance's final state to its own
// target.  Supported as for the single-mesh adjoint: Euler law (Roe, Rusanov, SLAU,
// AUSM+up or RoeUnprecWS; periodic, fixed, wall, Riemann and entropy boundaries) and
// scalar advection (Rusanov or central;
// periodic, fixed and Riemann boundaries); NoLimit1/2/3, van Albada, MinMod, van Leer; global
// timestep; HC_FP64 and HC_FP32 batches.  Scalar batches keep the pools' Euler slab
// layout (4 state planes per cell) and use their first 3 planes.
#include "hc_adjoint_driver.cuh"
#include "hc_batch.h"

#include <memory>

namespace hc {
namespace adj {

template <class R> struct BAdj : AdjCommon {
  hc_batch* b = nullptr;
  int ninst = 0;
  int nst = 4;
  RKTab tab{};
  size_t n = 0;  // cells of all instances
  R* sq[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  R* rbar[4] = {nullptr, nullptr, nullptr, nullptr};
  R* qm = nullptr;
  R* qmbar = nullptr;
  R* ai = nullptr;
  R* aj = nullptr;
  R* lam = nullptr;
  R* qbs = nullptr;
  R* q0bar = nullptr;
  R* refbar = nullptr;
  R* base = nullptr;
  R* snaps = nullptr;
  R* qnext = nullptr;  // the start states of the step reversed last
  std::vector<StageTape<R>> tapes;
  long long replays = 0;
  R* target = nullptr;
  R* part = nullptr;
  double* rates = nullptr;  // [step][instance]
  double* jacc = nullptr;   // one per instance
  int* seg_c = nullptr;     // cell-pass segments (256-thread blocks per instance)
  int* seg_f = nullptr;     // face-pass segments (kFaceThreads blocks per instance and direction)
  int blocks_c = 0, blocks_f = 0;
  std::vector<double> hrates;
  hc_objective obj{};
  int nsteps = 0;
  long long fwd_steps = 0, adj_steps = 0, launches = 0;
  size_t state_values() const { return 4 * n; }
  cudaStream_t s() const { return b->stream; }

  AdjBatchArgs<R> args() const {
    AdjBatchArgs<R> a{};
    a.inst = b->inst_d;
    a.gas = with_fixes(make_gas<R>(b->gamma, b->Rgas, b->minf), b->fixes);
    a.limiter = b->cfg.limiter;
    a.qm = qm;
    a.fi = (const R*)b->fi;
    a.fj = (const R*)b->fj;
    a.gref = (const R*)b->gref;
    a.refbar = refbar;
    a.ai = ai;
    a.aj = aj;
    a.qmbar = qmbar;
    return a;
  }
};

// one forward step of every instance from sq[0] to sq[nst]; record (rec) or replay
// the max rates of step `step`; nstages < nst runs only the first nstages stages
template <class R> int forward_step(BAdj<R>& A, int step, bool rec, int nstages = -1) {
  hc_batch* b = A.b;
  const BatchFn<R> euler_fn = batch_fn<R>(b->cfg.flux);
  auto fn = [b, euler_fn](const BatchArgs<R>& a, int tile, int grid, cudaStream_t st) -> cudaError_t {
    return b->scalar ? launch_scalar_batch_stage<R>(a, b->cfg.flux, tile, grid, st) : euler_fn(a, tile, grid, st);
  };
  // every tile a CTA: the stage launcher caps the persistent grid at full residency
  const int grid = std::max(1, b->nwork);
  const int tile = b->sched.tile;
  double* rates = A.rates + size_t(step) * A.ninst;
  const int ns = nstages < 0 ? A.nst : nstages;
  for (int s = 0; s < ns; ++s) {
    BatchArgs<R> a = batch_args<R>(b);
    a.q = A.sq[s];
    a.q0 = A.sq[0];
    a.stage = s;
    a.beta = R(A.tab.beta[s]);
    for (int k = 0; k <= s; ++k) a.alpha[k] = R(A.tab.alpha[s][k]);
    for (int k = 0; k < s; ++k) a.res_prev[k] = (const R*)b->res[k];
    a.res_out = (s < A.nst - 1) ? (R*)b->res[s] : nullptr;
    if (s == 0) {
      a.res_out = (R*)b->res[0];
      if (rec) {
        HC_CUDA(cudaMemset2DAsync(&b->info[0].maxrate, sizeof(StepInfo), 0, sizeof(unsigned long long), A.ninst,
                                  A.s()));
        a.mode = MODE_RES_MAXRATE;
        HC_CUDA(fn(a, tile, grid, A.s()));
        HC_CUDA(cudaMemcpy2DAsync(rates, sizeof(double), &b->info[0].maxrate, sizeof(StepInfo), sizeof(double),
                                  A.ninst, cudaMemcpyDeviceToDevice, A.s()));
      } else {
        HC_CUDA(cudaMemcpy2DAsync(&b->info[0].maxrate, sizeof(StepInfo), rates, sizeof(double), sizeof(double),
                                  A.ninst, cudaMemcpyDeviceToDevice, A.s()));
        a.mode = MODE_RESIDUAL;
        HC_CUDA(fn(a, tile, grid, A.s()));
      }
      a.q_out = A.sq[1];
      if (b->scalar)
        HC_CUDA(launch_scalar_batch_update0<R>(a, tile, grid, b->cfg.cfl, R(A.tab.alpha[0][0]), R(A.tab.beta[0]),
                                               A.s()));
      else
        HC_CUDA(launch_batch_update0<R>(a, tile, grid, b->cfg.cfl, R(A.tab.alpha[0][0]), R(A.tab.beta[0]), A.s()));
      A.launches += 2;
    } else {
      a.mode = MODE_FUSED_GLOBAL;
      a.q_out = A.sq[s + 1];
      HC_CUDA(fn(a, tile, grid, A.s()));
      A.launches += 1;
    }
  }
  A.fwd_steps += 1;
  return HC_OK;
}

// scalar law: qbar_out = (dRes/dq at q)^T rbar (+ qbar_add) for every instance, four launches
template <class R, int FK>
int residual_adjoint_scalar(BAdj<R>& A, const R* q, const R* rbar, const R* qbar_add, R* qbar_out) {
  AdjBatchArgs<R> a = A.args();
  a.q = q;
  a.rbar = rbar;
  a.qbar = qbar_out;
  a.qbar_add = qbar_add;
  a.seg = A.seg_c;
  a.nseg = A.ninst;
  AdjBatchArgs<R> af = a;
  af.seg = A.seg_f;
  af.nseg = 2 * A.ninst;
  adj_qm_batch_kernel<R, 3><<<A.blocks_c, 256, 0, A.s()>>>(a);
  adj_face_scalar_batch_kernel<R, FK><<<A.blocks_f, kFaceThreads, 0, A.s()>>>(af);
  adj_qmbar_batch_kernel<R, 3><<<A.blocks_c, 256, 0, A.s()>>>(a);
  adj_gather_batch_kernel<R, 3><<<A.blocks_c, 256, 0, A.s()>>>(a);
  A.launches += 4;
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

template <class R> int res_adj(BAdj<R>& A, const R* q, const R* rbar, const R* add, R* out) {
  if (A.b->cfg.flux == HC_FLUX_CENTRAL) return residual_adjoint_scalar<R, FLUX_CENTRAL>(A, q, rbar, add, out);
  return residual_adjoint_scalar<R, FLUX_RUSANOV>(A, q, rbar, add, out);
}

// lam holds the adjoint of every instance's q_{step+1}, sq[0] their q_step; on return
// lam holds the adjoint of q_step
template <class R> int adjoint_step_euler(BAdj<R>& A, int step);
template <class R> int adjoint_step(BAdj<R>& A, int step) {
  // stage states from the step's tape or a replay of its stages but the last (whose output
  // is the start state of the step reversed before, qnext)
  if (int st = stage_states(A, step)) return st;
  const size_t bytes4 = A.state_values() * sizeof(R);
  // q_{step+1} into sq[nst] by exchange with qnext; qnext takes q_step (sq[0]) the same way
  // when the step is done
  std::swap(A.sq[A.nst], A.qnext);
  if (!A.b->scalar) return adjoint_step_euler(A, step);
  for (int k = 0; k < A.nst; ++k) HC_CUDA(cudaMemsetAsync(A.rbar[k], 0, bytes4, A.s()));
  HC_CUDA(cudaMemsetAsync(A.q0bar, 0, bytes4, A.s()));
  for (int s = A.nst - 1; s >= 0; --s) {
    AdjUpdateBatch<R> u{};
    u.inst = A.b->inst_d;
    u.seg = A.seg_c;
    u.nseg = A.ninst;
    u.g = with_fixes(make_gas<R>(A.b->gamma, A.b->Rgas, A.b->minf), A.b->fixes);
    u.q_out = A.sq[s + 1];
    u.q0 = A.sq[0];
    u.vol = (const R*)A.b->vol;
    u.qbar_out = (s == A.nst - 1) ? A.lam : A.qbs;
    u.q0bar = A.q0bar;
    for (int k = 0; k < 4; ++k) {
      u.rbar[k] = A.rbar[k];
      u.alpha[k] = k <= s ? R(A.tab.alpha[s][k]) : R(0);
    }
    u.stage = s;
    u.beta = A.tab.beta[s];
    u.cfl = A.b->cfg.cfl;
    u.rates = A.rates + size_t(step) * A.ninst;
    adj_update_lin_batch_kernel<R><<<A.blocks_c, 256, 0, A.s()>>>(u);
    A.launches += 1;
    HC_CUDA(cudaGetLastError());
    if (int st = res_adj<R>(A, A.sq[s], A.rbar[s], s == 0 ? A.q0bar : nullptr, A.qbs)) return st;
  }
  HC_CUDA(cudaMemcpyAsync(A.lam, A.qbs, bytes4, cudaMemcpyDeviceToDevice, A.s()));
  std::swap(A.qnext, A.sq[0]);
  A.adj_steps += 1;
  return HC_OK;
}

// The Euler reverse of one step for every instance, as the single-mesh driver does it:
// per stage the face pass, the qmetric adjoint and the fused cell pass (gather of the
// stage, update reverse and qmetric of the stage before; at the first stage the gather
// with the update adjoints of q_step into lam), after one cell pass that reverses the
// last stage's update.
template <class R> int adjoint_step_euler(BAdj<R>& A, int step) {
  AdjCellBatch<R> ub{};
  ub.u.g = with_fixes(make_gas<R>(A.b->gamma, A.b->Rgas, A.b->minf), A.b->fixes);
  ub.u.q0 = A.sq[0];
  ub.u.vol = (const R*)A.b->vol;
  ub.u.q0bar = A.q0bar;
  for (int k = 0; k < 4; ++k) ub.u.rbar[k] = A.rbar[k];
  ub.cfl = A.b->cfg.cfl;
  ub.rates = A.rates + size_t(step) * A.ninst;
  auto update = [&](AdjCellBatch<R>& w, int s) {
    w.u.update = 1;
    w.u.q_out = A.sq[s + 1];
    for (int k = 0; k < 4; ++k) w.u.alpha[k] = k <= s ? R(A.tab.alpha[s][k]) : R(0);
    w.u.stage = s;
    w.beta = A.tab.beta[s];
  };
  AdjBatchArgs<R> a = A.args();
  a.seg = A.seg_c;
  a.nseg = A.ninst;
  {
    AdjCellBatch<R> w = ub;
    w.u.qbar_in = A.lam;
    update(w, A.nst - 1);
    w.u.first = 1;  // q0bar and every rbar_k written, not accumulated: no zeroing
    w.u.qm_q = A.sq[A.nst - 1];
    adj_cell_batch_kernel<R><<<A.blocks_c, 256, 0, A.s()>>>(a, w);
    A.launches += 1;
  }
  for (int s = A.nst - 1; s >= 0; --s) {
    a.q = A.sq[s];
    a.rbar = A.rbar[s];
    a.qbar_add = s == 0 ? A.q0bar : nullptr;
    AdjBatchArgs<R> af = a;
    af.seg = A.seg_f;
    af.nseg = 2 * A.ninst;
    if (flux_by_tangent(A.b->cfg.flux))
      HC_CUDA(launch_adj_face_tangent_batch<R>(A.b->cfg.flux, af, A.blocks_f, kFaceThreads, A.s()));
    else if (A.b->cfg.flux == HC_FLUX_ROE)
      adj_face_batch_kernel<R, FLUX_ROE><<<A.blocks_f, kFaceThreads, 0, A.s()>>>(af);
    else
      adj_face_batch_kernel<R, FLUX_RUSANOV><<<A.blocks_f, kFaceThreads, 0, A.s()>>>(af);
    adj_qmbar_batch_kernel<R><<<A.blocks_c, 256, 0, A.s()>>>(a);
    AdjCellBatch<R> w = ub;
    w.u.gather = 1;
    if (s > 0) {
      update(w, s - 1);
      w.u.qm_q = A.sq[s - 1];
    } else {
      w.u.qbar_out = A.lam;
    }
    adj_cell_batch_kernel<R><<<A.blocks_c, 256, 0, A.s()>>>(a, w);
    A.launches += 3;
    HC_CUDA(cudaGetLastError());
  }
  std::swap(A.qnext, A.sq[0]);
  A.adj_steps += 1;
  return HC_OK;
}

template <class R>
__global__ void l2_batch_kernel(const BatchInst* inst, const int* seg, int nseg, const R* q, const R* t, double w0,
                                double w1, double w2, double w3, R* part, int mode_grad, R* lam, int nv) {
  const int s = find_segment(seg, nseg, int(blockIdx.x));
  const BatchInst& in = inst[s];
  const long long c4 = 4 * in.cell;
  const size_t c = size_t(int(blockIdx.x) - seg[s]) * blockDim.x + threadIdx.x;
  l2_cell(q + c4, t + c4, size_t(in.ni) * in.nj, w0, w1, w2, w3, part ? part + in.cell : nullptr, mode_grad,
          lam ? lam + c4 : nullptr, c, nv);
}
// acc[k] += the sum of instance k's part values (one block per instance, the order
// of the single-mesh sum)
template <class R> __global__ void sum_batch_kernel(const BatchInst* inst, const R* part, double* acc) {
  const BatchInst& in = inst[blockIdx.x];
  block_sum_into(part + in.cell, in.ni * in.nj, acc + blockIdx.x);
}

template <class R> int l2_objective(BAdj<R>& A, bool grad) {
  const double* w = A.obj.weight;
  l2_batch_kernel<R><<<A.blocks_c, 256, 0, A.s()>>>(A.b->inst_d, A.seg_c, A.ninst, A.sq[0], A.target, w[0], w[1],
                                                     w[2], w[3], grad ? nullptr : A.part, grad ? 1 : 0,
                                                     grad ? A.lam : nullptr, A.b->nv);
  A.launches += 1;
  if (!grad) {
    sum_batch_kernel<R><<<A.ninst, 256, 0, A.s()>>>(A.b->inst_d, A.part, A.jacc);
    A.launches += 1;
  }
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

inline int check_batch_support(hc_batch* b) {
  if (b->cfg.basis != HC_BASIS_PRIMITIVE) return fail(HC_ERR_UNSUPPORTED, "the adjoint uses the primitive basis");
  if (b->scalar) {
    if (b->cfg.flux != HC_FLUX_RUSANOV && b->cfg.flux != HC_FLUX_CENTRAL)
      return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint supports the Rusanov and central fluxes");
    for (int t : b->bc)
      if (t != HC_BC_PERIODIC && t != HC_BC_FIXED && t != HC_BC_RIEMANN)
        return fail(HC_ERR_UNSUPPORTED, "the scalar-law adjoint supports periodic, fixed and Riemann boundaries");
  } else if (b->cfg.flux != HC_FLUX_ROE && b->cfg.flux != HC_FLUX_RUSANOV && !flux_by_tangent(b->cfg.flux)) {
    return fail(HC_ERR_UNSUPPORTED, "the Euler adjoint supports the Roe, Rusanov, SLAU, AUSM+up and RoeUnprecWS fluxes");
  }
  const int l = b->cfg.limiter;
  if (!(l == HC_LIM_NOLIMIT1 || l == HC_LIM_NOLIMIT2 || l == HC_LIM_NOLIMIT3 || l == HC_LIM_VANALBADA ||
        l == HC_LIM_MINMOD || l == HC_LIM_VANLEER))
    return fail(HC_ERR_UNSUPPORTED, "limiter not differentiated by the adjoint");
  if (b->cfg.dt_mode != HC_DT_GLOBAL) return fail(HC_ERR_UNSUPPORTED, "the adjoint uses the global timestep");

  return HC_OK;
}

template <class R>
int batch_setup(BAdj<R>& A, hc_batch* b, int nsteps, int nsnap, const hc_objective* obj,
                const double* const* targets) {
  if (nsteps < 1 || nsnap < 0 || !obj) return fail(HC_ERR_ARG, "bad adjoint arguments");
  if (obj->kind != HC_OBJ_L2) return fail(HC_ERR_UNSUPPORTED, "the batched adjoint takes the L2 objective");
  if (!targets) return fail(HC_ERR_ARG, "the L2 objective needs a target per instance");
  for (int k = 0; k < b->ninst; ++k)
    if (!targets[k]) return fail(HC_ERR_ARG, "instance " + std::to_string(k) + " has no target");
  if (int st = check_batch_support(b)) return st;
  A.b = b;
  A.ninst = b->ninst;
  A.tab = rk_table(b->cfg.rk);
  A.nst = A.tab.nst;
  A.n = b->ncell;
  A.obj = *obj;
  A.nsteps = nsteps;
  // segments of the cell and face passes
  std::vector<int> sc(1, 0), sf(1, 0);
  for (int k = 0; k < A.ninst; ++k) {
    const long long nc = b->icells(k);
    const long long nfi = (long long)(b->ni[k] + 1) * b->nj[k], nfj = (long long)b->ni[k] * (b->nj[k] + 1);
    const long long c = sc.back() + (nc + 255) / 256;
    const long long fi = sf.back() + (nfi + kFaceThreads - 1) / kFaceThreads;
    const long long fj = fi + (nfj + kFaceThreads - 1) / kFaceThreads;
    if (fj > 0x7fffffffLL) return fail(HC_ERR_UNSUPPORTED, "batch too large for one adjoint grid");
    sc.push_back(int(c));
    sf.push_back(int(fi));
    sf.push_back(int(fj));
  }
  A.blocks_c = sc.back();
  A.blocks_f = sf.back();
  const size_t n4 = A.state_values();
  if (int st = A.alloc(&A.seg_c, sc.size())) return st;
  if (int st = A.alloc(&A.seg_f, sf.size())) return st;
  HC_CUDA(cudaMemcpyAsync(A.seg_c, sc.data(), sc.size() * sizeof(int), cudaMemcpyHostToDevice, A.s()));
  HC_CUDA(cudaMemcpyAsync(A.seg_f, sf.data(), sf.size() * sizeof(int), cudaMemcpyHostToDevice, A.s()));
  for (int k = 0; k <= A.nst; ++k) if (int st = A.alloc(&A.sq[k], n4)) return st;
  for (int k = 0; k < 4; ++k) if (int st = A.alloc(&A.rbar[k], n4)) return st;
  if (int st = A.alloc(&A.qm, 8 * A.n)) return st;
  if (int st = A.alloc(&A.qmbar, 8 * A.n)) return st;
  if (int st = A.alloc(&A.ai, size_t(ADJ_FIELDS) * b->nfi)) return st;
  if (int st = A.alloc(&A.aj, size_t(ADJ_FIELDS) * b->nfj)) return st;
  if (int st = A.alloc(&A.lam, n4)) return st;
  if (int st = A.alloc(&A.qbs, n4)) return st;
  if (int st = A.alloc(&A.q0bar, n4)) return st;
  if (int st = A.alloc(&A.refbar, b->ngref)) return st;
  HC_CUDA(cudaMemsetAsync(A.refbar, 0, b->ngref * sizeof(R), A.s()));
  if (int st = A.alloc(&A.base, n4)) return st;
  if (int st = A.alloc(&A.qnext, n4)) return st;
  if (nsnap > 0) if (int st = A.alloc(&A.snaps, size_t(nsnap) * n4)) return st;
  if (int st = A.alloc(&A.rates, size_t(nsteps) * A.ninst)) return st;
  if (int st = A.alloc(&A.jacc, size_t(A.ninst))) return st;
  HC_CUDA(cudaMemsetAsync(A.jacc, 0, A.ninst * sizeof(double), A.s()));
  if (int st = A.alloc(&A.part, A.n)) return st;
  if (int st = A.alloc(&A.target, n4)) return st;
  // targets through the batch's FP64 staging buffer (one instance at a time)
  if (b->scalar) HC_CUDA(cudaMemsetAsync(A.target, 0, n4 * sizeof(R), A.s()));
  for (int k = 0; k < A.ninst; ++k) {
    const size_t m = size_t(b->nv) * b->icells(k);
    HC_CUDA(cudaMemcpyAsync(b->staging, targets[k], m * sizeof(double),
                            obj->target_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, A.s()));
    convert_kernel<R><<<512, 256, 0, A.s()>>>(b->staging, A.target + 4 * b->cell_off[k], m);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaStreamSynchronize(A.s()));  // targets[k] and the staging buffer are reused
  }
  HC_CUDA(cudaMemcpyAsync(A.base, b->q[0], n4 * sizeof(R), cudaMemcpyDeviceToDevice, A.s()));
  return HC_OK;
}

template <class R> int batch_forward_pass(BAdj<R>& A, const std::vector<std::pair<int, int>>& stores) {
  if (int st = restore(A, -1)) return st;
  const std::vector<char> keep = sweep_keeps(A.nsteps, stores, int(A.tapes.size()));
  size_t next = 0;
  for (int k = 0; k < A.nsteps; ++k) {
    if (int st = forward_step(A, k, true)) return st;
    if (keep[size_t(k)]) keep_stages(A, k);
    swap_out(A);
    while (next < stores.size() && stores[next].first == k + 1) {
      if (int st = store(A, stores[next].second)) return st;
      ++next;
    }
  }
  if (int st = l2_objective(A, false)) return st;
  A.hrates.resize(size_t(A.nsteps) * A.ninst);
  HC_CUDA(cudaMemcpyAsync(A.hrates.data(), A.rates, A.hrates.size() * sizeof(double), cudaMemcpyDeviceToHost,
                          A.s()));
  HC_CUDA(cudaStreamSynchronize(A.s()));
  return HC_OK;
}

// A recorded forward sweep: the adjoint buffers with the checkpoints of the schedule's
// first descent, the schedule and its free snapshot slots, kept between
// hc_batch_adjoint_record and hc_batch_adjoint_reverse.
struct BTapeBase {
  virtual ~BTapeBase() = default;
};
template <class R> struct BTape : BTapeBase {
  BAdj<R> A;
  Schedule sched;
  std::vector<int> stack;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~BTape() override {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};
inline void free_btape(void* p) { delete static_cast<BTapeBase*>(p); }

__global__ void to_double_kernel(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = double(a[k]);
}

// forward half: J per instance (host), the tape kept in the batch
template <class R>
int batch_record(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj, const double* const* targets,
                 double* J) {
  b->drop_adj_tape();
  std::unique_ptr<BTape<R>> T(new BTape<R>());
  BAdj<R>& A = T->A;
  if (int st = batch_setup(A, b, nsteps, snapshots, obj, targets)) return st;
  if (int st = alloc_tapes(A, b->adj_tapes, snapshots)) return st;
  HC_CUDA(cudaEventCreate(&T->e0));
  HC_CUDA(cudaEventCreate(&T->e1));
  for (int k = snapshots - 1; k >= 0; --k) T->stack.push_back(k);
  T->sched.build(nsteps, snapshots);
  const std::vector<std::pair<int, int>> stores = first_descent(T->sched, nsteps, snapshots, T->stack);
  cudaEventRecord(T->e0, A.s());
  if (int st = batch_forward_pass(A, stores)) return st;
  cudaEventRecord(T->e1, A.s());
  if (J) {
    HC_CUDA(cudaMemcpyAsync(J, A.jacc, A.ninst * sizeof(double), cudaMemcpyDeviceToHost, A.s()));
    HC_CUDA(cudaStreamSynchronize(A.s()));
  }
  b->adj_tape = T.release();
  b->adj_tape_free = free_btape;
  return HC_OK;
}

// reverse half: consumes the tape; q0_bar[k] (NULL entries skipped) in host memory or, with
// on_device, FP64 device memory written asynchronously on the batch's stream
template <class R> int batch_reverse(hc_batch* b, double* const* q0_bar, bool on_device, hc_adjoint_stats* stats) {
  BTape<R>* T = b->adj_tape ? dynamic_cast<BTape<R>*>(static_cast<BTapeBase*>(b->adj_tape)) : nullptr;
  if (!T) return fail(HC_ERR_ARG, "no recorded forward sweep of this batch's precision to reverse");
  std::unique_ptr<BTape<R>> own(T);
  b->adj_tape = nullptr;
  BAdj<R>& A = T->A;
  const int nsteps = A.nsteps;
  cudaEvent_t e2, er;
  HC_CUDA(cudaEventCreate(&e2));
  HC_CUDA(cudaEventCreate(&er));
  HC_CUDA(cudaEventRecord(er, A.s()));
  HC_CUDA(cudaMemcpyAsync(A.qnext, A.sq[0], A.state_values() * sizeof(R), cudaMemcpyDeviceToDevice, A.s()));
  if (int st = l2_objective(A, true)) return st;  // adjoint of the final states
  if (int st = reverse(A, T->sched, 0, nsteps, -1, T->stack, true)) return st;
  cudaEventRecord(e2, A.s());
  if (q0_bar) {
    for (int k = 0; k < A.ninst; ++k) {
      if (!q0_bar[k]) continue;
      const size_t m = size_t(b->nv) * b->icells(k);
      const R* src = A.lam + 4 * b->cell_off[k];
      if constexpr (std::is_same<R, double>::value) {
        HC_CUDA(cudaMemcpyAsync(q0_bar[k], src, m * sizeof(double),
                                on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, A.s()));
      } else if (on_device) {
        to_double_kernel<<<512, 256, 0, A.s()>>>(src, q0_bar[k], m);
        HC_CUDA(cudaGetLastError());
        A.launches += 1;
      } else {
        std::vector<R> tmp(m);
        HC_CUDA(cudaMemcpyAsync(tmp.data(), src, m * sizeof(R), cudaMemcpyDeviceToHost, A.s()));
        HC_CUDA(cudaStreamSynchronize(A.s()));
        for (size_t v = 0; v < m; ++v) q0_bar[k][v] = double(tmp[v]);
      }
    }
  }
  // the device's work and the tape's buffers end together: free them after the stream
  HC_CUDA(cudaStreamSynchronize(A.s()));
  float ms_f = 0, ms_t = 0, ms_r = 0;
  cudaEventElapsedTime(&ms_f, T->e0, T->e1);
  cudaEventElapsedTime(&ms_t, T->e0, e2);
  cudaEventElapsedTime(&ms_r, er, e2);
  cudaEventDestroy(e2);
  cudaEventDestroy(er);
  b->launches += A.launches;
  if (stats) {
    std::vector<double> jh(A.ninst);
    HC_CUDA(cudaMemcpy(jh.data(), A.jacc, A.ninst * sizeof(double), cudaMemcpyDeviceToHost));
    double jsum = 0;
    for (double v : jh) jsum += v;
    stats->J = jsum;
    stats->forward_steps = A.fwd_steps;
    stats->adjoint_steps = A.adj_steps;
    stats->kernel_launches = A.launches;
    stats->ms_forward = ms_f;
    stats->ms_total = ms_t;
    stats->ms_recompute = A.recompute_ms();
    stats->replays = A.replays;
    stats->stage_tapes = (long long)A.tapes.size();
    stats->ms_reverse = ms_r;
  }
  return HC_OK;
}

template <class R>
int batch_adjoint_gradient(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj,
                           const double* const* targets, double* J, double* const* q0_bar, hc_adjoint_stats* stats) {
  if (int st = batch_record<R>(b, nsteps, snapshots, obj, targets, J)) return st;
  return batch_reverse<R>(b, q0_bar, false, stats);
}

}  // namespace adj
}  // namespace hc

extern "C" int hc_batch_adjoint_gradient(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj,
                                         const double* const* targets, double* J, double* const* q0_bar,
                                         hc_adjoint_stats* stats) {
  if (!b) return hc::fail(HC_ERR_ARG, "null batch");
  if (b->fp32) return hc::adj::batch_adjoint_gradient<float>(b, nsteps, snapshots, obj, targets, J, q0_bar, stats);
  return hc::adj::batch_adjoint_gradient<double>(b, nsteps, snapshots, obj, targets, J, q0_bar, stats);
}

extern "C" int hc_batch_adjoint_record(hc_batch* b, int nsteps, int snapshots, const hc_objective* obj,
                                       const double* const* targets, double* J) {
  if (!b) return hc::fail(HC_ERR_ARG, "null batch");
  if (b->fp32) return hc::adj::batch_record<float>(b, nsteps, snapshots, obj, targets, J);
  return hc::adj::batch_record<double>(b, nsteps, snapshots, obj, targets, J);
}

extern "C" int hc_batch_adjoint_reverse(hc_batch* b, double* const* q0_bar, int on_device, hc_adjoint_stats* stats) {
  if (!b) return hc::fail(HC_ERR_ARG, "null batch");
  if (b->fp32) return hc::adj::batch_reverse<float>(b, q0_bar, on_device != 0, stats);
  return hc::adj::batch_reverse<double>(b, q0_bar, on_device != 0, stats);
}
