// hc_oned.cuh -- the one-dimensional Euler path: one fused RK stage per launch over
// tiles of TB cells (interiorResidual in 1D, spatial/residualCalc.h:74-127, with the
// 1D boundary loops and LSQ metrics of spatial/boundary/*.h and spatial/lsqMetrics.h).
// State: 3 planes {u, rho, p}; residual: 3 flux planes {rho u, rho, rho E} + the
// spectral-radius sum.  The fluxes and far-field updates are the 2D device functions
// with the second velocity 0 and face normals (+-1, 0): the reference's nDim = 1
// instantiations compute the same (pinned by the golden vectors).
#pragma once

#include "hc_kernels.cuh"

namespace hc {

// per-face 1D records (nc + 1 faces, face f at node f between cells f-1 and f)
enum Face1Field { F1_DL = 0, F1_DR, F1_IDLR, F1_WL, F1_SL, F1_WR, F1_SR, F1_DX, F1_WW, F1REC };

template <class R> struct Stage1DArgs {
  int nc;
  int bc[2];
  Gas<R> gas;
  int limiter;
  const R* q;       // stage state (3 planes)
  const R* q0;      // state at the start of the step
  const R* rec;     // F1REC planes of nc + 1 face records
  const R* vol;
  const R* gref[2]; // reference values of sides 0 / 1 (3 values)
  R* res_out;       // 4 planes or null
  const R* res_prev[4];
  R alpha[4];
  int stage, mode;
  R beta, cfl;
  StepInfo* info;
  R* q_out;
  int norm_stage0;
};

constexpr int kTile1D = 256;

template <class R> __device__ __forceinline__ St<R> st1(const Gas<R>& g, const R* q) {
  return prim_state(g, q[0], R(0), q[1], q[2]);
}

// cons(q0) + tot * fac -> {u, rho, p} (spatial/eulerForwardUpdate.h:76-85) through the 2D
// update with the second velocity and its flux 0
template <class R> __device__ __forceinline__ void update1(const Gas<R>& g, const R* q0, const R* tot, R fac, R* qn) {
  const R p4[4] = {q0[0], R(0), q0[1], q0[2]};
  const R t4[4] = {tot[0], R(0), tot[1], tot[2]};
  R n4[4];
  forward_update(g, p4, t4, fac, n4, false);
  qn[0] = n4[0]; qn[1] = n4[2]; qn[2] = n4[3];
}

template <class R, int FK> __global__ void __launch_bounds__(kTile1D) stage1d_kernel(const Stage1DArgs<R> a) {
  constexpr int TB = kTile1D, QN = TB + 4, MN = TB + 2, FN = TB + 1;
  __shared__ R sq[3 * QN];
  __shared__ R sm[3 * MN];
  __shared__ R sf[4 * FN];
  const int nc = a.nc, tid = threadIdx.x, i0 = blockIdx.x * TB;
  const bool per = a.bc[0] == BC_PERIODIC;
  const size_t n = size_t(nc);
  // phase 1: cells i0-2 .. i0+TB+1 (periodic wrap)
  for (int k = tid; k < QN; k += TB) {
    int c = i0 - 2 + k;
    bool ok = true;
    if (c < 0 || c >= nc) { if (per) c = wrapi(c, nc); else ok = false; }
#pragma unroll
    for (int v = 0; v < 3; ++v) sq[v * QN + k] = ok ? a.q[v * n + c] : R(0);
  }
  __syncthreads();
  auto Q = [&](int v, int la) -> R { return sq[v * QN + la + 2]; };
  auto rd = [&](int fld, int f) -> R { return a.rec[size_t(fld) * (nc + 1) + f]; };
  // phase 2: qmetric of cells i0-1 .. i0+TB (spatial/lsqMetrics.h qmetrics, D2)
  for (int k = tid; k < MN; k += TB) {
    const int la = k - 1;
    int c = i0 + la;
    bool ok = true;
    if (c < 0 || c >= nc) { if (per) c = wrapi(c, nc); else ok = false; }
    R m[3] = {R(0), R(0), R(0)};
    if (ok) {
      const int fl = c, fr = c + 1;  // left and right faces of the cell
      if ((fl > 0 && fl < nc) || per) {
        const R dx = rd(F1_DX, fl);
#pragma unroll
        for (int v = 0; v < 3; ++v) m[v] += (Q(v, la) - Q(v, la - 1)) * dx;
      }
      if (fr < nc || per) {
        const R dx = rd(F1_DX, fr);
#pragma unroll
        for (int v = 0; v < 3; ++v) m[v] += (Q(v, la + 1) - Q(v, la)) * dx;
      }
    }
#pragma unroll
    for (int v = 0; v < 3; ++v) sm[v * MN + k] = m[v];
  }
  __syncthreads();
  auto M = [&](int v, int la) -> R { return sm[v * MN + la + 1]; };
  // phase 3: faces i0 .. i0+TB
  const Gas<R> g = a.gas;
  const int lim = a.limiter;
  for (int k = tid; k < FN; k += TB) {
    const int f = i0 + k;
    Flux5<R> F;
    F.f[0] = F.f[1] = F.f[2] = F.f[3] = F.lam = R(0);
    if (f <= nc) {
      const bool bnd = (f == 0 || f == nc) && !per;
      if (!bnd) {
        R ql[3], qr[3], qL[3], qR[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) { ql[v] = Q(v, k - 1); qr[v] = Q(v, k); }
        if (lim != LIM_NOLIMIT1) {
          const R dl = rd(F1_DL, f), dr = rd(F1_DR, f), idlr = rd(F1_IDLR, f);
          const R wl = rd(F1_WL, f), sl = rd(F1_SL, f), wr = rd(F1_WR, f), sr = rd(F1_SR, f);
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const R dq = qr[v] - ql[v];
            const R gc = dq * idlr;
            const R gl = M(v, k - 1) * wl - dq * sl;
            const R gr = M(v, k) * wr - dq * sr;
            qL[v] = ql[v] + dl * limit<R>(lim, gc, gl);
            qR[v] = qr[v] - dr * limit<R>(lim, gc, gr);
          }
        } else {
#pragma unroll
          for (int v = 0; v < 3; ++v) { qL[v] = ql[v]; qR[v] = qr[v]; }
        }
        F = face_flux<R, FK>(g, R(1), R(0), R(1), st1(g, qL), st1(g, qR));
      } else {
        const int side = f == 0 ? 0 : 1;
        const bool int_right = side == 0;  // the interior cell is right of the left boundary
        const int li = int_right ? k : k - 1;
        R qi[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) qi[v] = Q(v, li);
        const int bct = a.bc[side];
        if (bct == BC_WALL) {
          // the interior state moved to the face with the cell's gradient; normal into the domain
          const R ww = rd(F1_WW, f);
          const R qw[4] = {qi[0] - M(0, li) * ww, R(0), qi[1] - M(1, li) * ww, qi[2] - M(2, li) * ww};
          F = wall_flux(g, int_right ? R(1) : R(-1), R(0), R(1), qw);
          if (!int_right) {  // res(interior) += F on both sides: stored as the face's (left - right) flux
#pragma unroll
            for (int v = 0; v < 4; ++v) F.f[v] = -F.f[v];
          }
        } else {
          R qg4[4];
          const R qi4[4] = {qi[0], R(0), qi[1], qi[2]};
          const R qf4[4] = {a.gref[side][0], R(0), a.gref[side][1], a.gref[side][2]};
          const R nin = int_right ? R(1) : R(-1);
          if (bct == BC_RIEMANN) farfield_update<R, BC_RIEMANN>(g, nin, R(0), qi4, qf4, qg4);
          else if (bct == BC_ENTROPY) farfield_update<R, BC_ENTROPY>(g, nin, R(0), qi4, qf4, qg4);
          else {
#pragma unroll
            for (int v = 0; v < 4; ++v) qg4[v] = qf4[v];
          }
          const R qg[3] = {qg4[0], qg4[2], qg4[3]};
          R qL[3], qR[3];
          if (lim != LIM_NOLIMIT1) {
            const R d = rd(F1_DL, f), idlr = rd(F1_IDLR, f), w = int_right ? rd(F1_WR, f) : rd(F1_WL, f);
#pragma unroll
            for (int v = 0; v < 3; ++v) {
              const R dq = int_right ? (qi[v] - qg[v]) : (qg[v] - qi[v]);
              const R s = limit<R>(lim, dq * idlr, M(v, li) * w);
              if (int_right) { qL[v] = qg[v]; qR[v] = qi[v] - d * s; }
              else { qL[v] = qi[v] + d * s; qR[v] = qg[v]; }
            }
          } else {
#pragma unroll
            for (int v = 0; v < 3; ++v) { qL[v] = int_right ? qg[v] : qi[v]; qR[v] = int_right ? qi[v] : qg[v]; }
          }
          F = face_flux<R, FK>(g, R(1), R(0), R(1), st1(g, qL), st1(g, qR));
        }
      }
    }
    sf[0 * FN + k] = F.f[0];
    sf[1 * FN + k] = F.f[2];
    sf[2 * FN + k] = F.f[3];
    sf[3 * FN + k] = F.lam;
  }
  __syncthreads();
  // phase 4: accumulate (res(c) += F(left face) - F(right face)) and update
  const int c = i0 + tid;
  const bool own = c < nc;
  R res[3] = {R(0), R(0), R(0)}, lam = R(0);
  if (own) {
#pragma unroll
    for (int v = 0; v < 3; ++v) res[v] = sf[v * FN + tid] - sf[v * FN + tid + 1];
    lam = sf[3 * FN + tid] + sf[3 * FN + tid + 1];
  }
  if (own && a.res_out) {
#pragma unroll
    for (int v = 0; v < 3; ++v) a.res_out[v * n + c] = res[v];
    a.res_out[3 * n + c] = lam;
  }
  if (a.mode == MODE_RES_MAXRATE || (a.mode == MODE_FUSED_LOCAL && a.norm_stage0 && a.stage == 0)) {
    R rate = own ? lam / a.vol[c] : R(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
    if ((tid & 31) == 0) atomic_max_rate<R>(a.info, rate);
  }
  if (a.norm_stage0 && a.stage == 0) {
    R r2 = own ? res[1] * res[1] : R(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    if ((tid & 31) == 0) atomicAdd(&a.info->resnorm2, double(r2));
  }
  if (a.mode == MODE_RES_MAXRATE || a.mode == MODE_RESIDUAL || !own) return;
  R tot[3] = {R(0), R(0), R(0)};
  for (int k = 0; k < a.stage; ++k)
#pragma unroll
    for (int v = 0; v < 3; ++v) tot[v] += a.alpha[k] * a.res_prev[k][v * n + c];
#pragma unroll
  for (int v = 0; v < 3; ++v) tot[v] += a.alpha[a.stage] * res[v];
  R fac;
  if (a.mode == MODE_FUSED_GLOBAL) {
    fac = (a.beta * R(a.info->dt)) / a.vol[c];
  } else {
    const R l0 = (a.stage == 0) ? lam : a.res_prev[0][3 * n + c];
    fac = (a.beta * a.cfl) / l0;
  }
  R q0[3], qn[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) q0[v] = a.q0[v * n + c];
  update1(g, q0, tot, fac, qn);
#pragma unroll
  for (int v = 0; v < 3; ++v) a.q_out[v * n + c] = qn[v];
  const R chk[4] = {qn[0], R(0), qn[1], qn[2]};
  flag_nonphysical(a.info, chk, c);
}

// stage-0 update of the 1D path with the global timestep
template <class R>
__global__ void update0_1d_kernel(int nc, Gas<R> g, const R* __restrict__ q0, const R* __restrict__ res0,
                                  const R* __restrict__ vol, R alpha00, R beta0, double cfl, StepInfo* info,
                                  R* __restrict__ q_out) {
  const R dt = global_dt<R>(info, cfl);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info->dt = double(dt);
    info->t += double(dt);
  }
  const size_t n = size_t(nc);
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
    R tot[3], q[3], qn[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) { tot[v] = R(0) + alpha00 * res0[v * n + c]; q[v] = q0[v * n + c]; }
    update1(g, q, tot, (beta0 * dt) / vol[c], qn);
#pragma unroll
    for (int v = 0; v < 3; ++v) q_out[v * n + c] = qn[v];
    const R chk[4] = {qn[0], R(0), qn[1], qn[2]};
    flag_nonphysical(info, chk, int(c));
  }
}

// Stage update of the 1D path from stored stage residuals (the update of the fused
// stage kernel as a kernel of its own, for residuals changed between the two: residual
// smoothing).  res[k] holds 4 planes (3 flux sums and lambda) of stage k; global dt: at
// stage 0 from the recorded max rate (and stored), later stages read it; local dt: the
// stage-0 lambda.
template <class R> struct Update1DArgs {
  int nc;
  Gas<R> gas;
  const R* q0;
  const R* res[4];
  R alpha[4];
  int stage;
  R beta;
  int global;
  double cfl;
  StepInfo* info;
  const R* vol;
  R* q_out;
};
template <class R> __global__ void update_stage_1d_kernel(const Update1DArgs<R> u) {
  const size_t n = size_t(u.nc);
  R dt = R(0);
  if (u.global) {
    if (u.stage == 0) {
      dt = global_dt<R>(u.info, u.cfl);
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        u.info->dt = double(dt);
        u.info->t += double(dt);
      }
    } else {
      dt = R(u.info->dt);
    }
  }
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < n; c += size_t(gridDim.x) * blockDim.x) {
    R tot[3] = {R(0), R(0), R(0)};
    for (int k = 0; k <= u.stage; ++k)
#pragma unroll
      for (int v = 0; v < 3; ++v) tot[v] += u.alpha[k] * u.res[k][v * n + c];
    const R fac = u.global ? (u.beta * dt) / u.vol[c] : (u.beta * R(u.cfl)) / u.res[0][3 * n + c];
    R q[3], qn[3];
#pragma unroll
    for (int v = 0; v < 3; ++v) q[v] = u.q0[v * n + c];
    update1(u.gas, q, tot, fac, qn);
#pragma unroll
    for (int v = 0; v < 3; ++v) u.q_out[v * n + c] = qn[v];
    const R chk[4] = {qn[0], R(0), qn[1], qn[2]};
    flag_nonphysical(u.info, chk, int(c));
  }
}

template <class R> cudaError_t launch_stage1d(const Stage1DArgs<R>& a, int flux, cudaStream_t s);

}  // namespace hc
