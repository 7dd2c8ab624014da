// hc_scalar.cuh -- stage kernel of the scalar advection law
// (conservationLaws/scalarAdvection/scalarAdvection.h:45-98): conserved set
// {u, v, q}, an advected scalar q with its advecting velocity (constant in time).
//
// Same tiling as the Euler stage kernel (hc_kernels.cuh): a TI x TJ tile with a
// 2-cell halo in shared memory, the LSQ qmetric of the tile and a 1-cell ring,
// every tile face once (MUSCL + limiter on the three conserved variables, the
// Rusanov or central flux, ghost faces with the Fixed or Riemann ghost value),
// gather accumulation, then the spectral-radius reduction or the alpha/beta RK
// update, which for this law acts on the conserved set directly.
//
// Layouts: state 3 planes {u, v, q}; residual 4 planes (3 flux sums + lambda);
// ghost reference 3 planes per side; face records as for the Euler path.
#pragma once

#include "hc_kernels.cuh"

namespace hc {

template <int TI, int TJ, class R> struct ScalarSmem {
  static constexpr int QI = TI + 4, QJ = TJ + 4;
  static constexpr int MI = TI + 2, MJ = TJ + 2;
  static constexpr size_t q_elems = size_t(3) * QI * QJ;
  static constexpr size_t m_elems = size_t(6) * MI * MJ;
  static constexpr size_t fi_elems = size_t(4) * (TI + 1) * TJ;
  static constexpr size_t fj_elems = size_t(4) * TI * (TJ + 1);
  static constexpr size_t bytes = (q_elems + m_elems + fi_elems + fj_elems) * sizeof(R);
};

template <class R> struct SFlux4 { R f[3]; R lam; };

// exactFlux (scalarAdvection/fluxes/exactFlux.ipp:8-21) summed into the central
// flux (conservationLaws/base/fluxes/centralFlux.ipp:2-14), plus the Rusanov
// dissipation (conservationLaws/base/fluxes/rusanovFlux.ipp:2-50) when FK is Rusanov
template <class R, int FK>
__device__ __forceinline__ SFlux4<R> scalar_face_flux(R nx, R ny, R A, const R* ql, const R* qr) {
  const R unl = nx * ql[0] + ny * ql[1];
  const R unr = nx * qr[0] + ny * qr[1];
  const R al = fabs(unl), ar = fabs(unr);
  SFlux4<R> o;
  o.f[0] = R(0);
  o.f[1] = R(0);
  o.f[2] = (R(0.5) * (unl * ql[2] + unr * qr[2])) * A;
  o.lam = fmax(al, ar) * A;
  if constexpr (FK == FLUX_RUSANOV) {
    const R c = R(-0.5) * (fmax(al, ar) * A);
#pragma unroll
    for (int v = 0; v < 3; ++v) o.f[v] += c * (qr[v] - ql[v]);
  }
  return o;
}

// Riemann ghost value (scalarAdvection/boundary/riemann.ipp): the face-averaged
// set rotated to the face frame, its velocity projected on the inward normal as
// written; inflow takes the boundary value, outflow the interior one.  Returns inflow.
template <class R>
__device__ __forceinline__ bool scalar_riemann_ghost(R nx, R ny, const R* qi, const R* qb, R* g) {
  const R au = qi[0] + R(0.5) * (qb[0] - qi[0]);
  const R av = qi[1] + R(0.5) * (qb[1] - qi[1]);
  const R tx = -ny, ty = nx;
  const R rn = nx * au + ny * av;   // normal component
  const R rt = tx * au + ty * av;   // tangential component
  const bool inflow = (nx * rn + ny * rt) > R(0);
#pragma unroll
  for (int v = 0; v < 3; ++v) g[v] = inflow ? qb[v] : qi[v];
  return inflow;
}

template <int TI, int TJ, class R, int FK>
__device__ __forceinline__ void scalar_stage_tile(const StageArgs<R>& a, int bi, int bj, unsigned char* smem_raw) {
  using SM = ScalarSmem<TI, TJ, R>;
  R* sq = reinterpret_cast<R*>(smem_raw);
  R* sm = sq + SM::q_elems;
  R* sfi = sm + SM::m_elems;
  R* sfj = sfi + SM::fi_elems;
  constexpr int QI = SM::QI, QJ = SM::QJ, MI = SM::MI, MJ = SM::MJ;
  constexpr int NT = TI * TJ;
  const int ni = a.ni, nj = a.nj;
  const size_t ncell = size_t(ni) * nj;
  const int i0 = bi * TI, j0 = bj * TJ;
  const int tid = threadIdx.x;
  const bool per_i = a.bc[0] == BC_PERIODIC, per_j = a.bc[2] == BC_PERIODIC;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);

  for (int k = tid; k < QI * QJ; k += NT) {
    const int la = k / QJ, lb = k % QJ;
    int gi = i0 - 2 + la, gj = j0 - 2 + lb;
    bool ok = true;
    if (gi < 0 || gi >= ni) { if (per_i) gi = wrapi(gi, ni); else ok = false; }
    if (gj < 0 || gj >= nj) { if (per_j) gj = wrapi(gj, nj); else ok = false; }
    const size_t c = size_t(gi) * nj + gj;
#pragma unroll
    for (int v = 0; v < 3; ++v) sq[(v * QI + la) * QJ + lb] = ok ? a.q[v * ncell + c] : R(0);
  }
  __syncthreads();

  auto Q = [&](int v, int la, int lb) -> R { return sq[(v * QI + la + 2) * QJ + lb + 2]; };
  auto M = [&](int k, int la, int lb) -> R& { return sm[(k * MI + la + 1) * MJ + lb + 1]; };

  for (int k = tid; k < MI * MJ; k += NT) {
    const int la = k / MJ - 1, lb = k % MJ - 1;
    const bool corner = (la < 0 || la >= TI) && (lb < 0 || lb >= TJ);
    int gi = i0 + la, gj = j0 + lb;
    bool ok = !corner;
    if (gi < 0 || gi >= ni) { if (per_i) gi = wrapi(gi, ni); else ok = false; }
    if (gj < 0 || gj >= nj) { if (per_j) gj = wrapi(gj, nj); else ok = false; }
    R m[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) m[q] = R(0);
    if (ok) {
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        const bool idir = f < 2;
        const int hi = f & 1;
        int fidx;
        bool pair;
        if (idir) {
          const int fi = gi + hi;
          pair = (fi > 0 && fi < ni) || per_i;
          fidx = fi * nj + gj;
        } else {
          const int fj = gj + hi;
          pair = (fj > 0 && fj < nj) || per_j;
          fidx = gi * (nj + 1) + fj;
        }
        if (!pair) continue;
        const R* rec = idir ? a.fi : a.fj;
        const int nf = idir ? nfi : nfj;
        const R dx = rec[size_t(F_DXX) * nf + fidx], dy = rec[size_t(F_DXY) * nf + fidx];
        const int na = la + (idir ? (hi ? 1 : -1) : 0), nb = lb + (idir ? 0 : (hi ? 1 : -1));
#pragma unroll
        for (int v = 0; v < 3; ++v) {
          const R dq = hi ? (Q(v, na, nb) - Q(v, la, lb)) : (Q(v, la, lb) - Q(v, na, nb));
          m[2 * v] += dq * dx;
          m[2 * v + 1] += dq * dy;
        }
      }
    }
    if (la >= -1 && la <= TI && lb >= -1 && lb <= TJ)
#pragma unroll
      for (int q = 0; q < 6; ++q) M(q, la, lb) = m[q];
  }
  __syncthreads();

  const int lim = a.limiter;
  constexpr int NFI = (TI + 1) * TJ, NFJ = TI * (TJ + 1);
  for (int k = tid; k < NFI + NFJ; k += NT) {
    const bool idir = k < NFI;
    int la, lb;
    if (idir) { la = k / TJ; lb = k % TJ; } else { const int kk = k - NFI; la = kk / (TJ + 1); lb = kk % (TJ + 1); }
    const int gi = i0 + la, gj = j0 + lb;
    const bool valid = idir ? (gi <= ni && gj < nj) : (gi < ni && gj <= nj);
    SFlux4<R> F;
    F.f[0] = F.f[1] = F.f[2] = F.lam = R(0);
    if (valid) {
      const R* rec = idir ? a.fi : a.fj;
      const int nf = idir ? nfi : nfj;
      const int fidx = idir ? gi * nj + gj : gi * (nj + 1) + gj;
      auto rd = [&](int fld) -> R { return rec[size_t(fld) * nf + fidx]; };
      const R nx = rd(F_NX), ny = rd(F_NY), A = rd(F_A);
      const int lo = idir ? gi : gj, nalong = idir ? ni : nj;
      const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
      const bool bnd = (lo == 0 || lo == nalong) && a.bc[side] != BC_PERIODIC;
      const int la_l = idir ? la - 1 : la, lb_l = idir ? lb : lb - 1;
      R qL[3], qR[3];
      if (!bnd) {
        R ql[3], qr[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) { ql[v] = Q(v, la_l, lb_l); qr[v] = Q(v, la, lb); }
        if (lim != LIM_NOLIMIT1) {
          const R dl = rd(F_DL), dr = rd(F_DR), idlr = rd(F_IDLR);
          const R wlx = rd(F_WLX), wly = rd(F_WLY), sl = rd(F_SL);
          const R wrx = rd(F_WRX), wry = rd(F_WRY), sr = rd(F_SR);
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const R dq = qr[v] - ql[v];
            const R gc = dq * idlr;
            const R gl = (M(2 * v, la_l, lb_l) * wlx + M(2 * v + 1, la_l, lb_l) * wly) - dq * sl;
            const R gr = (M(2 * v, la, lb) * wrx + M(2 * v + 1, la, lb) * wry) - dq * sr;
            qL[v] = ql[v] + dl * limit<R>(lim, gc, gl);
            qR[v] = qr[v] - dr * limit<R>(lim, gc, gr);
          }
        } else {
#pragma unroll
          for (int v = 0; v < 3; ++v) { qL[v] = ql[v]; qR[v] = qr[v]; }
        }
      } else {
        const bool int_right = lo == 0;
        const int ia = int_right ? la : la_l, ib = int_right ? lb : lb_l;
        R qi[3], qref[3], qg[3];
        const int kf = idir ? gj : gi;
        const int nfs = idir ? nj : ni;
#pragma unroll
        for (int v = 0; v < 3; ++v) { qi[v] = Q(v, ia, ib); qref[v] = a.gref[side][size_t(v) * nfs + kf]; }
        if (a.bc[side] == BC_RIEMANN) {
          const R sgn = int_right ? R(1) : R(-1);  // normal into the domain
          scalar_riemann_ghost(sgn * nx, sgn * ny, qi, qref, qg);
        } else {
#pragma unroll
          for (int v = 0; v < 3; ++v) qg[v] = qref[v];
        }
        if (lim != LIM_NOLIMIT1) {
          const R d = rd(F_DL), idlr = rd(F_IDLR);
          const R wx = int_right ? rd(F_WRX) : rd(F_WLX), wy = int_right ? rd(F_WRY) : rd(F_WLY);
#pragma unroll
          for (int v = 0; v < 3; ++v) {
            const R dq = int_right ? (qi[v] - qg[v]) : (qg[v] - qi[v]);
            const R gb = M(2 * v, ia, ib) * wx + M(2 * v + 1, ia, ib) * wy;
            const R s = limit<R>(lim, dq * idlr, gb);
            if (int_right) { qL[v] = qg[v]; qR[v] = qi[v] - d * s; }
            else { qL[v] = qi[v] + d * s; qR[v] = qg[v]; }
          }
        } else {
#pragma unroll
          for (int v = 0; v < 3; ++v) { qL[v] = int_right ? qg[v] : qi[v]; qR[v] = int_right ? qi[v] : qg[v]; }
        }
      }
      F = scalar_face_flux<R, FK>(nx, ny, A, qL, qR);
    }
    R* dst = idir ? sfi : sfj;
    const int slot = idir ? (la * TJ + lb) : (la * (TJ + 1) + lb);
    const int pl = idir ? NFI : NFJ;
#pragma unroll
    for (int v = 0; v < 3; ++v) dst[v * pl + slot] = F.f[v];
    dst[3 * pl + slot] = F.lam;
  }
  __syncthreads();

  const int la = tid / TJ, lb = tid % TJ;
  const int gi = i0 + la, gj = j0 + lb;
  const bool own = gi < ni && gj < nj;
  R res[3], lam = R(0);
  if (own) {
    const int s0 = la * TJ + lb, s1 = (la + 1) * TJ + lb;
    const int t0 = la * (TJ + 1) + lb, t1 = t0 + 1;
#pragma unroll
    for (int v = 0; v < 3; ++v) res[v] = ((sfi[v * NFI + s0] - sfi[v * NFI + s1]) + sfj[v * NFJ + t0]) - sfj[v * NFJ + t1];
    lam = ((sfi[3 * NFI + s0] + sfi[3 * NFI + s1]) + sfj[3 * NFJ + t0]) + sfj[3 * NFJ + t1];
  }
  const size_t c = size_t(gi) * nj + gj;
  if (own && a.res_out) {
#pragma unroll
    for (int v = 0; v < 3; ++v) a.res_out[v * ncell + c] = res[v];
    a.res_out[3 * ncell + c] = lam;
  }
  if (a.mode == MODE_RES_MAXRATE || (a.norm_stage0 && a.stage == 0)) {
    if (a.norm_stage0) {
      R r2 = own ? res[2] * res[2] : R(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
      if ((tid & 31) == 0) atomicAdd(&a.info->resnorm2, double(r2));
    }
    if (a.mode == MODE_RES_MAXRATE || a.mode == MODE_FUSED_LOCAL) {
      R rate = own ? lam / a.vol[c] : R(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
      if ((tid & 31) == 0) atomic_max_rate<R>(a.info, rate);
    }
  }
  if (a.mode == MODE_RES_MAXRATE || a.mode == MODE_RESIDUAL || !own) return;
  // rungeKuttaAccumulation and the forward update on the conserved set
  R tot[3] = {R(0), R(0), R(0)};
  for (int k = 0; k < a.stage; ++k)
#pragma unroll
    for (int v = 0; v < 3; ++v) tot[v] += a.alpha[k] * a.res_prev[k][v * ncell + c];
#pragma unroll
  for (int v = 0; v < 3; ++v) tot[v] += a.alpha[a.stage] * res[v];
  R fac;
  if (a.mode == MODE_FUSED_GLOBAL) {
    const R dts = a.beta * R(a.info->dt);
    fac = dts / a.vol[c];
  } else {
    const R l0 = (a.stage == 0) ? lam : a.res_prev[0][3 * ncell + c];
    const R cs = a.beta * a.cfl;
    fac = cs / l0;
  }
  R qn[3];
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    qn[v] = a.q0[v * ncell + c] + tot[v] * fac;
    a.q_out[v * ncell + c] = qn[v];
  }
  if (!isfinite(qn[0]) || !isfinite(qn[1]) || !isfinite(qn[2])) {
    if (atomicCAS(&a.info->status, ST_OK, ST_NONPHYSICAL) == ST_OK) a.info->bad_cell = int(c);
  }
}

template <int TI, int TJ, class R, int FK>
__global__ void __launch_bounds__(TI * TJ) scalar_stage_kernel(const StageArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  scalar_stage_tile<TI, TJ, R, FK>(a, blockIdx.y, blockIdx.x, smem_raw);
}

// Stage-0 update with the global dt on the conserved set
template <class R>
__global__ void scalar_update0_kernel(int ni, int nj, const R* __restrict__ q0, const R* __restrict__ res0,
                                      const R* __restrict__ vol, R alpha00, R beta0, double cfl, StepInfo* info,
                                      R* __restrict__ q_out, int advance_time) {
  const size_t ncell = size_t(ni) * nj;
  const R dt = global_dt<R>(info, cfl);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info->dt = double(dt);
    if (advance_time) info->t += double(dt);
  }
  const R dts = beta0 * dt;
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < ncell; c += size_t(gridDim.x) * blockDim.x) {
    const R fac = dts / vol[c];
#pragma unroll
    for (int v = 0; v < 3; ++v) q_out[v * ncell + c] = q0[v * ncell + c] + (R(0) + alpha00 * res0[v * ncell + c]) * fac;
  }
}

// ---- batched path (a batch of scalar-law instances; pools and work list as for the
// Euler batch, hc_kernels.cuh): each instance's slabs hold 4 state planes of which
// the law uses 3, and 5 residual planes of which it uses 4
template <class R, int NT> struct ScalarBatchResidency {
  static constexpr int value = (sizeof(R) == 4 ? 1024 : 512) / NT;
};

template <int TI, int TJ, class R, int FK>
__global__ void __launch_bounds__(TI * TJ, (ScalarBatchResidency<R, TI * TJ>::value))
    batch_scalar_stage_kernel(const BatchArgs<R> b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ StageArgs<R> sa;
  __shared__ int tile_ij[2];
  for (int w = blockIdx.x; w < b.nwork; w += gridDim.x) {
    __syncthreads();  // the previous work item may still read shared memory
    if (threadIdx.x == 0) {
      const int packed = b.order[w];
      const int k = packed >> 16, t = packed & 0xffff;
      const int tj = b.inst[k].tiles_j;
      sa = instance_args(b, k);
      tile_ij[0] = t / tj;
      tile_ij[1] = t % tj;
    }
    __syncthreads();
    scalar_stage_tile<TI, TJ, R, FK>(sa, tile_ij[0], tile_ij[1], smem_raw);
  }
}

// Stage-0 update of a scalar-law batch with each instance's own global dt
// (scalar_update0_kernel per work item)
template <int TI, int TJ, class R>
__global__ void __launch_bounds__(TI * TJ)
    batch_scalar_update0_kernel(const BatchArgs<R> b, double cfl, R alpha00, R beta0) {
  for (int w = blockIdx.x; w < b.nwork; w += gridDim.x) {
    const int packed = b.order[w];
    const int k = packed >> 16, t = packed & 0xffff;
    const BatchInst& in = b.inst[k];
    StepInfo* info = b.info + k;
    const R dt = global_dt<R>(info, cfl);
    if (t == 0 && threadIdx.x == 0) {
      info->dt = double(dt);
      info->t += double(dt);
    }
    const int bi = t / in.tiles_j, bj = t % in.tiles_j;
    const int gi = bi * TI + int(threadIdx.x) / TJ, gj = bj * TJ + int(threadIdx.x) % TJ;
    if (gi >= in.ni || gj >= in.nj) continue;
    const size_t ncell = size_t(in.ni) * in.nj;
    const size_t c = size_t(gi) * in.nj + gj;
    const R* q0 = b.q0 + 4 * in.cell;
    const R* res0 = b.res_out + 5 * in.cell;
    R* q_out = b.q_out + 4 * in.cell;
    const R fac = (beta0 * dt) / b.vol[in.cell + c];
#pragma unroll
    for (int v = 0; v < 3; ++v) q_out[v * ncell + c] = q0[v * ncell + c] + (R(0) + alpha00 * res0[v * ncell + c]) * fac;
  }
}

}  // namespace hc
