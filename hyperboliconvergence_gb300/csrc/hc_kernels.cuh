// hc_kernels.cuh -- CUDA kernels of the residual-and-timestep path.
//
//  * geometry kernels (once per mesh, always FP64): cell volumes/centres,
//    face normals/areas, least-squares metrics folded into per-face weights;
//  * stage kernel: one RK stage fused -- qmetric (LSQ) of every cell of a
//    halo tile, MUSCL reconstruction with the limiter, the face flux, face to
//    cell accumulation, and either the spectral-radius reduction (global dt,
//    stage 0) or the alpha/beta RK update (spatial/eulerForwardUpdate.h:38-168);
//  * update kernel: the stage-0 update once the global dt is known.
//
// Layouts in HBM (all SoA, cell (i,j) at i*nj+j, j fastest):
//   state      4 planes of ni*nj primitive values {u, v, rho, p}
//   residual   5 planes: 4 conserved flux sums + spectral-radius sum
//   i-faces    FREC planes of (ni+1)*nj records, face (i,j) between cells (i-1,j),(i,j)
//   j-faces    FREC planes of ni*(nj+1) records, face (i,j) between cells (i,j-1),(i,j)
#pragma once

#include "hc_physics.cuh"

#include <cuda.h>  // CUtensorMap (the tensor-map type of the TMA-staged FP32 stage kernel)

#include <cstdint>
#include <type_traits>

namespace hc {

// face record fields
enum FaceField { F_NX = 0, F_NY, F_A, F_DL, F_DR, F_IDLR, F_WLX, F_WLY, F_SL, F_WRX, F_WRY, F_SR, F_DXX, F_DXY,
                 FREC };

// Per-step scalars shared by the kernels of one RK step (device memory).
struct StepInfo {
  unsigned long long maxrate;  // max over cells of lambda/V as the bit pattern of a positive double
  double dt;                   // global timestep of the current step
  double t;                    // accumulated time
  int status;                  // 0 ok, 1 non-physical state produced
  int bad_cell;                // first cell found non-physical
  double resnorm2;             // sum over cells of the stage-0 density residual squared
};

// Status codes of the device-side checks
enum { ST_OK = 0, ST_NONPHYSICAL = 1, ST_TIMEOUT = 2 };

template <class R> struct StageArgs {
  int ni, nj;
  int bc[4];
  Gas<R> gas;
  int limiter;
  const R* q;         // input stage state
  const R* q0;        // state at the start of the step
  const R* fi;        // i-face records
  const R* fj;        // j-face records
  const void* fic;    // i-face records in the compute type when it differs from R
  const void* fjc;    // j-face records in the compute type when it differs from R
  const R* vol;       // cell volumes
  const R* gref[4];   // per side: far-field/fixed values in the solution basis, 4 planes of nface
  R* res_out;         // residual of this stage (5 planes) or null
  const R* res_prev[4];  // residuals of earlier stages (flux planes)
  R alpha[4];         // alpha[s][0..s]
  int stage;
  int mode;           // MODE_*
  R beta, cfl;
  StepInfo* info;
  R* q_out;           // next stage state (fused modes)
  int norm_stage0;    // accumulate the density-residual norm
  int basis;          // solution basis: 0 primitive, 1 conserved
  unsigned long long* sig_i;  // branch signatures of the i-faces / j-faces (recording kernels only)
  unsigned long long* sig_j;
  double* arg_i;              // with them (or null): the 8 limiter calls' (a, b) per face, 16 values
  double* arg_j;
  // dual time (null dual_src: off): the residual becomes dual_g0 R(q) - V dual_b0dt Q(q) +
  // dual_src, Q the conserved set, dual_src (4 planes) the earlier time levels' terms
  const R* dual_src;
  R dual_g0, dual_b0dt;
  int stall_copy;  // test hook (hc_inject_stalled_copy): the TMA-staged tile's records barrier
                   // expects 16 bytes its copy never delivers, so the bounded wait runs out
  int plain_loads; // host side: 1 keeps the FP32 launch on the plain-load kernel (hc_set_staged_loads)
};

// Branch signature of one face (recording kernels): bits 0-15 the limiter pieces of
// the left side's four variables (limit_piece, 4 bits each), 16-31 the right side's,
// 32-35 the flux branches (flux_bits), 36-37 the far-field path of a ghost face,
// 63 set when the face was evaluated.
enum : unsigned { SIG_FLUX_SHIFT = 32, SIG_BC_SHIFT = 36, SIG_VALID_SHIFT = 63 };

enum { MODE_RESIDUAL = 0, MODE_RES_MAXRATE = 1, MODE_FUSED_GLOBAL = 2, MODE_FUSED_LOCAL = 3 };

template <class R> __global__ void convert_kernel(const double* __restrict__ a, R* __restrict__ b, size_t n) {
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x)
    b[k] = R(a[k]);
}

// ---------------------------------------------------------------- stage kernel
// ---- TMA and mbarrier primitives (inline PTX) of the TMA-staged FP32 stage kernel
__device__ __forceinline__ unsigned smem_u32(const void* p) { return static_cast<unsigned>(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// a 3D box of the tensor map at (x, y, z) into shared memory, completing on bar
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wait for phase 0 of bar for at most one second: a copy that never lands marks the step
// ST_TIMEOUT (the host returns HC_ERR_TIMEOUT) instead of hanging the GPU
constexpr unsigned long long kCopyWaitNs = 1000000000ull;
__device__ __forceinline__ void mbar_wait_bounded(uint64_t* bar, StepInfo* info) {
  if (mbar_try_wait(bar, 0)) return;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, 0)) {
    if (globaltimer_ns() - t0 > kCopyWaitNs) {
      atomicCAS(&info->status, ST_OK, ST_TIMEOUT);
      return;
    }
  }
}

template <int TI, int TJ, class R> struct StageSmem {
  static constexpr int QI = TI + 4, QJ = TJ + 4;   // state tile with a 2-cell halo
  static constexpr int MI = TI + 2, MJ = TJ + 2;   // qmetric tile with a 1-cell halo
  static constexpr size_t q_elems = size_t(4) * QI * QJ;
  static constexpr size_t m_elems = size_t(8) * MI * MJ;
  static constexpr size_t fi_elems = size_t(5) * (TI + 1) * TJ;
  static constexpr size_t fj_elems = size_t(5) * TI * (TJ + 1);
  static constexpr size_t bytes = (q_elems + m_elems + fi_elems + fj_elems) * sizeof(R);
};

// Shared memory of the TMA-staged tile (FP32 or FP64): the state tile as the tensor copy lands
// it (rows of TJ + 8 values from column j0 - 4, so that each copy starts on a 16-byte
// boundary), the qmetric tile, the i-face records' first TMA_FIELDS fields (each face's fluxes
// later overwrite the first five fields of its own record), the j-face fluxes.
constexpr int TMA_FIELDS = 12;  // F_NX..F_SR: the fields the face phase reads
template <int TI, int TJ, class C = float> struct StageSmemTma {
  static constexpr int QI = TI + 4, QJ = TJ + 8;
  static constexpr size_t q_elems = size_t(4) * QI * QJ;
  static constexpr size_t m_elems = size_t(8) * (TI + 2) * (TJ + 2);
  static constexpr size_t ri_elems = size_t(TMA_FIELDS) * (TI + 1) * TJ;
  static constexpr size_t fj_elems = size_t(5) * TI * (TJ + 1);
  static constexpr size_t ri_offset = (q_elems + m_elems) * sizeof(C);
  static constexpr size_t bytes = (q_elems + m_elems + ri_elems + fj_elems) * sizeof(C);
  static_assert(ri_offset % 128 == 0, "the i-face records' tensor copy lands on a 128-byte boundary");
};

__device__ __forceinline__ int wrapi(int a, int n) {
  a %= n;
  return a < 0 ? a + n : a;
}

template <class R> __device__ __forceinline__ void atomic_max_rate(StepInfo* info, R v);
template <> __device__ __forceinline__ void atomic_max_rate<double>(StepInfo* info, double v) {
  if (v > 0.0) atomicMax(&info->maxrate, (unsigned long long)__double_as_longlong(v));
}
template <> __device__ __forceinline__ void atomic_max_rate<float>(StepInfo* info, float v) {
  const double d = double(v);
  if (d > 0.0) atomicMax(&info->maxrate, (unsigned long long)__double_as_longlong(d));
}

template <class R> __device__ __forceinline__ void flag_nonphysical(StepInfo* info, const R* q, int cell) {
  const bool bad = !(q[2] > R(0)) || !(q[3] > R(0)) || !isfinite(q[0]) || !isfinite(q[1]);
  if (bad) {
    if (atomicCAS(&info->status, ST_OK, ST_NONPHYSICAL) == ST_OK) info->bad_cell = cell;
  }
}

// cons(q0) + tot*fac -> solution basis (spatial/eulerForwardUpdate.h:76-85); a conserved
// field is its own conserved set (set2Set of the same type copies)
template <class R> __device__ __forceinline__ void forward_update(const Gas<R>& g, const R* q0, const R* tot, R fac,
                                                                  R* qn, bool cons) {
  if (cons) {
#pragma unroll
    for (int v = 0; v < 4; ++v) qn[v] = q0[v] + tot[v] * fac;
    return;
  }
  // conserved set of q0: r u, r v, r, r h - p = p/(gamma-1) + r |u|^2/2
  R qc[4];
  R u2 = q0[0] * q0[0];
  u2 += q0[1] * q0[1];
  qc[0] = q0[2] * q0[0]; qc[1] = q0[2] * q0[1]; qc[2] = q0[2];
  qc[3] = fma(q0[3], g.gamma1, q0[2] * (R(0.5) * u2));  // one contraction, whatever the kernel
#pragma unroll
  for (int v = 0; v < 4; ++v) qc[v] = qc[v] + tot[v] * fac;
  const St<R> s1 = cons_state(g, qc);
  qn[0] = s1.u; qn[1] = s1.v; qn[2] = s1.r; qn[3] = s1.p;
}

// the conserved set of a state in the solution basis
template <class R> __device__ __forceinline__ void basis_to_cons(const Gas<R>& g, const R* q, R* qc, bool cons) {
  if (cons) {
#pragma unroll
    for (int v = 0; v < 4; ++v) qc[v] = q[v];
    return;
  }
  R u2 = q[0] * q[0];
  u2 += q[1] * q[1];
  qc[0] = q[2] * q[0]; qc[1] = q[2] * q[1]; qc[2] = q[2];
  qc[3] = fma(q[3], g.gamma1, q[2] * (R(0.5) * u2));
}

// conversions between the storage type R and the compute type C of a stage
template <class To, class From> __device__ __forceinline__ To cvt(From x) { return To(x); }
template <> __device__ __forceinline__ double cvt<double, df64>(df64 x) { return x.to_double(); }
template <class C, class R> __device__ __forceinline__ Gas<C> gas_as(const Gas<R>& g) {
  Gas<C> o;
  o.gamma = cvt<C>(g.gamma); o.gm1 = cvt<C>(g.gm1); o.gamma1 = cvt<C>(g.gamma1);
  o.Rgas = cvt<C>(g.Rgas); o.minf = cvt<C>(g.minf); o.inv_gamma = cvt<C>(g.inv_gamma);
  o.lref_dt = cvt<C>(g.lref_dt); o.vscale = g.vscale; o.pscale = g.pscale; o.fixes = g.fixes;
  return o;
}

// One tile (TI x TJ cells, tile coordinates (bi, bj)) of one RK stage.  Called
// by every thread of the block; smem_raw holds StageSmem<TI,TJ,C>::bytes.
// R is the storage type (state, residuals, update); C the type the tile's
// gradients, reconstruction and fluxes are computed in (C = R, or double-float
// for FP64 storage, reading the face records from a.fic / a.fjc).
// REC: the recording instantiation also writes each face's branch signature to
// a.sig_i / a.sig_j (the production instantiations compile without it).  DUAL: dual-time
// terms are honoured (the batched instantiations, which have none, compile without them).
// LIM >= 0: the limiter is that compile-time constant (a.limiter must equal it), so its
// selection folds away; -1: a.limiter chosen at run time.
// TMA: the FP32 tile whose state tile (interior tiles) and i-face records arrive by tensor
// copies (tq, tfi; bars two mbarriers in shared memory), see stage_kernel_tma.
template <int TI, int TJ, class R, int FK, class C = R, bool REC = false, bool DUAL = true, int NTH = TI * TJ,
          int LIM = -1, bool TMA = false>
__device__ __forceinline__ void stage_tile(const StageArgs<R>& a, int bi, int bj, unsigned char* smem_raw,
                                           const CUtensorMap* tq = nullptr, const CUtensorMap* tfi = nullptr,
                                           uint64_t* bars = nullptr) {
  constexpr bool same = std::is_same<C, R>::value;
  using SM = StageSmem<TI, TJ, C>;
  static_assert(!TMA || std::is_same<C, R>::value, "the TMA-staged tile computes in its storage type");
  constexpr int QJT = TMA ? TJ + 8 : SM::QJ;  // row length of the state tile in shared memory
  constexpr int QSH = TMA ? 2 : 0;            // its column shift (the halo's column 0 at QSH)
  C* sq = reinterpret_cast<C*>(smem_raw);
  C* sm = sq + size_t(4) * SM::QI * QJT;
  C* sfi = sm + SM::m_elems;
  C* sfj = sfi + (TMA ? size_t(TMA_FIELDS) * (TI + 1) * TJ : SM::fi_elems);
  const C* cfi = same ? reinterpret_cast<const C*>(a.fi) : reinterpret_cast<const C*>(a.fic);
  const C* cfj = same ? reinterpret_cast<const C*>(a.fj) : reinterpret_cast<const C*>(a.fjc);
  constexpr int QI = SM::QI, QJ = SM::QJ, MI = SM::MI, MJ = SM::MJ;
  constexpr int NT = NTH;  // threads of the block: TI*TJ, or a divisor of it (several cells per thread)
  static_assert((TI * TJ) % NTH == 0 && NTH % 32 == 0, "threads must divide the tile's cells in whole warps");
  const int ni = a.ni, nj = a.nj;
  const size_t ncell = size_t(ni) * nj;
  const int i0 = bi * TI, j0 = bj * TJ;
  const int tid = threadIdx.x;
  const bool per_i = a.bc[0] == BC_PERIODIC, per_j = a.bc[2] == BC_PERIODIC;
  const int nfi = (ni + 1) * nj, nfj = ni * (nj + 1);

  // ---- phase 1: state tile with a 2-cell halo (periodic sides wrap)
  // A tile whose halo lies inside the mesh needs no wrap, bounds or pair-face tests in
  // phases 1-2 (uniform per block).  FP32 only: the FP64 stage is bound by its FP64 pipe
  // and gains nothing from fewer integer instructions.  Same sums in the same order.
  const bool interior =
      (std::is_same<C, float>::value || TMA) && i0 >= 2 && i0 + TI + 2 <= ni && j0 >= 2 && j0 + TJ + 2 <= nj;
  // TMA: one thread arms the two barriers and issues the tensor copies -- the interior tile's
  // state (4 planes x (TI + 4) rows x (TJ + 8) columns from (i0 - 2, j0 - 4); columns past the
  // mesh read zeros and are never used) and the i-face records (TMA_FIELDS fields x (TI + 1)
  // rows x TJ columns from (i0, j0); rows or columns past the mesh belong to no valid face);
  // they land while the threads run the halo and qmetric phases
  bool tma = false;
  if constexpr (TMA) {
    tma = tq != nullptr && tfi != nullptr && (smem_u32(sq) % 128u) == 0 && (smem_u32(sfi) % 128u) == 0;
    if (tma) {
      if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
      }
      __syncthreads();
      if (tid == 0) {
        // the block's earlier accesses to this shared memory (a persistent CTA's previous
        // work item) before the tensor copies overwrite it
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        if (interior) {
          mbar_expect_tx(&bars[0], unsigned(4 * QI * QJT * sizeof(C)));
          tma_load_3d(sq, tq, j0 - 4, i0 - 2, 0, &bars[0]);
        }
        mbar_expect_tx(&bars[1], unsigned(TMA_FIELDS * (TI + 1) * TJ * sizeof(C)) + (a.stall_copy ? 16u : 0u));
        tma_load_3d(sfi, tfi, j0, i0, 0, &bars[1]);
      }
    }
  }
  if (tma && interior) {
    mbar_wait_bounded(&bars[0], a.info);
  } else if (interior) {
    const R* qb = a.q + (size_t(i0 - 2) * nj + (j0 - 2));
    for (int k = tid; k < QI * QJ; k += NT) {
      const int la = k / QJ, lb = k % QJ;
      const size_t c = size_t(la) * nj + lb;
#pragma unroll
      for (int v = 0; v < 4; ++v) sq[(v * QI + la) * QJT + lb + QSH] = cvt<C>(qb[v * ncell + c]);
    }
  } else {
    for (int k = tid; k < QI * QJ; k += NT) {
      const int la = k / QJ, lb = k % QJ;
      int gi = i0 - 2 + la, gj = j0 - 2 + lb;
      bool ok = true;
      if (gi < 0 || gi >= ni) { if (per_i) gi = wrapi(gi, ni); else ok = false; }
      if (gj < 0 || gj >= nj) { if (per_j) gj = wrapi(gj, nj); else ok = false; }
      const size_t c = size_t(gi) * nj + gj;
#pragma unroll
      for (int v = 0; v < 4; ++v) sq[(v * QI + la) * QJT + lb + QSH] = ok ? cvt<C>(a.q[v * ncell + c]) : C(0);
    }
  }
  __syncthreads();

  auto Q = [&](int v, int la, int lb) -> C { return sq[(v * QI + la + 2) * QJT + lb + 2 + QSH]; };  // tile coords
  // the qmetric tile: FP32 keeps a cell's eight values as two float4 (the gradients of
  // variables 0-1, then 2-3), so that a face reads a cell's eight in two vector loads;
  // the other types keep one plane per value
  constexpr bool MV = std::is_same<C, float>::value;
  auto M = [&](int k, int la, int lb) -> C& {
    const int c = (la + 1) * MJ + lb + 1;
    return MV ? sm[((k >> 2) * MI * MJ + c) * 4 + (k & 3)] : sm[k * MI * MJ + c];
  };
  auto mload = [&](int la, int lb, C* m) {
    if constexpr (MV) {
      const float4* p = reinterpret_cast<const float4*>(sm) + (la + 1) * MJ + lb + 1;
      const float4 x = p[0], y = p[MI * MJ];
      m[0] = x.x; m[1] = x.y; m[2] = x.z; m[3] = x.w;
      m[4] = y.x; m[5] = y.y; m[6] = y.z; m[7] = y.w;
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) m[k] = M(k, la, lb);
    }
  };
  auto mstore = [&](int la, int lb, const C* m) {
    if constexpr (MV) {
      float4* p = reinterpret_cast<float4*>(sm) + (la + 1) * MJ + lb + 1;
      p[0] = make_float4(m[0], m[1], m[2], m[3]);
      p[MI * MJ] = make_float4(m[4], m[5], m[6], m[7]);
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) M(k, la, lb) = m[k];
    }
  };

  // ---- phase 2: qmetric of the tile cells and of the 1-cell halo strips
  // (lsq/qmetric.ipp via spatial/lsqMetrics.h:181-213; D2 periodic wrap)
  if (interior) {
    for (int k = tid; k < MI * MJ; k += NT) {
      const int la = k / MJ - 1, lb = k % MJ - 1;
      const bool corner = (la < 0 || la >= TI) && (lb < 0 || lb >= TJ);
      const int gi = i0 + la, gj = j0 + lb;
      C m[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) m[q] = C(0);
      if (!corner) {
        const int fi0 = gi * nj + gj, fj0 = gi * (nj + 1) + gj;
        const C dxi0 = cfi[size_t(F_DXX) * nfi + fi0], dyi0 = cfi[size_t(F_DXY) * nfi + fi0];
        const C dxi1 = cfi[size_t(F_DXX) * nfi + fi0 + nj], dyi1 = cfi[size_t(F_DXY) * nfi + fi0 + nj];
        const C dxj0 = cfj[size_t(F_DXX) * nfj + fj0], dyj0 = cfj[size_t(F_DXY) * nfj + fj0];
        const C dxj1 = cfj[size_t(F_DXX) * nfj + fj0 + 1], dyj1 = cfj[size_t(F_DXY) * nfj + fj0 + 1];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const C q0 = Q(v, la, lb);
          const C a0 = q0 - Q(v, la - 1, lb), a1 = Q(v, la + 1, lb) - q0;
          const C b0 = q0 - Q(v, la, lb - 1), b1 = Q(v, la, lb + 1) - q0;
          m[2 * v] += a0 * dxi0; m[2 * v + 1] += a0 * dyi0;
          m[2 * v] += a1 * dxi1; m[2 * v + 1] += a1 * dyi1;
          m[2 * v] += b0 * dxj0; m[2 * v + 1] += b0 * dyj0;
          m[2 * v] += b1 * dxj1; m[2 * v + 1] += b1 * dyj1;
        }
      }
      mstore(la, lb, m);
    }
  } else
  for (int k = tid; k < MI * MJ; k += NT) {
    const int la = k / MJ - 1, lb = k % MJ - 1;
    const bool corner = (la < 0 || la >= TI) && (lb < 0 || lb >= TJ);
    int gi = i0 + la, gj = j0 + lb;
    bool ok = !corner;
    if (gi < 0 || gi >= ni) { if (per_i) gi = wrapi(gi, ni); else ok = false; }
    if (gj < 0 || gj >= nj) { if (per_j) gj = wrapi(gj, nj); else ok = false; }
    C m[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) m[q] = C(0);
    if (ok) {
      // the cell's four faces: (face index, neighbour offset, is pair face)
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
        const C* rec = idir ? cfi : cfj;
        const int nf = idir ? nfi : nfj;
        const C dx = rec[size_t(F_DXX) * nf + fidx], dy = rec[size_t(F_DXY) * nf + fidx];
        const int na = la + (idir ? (hi ? 1 : -1) : 0), nb = lb + (idir ? 0 : (hi ? 1 : -1));
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          // (q_right - q_left) of the face
          const C dq = hi ? (Q(v, na, nb) - Q(v, la, lb)) : (Q(v, la, lb) - Q(v, na, nb));
          m[2 * v] += dq * dx;
          m[2 * v + 1] += dq * dy;
        }
      }
    }
    mstore(la, lb, m);
  }
  if (tma) mbar_wait_bounded(&bars[1], a.info);
  __syncthreads();

  // ---- phase 3: face fluxes (i-faces then j-faces of the tile, each once)
  const Gas<C> g = gas_as<C>(a.gas);
  const bool cons = a.basis != 0;  // conserved solution basis
  const int lim = LIM >= 0 ? LIM : a.limiter;
  constexpr int NFI = (TI + 1) * TJ, NFJ = TI * (TJ + 1);
  // one face: i-face kk (dir true) or j-face kk of the tile; dir is a bool, or a
  // std::integral_constant that makes the direction a compile-time constant
  auto face_body = [&](auto dir, const int kk) {
    const bool idir = static_cast<bool>(dir);
    // local coordinates of the face's right cell
    const int la = idir ? kk / TJ : kk / (TJ + 1), lb = idir ? kk % TJ : kk % (TJ + 1);
    const int gi = i0 + la, gj = j0 + lb;
    bool valid = idir ? (gi <= ni && gj < nj) : (gi < ni && gj <= nj);
    Flux5<C> F;
    F.f[0] = F.f[1] = F.f[2] = F.f[3] = F.lam = C(0);
    unsigned long long sg = 0;  // branch signature (REC)
    if (valid) {
      const C* rec = idir ? cfi : cfj;
      const int nf = idir ? nfi : nfj;
      const int fidx = idir ? gi * nj + gj : gi * (nj + 1) + gj;
      auto rd = [&](int fld) -> C {
        if constexpr (TMA) {
          if (idir && tma) return sfi[fld * NFI + la * TJ + lb];  // the tensor-copied i-face records
        }
        return rec[size_t(fld) * nf + fidx];
      };
      const C nx = rd(F_NX), ny = rd(F_NY), A = rd(F_A);
      const int lo = idir ? gi : gj, nalong = idir ? ni : nj;
      const int side = idir ? (lo == 0 ? 0 : 1) : (lo == 0 ? 2 : 3);
      const bool bnd = (lo == 0 || lo == nalong) && a.bc[side] != BC_PERIODIC;
      const int la_l = idir ? la - 1 : la, lb_l = idir ? lb : lb - 1;  // left cell
      if (!bnd) {
        C ql[4], qr[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) { ql[v] = Q(v, la_l, lb_l); qr[v] = Q(v, la, lb); }
        if (lim != LIM_NOLIMIT1) {
          const C dl = rd(F_DL), dr = rd(F_DR), idlr = rd(F_IDLR);
          const C wlx = rd(F_WLX), wly = rd(F_WLY), sl = rd(F_SL);
          const C wrx = rd(F_WRX), wry = rd(F_WRY), sr = rd(F_SR);
          C qL[4], qR[4];
          if constexpr (std::is_same<C, double>::value) {
            // FP64: the four variables of each side share the limiter's division
            C gc[4], gl[4], gr[4], sL[4], sR[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              const C dq = qr[v] - ql[v];
              gc[v] = dq * idlr;
              gl[v] = (M(2 * v, la_l, lb_l) * wlx + M(2 * v + 1, la_l, lb_l) * wly) - dq * sl;
              gr[v] = (M(2 * v, la, lb) * wrx + M(2 * v + 1, la, lb) * wry) - dq * sr;
            }
            limit4x2(lim, gc, gl, gr, sL, sR);
            if constexpr (REC) {
              double* ag = a.arg_i ? (idir ? a.arg_i + size_t(16) * fidx : a.arg_j + size_t(16) * fidx) : nullptr;
#pragma unroll
              for (int v = 0; v < 4; ++v) {
                sg |= ((unsigned long long)limit_piece<C>(lim, gc[v], gl[v]) << (4 * v)) |
                      ((unsigned long long)limit_piece<C>(lim, gc[v], gr[v]) << (16 + 4 * v));
                if (ag) {
                  ag[2 * v] = cvt<double>(gc[v]); ag[2 * v + 1] = cvt<double>(gl[v]);
                  ag[8 + 2 * v] = cvt<double>(gc[v]); ag[9 + 2 * v] = cvt<double>(gr[v]);
                }
              }
            }
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              qL[v] = ql[v] + dl * sL[v];
              qR[v] = qr[v] - dr * sR[v];
            }
          } else {
            C ml[8], mr[8];
            mload(la_l, lb_l, ml);
            mload(la, lb, mr);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              const C dq = qr[v] - ql[v];
              const C gc = dq * idlr;
              const C gl = (ml[2 * v] * wlx + ml[2 * v + 1] * wly) - dq * sl;
              const C gr = (mr[2 * v] * wrx + mr[2 * v + 1] * wry) - dq * sr;
              qL[v] = ql[v] + dl * limit<C>(lim, gc, gl);
              qR[v] = qr[v] - dr * limit<C>(lim, gc, gr);
              if constexpr (REC) {
                sg |= ((unsigned long long)limit_piece<C>(lim, gc, gl) << (4 * v)) |
                      ((unsigned long long)limit_piece<C>(lim, gc, gr) << (16 + 4 * v));
                if (a.arg_i) {
                  double* ag = idir ? a.arg_i + size_t(16) * fidx : a.arg_j + size_t(16) * fidx;
                  ag[2 * v] = cvt<double>(gc); ag[2 * v + 1] = cvt<double>(gl);
                  ag[8 + 2 * v] = cvt<double>(gc); ag[9 + 2 * v] = cvt<double>(gr);
                }
              }
            }
          }
          if constexpr (REC) {
            St<C> sL, sR;
            basis_state2(g, qL, qR, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
            sg |= (unsigned long long)flux_bits<C, FK>(g, nx, ny, sL, sR) << SIG_FLUX_SHIFT;
          } else {
            St<C> sL, sR;
            basis_state2(g, qL, qR, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
          }
        } else {
          if constexpr (REC) {
            St<C> sL, sR;
            basis_state2(g, ql, qr, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
            sg |= (unsigned long long)flux_bits<C, FK>(g, nx, ny, sL, sR) << SIG_FLUX_SHIFT;
          } else {
            St<C> sL, sR;
            basis_state2(g, ql, qr, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
          }
        }
      } else {
        // boundary face: interior cell is the right cell on sides 0/2, the left on 1/3
        const bool int_right = lo == 0;
        const int ia = int_right ? la : la_l, ib = int_right ? lb : lb_l;
        C qi[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) qi[v] = Q(v, ia, ib);
        const int kf = idir ? gj : gi;  // face index along the side
        const int bct = a.bc[side];
        if (bct == BC_WALL) {
          const C wx = int_right ? rd(F_WLX) : rd(F_WRX), wy = int_right ? rd(F_WLY) : rd(F_WRY);
          C qw[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) qw[v] = qi[v] - (M(2 * v, ia, ib) * wx + M(2 * v + 1, ia, ib) * wy);
          F = wall_flux(g, nx, ny, A, qw, cons);
        } else {
          const int nfs = idir ? nj : ni;
          C qg[4];
          // ghost state in the storage type (the far-field updates call pow)
          R qref[4], qgr[4], qir[4];
#pragma unroll
          for (int v = 0; v < 4; ++v) { qref[v] = a.gref[side][size_t(v) * nfs + kf]; qir[v] = cvt<R>(qi[v]); }
          const R sgn = int_right ? R(1) : R(-1);  // normal into the domain
          const R nxr = cvt<R>(nx), nyr = cvt<R>(ny);
          unsigned path = 0;
          unsigned* pathp = REC ? &path : nullptr;
          if (bct == BC_RIEMANN) {
            farfield_update<R, BC_RIEMANN>(a.gas, sgn * nxr, sgn * nyr, qir, qref, qgr, cons, pathp);
          } else if (bct == BC_ENTROPY) {
            farfield_update<R, BC_ENTROPY>(a.gas, sgn * nxr, sgn * nyr, qir, qref, qgr, cons, pathp);
          } else {
#pragma unroll
            for (int v = 0; v < 4; ++v) qgr[v] = qref[v];
          }
          if constexpr (REC) sg |= (unsigned long long)path << SIG_BC_SHIFT;
#pragma unroll
          for (int v = 0; v < 4; ++v) qg[v] = cvt<C>(qgr[v]);
          C qL[4], qR[4];
          if (lim != LIM_NOLIMIT1) {
            const C d = rd(F_DL), idlr = rd(F_IDLR);
            const C wx = int_right ? rd(F_WRX) : rd(F_WLX), wy = int_right ? rd(F_WRY) : rd(F_WLY);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              const C dq = int_right ? (qi[v] - qg[v]) : (qg[v] - qi[v]);
              const C gb = M(2 * v, ia, ib) * wx + M(2 * v + 1, ia, ib) * wy;
              const C s = limit<C>(lim, dq * idlr, gb);
              if (int_right) { qL[v] = qg[v]; qR[v] = qi[v] - d * s; }
              else { qL[v] = qi[v] + d * s; qR[v] = qg[v]; }
              if constexpr (REC) {  // the interior side's limiter, in its side's slot
                sg |= (unsigned long long)limit_piece<C>(lim, dq * idlr, gb) << ((int_right ? 16 : 0) + 4 * v);
                if (a.arg_i) {
                  double* ag = (idir ? a.arg_i : a.arg_j) + size_t(16) * fidx + (int_right ? 8 : 0);
                  ag[2 * v] = cvt<double>(dq * idlr); ag[2 * v + 1] = cvt<double>(gb);
                }
              }
            }
          } else {
#pragma unroll
            for (int v = 0; v < 4; ++v) { qL[v] = int_right ? qg[v] : qi[v]; qR[v] = int_right ? qi[v] : qg[v]; }
          }
          if constexpr (REC) {
            St<C> sL, sR;
            basis_state2(g, qL, qR, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
            sg |= (unsigned long long)flux_bits<C, FK>(g, nx, ny, sL, sR) << SIG_FLUX_SHIFT;
          } else {
            St<C> sL, sR;
            basis_state2(g, qL, qR, cons, sL, sR);
            F = face_flux<C, FK>(g, nx, ny, A, sL, sR);
          }
        }
      }
      if constexpr (REC) {
        const int fidx_s = idir ? gi * nj + gj : gi * (nj + 1) + gj;
        (idir ? a.sig_i : a.sig_j)[fidx_s] = sg | (1ull << SIG_VALID_SHIFT);
      }
    }
    C* dst = idir ? sfi : sfj;
    const int slot = idir ? (la * TJ + lb) : (la * (TJ + 1) + lb);
    const int pl = idir ? NFI : NFJ;
#pragma unroll
    for (int v = 0; v < 4; ++v) dst[v * pl + slot] = F.f[v];
    dst[4 * pl + slot] = F.lam;
  };
  // the i-faces then the j-faces, dealt round-robin to the threads as one list.  FP32: a
  // body per direction (the branch is uniform in every warp wholly inside one direction's
  // range; the issue-bound FP32 kernel saves the direction's selects); FP64 and
  // double-float: one body with the direction a run-time value (two bodies measured 4%
  // slower in the FP64-pipe-bound FP64 kernel)
  for (int k = tid; k < NFI + NFJ; k += NT) {
    if constexpr (std::is_same<C, float>::value) {
      if (k < NFI) face_body(std::true_type{}, k);
      else face_body(std::false_type{}, k - NFI);
    } else {
      const bool d = k < NFI;
      face_body(d, d ? k : k - NFI);
    }
  }
  __syncthreads();

  // ---- phase 4: accumulate to cells (residualCalc.h:199-253 signs) and update; with
  // fewer threads than cells each thread takes cells tid, tid + NT, ... (whole warps per
  // pass, so the warp reductions below see every lane)
  auto cell_update = [&](const int cidx) {
  const int la = cidx / TJ, lb = cidx % TJ;
  const int gi = i0 + la, gj = j0 + lb;
  const bool own = gi < ni && gj < nj;
  R res[4], lam = R(0);
  if (own) {
    const int s0 = la * TJ + lb, s1 = (la + 1) * TJ + lb;
    const int t0 = la * (TJ + 1) + lb, t1 = t0 + 1;
#pragma unroll
    for (int v = 0; v < 4; ++v)
      res[v] = cvt<R>(((sfi[v * NFI + s0] - sfi[v * NFI + s1]) + sfj[v * NFJ + t0]) - sfj[v * NFJ + t1]);
    lam = cvt<R>(((sfi[4 * NFI + s0] + sfi[4 * NFI + s1]) + sfj[4 * NFJ + t0]) + sfj[4 * NFJ + t1]);
  }
  const size_t c = size_t(gi) * nj + gj;
  if (DUAL && own && a.dual_src) {
    // dual time (ode.h:12-82, OLD.fieldOperations/dualTimeResidual.ipp): the physical-time
    // terms of the current iterate and of the earlier levels join the flux residual
    R qk[4], qc[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) qk[v] = a.q[v * ncell + c];
    basis_to_cons(a.gas, qk, qc, a.basis != 0);
    const R vb = a.vol[c] * a.dual_b0dt;
#pragma unroll
    for (int v = 0; v < 4; ++v) res[v] = a.dual_g0 * res[v] + (a.dual_src[v * ncell + c] - vb * qc[v]);
  }
  if (own && a.res_out) {
#pragma unroll
    for (int v = 0; v < 4; ++v) a.res_out[v * ncell + c] = res[v];
    a.res_out[4 * ncell + c] = lam;
  }
  if (a.mode == MODE_RES_MAXRATE) {
    // spectralRadius: max over cells of lambda/V (spatial/spectralRadius.h:19-48)
    R rate = own ? lam / a.vol[c] : R(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
    if ((tid & 31) == 0) atomic_max_rate<R>(a.info, rate);
    if (a.norm_stage0) {
      R r2 = own ? res[2] * res[2] : R(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
      if ((tid & 31) == 0) atomicAdd(&a.info->resnorm2, double(r2));
    }
    return;
  }
  if (a.mode == MODE_RESIDUAL) return;
  if (a.norm_stage0 && a.stage == 0) {
    R r2 = own ? res[2] * res[2] : R(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 += __shfl_xor_sync(0xffffffffu, r2, o);
    if ((tid & 31) == 0) atomicAdd(&a.info->resnorm2, double(r2));
    if (a.mode == MODE_FUSED_LOCAL) {
      // largest lambda/V: the smallest local timestep is cfl over it
      R rate = own ? lam / a.vol[c] : R(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) rate = fmax(rate, __shfl_xor_sync(0xffffffffu, rate, o));
      if ((tid & 31) == 0) atomic_max_rate<R>(a.info, rate);
    }
  }
  if (!own) return;
  // rungeKuttaAccumulation (timestepping/rungeKutta.h:172-197)
  R tot[4] = {R(0), R(0), R(0), R(0)};
  for (int k = 0; k < a.stage; ++k)
#pragma unroll
    for (int v = 0; v < 4; ++v) tot[v] += a.alpha[k] * a.res_prev[k][v * ncell + c];
#pragma unroll
  for (int v = 0; v < 4; ++v) tot[v] += a.alpha[a.stage] * res[v];
  R fac;
  if (a.mode == MODE_FUSED_GLOBAL) {
    const R dts = a.beta * R(a.info->dt);
    fac = qdiv(dts, a.vol[c]);
  } else {
    // local timestep from the stage-0 spectral radius sum (eulerForwardUpdate.h:155-161)
    const R l0 = (a.stage == 0) ? lam : a.res_prev[0][4 * ncell + c];
    const R cs = a.beta * a.cfl;
    // dual time: dtau / (1 + b0 dtau / dt), the physical-time term's share of the spectral radius
    fac = (DUAL && a.dual_src) ? cs / (l0 + a.cfl * a.vol[c] * a.dual_b0dt) : qdiv(cs, l0);
  }
  R q0[4], qn[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) q0[v] = a.q0[v * ncell + c];
  forward_update(a.gas, q0, tot, fac, qn, a.basis != 0);
#pragma unroll
  for (int v = 0; v < 4; ++v) a.q_out[v * ncell + c] = qn[v];
  flag_nonphysical(a.info, qn, int(c));
  };
#pragma unroll 1
  for (int cidx = tid; cidx < TI * TJ; cidx += NT) cell_update(cidx);
}

// Resident CTAs per SM the stage kernel is compiled for (measured on the 512x1024
// O-grid, 256-thread tiles): FP64 2 (its 122 registers; a looser bound lets the
// compiler take more and costs 13%), double-float 3 and FP32 5 (latency-bound
// kernels: the extra warps outweigh the few spilled registers, 10-12% faster).
template <class R, class C, int NT> struct StageResidency {
  static constexpr int value = std::is_same<R, float>::value ? 1280 / NT
                               : (std::is_same<C, R>::value ? 512 / NT : 768 / NT);
};

template <int TI, int TJ, class R, int FK, class C = R, int NT = TI * TJ, int LIM = -1>
__global__ void __launch_bounds__(NT, (StageResidency<R, C, NT>::value))
    stage_kernel(const StageArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_tile<TI, TJ, R, FK, C, false, true, NT, LIM>(a, blockIdx.y, blockIdx.x, smem_raw);
}

// The FP32 8x32 tile with its loads staged by the Tensor Memory Accelerator: the interior
// tile's state and every tile's i-face records arrive by cp.async.bulk.tensor copies on
// mbarriers, issued by one thread at the start, while the threads load the halo of edge
// tiles and form the qmetric; the j-face records and the earlier stages' residuals stay
// plain loads (the j-face planes' row pitch, (nj + 1) values, is not a multiple of 16 bytes).
// The tensor maps are kernel parameters (encoded per launch by the launcher, hc_tma.h).
template <int TI, int TJ, class R, int FK, int LIM, int NT = TI * TJ>
__global__ void __launch_bounds__(NT, (StageResidency<R, R, NT>::value))
    stage_kernel_tma(const StageArgs<R> a, const __grid_constant__ CUtensorMap tq,
                     const __grid_constant__ CUtensorMap tfi) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + StageSmemTma<TI, TJ, R>::bytes);
  stage_tile<TI, TJ, R, FK, R, false, true, NT, LIM, true>(a, blockIdx.y, blockIdx.x, smem_raw, &tq, &tfi, bars);
}

// the recording variant (a diagnostic, not on the stepping path): the same tile with
// each face's branch signature written out
template <int TI, int TJ, class R, int FK, class C = R>
__global__ void __launch_bounds__(TI * TJ) sig_kernel(const StageArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  stage_tile<TI, TJ, R, FK, C, true>(a, blockIdx.y, blockIdx.x, smem_raw);
}

// Stage-0 update of one cell with the global timestep dt = cfl / max(lambda/V)
// (timestepping/rungeKutta.h:131-154).
template <class R>
__device__ __forceinline__ void update0_cell(size_t c, size_t ncell, const Gas<R>& g, const R* __restrict__ q0,
                                             const R* __restrict__ res0, const R* __restrict__ vol, R alpha00,
                                             R dts, StepInfo* info, R* __restrict__ q_out, bool cons) {
  R tot[4], q[4], qn[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    tot[v] = R(0) + alpha00 * res0[v * ncell + c];
    q[v] = q0[v * ncell + c];
  }
  const R fac = dts / vol[c];
  forward_update(g, q, tot, fac, qn, cons);
#pragma unroll
  for (int v = 0; v < 4; ++v) q_out[v * ncell + c] = qn[v];
  flag_nonphysical(info, qn, int(c));
}

template <class R> __device__ __forceinline__ R global_dt(const StepInfo* info, double cfl) {
  const double rate = fmax(DBL_MIN, __longlong_as_double((long long)info->maxrate));
  return R(cfl / rate);
}
__host__ __device__ __forceinline__ double dual_step(double dtau, double b0dt) { return dtau / (1.0 + b0dt * dtau); }

template <class R>
__global__ void update0_kernel(int ni, int nj, Gas<R> g, const R* __restrict__ q0, const R* __restrict__ res0,
                               const R* __restrict__ vol, R alpha00, R beta0, double cfl, StepInfo* info,
                               R* __restrict__ q_out, int advance_time, int basis, double dual_b0dt) {
  const size_t ncell = size_t(ni) * nj;
  // dual time: the pseudo step dtau / (1 + b0 dtau / dt) (timestepping/dualTime.ipp:65-66)
  const R dt = dual_b0dt > 0.0 ? R(dual_step(double(global_dt<R>(info, cfl)), dual_b0dt)) : global_dt<R>(info, cfl);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    info->dt = double(dt);
    if (advance_time) info->t += double(dt);
  }
  const R dts = beta0 * dt;
  for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < ncell; c += size_t(gridDim.x) * blockDim.x)
    update0_cell(c, ncell, g, q0, res0, vol, alpha00, dts, info, q_out, basis != 0);
}

// ---------------------------------------------------------------- batched path
// Many independent meshes of uneven sizes advanced by one persistent launch per
// stage: the tiles of all instances form one work list that a grid of
// (SMs x ctas_per_sm) CTAs walks round-robin.  Per-instance data live at
// offsets in pooled buffers; each instance has its own StepInfo (global dt).
struct BatchInst {
  int ni, nj;
  int bc[4];
  int tiles_i, tiles_j;  // tile grid of this instance for the launch's tile shape
  long long cell;        // offset of the instance's cells in the cell pools
  long long fi, fj;      // offsets of its i-/j-face records (records, not values)
  long long gref[4];     // offsets of its ghost-reference planes (values)
};

template <class R> struct BatchArgs {
  const BatchInst* inst;
  const int* order;        // work list: packed (instance << 16 | tile index within the instance) entries
  int nwork;
  const int* tile_begin;   // not used by the kernels (host bookkeeping)
  Gas<R> gas;
  int limiter;
  const R* q;              // stage input pool
  const R* q0;
  R* q_out;
  R* res_out;
  const R* res_prev[4];
  const R* fi;
  const R* fj;
  const R* vol;
  const R* gref;
  R alpha[4];
  int stage, mode;
  R beta, cfl;
  StepInfo* info;          // one per instance
  int basis;               // solution basis: 0 primitive, 1 conserved
  // FP32 8x32 batches: per-instance tensor maps of the stage input buffer and of the i-face
  // records (device memory), or null (plain loads)
  const CUtensorMap* tmaps_q;
  const CUtensorMap* tmaps_fi;
};

template <class R> __device__ __forceinline__ StageArgs<R> instance_args(const BatchArgs<R>& b, int k) {
  const BatchInst& in = b.inst[k];
  StageArgs<R> a;
  a.ni = in.ni; a.nj = in.nj;
  for (int s = 0; s < 4; ++s) a.bc[s] = in.bc[s];
  a.gas = b.gas;
  a.limiter = b.limiter;
  a.basis = b.basis;
  a.sig_i = a.sig_j = nullptr;
  a.arg_i = a.arg_j = nullptr;
  a.dual_src = nullptr;  // batches have no dual time
  a.dual_g0 = R(1);
  a.dual_b0dt = R(0);
  a.stall_copy = 0;
  a.plain_loads = 0;
  a.fic = a.fjc = nullptr;  // batches compute in their storage type
  const long long n = (long long)in.ni * in.nj;
  const long long off4 = 4 * in.cell, off5 = 5 * in.cell;
  a.q = b.q + off4;
  a.q0 = b.q0 + off4;
  a.q_out = b.q_out ? b.q_out + off4 : nullptr;
  a.res_out = b.res_out ? b.res_out + off5 : nullptr;
  for (int s = 0; s < 4; ++s) a.res_prev[s] = b.res_prev[s] ? b.res_prev[s] + off5 : nullptr;
  const long long nfi = (long long)(in.ni + 1) * in.nj, nfj = (long long)in.ni * (in.nj + 1);
  (void)nfi; (void)nfj; (void)n;
  a.fi = b.fi + (long long)FREC * in.fi;
  a.fj = b.fj + (long long)FREC * in.fj;
  a.vol = b.vol + in.cell;
  for (int s = 0; s < 4; ++s) a.gref[s] = b.gref + in.gref[s];
  for (int s = 0; s < 4; ++s) a.alpha[s] = b.alpha[s];
  a.stage = b.stage;
  a.mode = b.mode;
  a.beta = b.beta;
  a.cfl = b.cfl;
  a.info = b.info + k;
  a.norm_stage0 = (b.stage == 0);
  return a;
}

// resident CTAs per SM the persistent kernel is compiled for (measured on the
// uneven 256-instance batch): FP32 4 -- 64 registers; its per-work-item loop
// spills more than the plain kernel at 5 CTAs/SM and runs 6% slower -- and FP64 2
template <class R, int NT> struct BatchResidency {
  static constexpr int value = (sizeof(R) == 4 ? 1024 : 512) / NT;
};

template <int TI, int TJ, class R, int FK, int LIM = -1>
__global__ void __launch_bounds__(TI * TJ, (BatchResidency<R, TI * TJ>::value))
    batch_stage_kernel(const BatchArgs<R> b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the work item's arguments live in shared memory, read field by field as the
  // tile needs them (a register or stack copy per thread costs occupancy)
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
    stage_tile<TI, TJ, R, FK, R, false, false, TI * TJ, LIM>(sa, tile_ij[0], tile_ij[1], smem_raw);
  }
}

// The persistent batch kernel with the TMA-staged FP32 8x32 tile (stage_kernel_tma): each
// work item's copies use its instance's tensor maps (b.tmaps_q, b.tmaps_fi); the tile
// re-arms its two mbarriers per item.
template <int FK, int LIM>
__global__ void __launch_bounds__(256, (BatchResidency<float, 256>::value))
    batch_stage_kernel_tma(const BatchArgs<float> b) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + StageSmemTma<8, 32>::bytes);
  __shared__ StageArgs<float> sa;
  __shared__ int item[3];  // instance, tile row, tile column
  for (int w = blockIdx.x; w < b.nwork; w += gridDim.x) {
    __syncthreads();  // the previous work item may still read shared memory
    if (threadIdx.x == 0) {
      const int packed = b.order[w];
      const int k = packed >> 16, t = packed & 0xffff;
      const int tj = b.inst[k].tiles_j;
      sa = instance_args(b, k);
      item[0] = k;
      item[1] = t / tj;
      item[2] = t % tj;
    }
    __syncthreads();
    const int k = item[0];
    stage_tile<8, 32, float, FK, float, false, false, 256, LIM, true>(sa, item[1], item[2], smem_raw,
                                                                      b.tmaps_q + k, b.tmaps_fi + k, bars);
  }
}

// Stage-0 update of the batch with each instance's own global dt.
template <int TI, int TJ, class R>
__global__ void __launch_bounds__(TI * TJ) batch_update0_kernel(const BatchArgs<R> b, double cfl, R alpha00, R beta0) {
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
    update0_cell(c, ncell, b.gas, b.q0 + 4 * in.cell, b.res_out + 5 * in.cell, b.vol + in.cell, alpha00,
                 beta0 * dt, info, b.q_out + 4 * in.cell, b.basis != 0);
  }
}

}  // namespace hc
