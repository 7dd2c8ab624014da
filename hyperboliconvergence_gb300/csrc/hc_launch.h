// hc_launch.h -- host-side launchers of the per-flux stage kernels.  Each
// flux is compiled in its own translation unit (hc_stage_<flux>.cu) so the
// build runs them in parallel.
#pragma once

#include "hc_kernels.cuh"
#include "hc_tma.h"

#include <algorithm>
#include <type_traits>
#include <vector>

namespace hc {

// Tile shapes the stage kernel is built for (cells along i x cells along j).
// TILE_16x16_H: 16 x 16 cells run by 128 threads (two cells a thread in the update)
enum TileShape { TILE_8x32 = 0, TILE_4x32 = 1, TILE_16x16 = 2, TILE_16x16_H = 3, TILE_COUNT = 4 };

template <class R, int FK> cudaError_t launch_stage(const StageArgs<R>& a, int tile, cudaStream_t s);
template <class R, int FK> cudaError_t prepare_stage();
// persistent batched stage: `grid` CTAs walk the work list of b
template <class R, int FK> cudaError_t launch_batch_stage(const BatchArgs<R>& b, int tile, int grid, cudaStream_t s);

// recording stage (hc_sig_*.cu): one residual evaluation of the 8x32 tile writing the
// face branch signatures to a.sig_i / a.sig_j; DF: double-float stage arithmetic
template <class R, bool DF> cudaError_t launch_sig_stage(const StageArgs<R>& a, int flux, cudaStream_t s);

// one-dimensional path (hc_oned.cu): host geometry of nc cells between nodes x[0..nc]
void oned_geometry(const double* x, int nc, const int bc[2], std::vector<double>& rec, std::vector<double>& vol);

// scalar advection law (hc_stage_scalar.cu): flux is FLUX_RUSANOV or FLUX_CENTRAL
template <class R> cudaError_t prepare_scalar_stage();
template <class R> cudaError_t launch_scalar_stage(const StageArgs<R>& a, int flux, int tile, cudaStream_t s);
template <class R>
cudaError_t launch_scalar_update0(int ni, int nj, const R* q0, const R* res0, const R* vol, R alpha00, R beta0,
                                  double cfl, StepInfo* info, R* q_out, int advance_time, cudaStream_t s);
// residual smoothing of the legacy 1D path (hc_smooth.cu): kind 0 implicit, 1 explicit;
// nplanes planes of n values at `stride`; implicit smoothing needs wrk and tmp of
// nplanes * n values and may run in place (r1 == r0); bc 'p', 'a' or other
template <class R>
cudaError_t launch_smooth_1d(int kind, const R* r0, R* r1, R* wrk, R* tmp, long long n, int nplanes, long long stride,
                             double alpha, int bc, cudaStream_t s);
// batches of scalar-law instances (pools as for the Euler batch)
template <class R>
cudaError_t launch_scalar_batch_stage(const BatchArgs<R>& b, int flux, int tile, int grid, cudaStream_t s);
template <class R>
cudaError_t launch_scalar_batch_update0(const BatchArgs<R>& b, int tile, int grid, double cfl, R alpha00, R beta0,
                                        cudaStream_t s);

inline void tile_dims(int tile, int* ti, int* tj) {
  switch (tile) {
    case TILE_4x32: *ti = 4; *tj = 32; break;
    case TILE_16x16:
    case TILE_16x16_H: *ti = 16; *tj = 16; break;
    default: *ti = 8; *tj = 32; break;
  }
}

}  // namespace hc

#define HC_STAGE_INSTANTIATE(FK)                                                                         \
  namespace hc {                                                                                         \
  template <class R, int TI, int TJ> static cudaError_t prep_one() {                                     \
    cudaError_t e = cudaFuncSetAttribute(stage_kernel<TI, TJ, R, FK>,                                    \
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,                    \
                                         int(StageSmem<TI, TJ, R>::bytes));                              \
    if (e != cudaSuccess) return e;                                                                      \
    if (std::is_same<R, double>::value && TI == 8 && TJ == 32) {                                          \
      e = cudaFuncSetAttribute(stage_kernel<8, 32, double, FK, df64>,                                    \
                               cudaFuncAttributeMaxDynamicSharedMemorySize,                              \
                               int(StageSmem<8, 32, df64>::bytes));                                      \
      if (e != cudaSuccess) return e;                                                                    \
    }                                                                                                    \
    return cudaFuncSetAttribute(batch_stage_kernel<TI, TJ, R, FK>,                                       \
                                cudaFuncAttributeMaxDynamicSharedMemorySize,                             \
                                int(StageSmem<TI, TJ, R>::bytes));                                       \
  }                                                                                                      \
  /* FP32 kernels with the limiter a compile-time constant (the FP32 stage is bound by */               \
  /* instruction issue; the run-time selection costs ~9% of it): the 8x32 single-mesh  */               \
  /* tile for the common limiters, and every batch tile for van Albada and NoLimit3     */               \
  /* with the state and i-face record loads staged by TMA where the mesh rows allow it */              \
  template <int LIM> static void go_lim(const StageArgs<float>& a, cudaStream_t s) {                     \
    const dim3 grid((a.nj + 31) / 32, (a.ni + 7) / 8);                                                   \
    CUtensorMap tq, tfi;                                                                                 \
    if (!a.plain_loads && stage_tma_maps(a, &tq, &tfi)) {                                                \
      stage_kernel_tma<8, 32, float, FK, LIM, 256>                                                       \
          <<<grid, 256, StageSmemTma<8, 32, float>::bytes + 2 * sizeof(uint64_t), s>>>(a, tq, tfi);      \
      return;                                                                                            \
    }                                                                                                    \
    stage_kernel<8, 32, float, FK, float, 256, LIM><<<grid, 256, StageSmem<8, 32, float>::bytes, s>>>(a); \
  }                                                                                                      \
  static bool go_fixed_lim(const StageArgs<float>& a, cudaStream_t s) {                                  \
    switch (a.limiter) {                                                                                 \
      case LIM_VANALBADA: go_lim<LIM_VANALBADA>(a, s); return true;                                      \
      case LIM_VANLEER: go_lim<LIM_VANLEER>(a, s); return true;                                          \
      case LIM_MINMOD: go_lim<LIM_MINMOD>(a, s); return true;                                            \
      case LIM_NOLIMIT2: go_lim<LIM_NOLIMIT2>(a, s); return true;                                        \
      case LIM_NOLIMIT3: go_lim<LIM_NOLIMIT3>(a, s); return true;                                        \
      default: return false;                                                                             \
    }                                                                                                    \
  }                                                                                                      \
  template <int LIM> static void gob_tma(const BatchArgs<float>& b, int grid, cudaStream_t s) {          \
    constexpr size_t smem = StageSmemTma<8, 32>::bytes + 2 * sizeof(uint64_t);                           \
    static int cap = 0;                                                                                  \
    if (cap == 0) {                                                                                      \
      int dev = 0, sms = 0, occ = 0;                                                                     \
      cudaGetDevice(&dev);                                                                               \
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                 \
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_stage_kernel_tma<FK, LIM>, 256, smem);   \
      cap = (sms > 0 && occ > 0) ? sms * occ : grid;                                                     \
    }                                                                                                    \
    batch_stage_kernel_tma<FK, LIM><<<std::min(grid, cap), 256, smem, s>>>(b);                           \
  }                                                                                                      \
  template <class R, int TI, int TJ, int LIM = -1>                                                        \
  static void gob(const BatchArgs<R>& b, int grid, cudaStream_t s) {                                     \
    /* the TMA-staged tile where the batch has tensor maps for this stage's input */                    \
    if constexpr (std::is_same<R, float>::value && TI == 8 && TJ == 32) {                                \
      if (b.tmaps_q && b.tmaps_fi) { gob_tma<LIM>(b, grid, s); return; }                                  \
    }                                                                                                    \
    /* a persistent grid larger than what stays resident would run a second, partial wave */           \
    static int cap = 0;                                                                                  \
    if (cap == 0) {                                                                                      \
      int dev = 0, sms = 0, occ = 0;                                                                     \
      cudaGetDevice(&dev);                                                                               \
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                 \
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_stage_kernel<TI, TJ, R, FK, LIM>, TI * TJ, \
                                                    StageSmem<TI, TJ, R>::bytes);                        \
      cap = (sms > 0 && occ > 0) ? sms * occ : grid;                                                     \
    }                                                                                                    \
    batch_stage_kernel<TI, TJ, R, FK, LIM><<<std::min(grid, cap), TI * TJ, StageSmem<TI, TJ, R>::bytes, s>>>( \
        b);                                                                                              \
  }                                                                                                      \
  template <int LIM> static void gob_tile(const BatchArgs<float>& b, int tile, int grid, cudaStream_t s) { \
    if (tile == TILE_4x32) gob<float, 4, 32, LIM>(b, grid, s);                                           \
    else if (tile == TILE_16x16) gob<float, 16, 16, LIM>(b, grid, s);                                    \
    else gob<float, 8, 32, LIM>(b, grid, s);                                                             \
  }                                                                                                      \
  template <> cudaError_t launch_batch_stage<double, FK>(const BatchArgs<double>& b, int tile, int grid, \
                                                         cudaStream_t s) {                               \
    if (tile == TILE_4x32) gob<double, 4, 32>(b, grid, s);                                               \
    else if (tile == TILE_16x16) gob<double, 16, 16>(b, grid, s);                                        \
    else gob<double, 8, 32>(b, grid, s);                                                                 \
    return cudaGetLastError();                                                                           \
  }                                                                                                      \
  template <> cudaError_t launch_batch_stage<float, FK>(const BatchArgs<float>& b, int tile, int grid,   \
                                                        cudaStream_t s) {                                \
    if (b.limiter == LIM_VANALBADA) gob_tile<LIM_VANALBADA>(b, tile, grid, s);                           \
    else if (b.limiter == LIM_NOLIMIT3) gob_tile<LIM_NOLIMIT3>(b, tile, grid, s);                        \
    else gob_tile<-1>(b, tile, grid, s);                                                                 \
    return cudaGetLastError();                                                                           \
  }                                                                                                      \
  template <class R, int TI, int TJ> static void go(const StageArgs<R>& a, cudaStream_t s) {             \
    const dim3 grid((a.nj + TJ - 1) / TJ, (a.ni + TI - 1) / TI);                                         \
    stage_kernel<TI, TJ, R, FK><<<grid, TI * TJ, StageSmem<TI, TJ, R>::bytes, s>>>(a);                   \
  }                                                                                                      \
  template <class R> static cudaError_t prep_half() {                                                   \
    return cudaFuncSetAttribute(stage_kernel<16, 16, R, FK, R, 128>,                                     \
                                cudaFuncAttributeMaxDynamicSharedMemorySize,                             \
                                int(StageSmem<16, 16, R>::bytes));                                       \
  }                                                                                                      \
  template <> cudaError_t prepare_stage<double, FK>() {                                                  \
    cudaError_t e = prep_one<double, 8, 32>();                                                           \
    if (e == cudaSuccess) e = prep_one<double, 4, 32>();                                                 \
    if (e == cudaSuccess) e = prep_one<double, 16, 16>();                                                \
    if (e == cudaSuccess) e = prep_half<double>();                                                       \
    return e;                                                                                            \
  }                                                                                                      \
  template <> cudaError_t prepare_stage<float, FK>() {                                                   \
    cudaError_t e = prep_one<float, 8, 32>();                                                            \
    if (e == cudaSuccess) e = prep_one<float, 4, 32>();                                                  \
    if (e == cudaSuccess) e = prep_one<float, 16, 16>();                                                 \
    if (e == cudaSuccess) e = prep_half<float>();                                                        \
    return e;                                                                                            \
  }                                                                                                      \
  template <class R> static cudaError_t dispatch(const StageArgs<R>& a, int tile, cudaStream_t s) {     \
    if (std::is_same<R, double>::value && a.fic) {                                                       \
      /* double-float compute type, 8x32 tiles */                                                        \
      const dim3 grid((a.nj + 31) / 32, (a.ni + 7) / 8);                                                 \
      stage_kernel<8, 32, double, FK, df64><<<grid, 256, StageSmem<8, 32, df64>::bytes, s>>>(           \
          *reinterpret_cast<const StageArgs<double>*>(&a));                                              \
      return cudaGetLastError();                                                                         \
    }                                                                                                    \
    if constexpr (std::is_same<R, float>::value) {                                                       \
      if ((tile == TILE_8x32 || tile < 0 || tile >= TILE_COUNT) && go_fixed_lim(a, s)) return cudaGetLastError(); \
    }                                                                                                    \
    if (tile == TILE_4x32) go<R, 4, 32>(a, s);                                                           \
    else if (tile == TILE_16x16) go<R, 16, 16>(a, s);                                                    \
    else if (tile == TILE_16x16_H) {                                                                     \
      const dim3 grid((a.nj + 15) / 16, (a.ni + 15) / 16);                                               \
      stage_kernel<16, 16, R, FK, R, 128><<<grid, 128, StageSmem<16, 16, R>::bytes, s>>>(a);             \
    } else go<R, 8, 32>(a, s);                                                                           \
    return cudaGetLastError();                                                                           \
  }                                                                                                      \
  template <> cudaError_t launch_stage<double, FK>(const StageArgs<double>& a, int tile, cudaStream_t s) { \
    return dispatch<double>(a, tile, s);                                                                 \
  }                                                                                                      \
  template <> cudaError_t launch_stage<float, FK>(const StageArgs<float>& a, int tile, cudaStream_t s) {   \
    return dispatch<float>(a, tile, s);                                                                  \
  }                                                                                                      \
  }
