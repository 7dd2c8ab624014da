// Stage kernels of the scalar advection law: Rusanov and central fluxes, FP64
// and FP32, all tile shapes, single-mesh and batched (persistent) launches.
#include "hc_scalar.cuh"
#include "hc_launch.h"

namespace hc {
namespace {

template <class R, int TI, int TJ, int FK> cudaError_t prep_one() {
  return cudaFuncSetAttribute(scalar_stage_kernel<TI, TJ, R, FK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(ScalarSmem<TI, TJ, R>::bytes));
}

template <class R, int TI, int TJ, int FK> cudaError_t prep_batch_one() {
  return cudaFuncSetAttribute(batch_scalar_stage_kernel<TI, TJ, R, FK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              int(ScalarSmem<TI, TJ, R>::bytes));
}

template <class R, int FK> cudaError_t prep_flux() {
  cudaError_t e = prep_one<R, 8, 32, FK>();
  if (e == cudaSuccess) e = prep_one<R, 4, 32, FK>();
  if (e == cudaSuccess) e = prep_one<R, 16, 16, FK>();
  if (e == cudaSuccess) e = prep_batch_one<R, 8, 32, FK>();
  if (e == cudaSuccess) e = prep_batch_one<R, 4, 32, FK>();
  if (e == cudaSuccess) e = prep_batch_one<R, 16, 16, FK>();
  return e;
}

// persistent launch; a grid larger than what stays resident would run a second, partial wave
template <class R, int TI, int TJ, int FK> void gob(const BatchArgs<R>& b, int grid, cudaStream_t s) {
  static int cap = 0;
  if (cap == 0) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_scalar_stage_kernel<TI, TJ, R, FK>, TI * TJ,
                                                  ScalarSmem<TI, TJ, R>::bytes);
    cap = (sms > 0 && occ > 0) ? sms * occ : grid;
  }
  batch_scalar_stage_kernel<TI, TJ, R, FK><<<std::min(grid, cap), TI * TJ, ScalarSmem<TI, TJ, R>::bytes, s>>>(b);
}

template <class R, int FK> void gob_tile(const BatchArgs<R>& b, int tile, int grid, cudaStream_t s) {
  if (tile == TILE_4x32) gob<R, 4, 32, FK>(b, grid, s);
  else if (tile == TILE_16x16) gob<R, 16, 16, FK>(b, grid, s);
  else gob<R, 8, 32, FK>(b, grid, s);
}

template <class R, int TI, int TJ, int FK> void go(const StageArgs<R>& a, cudaStream_t s) {
  const dim3 grid((a.nj + TJ - 1) / TJ, (a.ni + TI - 1) / TI);
  scalar_stage_kernel<TI, TJ, R, FK><<<grid, TI * TJ, ScalarSmem<TI, TJ, R>::bytes, s>>>(a);
}

template <class R, int FK> void go_tile(const StageArgs<R>& a, int tile, cudaStream_t s) {
  if (tile == TILE_4x32) go<R, 4, 32, FK>(a, s);
  else if (tile == TILE_16x16 || tile == TILE_16x16_H) go<R, 16, 16, FK>(a, s);
  else go<R, 8, 32, FK>(a, s);
}

}  // namespace

template <class R> cudaError_t prepare_scalar_stage() {
  cudaError_t e = prep_flux<R, FLUX_RUSANOV>();
  if (e == cudaSuccess) e = prep_flux<R, FLUX_CENTRAL>();
  return e;
}

template <class R> cudaError_t launch_scalar_stage(const StageArgs<R>& a, int flux, int tile, cudaStream_t s) {
  if (flux == FLUX_CENTRAL) go_tile<R, FLUX_CENTRAL>(a, tile, s);
  else go_tile<R, FLUX_RUSANOV>(a, tile, s);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_scalar_update0(int ni, int nj, const R* q0, const R* res0, const R* vol, R alpha00, R beta0,
                                  double cfl, StepInfo* info, R* q_out, int advance_time, cudaStream_t s) {
  const size_t n = size_t(ni) * nj;
  const unsigned grid = unsigned(std::min<size_t>((n + 255) / 256, 152 * 16));
  scalar_update0_kernel<R><<<grid, 256, 0, s>>>(ni, nj, q0, res0, vol, alpha00, beta0, cfl, info, q_out,
                                                advance_time);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_scalar_batch_stage(const BatchArgs<R>& b, int flux, int tile, int grid, cudaStream_t s) {
  if (flux == FLUX_CENTRAL) gob_tile<R, FLUX_CENTRAL>(b, tile, grid, s);
  else gob_tile<R, FLUX_RUSANOV>(b, tile, grid, s);
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_scalar_batch_update0(const BatchArgs<R>& b, int tile, int grid, double cfl, R alpha00, R beta0,
                                        cudaStream_t s) {
  if (tile == TILE_4x32) batch_scalar_update0_kernel<4, 32, R><<<grid, 128, 0, s>>>(b, cfl, alpha00, beta0);
  else if (tile == TILE_16x16) batch_scalar_update0_kernel<16, 16, R><<<grid, 256, 0, s>>>(b, cfl, alpha00, beta0);
  else batch_scalar_update0_kernel<8, 32, R><<<grid, 256, 0, s>>>(b, cfl, alpha00, beta0);
  return cudaGetLastError();
}

template cudaError_t launch_scalar_batch_stage<double>(const BatchArgs<double>&, int, int, int, cudaStream_t);
template cudaError_t launch_scalar_batch_stage<float>(const BatchArgs<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_scalar_batch_update0<double>(const BatchArgs<double>&, int, int, double, double, double,
                                                         cudaStream_t);
template cudaError_t launch_scalar_batch_update0<float>(const BatchArgs<float>&, int, int, double, float, float,
                                                        cudaStream_t);
template cudaError_t prepare_scalar_stage<double>();
template cudaError_t prepare_scalar_stage<float>();
template cudaError_t launch_scalar_stage<double>(const StageArgs<double>&, int, int, cudaStream_t);
template cudaError_t launch_scalar_stage<float>(const StageArgs<float>&, int, int, cudaStream_t);
template cudaError_t launch_scalar_update0<double>(int, int, const double*, const double*, const double*, double,
                                                   double, double, StepInfo*, double*, int, cudaStream_t);
template cudaError_t launch_scalar_update0<float>(int, int, const float*, const float*, const float*, float, float,
                                                  double, StepInfo*, float*, int, cudaStream_t);

}  // namespace hc
