// Face passes of the discrete adjoint for the Euler fluxes without a hand-written
// reverse (SLAU, SLAU as written, AUSM+up, RoeUnprecWS): the single-mesh and batched
// face kernels of hc_adjoint_kernels.cuh with the flux reversed by tangents
// (tangent_flux_adj, hc_tangent.cuh), FP64 and FP32.
#include "hc_adjoint_kernels.cuh"

namespace hc {

namespace {
template <class R, int FK>
void face_one(const AdjArgs<R>& a, int nbi, unsigned blocks, int threads, cudaStream_t s) {
  adj_face_kernel<R, FK><<<blocks, threads, 0, s>>>(a, nbi);
}
template <class R, int FK>
void face_batch(const AdjBatchArgs<R>& b, unsigned blocks, int threads, cudaStream_t s) {
  adj_face_batch_kernel<R, FK><<<blocks, threads, 0, s>>>(b);
}
}  // namespace

template <class R>
cudaError_t launch_adj_face_tangent(int flux, const AdjArgs<R>& a, int nbi, unsigned blocks, int threads,
                                    cudaStream_t s) {
  switch (flux) {
    case FLUX_SLAU: face_one<R, FLUX_SLAU>(a, nbi, blocks, threads, s); break;
    case FLUX_SLAU_REF: face_one<R, FLUX_SLAU_REF>(a, nbi, blocks, threads, s); break;
    case FLUX_AUSMPUP: face_one<R, FLUX_AUSMPUP>(a, nbi, blocks, threads, s); break;
    case FLUX_ROE_WS: face_one<R, FLUX_ROE_WS>(a, nbi, blocks, threads, s); break;
    case FLUX_ROE_FACE: face_one<R, FLUX_ROE_FACE>(a, nbi, blocks, threads, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class R>
cudaError_t launch_adj_face_tangent_batch(int flux, const AdjBatchArgs<R>& b, unsigned blocks, int threads,
                                          cudaStream_t s) {
  switch (flux) {
    case FLUX_SLAU: face_batch<R, FLUX_SLAU>(b, blocks, threads, s); break;
    case FLUX_SLAU_REF: face_batch<R, FLUX_SLAU_REF>(b, blocks, threads, s); break;
    case FLUX_AUSMPUP: face_batch<R, FLUX_AUSMPUP>(b, blocks, threads, s); break;
    case FLUX_ROE_WS: face_batch<R, FLUX_ROE_WS>(b, blocks, threads, s); break;
    case FLUX_ROE_FACE: face_batch<R, FLUX_ROE_FACE>(b, blocks, threads, s); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template cudaError_t launch_adj_face_tangent<double>(int, const AdjArgs<double>&, int, unsigned, int, cudaStream_t);
template cudaError_t launch_adj_face_tangent<float>(int, const AdjArgs<float>&, int, unsigned, int, cudaStream_t);
template cudaError_t launch_adj_face_tangent_batch<double>(int, const AdjBatchArgs<double>&, unsigned, int,
                                                           cudaStream_t);
template cudaError_t launch_adj_face_tangent_batch<float>(int, const AdjBatchArgs<float>&, unsigned, int,
                                                          cudaStream_t);

}  // namespace hc
