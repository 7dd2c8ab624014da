// Recording stage kernels (hc_face_signatures), storage float, stage arithmetic float.
#include "hc_sig.cuh"

namespace hc {
template <> cudaError_t launch_sig_stage<float, false>(const StageArgs<float>& a, int flux, cudaStream_t s) {
  return launch_sig_flux<float, float>(a, flux, s);
}
}  // namespace hc
