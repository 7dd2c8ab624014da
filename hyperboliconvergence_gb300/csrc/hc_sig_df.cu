// Recording stage kernels (hc_face_signatures), storage double, stage arithmetic df64.
#include "hc_sig.cuh"

namespace hc {
template <> cudaError_t launch_sig_stage<double, true>(const StageArgs<double>& a, int flux, cudaStream_t s) {
  return launch_sig_flux<double, df64>(a, flux, s);
}
}  // namespace hc
