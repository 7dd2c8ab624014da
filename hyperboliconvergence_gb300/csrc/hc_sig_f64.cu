// Recording stage kernels (hc_face_signatures), storage double, stage arithmetic double.
#include "hc_sig.cuh"

namespace hc {
template <> cudaError_t launch_sig_stage<double, false>(const StageArgs<double>& a, int flux, cudaStream_t s) {
  return launch_sig_flux<double, double>(a, flux, s);
}
}  // namespace hc
