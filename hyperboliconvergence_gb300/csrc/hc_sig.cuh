// hc_sig.cuh -- the recording stage kernels behind hc_face_signatures: one residual
// evaluation of the 8x32 tile that also writes each face's branch signature.  A
// diagnostic for the parity report, off the stepping path; each precision's
// instantiations live in a translation unit of their own (hc_sig_*.cu).
#pragma once

#include "hc_kernels.cuh"
#include "hc_launch.h"

namespace hc {

template <class R, int FK, class C> cudaError_t launch_sig_one(const StageArgs<R>& a, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(sig_kernel<8, 32, R, FK, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(StageSmem<8, 32, C>::bytes));
  if (e != cudaSuccess) return e;
  const dim3 grid((a.nj + 31) / 32, (a.ni + 7) / 8);
  sig_kernel<8, 32, R, FK, C><<<grid, 256, StageSmem<8, 32, C>::bytes, s>>>(a);
  return cudaGetLastError();
}

template <class R, class C> cudaError_t launch_sig_flux(const StageArgs<R>& a, int flux, cudaStream_t s) {
  switch (flux) {
    case FLUX_ROE: return launch_sig_one<R, FLUX_ROE, C>(a, s);
    case FLUX_SLAU: return launch_sig_one<R, FLUX_SLAU, C>(a, s);
    case FLUX_SLAU_REF: return launch_sig_one<R, FLUX_SLAU_REF, C>(a, s);
    case FLUX_AUSMPUP: return launch_sig_one<R, FLUX_AUSMPUP, C>(a, s);
    case FLUX_RUSANOV: return launch_sig_one<R, FLUX_RUSANOV, C>(a, s);
    case FLUX_ROE_WS: return launch_sig_one<R, FLUX_ROE_WS, C>(a, s);
    case FLUX_ROE_FACE: return launch_sig_one<R, FLUX_ROE_FACE, C>(a, s);
    default: return launch_sig_one<R, FLUX_CENTRAL, C>(a, s);
  }
}

}  // namespace hc
