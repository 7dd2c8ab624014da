// hc_host.h -- host-side helpers shared by the C-ABI translation units.
#pragma once

#include "../../include/hc.h"
#include "hc_launch.h"

#include <string>

namespace hc {

// last error of the calling thread (defined in hc_api.cu)
void set_last_error(const std::string& msg);

inline int fail(int code, const std::string& msg) {
  set_last_error(msg);
  return code;
}

#define HC_CUDA(call)                                                                                       \
  do {                                                                                                      \
    cudaError_t e_ = (call);                                                                                \
    if (e_ != cudaSuccess) return ::hc::fail(HC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// RK tables ssp11..ssp34 (ode.h:107-197)
struct RKTab {
  int nst;
  double alpha[4][4];
  double beta[4];
};
inline RKTab rk_table(int kind) {
  RKTab t{};
  if (kind == HC_RK_SSP11) {
    t.nst = 1; t.beta[0] = 1.0; t.alpha[0][0] = 1.0;
  } else if (kind == HC_RK_SSP22) {
    t.nst = 2; t.beta[0] = 1.0; t.beta[1] = 1.0;
    t.alpha[0][0] = 1.0; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
  } else if (kind == HC_RK_SSP33) {
    t.nst = 3; t.beta[0] = 1.0; t.beta[1] = 0.5; t.beta[2] = 1.0;
    t.alpha[0][0] = 1.; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
    t.alpha[2][0] = 1. / 6.; t.alpha[2][1] = 1. / 6.; t.alpha[2][2] = 2. / 3.;
  } else {
    t.nst = 4; t.beta[0] = 0.5; t.beta[1] = 1.0; t.beta[2] = 0.5; t.beta[3] = 1.0;
    t.alpha[0][0] = 1.0; t.alpha[1][0] = 0.5; t.alpha[1][1] = 0.5;
    t.alpha[2][0] = 1. / 3.; t.alpha[2][1] = 1. / 3.; t.alpha[2][2] = 1. / 3.;
    t.alpha[3][0] = 1. / 6.; t.alpha[3][1] = 1. / 6.; t.alpha[3][2] = 1. / 6.; t.alpha[3][3] = 1. / 2.;
  }
  return t;
}

template <class R> using StageFn = cudaError_t (*)(const StageArgs<R>&, int, cudaStream_t);
template <class R> using BatchFn = cudaError_t (*)(const BatchArgs<R>&, int tile, int grid, cudaStream_t);

template <class R> StageFn<R> stage_fn(int flux) {
  switch (flux) {
    case FLUX_ROE: return launch_stage<R, FLUX_ROE>;
    case FLUX_SLAU: return launch_stage<R, FLUX_SLAU>;
    case FLUX_SLAU_REF: return launch_stage<R, FLUX_SLAU_REF>;
    case FLUX_AUSMPUP: return launch_stage<R, FLUX_AUSMPUP>;
    case FLUX_RUSANOV: return launch_stage<R, FLUX_RUSANOV>;
    case FLUX_ROE_WS: return launch_stage<R, FLUX_ROE_WS>;
    case FLUX_ROE_FACE: return launch_stage<R, FLUX_ROE_FACE>;
    default: return launch_stage<R, FLUX_CENTRAL>;
  }
}
template <class R> BatchFn<R> batch_fn(int flux) {
  switch (flux) {
    case FLUX_ROE: return launch_batch_stage<R, FLUX_ROE>;
    case FLUX_SLAU: return launch_batch_stage<R, FLUX_SLAU>;
    case FLUX_SLAU_REF: return launch_batch_stage<R, FLUX_SLAU_REF>;
    case FLUX_AUSMPUP: return launch_batch_stage<R, FLUX_AUSMPUP>;
    case FLUX_RUSANOV: return launch_batch_stage<R, FLUX_RUSANOV>;
    case FLUX_ROE_WS: return launch_batch_stage<R, FLUX_ROE_WS>;
    case FLUX_ROE_FACE: return launch_batch_stage<R, FLUX_ROE_FACE>;
    default: return launch_batch_stage<R, FLUX_CENTRAL>;
  }
}
template <class R> cudaError_t prepare(int flux) {
  switch (flux) {
    case FLUX_ROE: return prepare_stage<R, FLUX_ROE>();
    case FLUX_SLAU: return prepare_stage<R, FLUX_SLAU>();
    case FLUX_SLAU_REF: return prepare_stage<R, FLUX_SLAU_REF>();
    case FLUX_AUSMPUP: return prepare_stage<R, FLUX_AUSMPUP>();
    case FLUX_RUSANOV: return prepare_stage<R, FLUX_RUSANOV>();
    case FLUX_ROE_WS: return prepare_stage<R, FLUX_ROE_WS>();
    case FLUX_ROE_FACE: return prepare_stage<R, FLUX_ROE_FACE>();
    default: return prepare_stage<R, FLUX_CENTRAL>();
  }
}

// geometry of one mesh (FP64 device buffers), built by hc_api.cu's kernels
struct GeomBuffers {
  double* nodes;   // (ni+1)*(nj+1)*2
  double* cx;
  double* cy;
  double* xm;      // 3 planes
  double* vol;     // ni*nj
  double* fi;      // FREC planes of (ni+1)*nj
  double* fj;      // FREC planes of ni*(nj+1)
};
// Enqueue the geometry kernels of one mesh on `s`; returns the number of launches.
int enqueue_geometry(const GeomBuffers& g, int ni, int nj, const int bc[4], cudaStream_t s);

}  // namespace hc
