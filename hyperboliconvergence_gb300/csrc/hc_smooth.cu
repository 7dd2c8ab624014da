// hc_smooth.cu -- residual smoothing of the reference's legacy 1D path on the device:
// centralImplicitSmoothing (OLD.fieldOperations/centralImplicitSmoothing.ipp:2-60: four
// weighted-Jacobi sweeps, omega 2/3, of (1 - beta delta^2) r1 = r0, beta = (alpha^2-1)/4,
// the result times alpha) and centralExplicitSmoothing (centralExplicitSmoothing.ipp:5-39).
// Ends: 'p' periodic, 'a' one-neighbour normalisation, otherwise unscaled (the
// reference's GridControls1D::boundaryCondition).  Products and sums are rounded one by
// one in the reference's order (no contraction), so FP64 results equal the oracle's.
#include "hc_launch.h"

namespace hc {
namespace {

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

// one CTA per plane: the sweeps need the whole line between them
template <class R>
__global__ void smooth_implicit_kernel(const R* r0, R* r1, R* wrk, R* tmp, long long n, long long stride, R alpha,
                                       int bc) {
  const R* a = r0 + blockIdx.x * stride;
  R* o = r1 + blockIdx.x * stride;
  R* w = wrk + blockIdx.x * n;
  R* t = tmp + blockIdx.x * n;
  const R beta = mul_rn(R(0.25), add_rn(mul_rn(alpha, alpha), R(-1)));
  const R c2 = div_rn(R(1), add_rn(R(1), mul_rn(R(2), beta)));
  const R c1 = div_rn(R(1), add_rn(R(1), beta));
  const R omega = R(2. / 3.), om1 = R(1. - 2. / 3.);
  for (long long i = threadIdx.x; i < n; i += blockDim.x) w[i] = a[i];
  __syncthreads();
  for (int j = 0; j < 4; ++j) {
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
      R x = a[i];
      if (i >= 1) x = add_rn(x, mul_rn(beta, w[i - 1]));
      if (i + 1 < n) x = add_rn(x, mul_rn(beta, w[i + 1]));
      if (i >= 1 && i + 1 < n) {
        x = mul_rn(x, c2);
      } else if (bc == 'p') {
        x = add_rn(x, mul_rn(beta, i == 0 ? w[n - 1] : w[0]));
        x = mul_rn(x, c2);
      } else if (bc == 'a') {
        x = mul_rn(x, c1);
      }
      t[i] = x;
    }
    __syncthreads();
    for (long long i = threadIdx.x; i < n; i += blockDim.x) w[i] = add_rn(mul_rn(om1, w[i]), mul_rn(omega, t[i]));
    __syncthreads();
  }
  for (long long i = threadIdx.x; i < n; i += blockDim.x) o[i] = mul_rn(w[i], alpha);
}

template <class R>
__global__ void smooth_explicit_kernel(const R* r0, R* r1, long long n, long long stride, int nplanes, R alpha,
                                       int bc) {
  const R beta = mul_rn(R(0.25), add_rn(mul_rn(alpha, alpha), R(-1)));
  const R gamma = mul_rn(R(0.25), add_rn(div_rn(add_rn(R(1), mul_rn(R(4), beta)), alpha), R(-1)));
  const long long total = n * nplanes;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k / n, i = k % n;
    const R* a = r0 + p * stride;
    R x = a[i];
    if (i >= 1) x = add_rn(x, mul_rn(gamma, add_rn(a[i], -a[i - 1])));
    if (i + 1 < n) x = add_rn(x, -mul_rn(gamma, add_rn(a[i + 1], -a[i])));
    if (bc == 'p') {
      const R dp = mul_rn(gamma, add_rn(a[0], -a[n - 1]));
      if (i == n - 1) x = add_rn(x, -dp);
      if (i == 0) x = add_rn(x, dp);
    }
    r1[p * stride + i] = x;
  }
}

}  // namespace

template <class R>
cudaError_t launch_smooth_1d(int kind, const R* r0, R* r1, R* wrk, R* tmp, long long n, int nplanes, long long stride,
                             double alpha, int bc, cudaStream_t s) {
  if (kind == 0) {
    smooth_implicit_kernel<R><<<nplanes, 1024, 0, s>>>(r0, r1, wrk, tmp, n, stride, R(alpha), bc);
  } else {
    const long long total = n * nplanes;
    const unsigned grid = unsigned(std::min<long long>((total + 255) / 256, 152 * 16));
    smooth_explicit_kernel<R><<<grid, 256, 0, s>>>(r0, r1, n, stride, nplanes, R(alpha), bc);
  }
  return cudaGetLastError();
}

template cudaError_t launch_smooth_1d<double>(int, const double*, double*, double*, double*, long long, int,
                                              long long, double, int, cudaStream_t);
template cudaError_t launch_smooth_1d<float>(int, const float*, float*, float*, float*, long long, int, long long,
                                             double, int, cudaStream_t);

}  // namespace hc
