// Device check of sqrt_rcp (hc_physics.cuh) at the edges of its fast path: the
// device must give what the host gives (s = sqrt(x), r = 1/s; zero gives s = 0,
// r = inf, not s = 0*inf = NaN).  Also prints the device Roe flux of zero-pressure
// and ordinary face states ("roe k f0 f1 f2 f3 lam", face normal (0.6, 0.8), area
// 1.5, gamma 1.4) for the caller to compare with the oracle.  Exits 1 on a
// sqrt_rcp mismatch.
#include "../../hyperboliconvergence_gb300/csrc/hc_physics.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace hc;

namespace {

constexpr int NX = 10;
constexpr int NF = 6;

__global__ void sqrt_rcp_kernel(const double* x, double* s, double* r, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) sqrt_rcp(x[k], s[k], r[k]);
}

__global__ void roe_kernel(const double* ql, const double* qr, double* out, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const Gas<double> g = make_gas<double>(1.4, 287.058, 0.3);
  const double* a = ql + 4 * k;
  const double* b = qr + 4 * k;
  const St<double> l = prim_state(g, a[0], a[1], a[2], a[3]);
  const St<double> r = prim_state(g, b[0], b[1], b[2], b[3]);
  const Flux5<double> f = roe_flux(g, 0.6, 0.8, 1.5, l, r);
  for (int v = 0; v < 4; ++v) out[5 * k + v] = f.f[v];
  out[5 * k + 4] = f.lam;
}

bool same(double dev, double host, double tol) {
  if (std::isnan(host) || std::isnan(dev)) return std::isnan(host) && std::isnan(dev);
  if (std::isinf(host) || std::isinf(dev)) return dev == host;
  return std::fabs(dev - host) <= tol * std::fmax(std::fabs(host), 1e-300);
}

#define CK(x)                                                               \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) {                                                \
      std::printf("cuda error %s at %d\n", cudaGetErrorString(e_), __LINE__); \
      return 2;                                                             \
    }                                                                       \
  } while (0)

}  // namespace

int main() {
  const double xs[NX] = {0.0, -0.0, 4.9e-324, 2.2250738585072014e-308, 1.0, 2.0, 1e300, INFINITY, NAN, -1.0};
  // zero-pressure pairs and ordinary ones: {u, v, rho, p} left, right
  const double qls[NF][4] = {{0, 0, 1, 0}, {0, 0, 1, 0}, {0.3, -0.2, 1, 0}, {0.1, 0.2, 1, 1}, {0, 0, 1, 1}, {0.5, 0, 1, 0}};
  const double qrs[NF][4] = {{0, 0, 2, 0}, {0, 0, 1, 0}, {0.3, -0.2, 1, 0}, {0.2, 0.1, 2, 0.5}, {0, 0, 1, 0}, {-0.5, 0, 1, 0}};

  double *dx, *ds, *dr, *dql, *dqr, *dout;
  CK(cudaMalloc(&dx, NX * sizeof(double)));
  CK(cudaMalloc(&ds, NX * sizeof(double)));
  CK(cudaMalloc(&dr, NX * sizeof(double)));
  CK(cudaMalloc(&dql, NF * 4 * sizeof(double)));
  CK(cudaMalloc(&dqr, NF * 4 * sizeof(double)));
  CK(cudaMalloc(&dout, NF * 5 * sizeof(double)));
  CK(cudaMemcpy(dx, xs, sizeof xs, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dql, qls, sizeof qls, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(dqr, qrs, sizeof qrs, cudaMemcpyHostToDevice));
  sqrt_rcp_kernel<<<1, 32>>>(dx, ds, dr, NX);
  roe_kernel<<<1, 32>>>(dql, dqr, dout, NF);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  double s[NX], r[NX], out[NF * 5];
  CK(cudaMemcpy(s, ds, sizeof s, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(r, dr, sizeof r, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(out, dout, sizeof out, cudaMemcpyDeviceToHost));

  int bad = 0;
  for (int k = 0; k < NX; ++k) {
    double hs, hr;
    sqrt_rcp(xs[k], hs, hr);  // host: sqrt and a division
    // the fast path rounds within 1.5 ulp; the guarded inputs must agree exactly
    const bool fast = xs[k] > 0 && std::isfinite(xs[k]);
    const double tol = fast ? 4e-16 : 0.0;
    if (!same(s[k], hs, tol) || !same(r[k], hr, tol)) {
      std::printf("sqrt_rcp(%.17g): device (%.17g, %.17g) host (%.17g, %.17g)\n", xs[k], s[k], r[k], hs, hr);
      ++bad;
    }
  }
  // the Roe fluxes go to the caller, which holds them to the oracle's
  for (int k = 0; k < NF; ++k)
    std::printf("roe %d %.17g %.17g %.17g %.17g %.17g\n", k, out[5 * k], out[5 * k + 1], out[5 * k + 2],
                out[5 * k + 3], out[5 * k + 4]);
  if (bad) return 1;
  std::printf("ok\n");
  return 0;
}
