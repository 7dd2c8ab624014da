// hc_reduce.cu -- context-free spectral radius: max over cells of lambda/V
// (spectralRadius, spatial/spectralRadius.h:19-48), the quantity the global
// timestep divides the CFL number by.  Two passes: every block reduces a fixed
// chunk of cells to one partial maximum, then one block reduces the partials.
#include "hc_host.h"

#include <cfloat>

namespace hc {

constexpr int SR_THREADS = 256;
constexpr int SR_PER_THREAD = 8;
constexpr long long SR_CHUNK = (long long)SR_THREADS * SR_PER_THREAD;  // cells per block

__device__ __forceinline__ double block_max(double m) {
  __shared__ double red[SR_THREADS / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double x = __shfl_xor_sync(0xffffffffu, m, o);
    m = (m < x) ? x : m;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < SR_THREADS / 32) ? red[threadIdx.x] : DBL_MIN;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double x = __shfl_xor_sync(0xffffffffu, m, o);
      m = (m < x) ? x : m;
    }
  }
  return m;
}

// partial[b] = max(DBL_MIN, max over the block's chunk of lambda/V); the fold
// starts at numeric_limits<double>::min() as the reference does.
__global__ void __launch_bounds__(SR_THREADS)
spectral_radius_partial(const double* __restrict__ lam, const double* __restrict__ vol, long long n,
                        double* __restrict__ partial) {
  double m = DBL_MIN;
  const long long base = blockIdx.x * SR_CHUNK;
#pragma unroll
  for (int k = 0; k < SR_PER_THREAD; ++k) {
    const long long c = base + (long long)k * SR_THREADS + threadIdx.x;
    if (c < n) {
      const double r = lam[c] / vol[c];
      m = (m < r) ? r : m;
    }
  }
  m = block_max(m);
  if (threadIdx.x == 0) partial[blockIdx.x] = m;
}

__global__ void __launch_bounds__(SR_THREADS)
spectral_radius_final(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  double m = DBL_MIN;
  for (int b = threadIdx.x; b < nb; b += SR_THREADS) m = (m < partial[b]) ? partial[b] : m;
  m = block_max(m);
  if (threadIdx.x == 0) out[0] = m;
}

// Scratch of hc_spectral_radius_noalloc: one partial maximum per block of
// SR_CHUNK cells, at most SR_NOALLOC_BLOCKS blocks (32 KiB).  It is static
// device memory, so every GPU that loads this library holds it until the
// process exits.  Each call writes every entry it later reads, so nothing has
// to be cleared between calls; calls that overlap on the GPU share the array
// and race.
constexpr int SR_NOALLOC_BLOCKS = 4096;
constexpr long long SR_NOALLOC_MAX_CELLS = SR_NOALLOC_BLOCKS * SR_CHUNK;  // 8,388,608
static __device__ __align__(256) double g_sr_noalloc_scratch[SR_NOALLOC_BLOCKS];

}  // namespace hc

#include <mutex>
#include <vector>

namespace {
std::mutex g_sr_scratch_mutex;
// Device address of the scratch array, per device, looked up once and kept for the life
// of the process.  cudaDeviceReset destroys the context the address belongs to, and this
// cache is not told: a process that resets a device must not call
// hc_spectral_radius_noalloc on that device again.
std::vector<double*> g_sr_scratch_ptr;
}  // namespace

using namespace hc;

extern "C" {

// The array's name is only a host-side stand-in for host code; its device
// address is looked up once per device (with that device current) on the
// first call made on the device, so that first call should come before any
// stream capture.
int hc_spectral_radius_noalloc(const double* lambda_sum, const double* vol, long long ncell, double* out,
                               void* stream) {
  if (!lambda_sum || !vol || !out) return fail(HC_ERR_ARG, "null pointer");
  if (ncell < 1) return fail(HC_ERR_ARG, "ncell must be positive");
  if (ncell > SR_NOALLOC_MAX_CELLS)
    return fail(HC_ERR_ARG, "ncell " + std::to_string(ncell) + " exceeds the no-allocation maximum of " +
                                std::to_string(SR_NOALLOC_MAX_CELLS) + " cells");
  int dev = 0;
  HC_CUDA(cudaGetDevice(&dev));
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_sr_scratch_mutex);
    if (g_sr_scratch_ptr.size() <= size_t(dev)) g_sr_scratch_ptr.resize(size_t(dev) + 1, nullptr);
    if (!g_sr_scratch_ptr[dev]) {
      void* p = nullptr;
      HC_CUDA(cudaGetSymbolAddress(&p, g_sr_noalloc_scratch));
      g_sr_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_sr_scratch_ptr[dev];
  }
  const long long nb = (ncell + SR_CHUNK - 1) / SR_CHUNK;
  const cudaStream_t s = (cudaStream_t)stream;
  spectral_radius_partial<<<unsigned(nb), SR_THREADS, 0, s>>>(lambda_sum, vol, ncell, scratch);
  spectral_radius_final<<<1, SR_THREADS, 0, s>>>(scratch, int(nb), out);
  HC_CUDA(cudaGetLastError());
  return HC_OK;
}

int hc_spectral_radius(const double* lambda_sum, const double* vol, long long ncell, double* out, void* stream) {
  if (!lambda_sum || !vol || !out) return fail(HC_ERR_ARG, "null pointer");
  if (ncell < 1) return fail(HC_ERR_ARG, "ncell must be positive");
  const long long nb = (ncell + SR_CHUNK - 1) / SR_CHUNK;
  if (nb > (1LL << 30)) return fail(HC_ERR_ARG, "ncell too large");
  const cudaStream_t s = (cudaStream_t)stream;
  double* partial = nullptr;
  HC_CUDA(cudaMallocAsync((void**)&partial, size_t(nb) * sizeof(double), s));
  spectral_radius_partial<<<unsigned(nb), SR_THREADS, 0, s>>>(lambda_sum, vol, ncell, partial);
  spectral_radius_final<<<1, SR_THREADS, 0, s>>>(partial, int(nb), out);
  const cudaError_t e = cudaGetLastError();
  cudaFreeAsync(partial, s);
  HC_CUDA(e);
  return HC_OK;
}

}  // extern "C"
