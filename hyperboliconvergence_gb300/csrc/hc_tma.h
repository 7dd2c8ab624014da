// hc_tma.h -- tensor maps of the TMA-staged FP32 stage kernel (stage_kernel_tma):
// cuTensorMapEncodeTiled, reached through the runtime's driver entry point (no link against
// the driver library), for the state planes and the i-face record planes of one launch.
#pragma once

#include "hc_kernels.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace hc {

using TmaEncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline TmaEncodeFn tma_encode_fn() {
  static TmaEncodeFn fn = []() -> TmaEncodeFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return reinterpret_cast<TmaEncodeFn>(p);
  }();
  return fn;
}

// a 3D FP32 tensor map: dims (x fastest) and byte pitches of the two outer dimensions
inline bool tma_encode_3d(CUtensorMap* map, const float* base, uint64_t nx, uint64_t ny, uint64_t nz, uint32_t bx,
                          uint32_t by, uint32_t bz) {
  const TmaEncodeFn fn = tma_encode_fn();
  if (!fn || (reinterpret_cast<uintptr_t>(base) % 16) != 0 || (nx * sizeof(float)) % 16 != 0) return false;
  const cuuint64_t dims[3] = {nx, ny, nz};
  const cuuint64_t pitch[2] = {nx * sizeof(float), nx * ny * sizeof(float)};
  const cuuint32_t box[3] = {bx, by, bz};
  const cuuint32_t estride[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, pitch, box, estride,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the two maps of an FP32 8x32 stage launch: the state (4 planes of ni x nj, box 4 x 12 x 40)
// and the i-face records (FREC planes of (ni + 1) x nj, box TMA_FIELDS x 9 x 32); false when
// the mesh's rows are not a multiple of 16 bytes or the driver entry point is missing (the
// launcher then takes the plain kernel)
inline bool stage_tma_maps(const StageArgs<float>& a, CUtensorMap* tq, CUtensorMap* tfi) {
  if (a.nj % 4 != 0 || a.ni < 1) return false;
  const uint64_t ni = uint64_t(a.ni), nj = uint64_t(a.nj);
  return tma_encode_3d(tq, a.q, nj, ni, 4, StageSmemTma<8, 32>::QJ, StageSmemTma<8, 32>::QI, 4) &&
         tma_encode_3d(tfi, reinterpret_cast<const float*>(a.fi), nj, ni + 1, FREC, 32, 9, TMA_FIELDS);
}

}  // namespace hc
