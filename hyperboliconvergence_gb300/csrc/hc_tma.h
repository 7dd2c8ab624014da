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

// a 3D FP32 or FP64 tensor map: dims (x fastest) and byte pitches of the two outer dimensions
template <class R>
inline bool tma_encode_3d(CUtensorMap* map, const R* base, uint64_t nx, uint64_t ny, uint64_t nz, uint32_t bx,
                          uint32_t by, uint32_t bz) {
  static_assert(sizeof(R) == 4 || sizeof(R) == 8, "FP32 or FP64 planes");
  const TmaEncodeFn fn = tma_encode_fn();
  if (!fn || (reinterpret_cast<uintptr_t>(base) % 16) != 0 || (nx * sizeof(R)) % 16 != 0) return false;
  const cuuint64_t dims[3] = {nx, ny, nz};
  const cuuint64_t pitch[2] = {nx * sizeof(R), nx * ny * sizeof(R)};
  const cuuint32_t box[3] = {bx, by, bz};
  const cuuint32_t estride[3] = {1, 1, 1};
  return fn(map, sizeof(R) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
            const_cast<R*>(base), dims, pitch, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the two maps of a TI x TJ stage launch: the state (4 planes of ni x nj, box 4 x (TI + 4) x
// (TJ + 8)) and the i-face records (FREC planes of (ni + 1) x nj, box TMA_FIELDS x (TI + 1) x
// TJ); false when the mesh's rows are not a multiple of 16 bytes or the driver entry point is
// missing (the launcher then takes the plain kernel)
template <class R, int TI = 8, int TJ = 32>
inline bool stage_tma_maps(const StageArgs<R>& a, CUtensorMap* tq, CUtensorMap* tfi) {
  if ((size_t(a.nj) * sizeof(R)) % 16 != 0 || a.ni < 1) return false;
  const uint64_t ni = uint64_t(a.ni), nj = uint64_t(a.nj);
  using SM = StageSmemTma<TI, TJ, R>;
  return tma_encode_3d<R>(tq, a.q, nj, ni, 4, SM::QJ, SM::QI, 4) &&
         tma_encode_3d<R>(tfi, reinterpret_cast<const R*>(a.fi), nj, ni + 1, FREC, TJ, TI + 1, TMA_FIELDS);
}

}  // namespace hc
