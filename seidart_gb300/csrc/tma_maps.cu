// Host side of the TMA-staged kernels: tensor-map descriptors over a handle's
// field array, encoded through the driver entry point the runtime exposes
// (no link against the driver library).
#include <cudaTypedefs.h>

#include <mutex>

#include "sfd_solvers.h"

namespace sfd {

bool encode_tiled(CUtensorMap* map, void* base, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                  const cuuint32_t* box) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void**)&encode, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      encode = nullptr;
  });
  if (!encode) return false;
  const cuuint32_t ones[5] = {1, 1, 1, 1, 1};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, (cuuint32_t)rank, base, dims, strides, box, ones,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_field_map(CUtensorMap* map, void* base, int NX, int NY, int NZ, int P, size_t field_stride, int nfields,
                      int box_x, int box_z, int box_f) {
  // (x, y, z, field), x extent NX: boxes reaching past the last column read zeros
  const cuuint64_t dims[4] = {(cuuint64_t)NX, (cuuint64_t)NY, (cuuint64_t)NZ, (cuuint64_t)nfields};
  const cuuint64_t strides[3] = {(cuuint64_t)P * 4, (cuuint64_t)NY * P * 4, (cuuint64_t)field_stride * 4};
  const cuuint32_t box[4] = {(cuuint32_t)box_x, 1, (cuuint32_t)box_z, (cuuint32_t)box_f};
  return encode_tiled(map, base, 4, dims, strides, box);
}

}  // namespace sfd
