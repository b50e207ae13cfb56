// Host side of the tensor copies: the tensor-map encoder and 2D maps.
#include "tma.cuh"

#include <mutex>

namespace rd {

EncodeTiled tensor_map_encoder() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

bool make_tensor_map_2d(CUtensorMap* map, CUtensorMapDataType type, int elem_bytes, const void* base, uint64_t width,
                        uint64_t height, uint64_t pitch_bytes, int box_w, int box_h) {
  if (reinterpret_cast<uintptr_t>(base) % 16 != 0 || pitch_bytes % 16 != 0 || ((uint64_t)box_w * elem_bytes) % 16 != 0)
    return false;
  if (box_w < 1 || box_w > 256 || box_h < 1 || box_h > 256 || width == 0 || height == 0) return false;
  const EncodeTiled enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)height};
  const cuuint64_t strides[1] = {(cuuint64_t)pitch_bytes};
  const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
  const cuuint32_t elem[2] = {1, 1};
  return enc(map, type, 2, const_cast<void*>(base), dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace rd
