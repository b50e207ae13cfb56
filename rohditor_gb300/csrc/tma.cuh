// Tensor-memory-access (TMA) tile copies and mbarriers for sm_103a, shared by
// the capture-sharpening and demosaic kernels.
//
// Device side: inline PTX for the mbarrier a copy completes on and for the 2D
// tensor copy itself (cp.async.bulk.tensor). Host side: tensor maps encoded
// through cuTensorMapEncodeTiled, reached by the runtime's driver entry-point
// query (no link against the driver library).
#pragma once

#include <cuda.h>  // CUtensorMap and its enums
#include <cuda_runtime.h>
#include <stdint.h>

namespace rd {

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Orders this thread's earlier generic-proxy shared-memory accesses before a
// tensor copy that writes the same shared memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// 2D tensor copy of the box at (x, y) into shared memory, completing on `bar`.
// The copy's x start times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// cuTensorMapEncodeTiled, or null when the driver does not provide it.
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled tensor_map_encoder();

// Tensor map of a row-major 2D array (`width` x `height` elements of
// `elem_bytes`, rows `pitch_bytes` apart) for box_w x box_h boxes; elements
// outside the array read as zero. False when TMA cannot address it: base not
// 16-byte aligned, pitch not a multiple of 16 bytes, a box row not a multiple
// of 16 bytes, or no encoder.
bool make_tensor_map_2d(CUtensorMap* map, CUtensorMapDataType type, int elem_bytes, const void* base, uint64_t width,
                        uint64_t height, uint64_t pitch_bytes, int box_w, int box_h);

}  // namespace rd
