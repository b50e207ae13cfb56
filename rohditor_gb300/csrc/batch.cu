// Batched develop of many mosaics of uneven sizes on one GPU.
//
// The reference develops one image per call (CpuPipeline / GpuSensorProcessor
// through SpatialCache::prepare_sensor, crates/engine/src/preview_cache/
// spatial.rs:475-600). For a queue of images this entry point keeps the GPU
// full: `lanes` host threads, each with its own context and stream, take the
// next image from a shared counter and run the whole path on it (develop,
// spatial pass, render with host outputs). The lanes' kernels overlap on the
// device, so one image's tail waves and host gaps are filled by another's work.
// Results (status, per-image time, outputs) are written into the items.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "rd_handles.cuh"

extern "C" rd_status rd_develop_batch(int device, rd_batch_item* items, int32_t count, int32_t lanes,
                                      double* wall_ms) {
  if (!items || count < 0 || lanes <= 0) return RD_INVALID_INPUT;
  if (wall_ms) *wall_ms = 0.0;
  if (count == 0) return RD_OK;
  lanes = std::min(lanes, count);
  std::vector<rd_ctx*> ctxs(lanes, nullptr);
  for (int l = 0; l < lanes; ++l) {
    const rd_status st = rd_ctx_create(device, 0, &ctxs[l]);
    if (st != RD_OK) {
      for (rd_ctx* c : ctxs)
        if (c) rd_ctx_destroy(c);
      return st;
    }
  }
  std::atomic<int> next{0};
  const auto t0 = std::chrono::steady_clock::now();
  auto lane = [&](rd_ctx* ctx) {
    for (int k = next++; k < count; k = next++) {
      rd_batch_item& it = items[k];
      const auto s0 = std::chrono::steady_clock::now();
      rd_source* src = nullptr;
      rd_base* base = nullptr;
      rd_status st = rd_develop(ctx, it.mosaic, it.row_stride, &it.sensor, &it.detail, nullptr, &src, nullptr);
      if (st == RD_OK)
        st = rd_spatial(ctx, src, &it.optics, it.target_width, it.target_height, it.wb_gains, it.camera_to_rec2020,
                        &base, nullptr);
      if (src) rd_source_release(src);
      if (st == RD_OK) st = rd_render(ctx, base, &it.color, it.srgb_out, it.hist, nullptr, nullptr);
      if (base) rd_base_release(base);
      it.status = st;
      it.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - s0).count();
    }
  };
  std::vector<std::thread> threads;
  for (int l = 1; l < lanes; ++l) threads.emplace_back(lane, ctxs[l]);
  lane(ctxs[0]);
  for (std::thread& t : threads) t.join();
  if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (rd_ctx* c : ctxs) rd_ctx_destroy(c);
  rd_status first = RD_OK;
  for (int k = 0; k < count && first == RD_OK; ++k) first = (rd_status)items[k].status;
  return first;
}
