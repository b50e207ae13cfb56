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
#include <cstring>
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

// The same batch as one captured CUDA graph. `chains` parallel branches each
// develop their share of the images one after another (develop, spatial
// pass, render: every device buffer allocated and freed inside the graph),
// with the host mosaics and outputs staged through pinned memory. The batch
// is captured once and runs as a single graph launch: no host thread turns
// around between the stages of an image, and the branches' kernels overlap on
// the device. Errors are read from each branch's error word after the launch.
// `capture_ms` receives the capture + instantiation time, `launch_ms` the
// graph launch to completion, `wall_ms` that plus the staging copies (none
// when `host_pinned`: the items' buffers are then pinned and used in place).
extern "C" rd_status rd_develop_batch_graph(int device, rd_batch_item* items, int32_t count, int32_t chains,
                                            int32_t host_pinned, double* wall_ms, double* capture_ms,
                                            double* launch_ms) {
  using Clock = std::chrono::steady_clock;
  if (!items || count < 0 || chains <= 0) return RD_INVALID_INPUT;
  if (wall_ms) *wall_ms = 0.0;
  if (capture_ms) *capture_ms = 0.0;
  if (launch_ms) *launch_ms = 0.0;
  if (count == 0) return RD_OK;
  chains = std::min(chains, count);
  std::vector<rd_ctx*> ctxs(chains, nullptr);
  rd_status status = RD_OK;
  // AMaZE scratch for the largest image: launches inside the capture never allocate.
  size_t max_tiles = 1;
  for (int k = 0; k < count; ++k)
    max_tiles = std::max(max_tiles, rd::amaze_tiles((int)items[k].sensor.crop_width, (int)items[k].sensor.crop_height));
  for (int c = 0; c < chains && status == RD_OK; ++c) {
    status = rd_ctx_create(device, 0, &ctxs[c]);
    if (status == RD_OK && !rd::reserve_amaze_scratch(ctxs[c]->c, max_tiles).ok()) status = RD_OVER_BUDGET;
    if (status == RD_OK && cudaStreamSynchronize(ctxs[c]->c.stream) != cudaSuccess) status = RD_SYNCHRONIZATION;
  }
  // Pinned staging for each image's mosaic, sRGB8 output and histogram,
  // unless the caller's buffers are pinned already (read and written in place).
  std::vector<size_t> in_off(count), out_off(count), hist_off(count);
  size_t total = 0;
  for (int k = 0; k < count && !host_pinned; ++k) {
    const rd_batch_item& it = items[k];
    in_off[k] = total;
    total += (sizeof(uint16_t) * it.row_stride * it.sensor.sensor_height + 255) & ~(size_t)255;
    out_off[k] = total;
    total += ((size_t)3 * it.target_width * it.target_height + 255) & ~(size_t)255;
    hist_off[k] = total;
    total += 1024 * sizeof(uint64_t);
  }
  unsigned char* stage = nullptr;
  if (status == RD_OK && !host_pinned &&
      cudaHostAlloc(reinterpret_cast<void**>(&stage), total, cudaHostAllocDefault) != cudaSuccess)
    status = RD_OVER_BUDGET;
  auto mosaic_of = [&](int k) {
    return host_pinned ? items[k].mosaic : reinterpret_cast<const uint16_t*>(stage + in_off[k]);
  };
  auto srgb_of = [&](int k) { return host_pinned ? items[k].srgb_out : stage + out_off[k]; };
  auto hist_of = [&](int k) {
    return host_pinned ? items[k].hist : reinterpret_cast<uint64_t*>(stage + hist_off[k]);
  };
  cudaStream_t main = nullptr;
  std::vector<cudaEvent_t> join(chains, nullptr);
  cudaEvent_t fork = nullptr;
  if (status == RD_OK && (cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking) != cudaSuccess ||
                          cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess))
    status = RD_SYNCHRONIZATION;
  for (int c = 0; c < chains && status == RD_OK; ++c)
    if (cudaEventCreateWithFlags(&join[c], cudaEventDisableTiming) != cudaSuccess) status = RD_SYNCHRONIZATION;
  for (int k = 0; k < count; ++k) items[k].status = RD_CANCELLED;

  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const auto c0 = Clock::now();
  if (status == RD_OK) {
    cudaSetDevice(device);
    if (cudaStreamBeginCapture(main, cudaStreamCaptureModeRelaxed) != cudaSuccess ||
        cudaEventRecord(fork, main) != cudaSuccess)
      status = RD_SYNCHRONIZATION;
    for (int c = 0; c < chains && status == RD_OK; ++c) {
      if (cudaStreamWaitEvent(ctxs[c]->c.stream, fork, 0) != cudaSuccess) status = RD_SYNCHRONIZATION;
      ctxs[c]->c.capturing = true;
    }
    for (int k = 0; k < count && status == RD_OK; ++k) {
      rd_batch_item& it = items[k];
      rd_ctx* ctx = ctxs[k % chains];
      const uint16_t* mosaic = mosaic_of(k);
      rd_source* src = nullptr;
      rd_base* base = nullptr;
      rd_status st = rd_develop(ctx, mosaic, it.row_stride, &it.sensor, &it.detail, nullptr, &src, nullptr);
      if (st == RD_OK)
        st = rd_spatial(ctx, src, &it.optics, it.target_width, it.target_height, it.wb_gains, it.camera_to_rec2020,
                        &base, nullptr);
      if (src) rd_source_release(src);
      if (st == RD_OK)
        st = rd_render(ctx, base, &it.color, srgb_of(k), hist_of(k), nullptr, nullptr);
      if (base) rd_base_release(base);
      if (st != RD_OK) status = st;
    }
    for (int c = 0; c < chains; ++c) {
      ctxs[c]->c.capturing = false;
      if (cudaEventRecord(join[c], ctxs[c]->c.stream) != cudaSuccess ||
          cudaStreamWaitEvent(main, join[c], 0) != cudaSuccess)
        if (status == RD_OK) status = RD_SYNCHRONIZATION;
    }
    const cudaError_t end = cudaStreamEndCapture(main, &graph);
    if (end != cudaSuccess && status == RD_OK) status = RD_SYNCHRONIZATION;
    if (status == RD_OK && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) status = RD_SYNCHRONIZATION;
    cudaGetLastError();
  }
  const auto c1 = Clock::now();
  if (capture_ms) *capture_ms = std::chrono::duration<double, std::milli>(c1 - c0).count();
  if (status == RD_OK) {
    const auto t0 = Clock::now();
    for (int k = 0; k < count && !host_pinned; ++k) {
      const rd_batch_item& it = items[k];
      std::memcpy(stage + in_off[k], it.mosaic, sizeof(uint16_t) * it.row_stride * it.sensor.sensor_height);
    }
    const auto l0 = Clock::now();
    if (cudaGraphLaunch(exec, main) != cudaSuccess || cudaStreamSynchronize(main) != cudaSuccess)
      status = RD_SYNCHRONIZATION;
    if (launch_ms) *launch_ms = std::chrono::duration<double, std::milli>(Clock::now() - l0).count();
    for (int c = 0; c < chains && status == RD_OK; ++c) {
      const rd::Status st = rd::check_kernel_error(ctxs[c]->c, "batch graph");
      if (!st.ok()) status = st.code;
    }
    if (status == RD_OK)
      for (int k = 0; k < count; ++k) {
        rd_batch_item& it = items[k];
        if (!host_pinned && it.srgb_out)
          std::memcpy(it.srgb_out, stage + out_off[k], (size_t)3 * it.target_width * it.target_height);
        if (!host_pinned && it.hist) std::memcpy(it.hist, stage + hist_off[k], 1024 * sizeof(uint64_t));
        it.status = RD_OK;
        it.ms = 0.0;
      }
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (cudaEvent_t e : join)
    if (e) cudaEventDestroy(e);
  if (fork) cudaEventDestroy(fork);
  if (main) cudaStreamDestroy(main);
  for (rd_ctx* c : ctxs)
    if (c) rd_ctx_destroy(c);
  if (stage) cudaFreeHost(stage);
  if (status != RD_OK)
    for (int k = 0; k < count; ++k)
      if (items[k].status == RD_OK) items[k].status = status;
  return status;
}
