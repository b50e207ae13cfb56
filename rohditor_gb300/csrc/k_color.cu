// White balance + camera matrix, the global adjustment chain, sRGB 8-bit
// output and the display histogram on sm_103a.
//
//  WB + matrix   crates/core/src/cpu/stages.rs:250-308 (dot order of matrix.rs:173-175)
//  adjustments   crates/core/src/cpu/stages.rs:380-528 and helpers :605-901
//                (exposure, base rendering LUT, tone curve LUT, saturation /
//                vibrance, 8-band HSL, 3-way grading; local masks are not part
//                of this path)
//  output        render_display8 (stages.rs:1028-1094): Rec.2020 -> XYZ ->
//                linear sRGB (Matrix3::then), hard clip, sRGB transfer,
//                round(v * 255), clamp
//  histogram     Histogram::count (crates/core/src/analysis/histogram.rs:92-128):
//                R, G, B and integer Rec.709 luma bins of the 8-bit output,
//                counted in shared memory and flushed once per CTA.
// The output kernel reads the planar base once and writes the interleaved u8
// image once; the histogram never leaves the SM until its final flush.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "color_chain.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

struct ColorParams {
  const float* in;   // planar [3][h][w]
  int W, H;
  int camera_native; // 1: apply WB + matrix first (stage entry point)
  float wb[3];
  float m[9];
  AdjustParams adj;
  float out_m[9];    // Rec.2020 -> linear sRGB
  unsigned char* out;
  unsigned long long* hist;  // 1024 bins
};

// The adjustment chain, output transform, sRGB8 quantisation and histogram
// bins of one base pixel (index i of a plane of `plane` pixels).
__device__ __forceinline__ void color_pixel(const ColorParams& p, long long i, long long plane, unsigned int* bins) {
  float v[3] = {p.in[i], p.in[plane + i], p.in[2 * plane + i]};
  if (p.camera_native) {
    v[0] *= p.wb[0];
    v[1] *= p.wb[1];
    v[2] *= p.wb[2];
    const float a = v[0], b = v[1], c = v[2];
    v[0] = p.m[0] * a + p.m[1] * b + p.m[2] * c;
    v[1] = p.m[3] * a + p.m[4] * b + p.m[5] * c;
    v[2] = p.m[6] * a + p.m[7] * b + p.m[8] * c;
  }
  apply_adjustments(p.adj, v);
  float lin[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float l = p.out_m[3 * r] * v[0] + p.out_m[3 * r + 1] * v[1] + p.out_m[3 * r + 2] * v[2];
    if (isnan(l) || l == -INFINITY) l = 0.0f;
    else if (l == INFINITY) l = 1.0f;
    else l = rclamp(l, 0.0f, 1.0f);
    lin[r] = l;
  }
  // (encoded * 255 + dither).round().clamp(0, 255) with DitherMode::None.
  float code[3];
  quantize_srgb3(lin, 255.0f, 0.0f, code);
  const unsigned char q[3] = {(unsigned char)code[0], (unsigned char)code[1], (unsigned char)code[2]};
  const long long y = i / p.W, x = i % p.W;
  unsigned char* o = p.out + y * 3 * p.W + 3 * x;
  o[0] = q[0];
  o[1] = q[1];
  o[2] = q[2];
  atomicAdd(&bins[q[0]], 1u);
  atomicAdd(&bins[256 + q[1]], 1u);
  atomicAdd(&bins[512 + q[2]], 1u);
  atomicAdd(&bins[768 + (2126u * q[0] + 7152u * q[1] + 722u * q[2] + 5000u) / 10000u], 1u);
}

__global__ void __launch_bounds__(256, 4) color_kernel(const ColorParams p) {
  __shared__ unsigned int bins[1024];
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) bins[k] = 0;
  __syncthreads();
  const long long plane = (long long)p.W * p.H;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += (long long)gridDim.x * blockDim.x)
    color_pixel(p, i, plane, bins);
  __syncthreads();
  for (int k = threadIdx.x; k < 1024; k += blockDim.x)
    if (bins[k]) atomicAdd(&p.hist[k], (unsigned long long)bins[k]);
}

// Several bases in one launch: blocks [block_start[k], block_start[k+1]) render
// image k with params[k]; each block stages its image's parameters in shared
// memory and flushes its histogram to that image's bins.
__global__ void __launch_bounds__(256) color_batch_kernel(const ColorParams* __restrict__ params,
                                                          const int* __restrict__ block_start, int n) {
  __shared__ unsigned int bins[1024];
  __shared__ ColorParams sp;
  const int b = blockIdx.x;
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (block_start[mid] <= b) lo = mid;
    else hi = mid;
  }
  if (threadIdx.x == 0) sp = params[lo];
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) bins[k] = 0;
  __syncthreads();
  const long long plane = (long long)sp.W * sp.H;
  const int first = block_start[lo], nb = block_start[lo + 1] - first;
  for (long long i = (long long)(b - first) * blockDim.x + threadIdx.x; i < plane; i += (long long)nb * blockDim.x)
    color_pixel(sp, i, plane, bins);
  __syncthreads();
  for (int k = threadIdx.x; k < 1024; k += blockDim.x)
    if (bins[k]) atomicAdd(&sp.hist[k], (unsigned long long)bins[k]);
}

__global__ void wb_matrix_kernel(float* rgb, long long plane, float g0, float g1, float g2, float m0, float m1, float m2,
                                 float m3, float m4, float m5, float m6, float m7, float m8) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= plane) return;
  const float a = rgb[i] * g0, b = rgb[plane + i] * g1, c = rgb[2 * plane + i] * g2;
  rgb[i] = m0 * a + m1 * b + m2 * c;
  rgb[plane + i] = m3 * a + m4 * b + m5 * c;
  rgb[2 * plane + i] = m6 * a + m7 * b + m8 * c;
}

}  // namespace

Status run_wb_matrix(Context& ctx, float* rgb, size_t pixels, const float g[3], const float m[9]) {
  RD_LAUNCH(ctx, K_WB_MATRIX, wb_matrix_kernel<<<(unsigned)((pixels + 255) / 256), 256, 0, ctx.stream>>>(
      rgb, (long long)pixels, g[0], g[1], g[2], m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]));
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

Status run_color_output(Context& ctx, const float* rgb, int W, int H, const rd_color_desc& c, bool camera_native,
                        uint8_t* srgb, unsigned long long* d_hist) {
  // LUTs live in one device buffer for the call.
  ColorParams p{};
  p.in = rgb;
  p.W = W;
  p.H = H;
  p.camera_native = camera_native ? 1 : 0;
  for (int k = 0; k < 3; ++k) p.wb[k] = c.wb_gains[k];
  for (int k = 0; k < 9; ++k) p.m[k] = c.camera_to_rec2020[k];
  p.adj = adjust_params(c);
  rec2020_to_display(XYZ_TO_SRGB, p.out_m);
  p.out = srgb;
  p.hist = d_hist;
  float* luts = nullptr;
  if (has_any_lut(c)) {
    void* d = nullptr;
    RD_TRY(device_alloc(ctx, LUT_SET_BYTES, &d));
    luts = static_cast<float*>(d);
    if (c.has_base_lut) RD_TRY(upload(ctx, luts, c.base_lut, sizeof(float) * LUT_ENTRIES));
    if (c.has_light_tone_lut) RD_TRY(upload(ctx, luts + LUT_ENTRIES, c.light_tone_lut, sizeof(float) * LUT_ENTRIES));
    if (c.has_tone_lut) RD_TRY(upload(ctx, luts + 2 * LUT_ENTRIES, c.tone_lut, sizeof(float) * LUT_ENTRIES));
  }
  set_lut_pointers(p.adj, c, luts);
  const long long pixels = (long long)W * H;
  // Grid-stride CTAs per SM: tuned across calls per image shape (the grid
  // changes only which CTA takes which pixels; the histogram is integer).
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const ShapeKey key{TUNE_COLOR, W, H, 0};
  const ShapePick pick = shape_begin(ctx, key, 8, {4, 16, 32});
  const int grid = (int)std::min<long long>((pixels + 255) / 256, (long long)sms * pick.value);
  RD_LAUNCH(ctx, K_COLOR, color_kernel<<<grid, 256, 0, ctx.stream>>>(p));
  shape_end(ctx, key, pick);
  const cudaError_t launch = cudaGetLastError();
  if (luts) device_free(ctx, luts, LUT_SET_BYTES);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

}  // namespace rd

// ---- several bases in one launch ---------------------------------------------
namespace rd {
namespace {

// Adjustment parameters of a non-camera-native render (the base already holds
// white-balanced Rec.2020); buffers and LUT pointers are filled by the caller.
ColorParams base_color_params(const rd_color_desc& c) {
  ColorParams p{};
  p.camera_native = 0;
  p.adj = adjust_params(c);
  rec2020_to_display(XYZ_TO_SRGB, p.out_m);
  return p;
}

constexpr int BATCH_PIXELS_PER_THREAD = 16;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

size_t color_batch_staging_bytes(int n) {
  return align256(sizeof(ColorParams) * n) + align256(sizeof(int) * (n + 1)) + LUT_SET_BYTES * (size_t)n;
}

Status run_color_batch(Context& ctx, const ColorBatchItem* items, int n, void* d_staging, void* h_staging) {
  if (n <= 0) return Status{};
  unsigned char* hb = static_cast<unsigned char*>(h_staging);
  unsigned char* db = static_cast<unsigned char*>(d_staging);
  ColorParams* hp = reinterpret_cast<ColorParams*>(hb);
  const size_t off_starts = align256(sizeof(ColorParams) * n);
  const size_t off_luts = off_starts + align256(sizeof(int) * (n + 1));
  int* hs = reinterpret_cast<int*>(hb + off_starts);
  float* hl = reinterpret_cast<float*>(hb + off_luts);
  float* dl = reinterpret_cast<float*>(db + off_luts);
  int blocks = 0;
  for (int k = 0; k < n; ++k) {
    const ColorBatchItem& it = items[k];
    ColorParams p = base_color_params(*it.color);
    p.in = it.rgb;
    p.W = it.width;
    p.H = it.height;
    p.out = it.srgb;
    p.hist = it.hist;
    stage_luts(*it.color, hl + (size_t)LUT_SET_ENTRIES * k);
    set_lut_pointers(p.adj, *it.color, dl + (size_t)LUT_SET_ENTRIES * k);
    hp[k] = p;
    hs[k] = blocks;
    const long long pixels = (long long)it.width * it.height;
    blocks += (int)((pixels + 256LL * BATCH_PIXELS_PER_THREAD - 1) / (256LL * BATCH_PIXELS_PER_THREAD));
  }
  hs[n] = blocks;
  RD_CUDA_TRY(cudaMemcpyAsync(d_staging, h_staging, color_batch_staging_bytes(n), cudaMemcpyHostToDevice, ctx.stream));
  for (int k = 0; k < n; ++k)
    RD_CUDA_TRY(cudaMemsetAsync(items[k].hist, 0, 1024 * sizeof(unsigned long long), ctx.stream));
  RD_LAUNCH(ctx, K_COLOR, color_batch_kernel<<<blocks, 256, 0, ctx.stream>>>(
                              reinterpret_cast<const ColorParams*>(db), reinterpret_cast<const int*>(db + off_starts), n));
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

}  // namespace rd

// ---- allocation-free render ------------------------------------------------
// rd_render_device_noalloc renders a base that the caller already holds in
// device memory into device buffers the caller owns, and allocates nothing.
// It is for callers that cannot allocate on the render path: an interactive
// editor re-renders the preview on every slider event, often from a UI or
// frame-callback thread, where a device allocation can block on the allocator
// or on device-wide synchronisation, and where the device working set has
// been sized and reserved up front under a fixed budget. The only per-call
// scratch of the render, the three 4096-entry LUTs, is staged in the
// file-scope array below instead of a stream-ordered buffer.
namespace rd {
namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
// One LUT set (base rendering, Light tone, tone curve; 48 KB), laid out as
// set_lut_pointers expects.
__device__ __align__(256) float g_noalloc_luts[LUT_SET_ENTRIES];

struct NoallocDevice {
  float* luts = nullptr;  // device address of g_noalloc_luts on this device
  int sm_count = 0;
};
std::mutex g_noalloc_mutex;
NoallocDevice g_noalloc_devices[NOALLOC_MAX_DEVICES];

// Resolves the array's address once per device, with that device current.
// The first call may load this file's module on the device.
rd_status noalloc_device(int device, NoallocDevice* out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoallocDevice& d = g_noalloc_devices[device];
  if (!d.luts) {
    float* p = nullptr;
    if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_luts) != cudaSuccess || !p) {
      cudaGetLastError();
      return RD_SYNCHRONIZATION;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
      cudaGetLastError();
      return RD_SYNCHRONIZATION;
    }
    d.luts = p;
    d.sm_count = sms;
  }
  *out = d;
  return RD_OK;
}

}  // namespace
}  // namespace rd

extern "C" rd_status rd_render_device_noalloc(const float* d_base, uint32_t width, uint32_t height,
                                              const rd_color_desc* color, uint8_t* d_srgb_out,
                                              uint64_t* d_hist, void* stream) {
  using namespace rd;
  if (!d_base || !color || !d_srgb_out || !d_hist) return RD_INVALID_INPUT;
  if (width == 0 || height == 0 || width > (uint32_t)INT32_MAX || height > (uint32_t)INT32_MAX)
    return RD_INVALID_INPUT;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) {
    cudaGetLastError();
    return RD_SYNCHRONIZATION;
  }
  if (device < 0 || device >= NOALLOC_MAX_DEVICES) return RD_INVALID_INPUT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The LUTs are copied from the caller's pageable descriptor on every call,
  // which a stream being captured cannot record: such a call is refused
  // before anything is enqueued.
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) {
    cudaGetLastError();
    return RD_INVALID_INPUT;
  }
  if (capture != cudaStreamCaptureStatusNone) return RD_INVALID_INPUT;
  NoallocDevice dev;
  const rd_status setup = noalloc_device(device, &dev);
  if (setup != RD_OK) return setup;
  const rd_color_desc& c = *color;
  ColorParams p{};
  p.in = d_base;
  p.W = (int)width;
  p.H = (int)height;
  p.camera_native = 0;
  p.adj = adjust_params(c);
  rec2020_to_display(XYZ_TO_SRGB, p.out_m);
  p.out = d_srgb_out;
  p.hist = reinterpret_cast<unsigned long long*>(d_hist);
  // The histogram accumulates with atomics, so it must start at zero; the LUTs
  // are overwritten whole before the kernel reads them.
  if (cudaMemsetAsync(d_hist, 0, 1024 * sizeof(uint64_t), s) != cudaSuccess) {
    cudaGetLastError();
    return RD_SYNCHRONIZATION;
  }
  const float* tables[3] = {c.has_base_lut ? c.base_lut : nullptr,
                            c.has_light_tone_lut ? c.light_tone_lut : nullptr,
                            c.has_tone_lut ? c.tone_lut : nullptr};
  for (int t = 0; t < 3; ++t) {
    if (tables[t] && cudaMemcpyAsync(dev.luts + t * LUT_ENTRIES, tables[t], sizeof(float) * LUT_ENTRIES,
                                     cudaMemcpyHostToDevice, s) != cudaSuccess) {
      cudaGetLastError();
      return RD_SYNCHRONIZATION;
    }
  }
  set_lut_pointers(p.adj, c, dev.luts);
  const long long pixels = (long long)width * height;
  const int grid = (int)std::min<long long>((pixels + 255) / 256, (long long)dev.sm_count * 8);
  color_kernel<<<grid, 256, 0, s>>>(p);
  if (cudaGetLastError() != cudaSuccess) return RD_SYNCHRONIZATION;
  return RD_OK;
}
