// Internal declarations shared by the library's translation units.
//
// Device layout conventions:
//  * mosaics: row-major, pitch = width (f32) or row_stride (u16 input);
//  * camera / Rec.2020 RGB: three planar f32 planes R, G, B, each [h][w],
//    allocated as one buffer of 3*w*h floats so a plane is `base + c*w*h`;
//  * sRGB8 output: interleaved u8 [h][3w], the host format.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/rd_gpu.h"

namespace rd {

// ------------------------------------------------------------------ errors
struct Status {
  rd_status code = RD_OK;
  std::string message;
  bool ok() const { return code == RD_OK; }
};

#define RD_CUDA_TRY(expr)                                                                        \
  do {                                                                                           \
    cudaError_t rd_err_ = (expr);                                                                \
    if (rd_err_ != cudaSuccess)                                                                  \
      return ::rd::Status{RD_SYNCHRONIZATION, std::string(#expr) + ": " + cudaGetErrorString(rd_err_)}; \
  } while (0)

#define RD_TRY(expr)                 \
  do {                               \
    ::rd::Status rd_st_ = (expr);    \
    if (!rd_st_.ok()) return rd_st_; \
  } while (0)

// ------------------------------------------------------------------ context
// Kernel families timed by the optional per-launch event bracketing.
enum KernelFamily {
  K_NORMALIZE, K_OPPOSED, K_MHC, K_RCD, K_AMAZE, K_RL_MASK, K_RL_ITER, K_RL_APPLY, K_VIGNETTE,
  K_OPTICS, K_AREA, K_WB_MATRIX, K_COLOR, K_SYNTH, K_OUTPUT, K_ENCODE, K_FAMILY_COUNT
};
static_assert(K_FAMILY_COUNT == RD_KERNEL_FAMILIES, "family table size");
const char* kernel_family_name(int family);

// Keys of the cross-call launch-shape tuner (see shape_begin below): the
// kernel and three shape parameters (width, height, radius or 0).
enum TunedKernel { TUNE_RL_PREP = 0, TUNE_COLOR = 1, TUNE_OPTICS = 2, TUNE_KERNEL_COUNT };
struct ShapeKey {
  int kernel, a, b, c;
  bool operator<(const ShapeKey& o) const {
    if (kernel != o.kernel) return kernel < o.kernel;
    if (a != o.a) return a < o.a;
    if (b != o.b) return b < o.b;
    return c < o.c;
  }
};
struct ShapePick {
  int value = 0;
  cudaEvent_t start = nullptr;  // set when this launch is timed
};
struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;     // 0 = unlimited
  uint64_t reserved = 0;   // bytes currently held by this context
  uint64_t launches = 0;   // kernels launched by this library on this context
  std::string last_error;
  // Error word written by kernels (bounds/footprint/non-finite), read after a stage.
  uint32_t* d_error = nullptr;
  // Work-item counter of the dynamically scheduled kernels (beside d_error):
  // zero between launches, put back to zero by each launch's last fetch.
  uint32_t* d_work = nullptr;
  // AMaZE per-CTA scratch slots (kept across calls).
  float* amaze_scratch = nullptr;
  size_t amaze_slots = 0;  // tiles the AMaZE scratch holds slabs and flags for
  size_t amaze_bytes = 0;
  int sm_count = 0;
  cudaEvent_t ev[8] = {};
  // Sizes of the allocations handed out through rd_device_alloc.
  std::unordered_map<void*, size_t> user_allocs;
  // Measurement: user event slots, an L2 flush buffer and per-family kernel timing.
  cudaEvent_t user_ev[64] = {};
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  bool timing = false;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  double family_ms[K_FAMILY_COUNT] = {};
  uint64_t family_launches[K_FAMILY_COUNT] = {};
  // While the stream is being captured into a CUDA graph: no host
  // synchronisation or readback (errors are read after the graph runs), and
  // host tables reach the device from pinned copies kept until the context
  // is destroyed.
  bool capturing = false;
  // A low-priority lane beside a latency-sensitive one: kernels that would
  // otherwise keep their CTAs resident across work items (AMaZE) end each CTA
  // after one item, so that a higher-priority stream's kernels get SMs within
  // one item.
  bool yield_sms = false;
  std::vector<void*> pinned_uploads;
  // Timed RL iterations of a launch-shape tuning run, resolved after the
  // stage's synchronisation: (candidate segment count, start, end).
  int tune_shape[3] = {0, 0, 0};
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> tune_runs;
  // Timed candidate launches of the cross-call shape tuner: (key, value, start, end).
  struct ShapeRun {
    ShapeKey key;
    int value;
    cudaEvent_t a, b;
  };
  std::vector<ShapeRun> shape_runs;
  // Bounded device waits (rd_ctx_set_wait_test): the iteration limit of each
  // wait, and which completion a test withholds so that a wait runs out.
  uint32_t wait_limit = 0;      // 0: the built-in limits
  int32_t wait_withhold = 0;    // RD_WAIT_* of include/rd_gpu.h
};

// Iteration limits of the device waits when no test sets one.
constexpr uint32_t AMAZE_DEFAULT_WAIT_TRIES = 1u << 22;
constexpr uint32_t RL_DEFAULT_WAIT_TRIES = 1u << 20;

// ---- launch-shape tuning across calls (tuner.cu) ----
// Kernels launched once per call whose launch shape (a work-item count or a
// grid size) changes only the schedule, never a value. The first calls for a
// (kernel, shape) key each launch one candidate, bracketed by events on the
// context stream and resolved at the call's synchronisation; once every
// candidate has been timed twice, the fastest is used for the key from then
// on, in every context of the process.
//
// The shape to launch with now: the tuned one, the next candidate still to
// time (start event recorded), or the default (under stream capture).
ShapePick shape_begin(Context& ctx, const ShapeKey& key, int default_value, const std::vector<int>& candidates);
// After the launch: records the end event of a timed launch.
void shape_end(Context& ctx, const ShapeKey& key, const ShapePick& pick);
// Folds the context's timed launches into the table (after a synchronisation).
void resolve_shape_tuning(Context& ctx);
// The table's entry for a key: tuned value, default, their best times; false until tuned.
bool shape_record(const ShapeKey& key, int* value, int* default_value, float* best_ms, float* default_ms);

// Brackets one kernel launch with events when kernel timing is enabled, and
// counts the launch either way.
struct LaunchScope {
  Context& ctx;
  int family;
  cudaEvent_t a = nullptr, b = nullptr;
  LaunchScope(Context& c, int f);
  ~LaunchScope();
};
// Resolves the pending launch events into per-family totals (after a sync).
void resolve_kernel_timing(Context& ctx);

#define RD_LAUNCH(ctx, family, ...)              \
  do {                                           \
    ::rd::LaunchScope rd_scope_((ctx), (family)); \
    __VA_ARGS__;                                 \
  } while (0)

// Host -> device copy of a host table on the context's stream. The source may
// be released as soon as the call returns (under capture it is copied into a
// pinned buffer that the graph reads).
Status upload(Context& ctx, void* dst, const void* src, size_t bytes);

Status reserve(Context& ctx, size_t bytes);
void release(Context& ctx, size_t bytes);
Status device_alloc(Context& ctx, size_t bytes, void** out);
void device_free(Context& ctx, void* ptr, size_t bytes);
Status check_kernel_error(Context& ctx, const char* stage);
Status set_stream_priority(Context& ctx, bool high);

// ------------------------------------------------------------------ mosaic source
// Per-sample view of the (cropped, normalized, highlight-processed) mosaic,
// optionally scaled by the demosaic channel balance. Either reads the raw u16
// sensor data and applies normalization + Clip on the fly (fused path), or
// reads an already reconstructed f32 mosaic (after Opposed).
struct MosaicSource {
  const uint16_t* raw;    // sensor samples, or null
  const float* f32;       // crop-sized normalized mosaic (pitch = width), or null
  long long row_stride;   // raw row stride in samples
  int crop_x, crop_y;
  int sensor_cfa;         // CFA at sensor (0,0)
  int width, height;      // crop size
  int cfa;                // CFA at crop (0,0)
  int black_w, black_h;
  int white_count;
  int clip;               // 1: apply Clip ceilings after normalization
  float clip_levels[3];
  float fwd[3];           // balance multipliers (1,1,1 when not balanced)
  float black[RD_MAX_LEVEL_PATTERN];
  float white[RD_MAX_LEVEL_PATTERN];
};

__host__ __device__ inline int color_at(int pattern, int x, int y) {
  // BayerPattern::color_at: RGGB, BGGR, GRBG, GBRG packed 2 bits per site.
  const unsigned table = pattern == 0 ? 0x94u : pattern == 1 ? 0x16u : pattern == 2 ? 0x61u : 0x49u;
  return (table >> (2 * (((y & 1) << 1) | (x & 1)))) & 3;
}

__host__ __device__ inline int shifted_cfa(int pattern, int x, int y) {
  const int px = x & 1, py = y & 1;
  if (!px && !py) return pattern;
  // A column shift maps RGGB<->GRBG and BGGR<->GBRG (p ^ 2); a row shift maps
  // RGGB<->GBRG and BGGR<->GRBG (3 - p).
  int p = pattern;
  if (px) p ^= 2;
  if (py) p = 3 - p;
  return p;
}

// NormalizationContract::normalize of one raw sample at sensor coordinates
// (sx, sy), with the black / white levels of that position.
__device__ __forceinline__ float normalize_raw(const MosaicSource& s, float sample, int sx, int sy) {
  // Level patterns repeat every 1, 2 or 4 samples in practice: mask instead of divide.
  const int by = (s.black_h & (s.black_h - 1)) == 0 ? (sy & (s.black_h - 1)) : sy % s.black_h;
  const int bx = (s.black_w & (s.black_w - 1)) == 0 ? (sx & (s.black_w - 1)) : sx % s.black_w;
  const int bi = by * s.black_w + bx;
  const float black = s.black[bi];
  float white;
  if (s.white_count == 1) white = s.white[0];
  else if (s.white_count == 3) white = s.white[color_at(s.sensor_cfa, sx, sy)];
  else white = s.white[bi];
  return __fdiv_rn(__fsub_rn(sample, black), __fsub_rn(white, black));
}

// Normalized sample at crop coordinates (x, y) before any highlight step:
// NormalizationContract::normalize with levels at sensor coordinates.
__device__ __forceinline__ float source_normalized(const MosaicSource& s, int x, int y) {
  if (s.f32) return s.f32[(long long)y * s.width + x];
  const int sx = s.crop_x + x, sy = s.crop_y + y;
  return normalize_raw(s, (float)s.raw[(long long)sy * s.row_stride + sx], sx, sy);
}

// Normalized, highlight-processed sample (Clip applied when selected), before balance.
__device__ __forceinline__ float source_linear(const MosaicSource& s, int x, int y) {
  float v = source_normalized(s, x, y);
  if (s.clip) {
    const float limit = s.clip_levels[color_at(s.cfa, x, y)];
    if (v > limit) v = limit;
  }
  return v;
}

__device__ __forceinline__ float source_balanced(const MosaicSource& s, int x, int y) {
  const float v = source_linear(s, x, y);
  return __fmul_rn(v, s.fwd[color_at(s.cfa, x, y)]);
}

// mirror_coordinate (whole-sample reflection, parity preserving).
__device__ __forceinline__ int mirror_index(int index, int length) {
  if (length <= 1) return 0;
  const int period = 2 * (length - 1);
  int w = index % period;
  if (w < 0) w += period;
  return w < period - w ? w : period - w;
}

// ------------------------------------------------------------------ stage launchers
// Each returns after enqueueing on ctx.stream. Planar RGB outputs.
Status launch_normalize(Context& ctx, const MosaicSource& src, float* out, unsigned long long* clip_stats);
// Opposed on the normalized samples of `src` (Clip is never applied here): the
// reconstructed crop-sized mosaic is written to `mosaic` (width*height f32).
// With src.f32 == mosaic the reconstruction is in place; otherwise the cell
// pass normalizes the raw samples and writes every one of them to `mosaic`.
Status run_opposed(Context& ctx, const MosaicSource& src, float* mosaic, const float levels[3], const float* ceiling,
                   unsigned long long* d_stats, uint32_t* region_count);
Status run_opposed_labels(Context& ctx, const MosaicSource& src, float* mosaic, const float levels[3],
                          const float* ceiling, unsigned long long* d_stats, uint32_t* labels_out,
                          uint32_t* region_count);
Status run_demosaic(Context& ctx, const MosaicSource& src, int algorithm, float* rgb, unsigned long long* clip_stats);
Status run_capture(Context& ctx, float* rgb, int width, int height, const rd_detail_desc& detail);
// Capture sharpening of several images (the batched develop's flat pass): the
// guide / mask pass image by image, every iteration of the images that share
// their taps in one launch over all their work items, then the gain image by
// image; each image ends bit for bit as run_capture leaves it. A job's status
// reports its own failure; the return value the first launch failure.
struct CaptureJob {
  float* rgb;
  int W, H;
  rd_detail_desc detail;
  Status st;
};
Status run_capture_images(Context& ctx, CaptureJob* jobs, int n);
// Vignetting multiplier plane (width*height f32) of an optics execution.
Status run_vignette_plane(Context& ctx, const rd_optics_desc& optics, float* mult);
// Radial multiplier table of one optics execution (RadialMultipliers,
// crates/optics/src/radial.rs:157-229): RADIAL_KNOTS knots of
// [m_red, m_green, m_blue, pin] at radii i * step, where pin is the break
// radius of a freeze boundary pinned inside segment [i, i + 1], or NaN.
constexpr int RADIAL_KNOTS = 1024;
enum {
  RD_RADIAL_NONE = -1,  // no radial work: the remap needs no table
  RD_RADIAL_ACCEPTED = 0,
  RD_RADIAL_NON_FINITE = 1,
  RD_RADIAL_TRIPWIRE = 2,
  RD_RADIAL_BREAK_COLLISION = 3,
  RD_RADIAL_FREEZE_AMBIGUITY = 4,
  RD_RADIAL_UNEXPLAINED_JUMP = 5,
};
struct RadialTable {
  int guard = RD_RADIAL_NONE;
  float step = 0.0f;
  std::vector<float> knots;  // 4 per knot
};
// The per-column then per-row input (lens) coordinates of an optics execution
// (plan.rs:119-130, narrowed to f32): width + height values.
std::vector<float> optics_input_coordinates(const rd_optics_desc& optics);
// `input_x` / `input_y`: the per-column and per-row input (lens) coordinates.
RadialTable build_radial_table(const rd_optics_desc& optics, const float* input_x, const float* input_y);
// Distortion / TCA gather; `mult` (optional) is the vignetting plane applied to
// each source sample as it is read.
Status run_optics_gather(Context& ctx, const rd_optics_desc& optics, const float* rgb_in, const float* mult,
                         float* rgb_out);
// Exact area reduction of planar RGB to tw x th (one pass, no intermediate
// plane); `mult` (optional) is applied to each source sample as it is read.
Status run_area_reduce(Context& ctx, const float* rgb, const float* mult, int width, int height, int tw, int th,
                       float* out);
Status run_wb_matrix(Context& ctx, float* rgb, size_t pixels, const float gains[3], const float matrix[9]);
Status run_color_output(Context& ctx, const float* rgb, int width, int height, const rd_color_desc& color,
                        bool camera_native, uint8_t* srgb, unsigned long long* d_hist);
Status run_synth(Context& ctx, const rd_synth_desc& desc, uint16_t* out);

// PNG encoding (k_encode.cu) of interleaved RGB rows, 8 or 16 bits per sample.
// png_header builds the signature, IHDR and the optional iCCP / eXIf chunks;
// png_bound is the largest file the encoder writes after that header;
// run_png_encode writes header + IDAT chunks + IEND into d_png and the file's
// byte count into *d_png_bytes (device memory), on the context's stream.
uint64_t png_stream_bytes(int W, int H, int depth);
Status png_header(int W, int H, int depth, const uint8_t* icc, size_t icc_len, const uint8_t* exif, size_t exif_len,
                  std::vector<uint8_t>* out);
uint64_t png_bound(int W, int H, int depth, uint64_t header_bytes);
bool png_metadata_ok(uint64_t icc_len, uint64_t exif_len);
uint64_t png_header_bytes(uint64_t icc_len, uint64_t exif_len);
Status run_png_encode(Context& ctx, const void* d_rgb, int W, int H, int depth, const std::vector<uint8_t>& header,
                      uint8_t* d_png, uint64_t* d_png_bytes);

// JPEG encoding (k_jpeg.cu) of interleaved 8-bit RGB rows at quality 1..100.
// jpeg_bound is the largest file; run_jpeg_encode writes the whole file into
// d_file and its byte count into *d_file_bytes (device memory). It reads the
// image's symbol counts back to build the Huffman tables, so it synchronises
// the stream once and cannot run under graph capture.
Status jpeg_check(int W, int H, int quality);
bool jpeg_metadata_ok(uint64_t icc_len, uint64_t exif_len);
uint64_t jpeg_bound(int W, int H, uint64_t icc_len, uint64_t exif_len);
Status run_jpeg_encode(Context& ctx, const uint8_t* d_rgb, int W, int H, int quality, const uint8_t* icc,
                       size_t icc_len, const uint8_t* exif, size_t exif_len, uint8_t* d_file, uint64_t* d_file_bytes);
// One launch rendering several bases (render path of the served loop). The
// staging buffers (host pinned and device, color_batch_staging_bytes(n) each)
// carry the per-image parameters and LUTs.
struct ColorBatchItem {
  const float* rgb;  // planar Rec.2020 base
  int width, height;
  const rd_color_desc* color;
  uint8_t* srgb;              // device [height][3 width]
  unsigned long long* hist;   // device 1024 bins, cleared by the call
};
size_t color_batch_staging_bytes(int n);
Status run_color_batch(Context& ctx, const ColorBatchItem* items, int n, void* d_staging, void* h_staging);

// Display / extended output (k_output.cu). The geometry is OutputGeometry of
// the reference resolved on the host: the axis swap and mirrors of the
// orientation, and the crop rectangle on the oriented canvas.
struct OutputGeometry {
  int swap, flip_h, flip_v;
  int src_w, src_h;
  int left, top, width, height;  // crop origin and output size
};
size_t output_bytes_per_pixel(int format);  // 0 for an unknown format
Status resolve_output_geometry(int width, int height, const rd_output_desc& output, OutputGeometry* g);
// rgb: planar linear Rec.2020 of g.src_w x g.src_h. d_hist (1024 bins, 8-bit
// output only) and d_gamut (5 counters) may be null; both are cleared first.
Status run_display_output(Context& ctx, const float* rgb, const rd_color_desc& color, const rd_output_desc& output,
                          const OutputGeometry& g, void* d_out, unsigned long long* d_hist,
                          unsigned long long* d_gamut);
// Exhaustive device checks of the correctly rounded arithmetic (rd_check_math).
Status run_math_check(Context& ctx, int which, uint64_t* result);
// Sampled device check of the optics branch's f32 hypot (rd_check_math 4).
Status run_hypot_check(Context& ctx, uint64_t* result);

// One image of a (multi-image) AMaZE launch: its mosaic source with the
// forward channel balance in fwd, the planar RGB output, and the inverse
// balance and clip point of demosaic_cancellable (crates/demosaic/src/lib.rs:302-392).
struct AmazeJob {
  MosaicSource src;
  float* rgb;
  int count_clip;
  unsigned long long* clip_stats;
  float gains[3];
  float clip_point;
};
// The launch parameters of demosaicing `src_in` (as-shot balance in fwd) with
// `algorithm` into `rgb`: the balanced source, inverse gains, clip point and
// whether Clip statistics are counted.
AmazeJob demosaic_job(const MosaicSource& src_in, int algorithm, float* rgb, unsigned long long* clip_stats);
// AMaZE of n images (each larger than 32x32) in one launch over a shared
// queue of half-tile work items.
Status run_amaze_images(Context& ctx, const AmazeJob* jobs, int n);
Status reserve_amaze_scratch(Context& ctx, size_t tiles);
// AMaZE tiles of a width x height mosaic (224-pixel cores).
size_t amaze_tiles(int width, int height);
// Folds the timed RL iterations of a tuning run into the process-wide table of
// launch shapes (k_capture.cu); called after a synchronisation.
void resolve_rl_tuning(Context& ctx);

// Host contract helpers.
int gaussian_kernel(float sigma, float* weights, int max_taps);
Status optics_plan(rd_optics_desc& optics, float crop, float real_focal, float cx, float cy);
void standard_base_lut(float* lut);
void light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks, float* lut);

}  // namespace rd
