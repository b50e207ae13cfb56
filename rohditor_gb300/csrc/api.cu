// The C ABI (include/rd_gpu.h): context, processor API, stage entry points and
// host contract helpers. Everything device-side is ordered on the context's
// stream; device memory comes from the stream-ordered pool (cudaMallocAsync)
// and is charged against the context's byte budget before it is taken, like
// the reference's logical reservations (crates/gpu/src/memory.rs:44-60).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "rd_internal.cuh"

#include "rd_handles.cuh"

namespace rd {

Status run_amaze(Context& ctx, const MosaicSource& src, const float gains[3], float clip_point, float* rgb,
                 int count_clip, unsigned long long* clip_stats);

Status reserve(Context& ctx, size_t bytes) {
  if (ctx.budget && ctx.reserved + bytes > ctx.budget)
    return Status{RD_OVER_BUDGET, "device working set of " + std::to_string(ctx.reserved + bytes) +
                                      " bytes exceeds the budget of " + std::to_string(ctx.budget)};
  ctx.reserved += bytes;
  return Status{};
}
void release(Context& ctx, size_t bytes) { ctx.reserved -= std::min<uint64_t>(bytes, ctx.reserved); }

Status device_alloc(Context& ctx, size_t bytes, void** out) {
  *out = nullptr;
  if (bytes == 0) bytes = 16;
  RD_TRY(reserve(ctx, bytes));
  const cudaError_t e = cudaMallocAsync(out, bytes, ctx.stream);
  if (e != cudaSuccess) {
    release(ctx, bytes);
    cudaGetLastError();
    return Status{RD_OVER_BUDGET, std::string("device allocation failed: ") + cudaGetErrorString(e)};
  }
  return Status{};
}
void device_free(Context& ctx, void* ptr, size_t bytes) {
  if (!ptr) return;
  cudaFreeAsync(ptr, ctx.stream);
  release(ctx, bytes == 0 ? 16 : bytes);
}

const char* kernel_family_name(int family) {
  static const char* names[K_FAMILY_COUNT] = {
      "normalize", "opposed", "mhc_bilinear", "rcd", "amaze", "rl_mask", "rl_iteration",
      "rl_apply", "vignetting", "optics_gather", "area_reduce", "wb_matrix",
      "color_output", "synth", "display_output", "file_encode"};
  return family >= 0 && family < K_FAMILY_COUNT ? names[family] : "unknown";
}

LaunchScope::LaunchScope(Context& c, int f) : ctx(c), family(f) {
  ctx.launches++;
  ctx.family_launches[f]++;
  if (!ctx.timing) return;
  auto take = [&]() {
    cudaEvent_t e = nullptr;
    if (!ctx.event_pool.empty()) {
      e = ctx.event_pool.back();
      ctx.event_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  };
  a = take();
  b = take();
  cudaEventRecord(a, ctx.stream);
}

LaunchScope::~LaunchScope() {
  if (!a) return;
  cudaEventRecord(b, ctx.stream);
  ctx.pending.push_back({family, {a, b}});
}

void resolve_kernel_timing(Context& ctx) {
  for (auto& p : ctx.pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess) ctx.family_ms[p.first] += ms;
    ctx.event_pool.push_back(p.second.first);
    ctx.event_pool.push_back(p.second.second);
  }
  ctx.pending.clear();
  cudaGetLastError();
}

// Reads and clears the kernels' error word; one synchronization point per call.
// Recreates the context's stream at the device's highest (or lowest) priority;
// the stream must be idle.
Status set_stream_priority(Context& c, bool high) {
  int least = 0, greatest = 0;
  RD_CUDA_TRY(cudaSetDevice(c.device));
  RD_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  RD_CUDA_TRY(cudaStreamSynchronize(c.stream));
  cudaStream_t s = nullptr;
  RD_CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, high ? greatest : least));
  cudaStreamDestroy(c.stream);
  c.stream = s;
  return Status{};
}

Status upload(Context& ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx.capturing) {
    RD_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx.stream));
    return Status{};
  }
  void* pinned = nullptr;
  RD_CUDA_TRY(cudaHostAlloc(&pinned, bytes, cudaHostAllocDefault));
  ctx.pinned_uploads.push_back(pinned);
  std::memcpy(pinned, src, bytes);
  RD_CUDA_TRY(cudaMemcpyAsync(dst, pinned, bytes, cudaMemcpyHostToDevice, ctx.stream));
  return Status{};
}

Status check_kernel_error(Context& ctx, const char* stage) {
  if (ctx.capturing) return Status{};  // read after the graph has run
  uint32_t word = 0;
  RD_CUDA_TRY(cudaMemcpyAsync(&word, ctx.d_error, sizeof(word), cudaMemcpyDeviceToHost, ctx.stream));
  RD_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
  if (!ctx.pending.empty()) resolve_kernel_timing(ctx);
  if (!ctx.tune_runs.empty()) resolve_rl_tuning(ctx);
  if (!ctx.shape_runs.empty()) resolve_shape_tuning(ctx);
  if (word) {
    RD_CUDA_TRY(cudaMemsetAsync(ctx.d_error, 0, sizeof(uint32_t), ctx.stream));
    std::string what;
    if (word & 1u) what += " non-finite demosaic output;";
    if (word & 2u) what += " non-finite capture input;";
    if (word & 4u) what += " invalid vignetting gain;";
    if (word & 8u) what += " optics footprint outside the image or non-finite coordinate;";
    if (word & 16u) what += " highlight reconstruction failed;";
    if (word & 32u) what += " capture-sharpening tensor copy timed out;";
    if (word & 64u) what += " demosaic tile wait timed out;";
    if (word & 128u) what += " demosaic tile copy timed out;";
    return Status{RD_INVALID_INPUT, std::string(stage) + ":" + what};
  }
  return Status{};
}

// ------------------------------------------------------------- host contracts
static void validate_sensor(const rd_sensor_desc& s, Status& st) {
  auto bad = [&](const char* why) {
    if (st.ok()) st = Status{RD_INVALID_INPUT, why};
  };
  if (s.sensor_width < 2 || s.sensor_height < 2) bad("sensor must be at least 2x2");
  if (s.crop_width < 2 || s.crop_height < 2) bad("crop must be at least 2x2");
  if ((uint64_t)s.crop_x + s.crop_width > s.sensor_width || (uint64_t)s.crop_y + s.crop_height > s.sensor_height)
    bad("crop lies outside the sensor");
  if (s.cfa < 0 || s.cfa > 3) bad("unknown CFA pattern");
  const uint64_t n = (uint64_t)s.black_repeat_w * s.black_repeat_h;
  if (n == 0 || n > RD_MAX_LEVEL_PATTERN) bad("black repeat pattern must hold 1..64 values");
  if (!(s.white_count == 1 || s.white_count == 3 || s.white_count == n)) bad("white levels must be 1, 3 or per pattern");
  for (uint64_t k = 0; k < n && k < RD_MAX_LEVEL_PATTERN; ++k)
    if (!std::isfinite(s.black[k])) bad("black levels must be finite");
  for (uint32_t k = 0; k < s.white_count && k < RD_MAX_LEVEL_PATTERN; ++k)
    if (!std::isfinite(s.white[k])) bad("white levels must be finite");
  if (st.ok()) {
    // validate_levels (sensor.rs:532-561): white must exceed black over the pattern.
    for (uint32_t y = 0; y < s.black_repeat_h; ++y)
      for (uint32_t x = 0; x < s.black_repeat_w; ++x) {
        const uint32_t i = y * s.black_repeat_w + x;
        const float black = s.black[i];
        const float white = s.white_count == 1 ? s.white[0]
                            : s.white_count == 3 ? s.white[color_at(s.cfa, (int)x, (int)y)]
                                                 : s.white[i];
        if (!(white > black)) bad("white level must exceed black level");
      }
  }
  if (s.highlight < 0 || s.highlight > 2) bad("unknown highlight method");
  const float* lv = s.highlight == RD_HIGHLIGHT_CLIP ? s.clip_levels : s.detection_levels;
  if (s.highlight != RD_HIGHLIGHT_OFF)
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(lv[c]) || !(lv[c] > 0.0f)) bad("highlight levels must be finite and positive");
  if (s.highlight == RD_HIGHLIGHT_OPPOSED && s.has_neutral_ceiling)
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(s.neutral_ceiling[c]) || !(s.neutral_ceiling[c] > 0.0f))
        bad("neutral ceiling must be finite and positive");
  if (s.demosaic < 0 || s.demosaic > 3) bad("unknown demosaic algorithm");
  for (int c = 0; c < 3; ++c)
    if (!std::isfinite(s.demosaic_balance[c]) || !(s.demosaic_balance[c] > 0.0f))
      bad("demosaic balance must be finite and positive");
}

static MosaicSource make_source(const rd_sensor_desc& s, const uint16_t* d_raw, size_t row_stride) {
  MosaicSource m{};
  m.raw = d_raw;
  m.f32 = nullptr;
  m.row_stride = (long long)row_stride;
  m.crop_x = (int)s.crop_x;
  m.crop_y = (int)s.crop_y;
  m.sensor_cfa = s.cfa;
  m.width = (int)s.crop_width;
  m.height = (int)s.crop_height;
  m.cfa = shifted_cfa(s.cfa, (int)s.crop_x, (int)s.crop_y);
  m.black_w = (int)s.black_repeat_w;
  m.black_h = (int)s.black_repeat_h;
  m.white_count = (int)s.white_count;
  m.clip = s.highlight == RD_HIGHLIGHT_CLIP ? 1 : 0;
  for (int c = 0; c < 3; ++c) {
    m.clip_levels[c] = s.clip_levels[c];
    m.fwd[c] = s.demosaic_balance[c];  // run_demosaic normalizes it
  }
  for (int k = 0; k < RD_MAX_LEVEL_PATTERN; ++k) {
    m.black[k] = s.black[k];
    m.white[k] = s.white[k];
  }
  return m;
}

// build_plan (crates/optics/src/plan.rs:173-231) and find_scale (:521-559).
namespace {
bool map_coords(const rd_optics_desc& p, double x, double y, float scale, float out[6]);
}

Status optics_plan(rd_optics_desc& p, float crop, float real_focal, float lens_cx, float lens_cy) {
  if (p.width < 4 || p.height < 4) return Status{RD_INVALID_DIMENSIONS, "optics needs at least 4x4 pixels"};
  if (!(crop > 0.0f) || !std::isfinite(crop) || !(real_focal > 0.0f) || !std::isfinite(real_focal))
    return Status{RD_INVALID_INPUT, "crop factor and focal length must be finite and positive"};
  const double wf = p.width >= 2 ? (double)(p.width - 1) : 1.0;
  const double hf = p.height >= 2 ? (double)(p.height - 1) : 1.0;
  p.norm_scale = std::hypot(36.0, 24.0) / (double)crop / std::hypot(wf + 1.0, hf + 1.0) / (double)real_focal;
  p.norm_unscale = 1.0 / p.norm_scale;
  const double lens_size = std::min(wf, hf);
  p.center_x = (wf / 2.0 + lens_size / 2.0 * (double)lens_cx) * p.norm_scale;
  p.center_y = (hf / 2.0 + lens_size / 2.0 * (double)lens_cy) * p.norm_scale;
  p.scale = 1.0f;
  if (p.distortion_model == RD_DISTORTION_NONE && p.tca_model == RD_TCA_NONE) return Status{};
  float scale = 1.0f;
  for (int i = 0; i < 160; ++i) {
    bool safe = true;
    const int max_x = (int)p.width - 1, max_y = (int)p.height - 1;
    for (int index = 0; index < 64 && safe; ++index) {
      const float t = (float)index / 63.0f;
      const float pts[4][2] = {{t * (float)max_x, 0.0f},
                               {t * (float)max_x, (float)max_y},
                               {0.0f, t * (float)max_y},
                               {(float)max_x, t * (float)max_y}};
      for (auto& pt : pts) {
        float c[6];
        if (!map_coords(p, (double)(size_t)pt[0], (double)(size_t)pt[1], scale, c)) {
          safe = false;
          break;
        }
        for (int k = 0; k < 3; ++k)
          if (!(c[2 * k] >= 1.0f && c[2 * k + 1] >= 1.0f && c[2 * k] <= (float)(p.width - 2) &&
                c[2 * k + 1] <= (float)(p.height - 2)))
            safe = false;
        if (!safe) break;
      }
    }
    if (safe) {
      p.scale = scale;
      return Status{};
    }
    scale *= 1.025f;
  }
  return Status{RD_INVALID_INPUT, "no automatic scale keeps the cubic footprint inside the image"};
}

namespace {
constexpr double NEWTON_EPS = 0.00001;
void undist(const rd_optics_desc& p, float x, float y, float* ox, float* oy) {
  *ox = x;
  *oy = y;
  if (p.distortion_model == RD_DISTORTION_NONE) return;
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double a = p.distortion[0], b = p.distortion[1], c = p.distortion[2];
  double ru = rd;
  bool converged = false;
  if (p.distortion_model == RD_DISTORTION_POLY3) {
    const double inv_k1 = (double)(1.0f / p.distortion[0]);
    const double rd_div_k1 = (double)(float)(rd * inv_k1);
    for (int s = 0; s < 7; ++s) {
      const double f = ru * ru * ru + ru * inv_k1 - rd_div_k1;
      if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
      ru -= f / (3.0 * ru * ru + inv_k1);
    }
    if (!converged || ru < 0.0) { *ox = NAN; *oy = NAN; return; }
  } else if (p.distortion_model == RD_DISTORTION_POLY5) {
    for (int s = 0; s < 7; ++s) {
      const double ru2 = ru * ru;
      const double f = ru * (1.0 + a * ru2 + b * ru2 * ru2) - rd;
      if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
      ru -= f / (1.0 + 3.0 * a * ru2 + 5.0 * b * ru2 * ru2);
    }
    if (!converged || ru < 0.0) return;
  } else {
    for (int s = 0; s < 7; ++s) {
      const double f = ru * (a * ru * ru * ru + b * ru * ru + c * ru + 1.0) - rd;
      if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
      ru -= f / (4.0 * a * ru * ru * ru + 3.0 * b * ru * ru + 2.0 * c * ru + 1.0);
    }
    if (!converged || ru < 0.0) return;
  }
  const double ratio = ru / rd;
  *ox = (float)((double)x * ratio);
  *oy = (float)((double)y * ratio);
}
void tca3(const float* ch, float x, float y, float* ox, float* oy) {
  *ox = x;
  *oy = y;
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double v = ch[0], c = ch[1], b = ch[2];
  double ru = rd;
  bool converged = false;
  for (int s = 0; s < 7; ++s) {
    const double ru2 = ru * ru;
    const double f = b * ru2 * ru + c * ru2 + v * ru - rd;
    if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
    ru -= f / (3.0 * b * ru2 + 2.0 * c * ru + v);
  }
  if (!converged || ru <= 0.0) return;
  const double ratio = ru / rd;
  *ox = (float)((double)x * ratio);
  *oy = (float)((double)y * ratio);
}
bool map_coords(const rd_optics_desc& p, double x, double y, float scale, float out[6]) {
  const double cpx = p.center_x * p.norm_unscale, cpy = p.center_y * p.norm_unscale;
  const double mx = cpx + (x - cpx) / (double)scale, my = cpy + (y - cpy) / (double)scale;
  const double ix = mx * p.norm_scale - p.center_x, iy = my * p.norm_scale - p.center_y;
  float gx, gy;
  undist(p, (float)ix, (float)iy, &gx, &gy);
  if (!std::isfinite(gx) || !std::isfinite(gy)) return false;
  float n[6] = {gx, gy, gx, gy, gx, gy};
  if (p.tca_model == RD_TCA_LINEAR) {
    n[0] = gx * p.tca_red[0];
    n[1] = gy * p.tca_red[0];
    n[4] = gx * p.tca_blue[0];
    n[5] = gy * p.tca_blue[0];
  } else if (p.tca_model == RD_TCA_POLY3) {
    tca3(p.tca_red, gx, gy, &n[0], &n[1]);
    tca3(p.tca_blue, gx, gy, &n[4], &n[5]);
  }
  for (int c = 0; c < 3; ++c) {
    out[2 * c] = (float)(((double)n[2 * c] + p.center_x) * p.norm_unscale);
    out[2 * c + 1] = (float)(((double)n[2 * c + 1] + p.center_y) * p.norm_unscale);
    if (!std::isfinite(out[2 * c]) || !std::isfinite(out[2 * c + 1])) return false;
  }
  return true;
}
}  // namespace

// BaseRenderingLut::standard_v1 (crates/core/src/rendering.rs:36-50, 223-234).
void standard_base_lut(float* lut) {
  const float anchor = std::pow(0.18f, 1.45f - 1.0f) * (1.0f - 0.18f);
  for (int i = 0; i < 4096; ++i) {
    if (i == 4095) {
      lut[i] = 1.0f;
      continue;
    }
    const float coordinate = (float)i / 4095.0f;
    const float input = coordinate / (1.0f - coordinate);
    if (input == 0.0f) {
      lut[i] = 0.0f;
      continue;
    }
    const float numerator = std::pow(input, 1.45f);
    lut[i] = numerator / (numerator + anchor);
  }
}

// LightToneLut::new (crates/edit/src/light.rs:27-47) with evaluate_light_tone
// (:90-117), protected_contrast (:119-129), bounded_move (:131-137) and
// smoothstep (:139-142), in f32 with each operation rounded on its own.
namespace {
constexpr float LIGHT_CONTRAST_PIVOT = 0.18f;
constexpr float LIGHT_SHADOW_STRENGTH = 0.45f, LIGHT_HIGHLIGHT_STRENGTH = 0.45f;
constexpr float LIGHT_BLACK_STRENGTH = 0.25f, LIGHT_WHITE_STRENGTH = 0.25f;

float light_smoothstep(float edge0, float edge1, float v) {
  float n = (v - edge0) / (edge1 - edge0);
  if (n < 0.0f) n = 0.0f;
  if (n > 1.0f) n = 1.0f;
  return n * n * (3.0f - 2.0f * n);
}
float light_bounded_move(float value, float amount, float weight) {
  return amount >= 0.0f ? value + (1.0f - value) * amount * weight : value + value * amount * weight;
}
float light_contrast(float input, float contrast) {
  if (contrast == 0.0f) return input;
  const float exponent = std::exp2(contrast);
  if (input <= LIGHT_CONTRAST_PIVOT) return LIGHT_CONTRAST_PIVOT * std::pow(input / LIGHT_CONTRAST_PIVOT, exponent);
  return 1.0f - (1.0f - LIGHT_CONTRAST_PIVOT) * std::pow((1.0f - input) / (1.0f - LIGHT_CONTRAST_PIVOT), exponent);
}
}  // namespace

void light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks, float* lut) {
  for (int i = 0; i < 4096; ++i) {
    const float input = (float)i / 4095.0f;
    float out = light_contrast(input, contrast);
    const float shadow_w = light_smoothstep(0.0f, 0.16f, input) * (1.0f - light_smoothstep(0.38f, 0.68f, input));
    const float highlight_w = light_smoothstep(0.32f, 0.62f, input) * (1.0f - light_smoothstep(0.84f, 1.0f, input));
    out = light_bounded_move(out, shadows, LIGHT_SHADOW_STRENGTH * shadow_w);
    out = light_bounded_move(out, highlights, LIGHT_HIGHLIGHT_STRENGTH * highlight_w);
    const float black_w = 1.0f - light_smoothstep(0.0f, 0.32f, input);
    const float white_w = light_smoothstep(0.68f, 1.0f, input);
    out = light_bounded_move(out, blacks, LIGHT_BLACK_STRENGTH * black_w);
    out = light_bounded_move(out, whites, LIGHT_WHITE_STRENGTH * white_w);
    if (out < 0.0f) out = 0.0f;
    if (out > 1.0f) out = 1.0f;
    lut[i] = out;
  }
  // Monotone projection: each value is at least its predecessor (f32::max,
  // which returns the other operand for a NaN).
  float previous = lut[0];
  for (int i = 1; i < 4096; ++i) {
    if (std::isnan(lut[i]) || previous > lut[i]) lut[i] = previous;
    previous = lut[i];
  }
}

}  // namespace rd

using rd::Status;

namespace {

rd_status finish(rd_ctx* ctx, const Status& st) {
  if (ctx) ctx->c.last_error = st.message;
  return st.code;
}

struct Timer {
  rd::Context& c;
  int n = 0;
  explicit Timer(rd::Context& ctx) : c(ctx) {}
  void mark() {
    if (n < 8 && !c.capturing) cudaEventRecord(c.ev[n++], c.stream);
  }
  float span(int a, int b) const {
    float ms = 0.0f;
    if (a < n && b < n) cudaEventElapsedTime(&ms, c.ev[a], c.ev[b]);
    return ms;
  }
};

// Sensor development on a resident mosaic: normalize + highlight + demosaic,
// then capture sharpening. Returns a new rd_source.
Status develop_impl(rd_ctx* h, const uint16_t* d_raw, size_t row_stride, const rd_sensor_desc& s,
                    const rd_detail_desc* detail, const volatile uint32_t* cancel, rd_source** out,
                    rd_metrics* metrics) {
  rd::Context& ctx = h->c;
  Status st;
  validate_sensor(s, st);
  if (!st.ok()) return st;
  if (row_stride < s.sensor_width) return Status{RD_INVALID_DIMENSIONS, "row stride is shorter than the sensor width"};
  if (cancel && *cancel) return Status{RD_CANCELLED, "cancelled"};
  const int W = (int)s.crop_width, H = (int)s.crop_height;
  const long long plane = (long long)W * H;
  rd::MosaicSource src = rd::make_source(s, d_raw, row_stride);
  Timer tm(ctx);
  tm.mark();
  unsigned long long* d_stats = nullptr;
  void* p = nullptr;
  RD_TRY(rd::device_alloc(ctx, sizeof(unsigned long long) * 16, &p));
  d_stats = static_cast<unsigned long long*>(p);
  RD_CUDA_TRY(cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 16, ctx.stream));
  float* d_mosaic = nullptr;
  const size_t mosaic_bytes = sizeof(float) * (size_t)plane;
  if (s.highlight == RD_HIGHLIGHT_OPPOSED) {
    st = rd::device_alloc(ctx, mosaic_bytes, &p);
    if (st.ok()) {
      d_mosaic = static_cast<float*>(p);
      // The cell pass of Opposed normalizes the raw samples into d_mosaic.
      st = rd::run_opposed(ctx, src, d_mosaic, s.detection_levels,
                           s.has_neutral_ceiling ? s.neutral_ceiling : nullptr, d_stats, nullptr);
    }
    src.f32 = d_mosaic;
    src.clip = 0;
  }
  tm.mark();
  rd_source* result = nullptr;
  if (st.ok() && cancel && *cancel) st = Status{RD_CANCELLED, "cancelled"};
  if (st.ok()) {
    result = new (std::nothrow) rd_source{h, nullptr, W, H, sizeof(float) * 3 * (size_t)plane};
    if (!result) st = Status{RD_OVER_BUDGET, "host allocation failed"};
  }
  if (st.ok()) {
    st = rd::device_alloc(ctx, result->bytes, &p);
    if (st.ok()) result->rgb = static_cast<float*>(p);
  }
  if (st.ok()) st = rd::run_demosaic(ctx, src, s.demosaic, result->rgb, d_stats);
  tm.mark();
  if (st.ok() && cancel && *cancel) st = Status{RD_CANCELLED, "cancelled"};
  if (st.ok() && detail) st = rd::run_capture(ctx, result->rgb, W, H, *detail);
  tm.mark();
  if (d_mosaic) rd::device_free(ctx, d_mosaic, mosaic_bytes);
  uint64_t host_stats[16] = {};
  if (st.ok() && !ctx.capturing) {
    const cudaError_t e = cudaMemcpyAsync(host_stats, d_stats, sizeof(host_stats), cudaMemcpyDeviceToHost, ctx.stream);
    if (e != cudaSuccess) st = Status{RD_READBACK, cudaGetErrorString(e)};
  }
  rd::device_free(ctx, d_stats, sizeof(unsigned long long) * 16);
  if (st.ok()) st = rd::check_kernel_error(ctx, "develop");
  if (st.ok() && cancel && *cancel) st = Status{RD_CANCELLED, "cancelled"};
  if (!st.ok()) {
    if (result) {
      if (result->rgb) rd::device_free(ctx, result->rgb, result->bytes);
      delete result;
    }
    cudaStreamSynchronize(ctx.stream);
    return st;
  }
  if (metrics) {
    metrics->normalize_highlight_ms = tm.span(0, 1);
    metrics->demosaic_ms = tm.span(1, 2);
    metrics->capture_ms = tm.span(2, 3);
    metrics->total_ms = tm.span(0, 3);
    for (int k = 0; k < 9; ++k) metrics->highlight_stats[k] = host_stats[k];
    metrics->kernel_launches = ctx.launches;
    metrics->device_bytes = ctx.reserved;
  }
  *out = result;
  return Status{};
}

}  // namespace

extern "C" {

int rd_status_is_routing(rd_status status) {
  return status == RD_UNSUPPORTED_EDITS || status == RD_OVER_BUDGET;
}

const char* rd_status_name(rd_status status) {
  switch (status) {
    case RD_OK: return "Ok";
    case RD_CANCELLED: return "Cancelled";
    case RD_UNSUPPORTED: return "Unsupported";
    case RD_OVER_BUDGET: return "OverBudget";
    case RD_INVALID_DIMENSIONS: return "InvalidDimensions";
    case RD_BASE_MISMATCH: return "BaseMismatch";
    case RD_UNSUPPORTED_EDITS: return "UnsupportedEdits";
    case RD_SYNCHRONIZATION: return "Synchronization";
    case RD_INVALID_INPUT: return "InvalidInput";
    case RD_READBACK: return "Readback";
  }
  return "Unknown";
}

rd_status rd_ctx_create(int device, uint64_t budget_bytes, rd_ctx** out) {
  if (!out) return RD_INVALID_INPUT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return RD_UNSUPPORTED;
  }
  if (cudaSetDevice(device) != cudaSuccess) return RD_SYNCHRONIZATION;
  rd_ctx* h = new (std::nothrow) rd_ctx();
  if (!h) return RD_OVER_BUDGET;
  rd::Context& c = h->c;
  c.device = device;
  c.budget = budget_bytes;
  cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return RD_SYNCHRONIZATION;
  }
  for (auto& e : c.ev) cudaEventCreate(&e);
  if (cudaMalloc(&c.d_error, 4 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemsetAsync(c.d_error, 0, 4 * sizeof(uint32_t), c.stream) != cudaSuccess) {
    cudaStreamDestroy(c.stream);
    delete h;
    return RD_SYNCHRONIZATION;
  }
  c.d_work = c.d_error + 1;
  // Keep freed pool memory cached between calls instead of returning it to the driver.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t threshold = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  cudaStreamSynchronize(c.stream);
  *out = h;
  return RD_OK;
}


void rd_ctx_destroy(rd_ctx* h) {
  if (!h) return;
  rd::Context& c = h->c;
  cudaSetDevice(c.device);
  if (c.amaze_scratch) rd::device_free(c, c.amaze_scratch, c.amaze_bytes);
  if (c.flush_buf) rd::device_free(c, c.flush_buf, c.flush_bytes);
  cudaStreamSynchronize(c.stream);
  for (void* p : c.pinned_uploads) cudaFreeHost(p);
  rd::resolve_kernel_timing(c);
  for (auto& r : c.tune_runs) {
    cudaEventDestroy(r.second.first);
    cudaEventDestroy(r.second.second);
  }
  for (auto& r : c.shape_runs) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : c.event_pool) cudaEventDestroy(e);
  for (auto& e : c.user_ev)
    if (e) cudaEventDestroy(e);
  cudaFree(c.d_error);
  for (auto& e : c.ev) cudaEventDestroy(e);
  cudaStreamDestroy(c.stream);
  delete h;
}

rd_status rd_ctx_set_budget(rd_ctx* h, uint64_t budget_bytes) {
  if (!h) return RD_INVALID_INPUT;
  h->c.budget = budget_bytes;
  return RD_OK;
}

const char* rd_ctx_last_error(const rd_ctx* h) { return h ? h->c.last_error.c_str() : "no context"; }

rd_status rd_ctx_synchronize(rd_ctx* h) {
  if (!h) return RD_INVALID_INPUT;
  return cudaStreamSynchronize(h->c.stream) == cudaSuccess ? RD_OK : RD_SYNCHRONIZATION;
}

uint64_t rd_ctx_kernel_launches(const rd_ctx* h) { return h ? h->c.launches : 0; }

rd_status rd_ctx_set_wait_test(rd_ctx* h, uint32_t wait_limit, int32_t withhold) {
  if (!h) return RD_INVALID_INPUT;
  if (withhold < RD_WAIT_NONE || withhold > RD_WAIT_AMAZE_COPY)
    return finish(h, Status{RD_INVALID_INPUT, "unknown withheld completion"});
  h->c.wait_limit = wait_limit;
  h->c.wait_withhold = withhold;
  return RD_OK;
}

int rd_supports(const rd_sensor_desc* s) {
  if (!s) return 0;
  Status st;
  rd::validate_sensor(*s, st);
  return st.ok() ? 1 : 0;
}

rd_status rd_develop(rd_ctx* h, const uint16_t* mosaic, size_t row_stride, const rd_sensor_desc* sensor,
                     const rd_detail_desc* detail, const volatile uint32_t* cancel, rd_source** out,
                     rd_metrics* metrics) {
  if (!h || !mosaic || !sensor || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  *out = nullptr;
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const size_t bytes = sizeof(uint16_t) * row_stride * sensor->sensor_height;
  void* p = nullptr;
  Status st = rd::device_alloc(ctx, bytes, &p);
  if (!st.ok()) return finish(h, st);
  if (cudaMemcpyAsync(p, mosaic, bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "mosaic upload failed"};
  if (st.ok()) st = develop_impl(h, static_cast<const uint16_t*>(p), row_stride, *sensor, detail, cancel, out, metrics);
  rd::device_free(ctx, p, bytes);
  return finish(h, st);
}

rd_status rd_develop_device(rd_ctx* h, const uint16_t* d_mosaic, size_t row_stride, const rd_sensor_desc* sensor,
                            const rd_detail_desc* detail, const volatile uint32_t* cancel, rd_source** out,
                            rd_metrics* metrics) {
  if (!h || !d_mosaic || !sensor || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  *out = nullptr;
  cudaSetDevice(h->c.device);
  return finish(h, develop_impl(h, d_mosaic, row_stride, *sensor, detail, cancel, out, metrics));
}

rd_status rd_spatial(rd_ctx* h, const rd_source* source, const rd_optics_desc* optics, uint32_t tw, uint32_t th,
                     const float wb_gains[3], const float cam[9], rd_base** out, rd_metrics* metrics) {
  if (!h || !source || !out || !wb_gains || !cam) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  *out = nullptr;
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const int W = source->W, H = source->H;
  if (tw == 0 || th == 0 || (int)tw > W || (int)th > H)
    return finish(h, Status{RD_INVALID_DIMENSIONS, "area reduction cannot upscale or produce an empty image"});
  if (optics && ((int)optics->width != W || (int)optics->height != H))
    return finish(h, Status{RD_BASE_MISMATCH, "optics execution was resolved for another image size"});
  for (int c = 0; c < 3; ++c)
    if (!std::isfinite(wb_gains[c]) || !(wb_gains[c] > 0.0f))
      return finish(h, Status{RD_INVALID_INPUT, "white-balance gains must be finite and positive"});
  const long long plane = (long long)W * H;
  Timer tm(ctx);
  tm.mark();
  Status st;
  const bool vig = optics && optics->vignetting == 1;
  const bool warp = optics && (optics->distortion_model != RD_DISTORTION_NONE || optics->tca_model != RD_TCA_NONE);
  void* p = nullptr;
  float* mult = nullptr;
  float* warped = nullptr;
  // Vignetting multiplies the source in place before the warp
  // (correction.rs:70-211); the source stays reusable here, so the gather and
  // the area reduction apply the multiplier plane to each sample they read.
  if (vig) {
    st = rd::device_alloc(ctx, sizeof(float) * plane, &p);
    if (st.ok()) {
      mult = static_cast<float*>(p);
      st = rd::run_vignette_plane(ctx, *optics, mult);
    }
  }
  const float* reduce_in = source->rgb;
  const float* reduce_mult = mult;
  if (st.ok() && warp) {
    st = rd::device_alloc(ctx, sizeof(float) * 3 * plane, &p);
    if (st.ok()) {
      warped = static_cast<float*>(p);
      st = rd::run_optics_gather(ctx, *optics, source->rgb, mult, warped);
      reduce_in = warped;
      reduce_mult = nullptr;
    }
  }
  tm.mark();
  rd_base* base = nullptr;
  if (st.ok()) {
    base = new (std::nothrow) rd_base{h, nullptr, (int)tw, (int)th, sizeof(float) * 3 * (size_t)tw * th, nullptr, nullptr, 0};
    if (!base) st = Status{RD_OVER_BUDGET, "host allocation failed"};
  }
  if (st.ok()) {
    st = rd::device_alloc(ctx, base->bytes, &p);
    if (st.ok()) base->rgb = static_cast<float*>(p);
  }
  if (st.ok()) {
    if ((int)tw == W && (int)th == H && !reduce_mult) {
      if (cudaMemcpyAsync(base->rgb, reduce_in, base->bytes, cudaMemcpyDeviceToDevice, ctx.stream) != cudaSuccess)
        st = Status{RD_SYNCHRONIZATION, "copy failed"};
    } else {
      st = rd::run_area_reduce(ctx, reduce_in, reduce_mult, W, H, (int)tw, (int)th, base->rgb);
    }
  }
  tm.mark();
  if (st.ok()) st = rd::run_wb_matrix(ctx, base->rgb, (size_t)tw * th, wb_gains, cam);
  tm.mark();
  if (mult) rd::device_free(ctx, mult, sizeof(float) * plane);
  if (warped) rd::device_free(ctx, warped, sizeof(float) * 3 * plane);
  if (st.ok()) st = rd::check_kernel_error(ctx, "spatial");
  if (!st.ok()) {
    if (base) {
      if (base->rgb) rd::device_free(ctx, base->rgb, base->bytes);
      delete base;
    }
    cudaStreamSynchronize(ctx.stream);
    return finish(h, st);
  }
  if (metrics) {
    metrics->optics_ms = tm.span(0, 1);
    metrics->reduce_ms = tm.span(1, 2);
    metrics->color_ms = tm.span(2, 3);
    metrics->total_ms = tm.span(0, 3);
    metrics->kernel_launches = ctx.launches;
    metrics->device_bytes = ctx.reserved;
  }
  *out = base;
  return finish(h, Status{});
}

static Status ensure_outputs(rd_base* base) {
  rd::Context& ctx = base->ctx->c;
  if (base->d_srgb) return Status{};
  base->out_bytes = (size_t)3 * base->W * base->H + 1024 * sizeof(unsigned long long) + 16;
  void* p = nullptr;
  RD_TRY(rd::device_alloc(ctx, base->out_bytes, &p));
  base->d_hist = static_cast<unsigned long long*>(p);
  base->d_srgb = reinterpret_cast<uint8_t*>(base->d_hist + 1024);
  return Status{};
}

rd_status rd_render_device(rd_ctx* h, rd_base* base, const rd_color_desc* color, rd_metrics* metrics) {
  if (!h || !base || !color) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (base->ctx != h) return finish(h, Status{RD_BASE_MISMATCH, "base belongs to another context"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  Status st = ensure_outputs(base);
  if (!st.ok()) return finish(h, st);
  Timer tm(ctx);
  tm.mark();
  if (cudaMemsetAsync(base->d_hist, 0, 1024 * sizeof(unsigned long long), ctx.stream) != cudaSuccess)
    return finish(h, Status{RD_SYNCHRONIZATION, "memset failed"});
  st = rd::run_color_output(ctx, base->rgb, base->W, base->H, *color, false, base->d_srgb, base->d_hist);
  tm.mark();
  if (st.ok()) st = rd::check_kernel_error(ctx, "render");
  if (st.ok() && metrics) {
    metrics->color_ms = tm.span(0, 1);
    metrics->total_ms = metrics->color_ms;
    metrics->kernel_launches = ctx.launches;
  }
  return finish(h, st);
}

rd_status rd_render(rd_ctx* h, const rd_base* cbase, const rd_color_desc* color, uint8_t* srgb_out, uint64_t* hist,
                    uint64_t* clipped, rd_metrics* metrics) {
  rd_base* base = const_cast<rd_base*>(cbase);
  rd_status s = rd_render_device(h, base, color, metrics);
  if (s != RD_OK) return s;
  rd::Context& ctx = h->c;
  if (ctx.capturing) {
    // Graph capture: copies straight into the caller's (pinned) buffers, which
    // must live until the graph has run; clip counts come from the histogram.
    if (clipped) return finish(h, Status{RD_INVALID_INPUT, "clip counts are not read back under graph capture"});
    Status cs;
    if (srgb_out && cudaMemcpyAsync(srgb_out, base->d_srgb, (size_t)3 * base->W * base->H, cudaMemcpyDeviceToHost,
                                    ctx.stream) != cudaSuccess)
      cs = Status{RD_READBACK, "output readback failed"};
    if (cs.ok() && hist &&
        cudaMemcpyAsync(hist, base->d_hist, 1024 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess)
      cs = Status{RD_READBACK, "histogram readback failed"};
    return finish(h, cs);
  }
  uint64_t bins[1024];
  Status st;
  if (srgb_out &&
      cudaMemcpyAsync(srgb_out, base->d_srgb, (size_t)3 * base->W * base->H, cudaMemcpyDeviceToHost, ctx.stream) !=
          cudaSuccess)
    st = Status{RD_READBACK, "output readback failed"};
  if (st.ok() && cudaMemcpyAsync(bins, base->d_hist, sizeof(bins), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess)
    st = Status{RD_READBACK, "histogram readback failed"};
  if (st.ok() && cudaStreamSynchronize(ctx.stream) != cudaSuccess) st = Status{RD_READBACK, "readback failed"};
  if (st.ok()) {
    if (hist) std::memcpy(hist, bins, sizeof(bins));
    // Histogram::count_clipped (histogram.rs:110-121): bins 0 and 255.
    if (clipped)
      for (int c = 0; c < 3; ++c) {
        clipped[c] = bins[256 * c];
        clipped[3 + c] = bins[256 * c + 255];
      }
  }
  return finish(h, st);
}

rd_status rd_output_dimensions(uint32_t width, uint32_t height, const rd_output_desc* output, uint32_t* out_width,
                               uint32_t* out_height, uint32_t* bytes_per_pixel) {
  if (!output || !out_width || !out_height) return RD_INVALID_INPUT;
  if (width == 0 || height == 0 || width > (uint32_t)INT32_MAX || height > (uint32_t)INT32_MAX)
    return RD_INVALID_DIMENSIONS;
  rd::OutputGeometry g;
  const Status st = rd::resolve_output_geometry((int)width, (int)height, *output, &g);
  if (!st.ok()) return st.code;
  *out_width = (uint32_t)g.width;
  *out_height = (uint32_t)g.height;
  if (bytes_per_pixel) *bytes_per_pixel = (uint32_t)rd::output_bytes_per_pixel(output->format);
  return RD_OK;
}

rd_status rd_render_output_device(rd_ctx* h, const rd_base* base, const rd_color_desc* color,
                                  const rd_output_desc* output, void* d_out, uint64_t* d_hist, uint64_t* d_gamut,
                                  rd_metrics* metrics) {
  if (!h || !base || !color || !output || !d_out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (base->ctx != h) return finish(h, Status{RD_BASE_MISMATCH, "base belongs to another context"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  rd::OutputGeometry g;
  Status st = rd::resolve_output_geometry(base->W, base->H, *output, &g);
  if (st.ok() && d_hist && output->format != RD_OUTPUT_SRGB8)
    st = Status{RD_INVALID_INPUT, "the histogram is counted on the 8-bit output only"};
  if (!st.ok()) return finish(h, st);
  Timer tm(ctx);
  tm.mark();
  st = rd::run_display_output(ctx, base->rgb, *color, *output, g, d_out,
                              reinterpret_cast<unsigned long long*>(d_hist),
                              reinterpret_cast<unsigned long long*>(d_gamut));
  tm.mark();
  if (st.ok()) st = rd::check_kernel_error(ctx, "output");
  if (st.ok() && metrics) {
    metrics->color_ms = tm.span(0, 1);
    metrics->total_ms = metrics->color_ms;
    metrics->kernel_launches = ctx.launches;
  }
  return finish(h, st);
}

// Device output + readback into host buffers. The device output, histogram and
// counters share one allocation of the context.
static Status render_output_host(rd_ctx* h, const float* d_rgb, int W, int H, const rd_color_desc& color,
                                 const rd_output_desc& output, void* out, size_t out_capacity, uint64_t* hist,
                                 uint64_t* gamut, float* color_ms) {
  rd::Context& ctx = h->c;
  rd::OutputGeometry g;
  RD_TRY(rd::resolve_output_geometry(W, H, output, &g));
  if (hist && output.format != RD_OUTPUT_SRGB8)
    return Status{RD_INVALID_INPUT, "the histogram is counted on the 8-bit output only"};
  const size_t out_bytes = (size_t)g.width * g.height * rd::output_bytes_per_pixel(output.format);
  if (out_capacity < out_bytes) return Status{RD_INVALID_DIMENSIONS, "output buffer is smaller than the output"};
  const size_t counters = 1024 + 8;  // histogram, gamut counters (padded)
  const size_t total = counters * sizeof(unsigned long long) + out_bytes;
  void* p = nullptr;
  RD_TRY(rd::device_alloc(ctx, total, &p));
  unsigned long long* d_hist = static_cast<unsigned long long*>(p);
  unsigned long long* d_gamut = d_hist + 1024;
  void* d_out = d_hist + counters;
  Timer tm(ctx);
  tm.mark();
  Status st = rd::run_display_output(ctx, d_rgb, color, output, g, d_out, hist ? d_hist : nullptr, d_gamut);
  tm.mark();
  uint64_t bins[1024];
  uint64_t diag[5];
  if (st.ok() && (cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaMemcpyAsync(diag, d_gamut, sizeof(diag), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  (hist && cudaMemcpyAsync(bins, d_hist, sizeof(bins), cudaMemcpyDeviceToHost, ctx.stream) !=
                               cudaSuccess)))
    st = Status{RD_READBACK, "output readback failed"};
  if (st.ok() && cudaStreamSynchronize(ctx.stream) != cudaSuccess) st = Status{RD_READBACK, "readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "output");
  if (st.ok()) {
    if (hist) std::memcpy(hist, bins, sizeof(bins));
    if (gamut) std::memcpy(gamut, diag, sizeof(diag));
    if (color_ms) *color_ms = tm.span(0, 1);
  }
  rd::device_free(ctx, p, total);
  return st;
}

rd_status rd_render_output(rd_ctx* h, const rd_base* base, const rd_color_desc* color, const rd_output_desc* output,
                           void* out, size_t out_capacity, uint64_t* hist, uint64_t* gamut, rd_metrics* metrics) {
  if (!h || !base || !color || !output || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (base->ctx != h) return finish(h, Status{RD_BASE_MISMATCH, "base belongs to another context"});
  cudaSetDevice(h->c.device);
  float ms = 0.0f;
  const Status st = render_output_host(h, base->rgb, base->W, base->H, *color, *output, out, out_capacity, hist,
                                       gamut, &ms);
  if (st.ok() && metrics) {
    metrics->color_ms = ms;
    metrics->total_ms = ms;
    metrics->kernel_launches = h->c.launches;
  }
  return finish(h, st);
}

// ---- PNG encode ----------------------------------------------------------
static Status png_args(const void* rgb, uint32_t width, uint32_t height, uint64_t row_stride, int32_t bit_depth,
                       const uint8_t* icc, uint64_t icc_len, const uint8_t* exif, uint64_t exif_len) {
  if (!rgb || (icc_len && !icc) || (exif_len && !exif)) return Status{RD_INVALID_INPUT, "null argument"};
  if (bit_depth != 8 && bit_depth != 16) return Status{RD_INVALID_INPUT, "PNG samples are 8 or 16 bits"};
  if (width == 0 || height == 0 || width > (uint32_t)INT32_MAX || height > (uint32_t)INT32_MAX)
    return Status{RD_INVALID_DIMENSIONS, "PNG dimensions out of range"};
  // ExportError::InvalidImageLayout (crates/core/src/export.rs:136-150).
  if (row_stride != 3ull * width)
    return Status{RD_INVALID_INPUT, "encoders require tightly packed RGB rows"};
  if (bit_depth == 16 && reinterpret_cast<uintptr_t>(rgb) % 2)
    return Status{RD_INVALID_INPUT, "16-bit rows must be 2-byte aligned"};
  if (!rd::png_metadata_ok(icc_len, exif_len)) return Status{RD_INVALID_INPUT, "metadata too large for a PNG chunk"};
  return Status{};
}

uint64_t rd_png_bound(uint32_t width, uint32_t height, int32_t bit_depth, uint64_t icc_len, uint64_t exif_len) {
  if ((bit_depth != 8 && bit_depth != 16) || width == 0 || height == 0 || width > (uint32_t)INT32_MAX ||
      height > (uint32_t)INT32_MAX)
    return 0;
  if (!rd::png_metadata_ok(icc_len, exif_len)) return 0;
  return rd::png_bound((int)width, (int)height, bit_depth, rd::png_header_bytes(icc_len, exif_len));
}

rd_status rd_encode_png_device(rd_ctx* h, const void* d_rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                               int32_t bit_depth, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                               uint64_t exif_len, uint8_t* d_png, uint64_t capacity, uint64_t* d_png_bytes) {
  if (!h || !d_png || !d_png_bytes) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  Status st = png_args(d_rgb, width, height, row_stride, bit_depth, icc, icc_len, exif, exif_len);
  if (st.ok() && (reinterpret_cast<uintptr_t>(d_png) % 4 || reinterpret_cast<uintptr_t>(d_png_bytes) % 8))
    st = Status{RD_INVALID_INPUT, "the PNG buffer must be 4-byte aligned and its byte count 8-byte aligned"};
  if (!st.ok()) return finish(h, st);
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  std::vector<uint8_t> header;
  st = rd::png_header((int)width, (int)height, bit_depth, icc, icc_len, exif, exif_len, &header);
  if (st.ok() && capacity < rd::png_bound((int)width, (int)height, bit_depth, header.size()))
    st = Status{RD_INVALID_DIMENSIONS, "the PNG buffer is smaller than rd_png_bound"};
  if (st.ok()) st = rd::run_png_encode(ctx, d_rgb, (int)width, (int)height, bit_depth, header, d_png, d_png_bytes);
  if (st.ok()) st = rd::check_kernel_error(ctx, "png encode");
  return finish(h, st);
}

rd_status rd_encode_png(rd_ctx* h, const void* rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                        int32_t bit_depth, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                        uint64_t exif_len, uint8_t* png, uint64_t capacity, uint64_t* png_bytes,
                        rd_metrics* metrics) {
  if (!h || !png || !png_bytes) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  Status st = png_args(rgb, width, height, row_stride, bit_depth, icc, icc_len, exif, exif_len);
  if (!st.ok()) return finish(h, st);
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  std::vector<uint8_t> header;
  st = rd::png_header((int)width, (int)height, bit_depth, icc, icc_len, exif, exif_len, &header);
  if (!st.ok()) return finish(h, st);
  const uint64_t in_bytes = 3ull * width * height * (uint64_t)(bit_depth / 8);
  const uint64_t in_room = (in_bytes + 255) & ~255ull;
  const uint64_t bound = rd::png_bound((int)width, (int)height, bit_depth, header.size());
  const uint64_t total = in_room + ((bound + 255) & ~255ull) + 16;
  void* p = nullptr;
  st = rd::device_alloc(ctx, total, &p);
  if (!st.ok()) return finish(h, st);
  uint8_t* d_in = static_cast<uint8_t*>(p);
  uint8_t* d_png = d_in + in_room;
  uint64_t* d_size = reinterpret_cast<uint64_t*>(d_png + ((bound + 255) & ~255ull));
  Timer tm(ctx);
  if (cudaMemcpyAsync(d_in, rgb, in_bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "image upload failed"};
  tm.mark();
  if (st.ok()) st = rd::run_png_encode(ctx, d_in, (int)width, (int)height, bit_depth, header, d_png, d_size);
  tm.mark();
  uint64_t size = 0;
  if (st.ok() && (cudaMemcpyAsync(&size, d_size, sizeof(size), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaStreamSynchronize(ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "PNG size readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "png encode");
  if (st.ok()) {
    *png_bytes = size;
    if (size > capacity) st = Status{RD_INVALID_DIMENSIONS, "the PNG buffer is smaller than the file"};
  }
  if (st.ok() && (cudaMemcpyAsync(png, d_png, size, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaStreamSynchronize(ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "PNG readback failed"};
  if (st.ok() && metrics) {
    std::memset(metrics, 0, sizeof(*metrics));
    metrics->total_ms = tm.span(0, 1);
    metrics->kernel_launches = ctx.launches;
  }
  rd::device_free(ctx, p, total);
  return finish(h, st);
}

// ---- JPEG encode ---------------------------------------------------------
static Status jpeg_args(const void* rgb, uint32_t width, uint32_t height, uint64_t row_stride, int32_t quality,
                        const uint8_t* icc, uint64_t icc_len, const uint8_t* exif, uint64_t exif_len) {
  // The JPEG arm takes 8-bit rows only (export.rs:166 matches ExportImage::Rgb8).
  RD_TRY(png_args(rgb, width, height, row_stride, 8, icc, icc_len, exif, exif_len));
  if (!rd::jpeg_metadata_ok(icc_len, exif_len)) return Status{RD_INVALID_INPUT, "metadata too large for JPEG segments"};
  return rd::jpeg_check((int)width, (int)height, quality);
}

uint64_t rd_jpeg_bound(uint32_t width, uint32_t height, uint64_t icc_len, uint64_t exif_len) {
  if (width == 0 || height == 0 || width > 65535 || height > 65535 || !rd::jpeg_metadata_ok(icc_len, exif_len))
    return 0;
  return rd::jpeg_bound((int)width, (int)height, icc_len, exif_len);
}

rd_status rd_encode_jpeg_device(rd_ctx* h, const uint8_t* d_rgb, uint32_t width, uint32_t height,
                                uint64_t row_stride, int32_t quality, const uint8_t* icc, uint64_t icc_len,
                                const uint8_t* exif, uint64_t exif_len, uint8_t* d_jpeg, uint64_t capacity,
                                uint64_t* d_jpeg_bytes) {
  if (!h || !d_jpeg || !d_jpeg_bytes) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  Status st = jpeg_args(d_rgb, width, height, row_stride, quality, icc, icc_len, exif, exif_len);
  if (st.ok() && reinterpret_cast<uintptr_t>(d_jpeg_bytes) % 8)
    st = Status{RD_INVALID_INPUT, "the byte count must be 8-byte aligned"};
  if (st.ok() && capacity < rd::jpeg_bound((int)width, (int)height, icc_len, exif_len))
    st = Status{RD_INVALID_DIMENSIONS, "the JPEG buffer is smaller than rd_jpeg_bound"};
  if (!st.ok()) return finish(h, st);
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  st = rd::run_jpeg_encode(ctx, d_rgb, (int)width, (int)height, quality, icc, icc_len, exif, exif_len, d_jpeg,
                           d_jpeg_bytes);
  if (st.ok()) st = rd::check_kernel_error(ctx, "jpeg encode");
  return finish(h, st);
}

rd_status rd_encode_jpeg(rd_ctx* h, const uint8_t* rgb, uint32_t width, uint32_t height, uint64_t row_stride,
                         int32_t quality, const uint8_t* icc, uint64_t icc_len, const uint8_t* exif,
                         uint64_t exif_len, uint8_t* jpeg, uint64_t capacity, uint64_t* jpeg_bytes,
                         rd_metrics* metrics) {
  if (!h || !jpeg || !jpeg_bytes) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  Status st = jpeg_args(rgb, width, height, row_stride, quality, icc, icc_len, exif, exif_len);
  if (!st.ok()) return finish(h, st);
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const uint64_t in_bytes = 3ull * width * height;
  const uint64_t in_room = (in_bytes + 255) & ~255ull;
  const uint64_t bound = rd::jpeg_bound((int)width, (int)height, icc_len, exif_len);
  const uint64_t out_room = (bound + 255) & ~255ull;
  const uint64_t total = in_room + out_room + 16;
  void* p = nullptr;
  st = rd::device_alloc(ctx, total, &p);
  if (!st.ok()) return finish(h, st);
  uint8_t* d_in = static_cast<uint8_t*>(p);
  uint8_t* d_file = d_in + in_room;
  uint64_t* d_size = reinterpret_cast<uint64_t*>(d_file + out_room);
  Timer tm(ctx);
  if (cudaMemcpyAsync(d_in, rgb, in_bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "image upload failed"};
  tm.mark();
  if (st.ok())
    st = rd::run_jpeg_encode(ctx, d_in, (int)width, (int)height, quality, icc, icc_len, exif, exif_len, d_file,
                             d_size);
  tm.mark();
  uint64_t size = 0;
  if (st.ok() && (cudaMemcpyAsync(&size, d_size, sizeof(size), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaStreamSynchronize(ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "JPEG size readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "jpeg encode");
  if (st.ok()) {
    *jpeg_bytes = size;
    if (size > capacity) st = Status{RD_INVALID_DIMENSIONS, "the JPEG buffer is smaller than the file"};
  }
  if (st.ok() && (cudaMemcpyAsync(jpeg, d_file, size, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaStreamSynchronize(ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "JPEG readback failed"};
  if (st.ok() && metrics) {
    std::memset(metrics, 0, sizeof(*metrics));
    metrics->total_ms = tm.span(0, 1);
    metrics->kernel_launches = ctx.launches;
  }
  rd::device_free(ctx, p, total);
  return finish(h, st);
}

rd_status rd_check_math(rd_ctx* h, int32_t which, uint64_t* result) {
  if (!h || !result || which < 0 || which > 4) return finish(h, Status{RD_INVALID_INPUT, "bad argument"});
  cudaSetDevice(h->c.device);
  if (which == 4) return finish(h, rd::run_hypot_check(h->c, result));
  return finish(h, rd::run_math_check(h->c, which, result));
}

rd_status rd_source_dimensions(const rd_source* s, uint32_t* w, uint32_t* hgt) {
  if (!s || !w || !hgt) return RD_INVALID_INPUT;
  *w = (uint32_t)s->W;
  *hgt = (uint32_t)s->H;
  return RD_OK;
}
rd_status rd_base_dimensions(const rd_base* b, uint32_t* w, uint32_t* hgt) {
  if (!b || !w || !hgt) return RD_INVALID_INPUT;
  *w = (uint32_t)b->W;
  *hgt = (uint32_t)b->H;
  return RD_OK;
}

static rd_status download_planar(rd_ctx* h, const float* d, int W, int H, float* out) {
  rd::Context& ctx = h->c;
  const size_t plane = (size_t)W * H;
  std::vector<float> tmp(3 * plane);
  if (cudaMemcpyAsync(tmp.data(), d, sizeof(float) * 3 * plane, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx.stream) != cudaSuccess)
    return finish(h, Status{RD_READBACK, "readback failed"});
  for (size_t i = 0; i < plane; ++i) {
    out[3 * i] = tmp[i];
    out[3 * i + 1] = tmp[plane + i];
    out[3 * i + 2] = tmp[2 * plane + i];
  }
  return RD_OK;
}

rd_status rd_source_download(rd_ctx* h, const rd_source* s, float* out) {
  if (!h || !s || !out) return RD_INVALID_INPUT;
  return download_planar(h, s->rgb, s->W, s->H, out);
}
rd_status rd_base_download(rd_ctx* h, const rd_base* b, float* out) {
  if (!h || !b || !out) return RD_INVALID_INPUT;
  return download_planar(h, b->rgb, b->W, b->H, out);
}
void rd_source_release(rd_source* s) {
  if (!s) return;
  rd::device_free(s->ctx->c, s->rgb, s->bytes);
  delete s;
}
void rd_base_release(rd_base* b) {
  if (!b) return;
  rd::device_free(b->ctx->c, b->rgb, b->bytes);
  if (b->d_hist) rd::device_free(b->ctx->c, b->d_hist, b->out_bytes);
  delete b;
}

// ------------------------------------------------------------------ stages
static Status upload_planar(rd::Context& ctx, const float* interleaved, int W, int H, float** out, size_t* bytes) {
  const size_t plane = (size_t)W * H;
  std::vector<float> tmp(3 * plane);
  for (size_t i = 0; i < plane; ++i) {
    tmp[i] = interleaved[3 * i];
    tmp[plane + i] = interleaved[3 * i + 1];
    tmp[2 * plane + i] = interleaved[3 * i + 2];
  }
  *bytes = sizeof(float) * 3 * plane;
  void* p = nullptr;
  RD_TRY(rd::device_alloc(ctx, *bytes, &p));
  *out = static_cast<float*>(p);
  RD_CUDA_TRY(cudaMemcpyAsync(*out, tmp.data(), *bytes, cudaMemcpyHostToDevice, ctx.stream));
  RD_CUDA_TRY(cudaStreamSynchronize(ctx.stream));
  return Status{};
}

rd_status rd_stage_highlight(rd_ctx* h, const uint16_t* mosaic, size_t row_stride, const rd_sensor_desc* s,
                             float* out, uint64_t* stats) {
  if (!h || !mosaic || !s || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  Status st;
  rd::validate_sensor(*s, st);
  if (!st.ok()) return finish(h, st);
  const size_t raw_bytes = sizeof(uint16_t) * row_stride * s->sensor_height;
  const int W = (int)s->crop_width, H = (int)s->crop_height;
  const size_t out_bytes = sizeof(float) * (size_t)W * H;
  void *praw = nullptr, *pout = nullptr, *pst = nullptr;
  st = rd::device_alloc(ctx, raw_bytes, &praw);
  if (st.ok()) st = rd::device_alloc(ctx, out_bytes, &pout);
  if (st.ok()) st = rd::device_alloc(ctx, 16 * sizeof(unsigned long long), &pst);
  if (st.ok() && cudaMemcpyAsync(praw, mosaic, raw_bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "upload failed"};
  if (st.ok() && cudaMemsetAsync(pst, 0, 16 * sizeof(unsigned long long), ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "memset failed"};
  if (st.ok()) {
    rd::MosaicSource src = rd::make_source(*s, static_cast<const uint16_t*>(praw), row_stride);
    if (s->highlight == RD_HIGHLIGHT_OPPOSED)
      st = rd::run_opposed(ctx, src, static_cast<float*>(pout), s->detection_levels,
                           s->has_neutral_ceiling ? s->neutral_ceiling : nullptr,
                           static_cast<unsigned long long*>(pst), nullptr);
    else
      st = rd::launch_normalize(ctx, src, static_cast<float*>(pout), static_cast<unsigned long long*>(pst));
  }
  uint64_t host_stats[16] = {};
  if (st.ok() && (cudaMemcpyAsync(out, pout, out_bytes, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaMemcpyAsync(host_stats, pst, sizeof(host_stats), cudaMemcpyDeviceToHost, ctx.stream) !=
                      cudaSuccess))
    st = Status{RD_READBACK, "readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "highlight");
  if (st.ok() && stats) std::memcpy(stats, host_stats, sizeof(uint64_t) * 9);
  rd::device_free(ctx, praw, raw_bytes);
  rd::device_free(ctx, pout, out_bytes);
  rd::device_free(ctx, pst, 16 * sizeof(unsigned long long));
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_opposed(rd_ctx* h, const float* mosaic, uint32_t W, uint32_t H, int32_t cfa,
                           const float levels[3], const float* ceiling, float* out, uint64_t* stats,
                           uint32_t* labels, uint32_t* region_count) {
  if (!h || !mosaic || !levels || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (W < 1 || H < 1 || cfa < 0 || cfa > 3) return finish(h, Status{RD_INVALID_DIMENSIONS, "bad mosaic"});
  for (int c = 0; c < 3; ++c) {
    if (!std::isfinite(levels[c]) || !(levels[c] > 0.0f))
      return finish(h, Status{RD_INVALID_INPUT, "detection levels must be finite and positive"});
    if (ceiling && (!std::isfinite(ceiling[c]) || !(ceiling[c] > 0.0f)))
      return finish(h, Status{RD_INVALID_INPUT, "neutral ceiling must be finite and positive"});
  }
  for (size_t i = 0; i < (size_t)W * H; ++i)
    if (!std::isfinite(mosaic[i])) return finish(h, Status{RD_INVALID_INPUT, "non-finite sample"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const size_t bytes = sizeof(float) * (size_t)W * H;
  const size_t cells = (size_t)(W / 2 + W % 2) * (H / 2 + H % 2);
  void *pm = nullptr, *ps = nullptr, *pl = nullptr;
  Status st = rd::device_alloc(ctx, bytes, &pm);
  if (st.ok()) st = rd::device_alloc(ctx, 16 * sizeof(unsigned long long), &ps);
  if (st.ok() && labels) st = rd::device_alloc(ctx, sizeof(uint32_t) * cells, &pl);
  if (st.ok() && (cudaMemcpyAsync(pm, mosaic, bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess ||
                  cudaMemsetAsync(ps, 0, 16 * sizeof(unsigned long long), ctx.stream) != cudaSuccess))
    st = Status{RD_SYNCHRONIZATION, "upload failed"};
  uint32_t count = 0;
  if (st.ok()) {
    // The normalized mosaic is the source and is reconstructed in place.
    rd::MosaicSource src{};
    src.f32 = static_cast<const float*>(pm);
    src.width = (int)W;
    src.height = (int)H;
    src.cfa = cfa;
    src.black_w = src.black_h = 1;
    src.white_count = 1;
    st = rd::run_opposed_labels(ctx, src, static_cast<float*>(pm), levels, ceiling,
                                static_cast<unsigned long long*>(ps), static_cast<uint32_t*>(pl), &count);
  }
  uint64_t host_stats[16] = {};
  if (st.ok() && (cudaMemcpyAsync(out, pm, bytes, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaMemcpyAsync(host_stats, ps, sizeof(host_stats), cudaMemcpyDeviceToHost, ctx.stream) !=
                      cudaSuccess ||
                  (labels && cudaMemcpyAsync(labels, pl, sizeof(uint32_t) * cells, cudaMemcpyDeviceToHost,
                                             ctx.stream) != cudaSuccess)))
    st = Status{RD_READBACK, "readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "opposed");
  if (st.ok()) {
    if (stats) std::memcpy(stats, host_stats, sizeof(uint64_t) * 9);
    if (region_count) *region_count = count;
  }
  rd::device_free(ctx, pm, bytes);
  rd::device_free(ctx, ps, 16 * sizeof(unsigned long long));
  if (pl) rd::device_free(ctx, pl, sizeof(uint32_t) * cells);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_demosaic(rd_ctx* h, const float* mosaic, uint32_t W, uint32_t H, int32_t cfa, int32_t algorithm,
                            const float balance[3], float* out) {
  if (!h || !mosaic || !balance || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (W < 2 || H < 2) return finish(h, Status{RD_INVALID_DIMENSIONS, "demosaicing requires at least 2x2 samples"});
  if (cfa < 0 || cfa > 3 || algorithm < 0 || algorithm > 3)
    return finish(h, Status{RD_INVALID_INPUT, "unknown CFA or algorithm"});
  for (int c = 0; c < 3; ++c)
    if (!std::isfinite(balance[c]) || !(balance[c] > 0.0f))
      return finish(h, Status{RD_INVALID_INPUT, "balance must be finite and positive"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const size_t in_bytes = sizeof(float) * (size_t)W * H, out_bytes = 3 * in_bytes;
  void *pin = nullptr, *pout = nullptr;
  Status st = rd::device_alloc(ctx, in_bytes, &pin);
  if (st.ok()) st = rd::device_alloc(ctx, out_bytes, &pout);
  if (st.ok() && cudaMemcpyAsync(pin, mosaic, in_bytes, cudaMemcpyHostToDevice, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "upload failed"};
  if (st.ok()) {
    rd::MosaicSource src{};
    src.f32 = static_cast<const float*>(pin);
    src.width = (int)W;
    src.height = (int)H;
    src.cfa = cfa;
    src.black_w = src.black_h = 1;
    src.white_count = 1;
    for (int c = 0; c < 3; ++c) src.fwd[c] = balance[c];
    st = rd::run_demosaic(ctx, src, algorithm, static_cast<float*>(pout), nullptr);
  }
  if (st.ok()) st = rd::check_kernel_error(ctx, "demosaic");
  rd_status rs = st.code;
  if (st.ok()) rs = download_planar(h, static_cast<float*>(pout), (int)W, (int)H, out);
  rd::device_free(ctx, pin, in_bytes);
  rd::device_free(ctx, pout, out_bytes);
  cudaStreamSynchronize(ctx.stream);
  if (rs != RD_OK && st.ok()) return rs;
  return finish(h, st);
}

rd_status rd_stage_capture(rd_ctx* h, float* rgb, uint32_t W, uint32_t H, const rd_detail_desc* detail) {
  if (!h || !rgb || !detail) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  float* d = nullptr;
  size_t bytes = 0;
  Status st = upload_planar(ctx, rgb, (int)W, (int)H, &d, &bytes);
  if (st.ok()) st = rd::run_capture(ctx, d, (int)W, (int)H, *detail);
  if (st.ok()) st = rd::check_kernel_error(ctx, "capture");
  if (st.ok() && download_planar(h, d, (int)W, (int)H, rgb) != RD_OK) st = Status{RD_READBACK, "readback failed"};
  if (d) rd::device_free(ctx, d, bytes);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_optics(rd_ctx* h, const rd_optics_desc* o, const float* rgb_in, float* rgb_out) {
  if (!h || !o || !rgb_in || !rgb_out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (o->width < 4 || o->height < 4) return finish(h, Status{RD_INVALID_DIMENSIONS, "optics needs at least 4x4"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const int W = (int)o->width, H = (int)o->height;
  const size_t plane = (size_t)W * H;
  float* d = nullptr;
  size_t bytes = 0;
  void* p = nullptr;
  float* mult = nullptr;
  float* warped = nullptr;
  Status st = upload_planar(ctx, rgb_in, W, H, &d, &bytes);
  if (st.ok() && o->vignetting == 1) {
    st = rd::device_alloc(ctx, sizeof(float) * plane, &p);
    if (st.ok()) {
      mult = static_cast<float*>(p);
      st = rd::run_vignette_plane(ctx, *o, mult);
    }
  }
  const bool warp = o->distortion_model != RD_DISTORTION_NONE || o->tca_model != RD_TCA_NONE;
  if (st.ok()) {
    st = rd::device_alloc(ctx, bytes, &p);
    if (st.ok()) warped = static_cast<float*>(p);
  }
  if (st.ok()) {
    if (warp) {
      st = rd::run_optics_gather(ctx, *o, d, mult, warped);
    } else {
      // Vignetting only: the reduction kernel at 1:1 applies the multiplier exactly.
      st = rd::run_area_reduce(ctx, d, mult, W, H, W, H, warped);
    }
  }
  if (st.ok()) st = rd::check_kernel_error(ctx, "optics");
  if (st.ok() && download_planar(h, warped, W, H, rgb_out) != RD_OK) st = Status{RD_READBACK, "readback failed"};
  if (d) rd::device_free(ctx, d, bytes);
  if (warped) rd::device_free(ctx, warped, bytes);
  if (mult) rd::device_free(ctx, mult, sizeof(float) * plane);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_area_reduce(rd_ctx* h, const float* rgb_in, uint32_t W, uint32_t H, uint32_t tw, uint32_t th,
                               float* rgb_out) {
  if (!h || !rgb_in || !rgb_out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (tw == 0 || th == 0 || tw > W || th > H)
    return finish(h, Status{RD_INVALID_DIMENSIONS, "area reduction cannot upscale or produce an empty image"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  float* d = nullptr;
  size_t bytes = 0;
  void* p = nullptr;
  const size_t out_bytes = sizeof(float) * 3 * (size_t)tw * th;
  Status st = upload_planar(ctx, rgb_in, (int)W, (int)H, &d, &bytes);
  if (st.ok()) st = rd::device_alloc(ctx, out_bytes, &p);
  if (st.ok())
    st = rd::run_area_reduce(ctx, d, nullptr, (int)W, (int)H, (int)tw, (int)th, static_cast<float*>(p));
  if (st.ok()) st = rd::check_kernel_error(ctx, "area reduce");
  if (st.ok() && download_planar(h, static_cast<float*>(p), (int)tw, (int)th, rgb_out) != RD_OK)
    st = Status{RD_READBACK, "readback failed"};
  if (d) rd::device_free(ctx, d, bytes);
  if (p) rd::device_free(ctx, p, out_bytes);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_color(rd_ctx* h, const float* rgb_in, uint32_t W, uint32_t H, const rd_color_desc* color,
                         uint8_t* srgb_out, uint64_t* hist, uint64_t* clipped) {
  if (!h || !rgb_in || !color || !srgb_out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  float* d = nullptr;
  size_t bytes = 0;
  void* p = nullptr;
  const size_t out_bytes = (size_t)3 * W * H + 1024 * sizeof(unsigned long long);
  Status st = upload_planar(ctx, rgb_in, (int)W, (int)H, &d, &bytes);
  if (st.ok()) st = rd::device_alloc(ctx, out_bytes, &p);
  unsigned long long* d_hist = static_cast<unsigned long long*>(p);
  uint8_t* d_out = reinterpret_cast<uint8_t*>(d_hist + 1024);
  if (st.ok() && cudaMemsetAsync(d_hist, 0, 1024 * sizeof(unsigned long long), ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "memset failed"};
  if (st.ok()) st = rd::run_color_output(ctx, d, (int)W, (int)H, *color, true, d_out, d_hist);
  uint64_t bins[1024];
  if (st.ok() && (cudaMemcpyAsync(srgb_out, d_out, (size_t)3 * W * H, cudaMemcpyDeviceToHost, ctx.stream) !=
                      cudaSuccess ||
                  cudaMemcpyAsync(bins, d_hist, sizeof(bins), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "readback failed"};
  if (st.ok()) st = rd::check_kernel_error(ctx, "color");
  if (st.ok()) {
    if (hist) std::memcpy(hist, bins, sizeof(bins));
    if (clipped)
      for (int c = 0; c < 3; ++c) {
        clipped[c] = bins[256 * c];
        clipped[3 + c] = bins[256 * c + 255];
      }
  }
  if (d) rd::device_free(ctx, d, bytes);
  if (p) rd::device_free(ctx, p, out_bytes);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_stage_output(rd_ctx* h, const float* rgb_in, uint32_t W, uint32_t H, const rd_color_desc* color,
                          const rd_output_desc* output, void* out, size_t out_capacity, uint64_t* hist,
                          uint64_t* gamut) {
  if (!h || !rgb_in || !color || !output || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  if (W == 0 || H == 0 || W > (uint32_t)INT32_MAX || H > (uint32_t)INT32_MAX)
    return finish(h, Status{RD_INVALID_DIMENSIONS, "empty image"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  float* d = nullptr;
  size_t bytes = 0;
  Status st = upload_planar(ctx, rgb_in, (int)W, (int)H, &d, &bytes);
  if (st.ok()) st = render_output_host(h, d, (int)W, (int)H, *color, *output, out, out_capacity, hist, gamut, nullptr);
  if (d) rd::device_free(ctx, d, bytes);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_optics_plan(rd_optics_desc* o, float crop, float real_focal, float cx, float cy) {
  if (!o) return RD_INVALID_INPUT;
  return rd::optics_plan(*o, crop, real_focal, cx, cy).code;
}

rd_status rd_optics_radial_table(const rd_optics_desc* o, float* knots, float* step, int32_t* guard) {
  if (!o || !guard || o->width == 0 || o->height == 0) return RD_INVALID_INPUT;
  const std::vector<float> tab = rd::optics_input_coordinates(*o);
  const rd::RadialTable t = rd::build_radial_table(*o, tab.data(), tab.data() + o->width);
  *guard = t.guard;
  if (step) *step = t.step;
  if (knots && t.guard >= 0) std::copy(t.knots.begin(), t.knots.end(), knots);
  return RD_OK;
}

void rd_standard_base_lut(float* lut) {
  if (lut) rd::standard_base_lut(lut);
}

void rd_light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks, float* lut) {
  if (lut) rd::light_tone_lut(contrast, highlights, shadows, whites, blacks, lut);
}

rd_status rd_synth_mosaic_device(rd_ctx* h, const rd_synth_desc* d, uint16_t* d_out) {
  if (!h || !d || !d_out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  cudaSetDevice(h->c.device);
  Status st = rd::run_synth(h->c, *d, d_out);
  if (st.ok() && cudaStreamSynchronize(h->c.stream) != cudaSuccess) st = Status{RD_SYNCHRONIZATION, "sync failed"};
  return finish(h, st);
}

rd_status rd_synth_mosaic(rd_ctx* h, const rd_synth_desc* d, uint16_t* out) {
  if (!h || !d || !out) return finish(h, Status{RD_INVALID_INPUT, "null argument"});
  rd::Context& ctx = h->c;
  cudaSetDevice(ctx.device);
  const size_t bytes = sizeof(uint16_t) * d->width * d->height;
  void* p = nullptr;
  Status st = rd::device_alloc(ctx, bytes, &p);
  if (st.ok()) st = rd::run_synth(ctx, *d, static_cast<uint16_t*>(p));
  if (st.ok() && (cudaMemcpyAsync(out, p, bytes, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
                  cudaStreamSynchronize(ctx.stream) != cudaSuccess))
    st = Status{RD_READBACK, "readback failed"};
  if (p) rd::device_free(ctx, p, bytes);
  cudaStreamSynchronize(ctx.stream);
  return finish(h, st);
}

rd_status rd_ctx_event_record(rd_ctx* h, int slot) {
  if (!h || slot < 0 || slot >= 64) return RD_INVALID_INPUT;
  rd::Context& c = h->c;
  if (!c.user_ev[slot] && cudaEventCreate(&c.user_ev[slot]) != cudaSuccess) return RD_SYNCHRONIZATION;
  return cudaEventRecord(c.user_ev[slot], c.stream) == cudaSuccess ? RD_OK : RD_SYNCHRONIZATION;
}

rd_status rd_ctx_event_elapsed(rd_ctx* h, int a, int b, float* ms) {
  if (!h || !ms || a < 0 || b < 0 || a >= 64 || b >= 64 || !h->c.user_ev[a] || !h->c.user_ev[b])
    return RD_INVALID_INPUT;
  if (cudaEventSynchronize(h->c.user_ev[b]) != cudaSuccess) return RD_SYNCHRONIZATION;
  return cudaEventElapsedTime(ms, h->c.user_ev[a], h->c.user_ev[b]) == cudaSuccess ? RD_OK : RD_SYNCHRONIZATION;
}

rd_status rd_ctx_flush_l2(rd_ctx* h) {
  if (!h) return RD_INVALID_INPUT;
  rd::Context& c = h->c;
  if (!c.flush_buf) {
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c.device);
    c.flush_bytes = std::max<size_t>((size_t)l2 * 2, (size_t)256 << 20);
    Status st = rd::device_alloc(c, c.flush_bytes, &c.flush_buf);
    if (!st.ok()) return finish(h, st);
  }
  return cudaMemsetAsync(c.flush_buf, 0x5a, c.flush_bytes, c.stream) == cudaSuccess ? RD_OK : RD_SYNCHRONIZATION;
}

rd_status rd_ctx_enable_kernel_timing(rd_ctx* h, int enable) {
  if (!h) return RD_INVALID_INPUT;
  cudaStreamSynchronize(h->c.stream);
  rd::resolve_kernel_timing(h->c);
  h->c.timing = enable != 0;
  return RD_OK;
}

rd_status rd_ctx_kernel_timing(const rd_ctx* h, int family, const char** name, double* total_ms,
                               uint64_t* launches) {
  if (!h || family < 0 || family >= RD_KERNEL_FAMILIES) return RD_INVALID_INPUT;
  if (name) *name = rd::kernel_family_name(family);
  if (total_ms) *total_ms = h->c.family_ms[family];
  if (launches) *launches = h->c.family_launches[family];
  return RD_OK;
}

rd_status rd_ctx_reset_kernel_timing(rd_ctx* h) {
  if (!h) return RD_INVALID_INPUT;
  cudaStreamSynchronize(h->c.stream);
  rd::resolve_kernel_timing(h->c);
  for (int k = 0; k < RD_KERNEL_FAMILIES; ++k) {
    h->c.family_ms[k] = 0.0;
    h->c.family_launches[k] = 0;
  }
  return RD_OK;
}

rd_status rd_host_alloc(size_t bytes, void** out) {
  if (!out) return RD_INVALID_INPUT;
  return cudaMallocHost(out, bytes) == cudaSuccess ? RD_OK : RD_OVER_BUDGET;
}

void rd_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
}

rd_status rd_device_alloc(rd_ctx* h, size_t bytes, void** out) {
  if (!h || !out) return RD_INVALID_INPUT;
  cudaSetDevice(h->c.device);
  Status st = rd::device_alloc(h->c, bytes, out);
  if (st.ok()) {
    h->c.user_allocs[*out] = bytes;
    cudaStreamSynchronize(h->c.stream);
  }
  return finish(h, st);
}
rd_status rd_device_free(rd_ctx* h, void* ptr) {
  if (!h) return RD_INVALID_INPUT;
  if (!ptr) return RD_OK;
  auto it = h->c.user_allocs.find(ptr);
  if (it == h->c.user_allocs.end()) return finish(h, Status{RD_INVALID_INPUT, "pointer was not allocated here"});
  rd::device_free(h->c, ptr, it->second);
  h->c.user_allocs.erase(it);
  cudaStreamSynchronize(h->c.stream);
  return RD_OK;
}
rd_status rd_copy_to_device(rd_ctx* h, void* dst, const void* src, size_t bytes) {
  if (!h) return RD_INVALID_INPUT;
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->c.stream) != cudaSuccess ||
      cudaStreamSynchronize(h->c.stream) != cudaSuccess)
    return RD_SYNCHRONIZATION;
  return RD_OK;
}
rd_status rd_copy_to_host(rd_ctx* h, void* dst, const void* src, size_t bytes) {
  if (!h) return RD_INVALID_INPUT;
  if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->c.stream) != cudaSuccess ||
      cudaStreamSynchronize(h->c.stream) != cudaSuccess)
    return RD_READBACK;
  return RD_OK;
}

}  // extern "C"

// ---- batched develop over one AMaZE work queue -------------------------------
// rd_develop_batch_flat: the batch stage by stage. Lanes (contexts on their own
// streams, one host thread each) upload their images and normalize / Opposed
// them; one AMaZE launch then takes the half-tile work items of every image
// from a shared counter (run_amaze_images), so no image's last wave leaves SMs
// idle; capture sharpening follows on the same stream, each RL iteration one
// launch over the work items of every image that shares its taps
// (run_capture_images); the lanes finish their images (spatial pass, render
// with host outputs). Image k belongs to lane k % lanes throughout, and its
// device buffers come from that lane's pool.
namespace {

struct FlatJob {
  uint16_t* d_raw = nullptr;
  size_t raw_bytes = 0;
  float* d_mosaic = nullptr;
  size_t mosaic_bytes = 0;
  unsigned long long* d_stats = nullptr;
  rd::MosaicSource src{};
  rd_source* source = nullptr;
  Status st;
};

Status flat_prepare(rd_ctx* h, const rd_batch_item& it, FlatJob& j) {
  rd::Context& ctx = h->c;
  const rd_sensor_desc& s = it.sensor;
  Status st;
  validate_sensor(s, st);
  if (!st.ok()) return st;
  if (!it.mosaic) return Status{RD_INVALID_INPUT, "null mosaic"};
  if (it.row_stride < s.sensor_width) return Status{RD_INVALID_DIMENSIONS, "row stride is shorter than the sensor width"};
  const int W = (int)s.crop_width, H = (int)s.crop_height;
  void* p = nullptr;
  j.raw_bytes = sizeof(uint16_t) * it.row_stride * s.sensor_height;
  RD_TRY(rd::device_alloc(ctx, j.raw_bytes, &p));
  j.d_raw = static_cast<uint16_t*>(p);
  RD_CUDA_TRY(cudaMemcpyAsync(j.d_raw, it.mosaic, j.raw_bytes, cudaMemcpyHostToDevice, ctx.stream));
  RD_TRY(rd::device_alloc(ctx, sizeof(unsigned long long) * 16, &p));
  j.d_stats = static_cast<unsigned long long*>(p);
  RD_CUDA_TRY(cudaMemsetAsync(j.d_stats, 0, sizeof(unsigned long long) * 16, ctx.stream));
  j.src = rd::make_source(s, j.d_raw, it.row_stride);
  if (s.highlight == RD_HIGHLIGHT_OPPOSED) {
    j.mosaic_bytes = sizeof(float) * (size_t)W * H;
    RD_TRY(rd::device_alloc(ctx, j.mosaic_bytes, &p));
    j.d_mosaic = static_cast<float*>(p);
    RD_TRY(rd::run_opposed(ctx, j.src, j.d_mosaic, s.detection_levels,
                           s.has_neutral_ceiling ? s.neutral_ceiling : nullptr, j.d_stats, nullptr));
    j.src.f32 = j.d_mosaic;
    j.src.clip = 0;
  }
  j.source = new (std::nothrow) rd_source{h, nullptr, W, H, sizeof(float) * 3 * (size_t)W * H};
  if (!j.source) return Status{RD_OVER_BUDGET, "host allocation failed"};
  RD_TRY(rd::device_alloc(ctx, j.source->bytes, &p));
  j.source->rgb = static_cast<float*>(p);
  return Status{};
}

void flat_release_staging(rd_ctx* h, FlatJob& j) {
  rd::Context& ctx = h->c;
  if (j.d_mosaic) rd::device_free(ctx, j.d_mosaic, j.mosaic_bytes);
  if (j.d_raw) rd::device_free(ctx, j.d_raw, j.raw_bytes);
  if (j.d_stats) rd::device_free(ctx, j.d_stats, sizeof(unsigned long long) * 16);
  j.d_mosaic = nullptr;
  j.d_raw = nullptr;
  j.d_stats = nullptr;
}

}  // namespace

extern "C" rd_status rd_develop_batch_flat(int device, rd_batch_item* items, int32_t count, int32_t lanes,
                                           double* wall_ms) {
  using Clock = std::chrono::steady_clock;
  if (!items || count < 0 || lanes <= 0) return RD_INVALID_INPUT;
  if (wall_ms) *wall_ms = 0.0;
  if (count == 0) return RD_OK;
  lanes = std::min(lanes, count);
  std::vector<rd_ctx*> ctxs(lanes, nullptr);
  std::vector<cudaEvent_t> prepared(lanes, nullptr);
  cudaEvent_t demosaiced = nullptr;
  rd_status status = RD_OK;
  for (int l = 0; l < lanes && status == RD_OK; ++l) {
    status = rd_ctx_create(device, 0, &ctxs[l]);
    if (status == RD_OK && cudaEventCreateWithFlags(&prepared[l], cudaEventDisableTiming) != cudaSuccess)
      status = RD_SYNCHRONIZATION;
  }
  if (status == RD_OK && cudaEventCreateWithFlags(&demosaiced, cudaEventDisableTiming) != cudaSuccess)
    status = RD_SYNCHRONIZATION;
  std::vector<FlatJob> jobs((size_t)count);
  const auto t0 = Clock::now();
  auto on_lanes = [&](auto&& body) {
    std::vector<std::thread> threads;
    for (int l = 1; l < lanes; ++l) threads.emplace_back(body, l);
    body(0);
    for (std::thread& t : threads) t.join();
  };
  if (status == RD_OK) {
    // 1. upload + normalize + highlight, lane by lane.
    on_lanes([&](int l) {
      rd_ctx* h = ctxs[l];
      cudaSetDevice(h->c.device);
      for (int k = l; k < count; k += lanes) jobs[k].st = flat_prepare(h, items[k], jobs[k]);
      cudaEventRecord(prepared[l], h->c.stream);
    });
    // 2. demosaic on lane 0: AMaZE of every image larger than 32x32 in one launch.
    rd::Context& c0 = ctxs[0]->c;
    cudaSetDevice(c0.device);
    for (int l = 1; l < lanes; ++l) cudaStreamWaitEvent(c0.stream, prepared[l], 0);
    std::vector<rd::AmazeJob> amaze;
    std::vector<int> amaze_images;
    Status dm;
    for (int k = 0; k < count && dm.ok(); ++k) {
      FlatJob& j = jobs[k];
      if (!j.st.ok()) continue;
      const int alg = items[k].sensor.demosaic;
      if (alg == RD_DEMOSAIC_AMAZE && j.source->W > 32 && j.source->H > 32) {
        amaze.push_back(rd::demosaic_job(j.src, alg, j.source->rgb, j.d_stats));
        amaze_images.push_back(k);
      } else {
        j.st = rd::run_demosaic(c0, j.src, alg, j.source->rgb, j.d_stats);
      }
    }
    if (!amaze.empty()) dm = rd::run_amaze_images(c0, amaze.data(), (int)amaze.size());
    if (dm.ok()) dm = rd::check_kernel_error(c0, "batch demosaic");
    if (!dm.ok())
      for (int k : amaze_images)
        if (jobs[k].st.ok()) jobs[k].st = dm;
    // 3. capture sharpening on lane 0: each iteration of every image that
    //    shares its taps in one launch over all their work items.
    std::vector<rd::CaptureJob> capture;
    std::vector<int> capture_images;
    for (int k = 0; k < count; ++k) {
      FlatJob& j = jobs[k];
      if (!j.st.ok()) continue;
      capture.push_back(rd::CaptureJob{j.source->rgb, j.source->W, j.source->H, items[k].detail, Status{}});
      capture_images.push_back(k);
    }
    Status cs;
    if (!capture.empty()) cs = rd::run_capture_images(c0, capture.data(), (int)capture.size());
    if (cs.ok()) cs = rd::check_kernel_error(c0, "batch capture");
    for (size_t i = 0; i < capture.size(); ++i) {
      FlatJob& j = jobs[capture_images[i]];
      if (!capture[i].st.ok()) j.st = capture[i].st;
      else if (!cs.ok()) j.st = cs;
    }
    cudaEventRecord(demosaiced, c0.stream);
    // 4. spatial pass and render, lane by lane.
    on_lanes([&](int l) {
      rd_ctx* h = ctxs[l];
      rd::Context& ctx = h->c;
      cudaSetDevice(ctx.device);
      cudaStreamWaitEvent(ctx.stream, demosaiced, 0);
      for (int k = l; k < count; k += lanes) {
        FlatJob& j = jobs[k];
        rd_batch_item& it = items[k];
        const auto s0 = Clock::now();
        Status st = j.st;
        flat_release_staging(h, j);
        if (st.ok()) st = rd::check_kernel_error(ctx, "batch develop");
        rd_status code = finish(h, st);
        rd_base* base = nullptr;
        if (code == RD_OK)
          code = rd_spatial(h, j.source, &it.optics, it.target_width, it.target_height, it.wb_gains,
                            it.camera_to_rec2020, &base, nullptr);
        if (j.source) {
          if (j.source->rgb) {
            rd_source_release(j.source);
          } else {
            delete j.source;
          }
          j.source = nullptr;
        }
        if (code == RD_OK) code = rd_render(h, base, &it.color, it.srgb_out, it.hist, nullptr, nullptr);
        if (base) rd_base_release(base);
        it.status = code;
        it.ms = std::chrono::duration<double, std::milli>(Clock::now() - s0).count();
      }
    });
  }
  if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
  for (FlatJob& j : jobs)
    if (j.source) {
      if (j.source->rgb) rd_source_release(j.source);
      else delete j.source;
    }
  for (int l = 0; l < lanes; ++l) {
    if (prepared[l]) cudaEventDestroy(prepared[l]);
  }
  if (demosaiced) cudaEventDestroy(demosaiced);
  for (int l = 0; l < lanes; ++l)
    if (ctxs[l]) {
      for (int k = l; k < count; k += lanes) flat_release_staging(ctxs[l], jobs[k]);
      rd_ctx_destroy(ctxs[l]);
    }
  if (status != RD_OK) return status;
  for (int k = 0; k < count; ++k)
    if (items[k].status != RD_OK) return (rd_status)items[k].status;
  return RD_OK;
}

// rd_develop_batch_flat_graph: the stage-by-stage batch captured into one CUDA
// graph. Branches (one context and stream each, image k on branch k %
// chains) upload and normalize / highlight their images; after a join, branch
// 0 runs the one AMaZE launch over every image's half-tile items and the
// capture sharpening with one launch per RL iteration over the batch; after a
// fork the branches finish their images (spatial pass, render into pinned
// outputs). Every device buffer is allocated and freed inside the graph;
// the AMaZE scratch for the whole batch is reserved before the capture.
extern "C" rd_status rd_develop_batch_flat_graph(int device, rd_batch_item* items, int32_t count, int32_t chains,
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
  size_t all_tiles = 1;
  for (int k = 0; k < count; ++k)
    all_tiles += rd::amaze_tiles((int)items[k].sensor.crop_width, (int)items[k].sensor.crop_height);
  for (int c = 0; c < chains && status == RD_OK; ++c) {
    status = rd_ctx_create(device, 0, &ctxs[c]);
    if (status == RD_OK && c == 0 && !rd::reserve_amaze_scratch(ctxs[c]->c, all_tiles).ok()) status = RD_OVER_BUDGET;
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
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr, mid = nullptr;
  std::vector<cudaEvent_t> join(chains, nullptr), prepared(chains, nullptr);
  if (status == RD_OK && (cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking) != cudaSuccess ||
                          cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess ||
                          cudaEventCreateWithFlags(&mid, cudaEventDisableTiming) != cudaSuccess))
    status = RD_SYNCHRONIZATION;
  for (int c = 0; c < chains && status == RD_OK; ++c)
    if (cudaEventCreateWithFlags(&join[c], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&prepared[c], cudaEventDisableTiming) != cudaSuccess)
      status = RD_SYNCHRONIZATION;
  for (int k = 0; k < count; ++k) items[k].status = RD_CANCELLED;
  std::vector<FlatJob> jobs((size_t)count);
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
    // 1. upload + normalize + highlight on the branches.
    for (int k = 0; k < count && status == RD_OK; ++k) {
      rd_batch_item it = items[k];
      if (!host_pinned) it.mosaic = reinterpret_cast<const uint16_t*>(stage + in_off[k]);
      const Status st = flat_prepare(ctxs[k % chains], it, jobs[k]);
      if (!st.ok()) status = st.code;
    }
    for (int c = 0; c < chains && status == RD_OK; ++c)
      if (cudaEventRecord(prepared[c], ctxs[c]->c.stream) != cudaSuccess ||
          cudaStreamWaitEvent(ctxs[0]->c.stream, prepared[c], 0) != cudaSuccess)
        status = RD_SYNCHRONIZATION;
    // 2. demosaic and capture sharpening over the batch on branch 0.
    rd::Context& b0 = ctxs[0]->c;
    if (status == RD_OK) {
      std::vector<rd::AmazeJob> amaze;
      Status st;
      for (int k = 0; k < count && st.ok(); ++k) {
        FlatJob& j = jobs[k];
        const int alg = items[k].sensor.demosaic;
        if (alg == RD_DEMOSAIC_AMAZE && j.source->W > 32 && j.source->H > 32)
          amaze.push_back(rd::demosaic_job(j.src, alg, j.source->rgb, j.d_stats));
        else
          st = rd::run_demosaic(b0, j.src, alg, j.source->rgb, j.d_stats);
      }
      if (st.ok() && !amaze.empty()) st = rd::run_amaze_images(b0, amaze.data(), (int)amaze.size());
      std::vector<rd::CaptureJob> capture;
      for (int k = 0; k < count && st.ok(); ++k)
        capture.push_back(
            rd::CaptureJob{jobs[k].source->rgb, jobs[k].source->W, jobs[k].source->H, items[k].detail, Status{}});
      if (st.ok() && !capture.empty()) st = rd::run_capture_images(b0, capture.data(), (int)capture.size());
      for (const rd::CaptureJob& cj : capture)
        if (st.ok() && !cj.st.ok()) st = cj.st;
      if (!st.ok()) status = st.code;
    }
    if (status == RD_OK && cudaEventRecord(mid, b0.stream) != cudaSuccess) status = RD_SYNCHRONIZATION;
    for (int c = 1; c < chains && status == RD_OK; ++c)
      if (cudaStreamWaitEvent(ctxs[c]->c.stream, mid, 0) != cudaSuccess) status = RD_SYNCHRONIZATION;
    // 3. spatial pass and render on the branches.
    for (int k = 0; k < count && status == RD_OK; ++k) {
      rd_batch_item& it = items[k];
      rd_ctx* h = ctxs[k % chains];
      FlatJob& j = jobs[k];
      flat_release_staging(h, j);
      rd_base* base = nullptr;
      rd_status st = rd_spatial(h, j.source, &it.optics, it.target_width, it.target_height, it.wb_gains,
                                it.camera_to_rec2020, &base, nullptr);
      rd_source_release(j.source);
      j.source = nullptr;
      uint8_t* srgb = host_pinned ? it.srgb_out : stage + out_off[k];
      uint64_t* hist = host_pinned ? it.hist : reinterpret_cast<uint64_t*>(stage + hist_off[k]);
      if (st == RD_OK) st = rd_render(h, base, &it.color, srgb, hist, nullptr, nullptr);
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
      const Status st = rd::check_kernel_error(ctxs[c]->c, "batch flat graph");
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
  // A capture that failed part way leaves host-side handles behind; their
  // device buffers were graph allocations that no launch made.
  for (FlatJob& j : jobs) delete j.source;
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (cudaEvent_t e : join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : prepared)
    if (e) cudaEventDestroy(e);
  if (fork) cudaEventDestroy(fork);
  if (mid) cudaEventDestroy(mid);
  if (main) cudaStreamDestroy(main);
  for (rd_ctx* c : ctxs)
    if (c) rd_ctx_destroy(c);
  if (stage) cudaFreeHost(stage);
  if (status != RD_OK)
    for (int k = 0; k < count; ++k)
      if (items[k].status == RD_OK) items[k].status = status;
  return status;
}

