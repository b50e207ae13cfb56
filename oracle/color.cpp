// CPU oracle: white balance, camera matrix, global adjustments, sRGB 8-bit
// output and the display histogram. Test infrastructure only.
//
//  white balance / matrix  crates/core/src/cpu/stages.rs:250-308, crates/color/src/matrix.rs:45-61,173-175
//  adjustments             crates/core/src/cpu/stages.rs:380-901
//  base rendering LUT      crates/core/src/rendering.rs:36-92, 223-234
//  LUT sampling            crates/edit/src/light.rs:49-88
//  Light tone LUT          crates/edit/src/light.rs:27-47, 90-142; applied at stages.rs:631-645
//  output                  crates/core/src/cpu/stages.rs:1028-1094, crates/core/src/color/display_output.rs:24-59,
//                          crates/color/src/gamut.rs:110-122,209-222, crates/color/src/transfer.rs:5-11
//  histogram               crates/core/src/analysis/histogram.rs:92-128, clipping.rs:12-22
#include <cmath>
#include <cstring>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

namespace {
constexpr float F32_EPSILON = 1.1920929e-7f;
constexpr float LUM[3] = {0.2627f, 0.6780f, 0.0593f};        // REC2020_LUMINANCE
constexpr float TRANSITION = 0.02f;                           // LUMINANCE_RATIO_TRANSITION
constexpr float HSL_CENTERS[8] = {0.0f, 30.0f / 360.0f, 60.0f / 360.0f, 120.0f / 360.0f,
                                  180.0f / 360.0f, 240.0f / 360.0f, 270.0f / 360.0f, 300.0f / 360.0f};
constexpr float HUE_SHIFT = 0.125f;

// crates/color/src/matrix.rs:103-121
constexpr float REC2020_TO_XYZ[3][3] = {{0.63695806f, 0.1446169f, 0.16888097f},
                                        {0.2627002f, 0.67799807f, 0.059301715f},
                                        {0.0f, 0.028072694f, 1.0609851f}};
constexpr float XYZ_TO_SRGB[3][3] = {{3.24097f, -1.5373832f, -0.49861076f},
                                     {-0.96924365f, 1.8759675f, 0.04155506f},
                                     {0.05563008f, -0.20397696f, 1.0569715f}};

inline float luminance(const float* p) { return p[0] * LUM[0] + p[1] * LUM[1] + p[2] * LUM[2]; }
inline float smoothstep(float e0, float e1, float v) {
  const float n = rclamp((v - e0) / (e1 - e0), 0.0f, 1.0f);
  return n * n * (3.0f - 2.0f * n);
}
inline float rem_euclid(float x, float m) {
  const float r = std::fmod(x, m);
  return r < 0.0f ? r + std::fabs(m) : r;
}
inline float signum(float v) { return std::isnan(v) ? v : (std::signbit(v) ? -1.0f : 1.0f); }

float base_sample(const float* values, float input) {
  if (!std::isfinite(input) || input <= 0.0f) return input;
  const float coordinate = input / (1.0f + input);
  const float position = coordinate * 4095.0f;
  std::size_t lower = (std::size_t)std::floor(position);
  if (lower > 4095) lower = 4095;
  const std::size_t upper = lower + 1 > 4095 ? 4095 : lower + 1;
  const float fraction = position - (float)lower;
  return values[lower] + (values[upper] - values[lower]) * fraction;
}
float lut_sample(const float* values, float input) {
  if (!(input >= 0.0f && input <= 1.0f)) return input;
  const float position = input * 4095.0f;
  const std::size_t lower = (std::size_t)std::floor(position);
  const std::size_t upper = lower + 1 > 4095 ? 4095 : lower + 1;
  const float fraction = position - (float)lower;
  return values[lower] + (values[upper] - values[lower]) * fraction;
}

// stages.rs:657-701
void apply_luminance_delta(float* p, float current, float target) {
  if (!std::isfinite(current) || !std::isfinite(target)) return;
  if ((current > 1.0e-6f && target >= TRANSITION) || (current < -1.0e-6f && target <= -TRANSITION)) {
    const float scale = target / current;
    const float u[3] = {p[0] * scale, p[1] * scale, p[2] * scale};
    if (std::isfinite(u[0]) && std::isfinite(u[1]) && std::isfinite(u[2])) {
      std::memcpy(p, u, sizeof(u));
      return;
    }
  }
  const float delta = target - current;
  if (!std::isfinite(delta)) return;
  const float add[3] = {p[0] + delta, p[1] + delta, p[2] + delta};
  if (!std::isfinite(add[0]) || !std::isfinite(add[1]) || !std::isfinite(add[2])) return;
  if (std::fabs(current) <= 1.0e-6f || signum(current) != signum(target)) {
    std::memcpy(p, add, sizeof(add));
    return;
  }
  const float rw = smoothstep(0.0f, TRANSITION, std::fabs(target));
  if (rw <= F32_EPSILON) {
    std::memcpy(p, add, sizeof(add));
    return;
  }
  const float scale = target / current;
  const float sc[3] = {p[0] * scale, p[1] * scale, p[2] * scale};
  const float u[3] = {add[0] + (sc[0] - add[0]) * rw, add[1] + (sc[1] - add[1]) * rw, add[2] + (sc[2] - add[2]) * rw};
  if (std::isfinite(u[0]) && std::isfinite(u[1]) && std::isfinite(u[2])) std::memcpy(p, u, sizeof(u));
}

void apply_lut_tone(float* p, const float* lut, bool base) {
  const float current = luminance(p);
  const float target = base ? base_sample(lut, current) : lut_sample(lut, current);
  if (!std::isfinite(target) || std::fabs(target - current) <= F32_EPSILON) return;
  apply_luminance_delta(p, current, target);
}

// stages.rs:848-867
void rgb_to_hsl(const float* c, float* out) {
  const float mx = rmax(rmax(c[0], c[1]), c[2]);
  const float mn = rmin(rmin(c[0], c[1]), c[2]);
  const float l = (mx + mn) * 0.5f;
  const float chroma = mx - mn;
  if (chroma <= F32_EPSILON) { out[0] = 0.0f; out[1] = 0.0f; out[2] = l; return; }
  const float s = chroma / (1.0f - std::fabs(2.0f * l - 1.0f));
  float hue;
  if (mx == c[0]) hue = rem_euclid((c[1] - c[2]) / chroma, 6.0f) / 6.0f;
  else if (mx == c[1]) hue = ((c[2] - c[0]) / chroma + 2.0f) / 6.0f;
  else hue = ((c[0] - c[1]) / chroma + 4.0f) / 6.0f;
  out[0] = hue; out[1] = s; out[2] = l;
}
// stages.rs:869-886
void hsl_to_rgb(float h, float s, float l, float* out) {
  if (s <= F32_EPSILON) { out[0] = out[1] = out[2] = l; return; }
  const float chroma = (1.0f - std::fabs(2.0f * l - 1.0f)) * s;
  const float hp = h * 6.0f;
  const float sec = chroma * (1.0f - std::fabs(rem_euclid(hp, 2.0f) - 1.0f));
  float r, g, b;
  if (hp < 1.0f) { r = chroma; g = sec; b = 0.0f; }
  else if (hp < 2.0f) { r = sec; g = chroma; b = 0.0f; }
  else if (hp < 3.0f) { r = 0.0f; g = chroma; b = sec; }
  else if (hp < 4.0f) { r = 0.0f; g = sec; b = chroma; }
  else if (hp < 5.0f) { r = sec; g = 0.0f; b = chroma; }
  else { r = chroma; g = 0.0f; b = sec; }
  const float m = l - chroma * 0.5f;
  out[0] = r + m; out[1] = g + m; out[2] = b + m;
}
// stages.rs:758-784
void hsl_weights(float hue, float* w) {
  for (int k = 0; k < 8; ++k) w[k] = 0.0f;
  if (!std::isfinite(hue)) return;
  hue = rem_euclid(hue, 1.0f);
  int left = 7, right = 0;
  float start = HSL_CENTERS[7], end = 1.0f;
  for (int k = 0; k < 7; ++k)
    if (hue >= HSL_CENTERS[k] && hue < HSL_CENTERS[k + 1]) {
      left = k; right = k + 1; start = HSL_CENTERS[k]; end = HSL_CENTERS[k + 1];
      break;
    }
  const float fraction = rclamp((hue - start) / (end - start), 0.0f, 1.0f);
  w[left] = 1.0f - fraction;
  w[right] = fraction;
}
// stages.rs:703-749
void apply_hsl(float* p, const float (*hsl)[3]) {
  const float r = p[0], g = p[1], b = p[2];
  if (!std::isfinite(r) || !std::isfinite(g) || !std::isfinite(b)) return;
  const float offset = rmax(-rmin(rmin(r, g), b), 0.0f);
  const float sh[3] = {r + offset, g + offset, b + offset};
  if (!std::isfinite(sh[0]) || !std::isfinite(sh[1]) || !std::isfinite(sh[2])) return;
  float scale = 0.0f;
  for (float v : sh) scale = rmax(scale, v);
  if (!std::isfinite(scale) || scale <= F32_EPSILON) return;
  const float norm[3] = {sh[0] / scale, sh[1] / scale, sh[2] / scale};
  float hsl_v[3];
  rgb_to_hsl(norm, hsl_v);
  float hue = hsl_v[0], sat = hsl_v[1], light = hsl_v[2];
  const float cw = smoothstep(0.0f, 0.05f, sat);
  if (cw <= F32_EPSILON) return;
  float weights[8];
  hsl_weights(hue, weights);
  float hs = 0.0f, ss = 0.0f, ls = 0.0f;
  for (int k = 0; k < 8; ++k) {
    const float wgt = weights[k] * cw;
    hs += hsl[k][0] * HUE_SHIFT * wgt;
    ss += hsl[k][1] * 0.5f * wgt;
    ls += hsl[k][2] * 0.25f * wgt;
  }
  if (hs == 0.0f && ss == 0.0f && ls == 0.0f) return;
  hue = rem_euclid(hue + hs, 1.0f);
  sat = rclamp(sat + ss, 0.0f, 1.0f);
  light = rclamp(light + ls, 0.0f, 1.0f);
  float conv[3];
  hsl_to_rgb(hue, sat, light, conv);
  const float rest[3] = {conv[0] * scale - offset, conv[1] * scale - offset, conv[2] * scale - offset};
  if (std::isfinite(rest[0]) && std::isfinite(rest[1]) && std::isfinite(rest[2])) std::memcpy(p, rest, sizeof(rest));
}
// stages.rs:805-844
void apply_grading(float* p, const float (*gr)[3]) {
  const float value = rclamp(luminance(p), 0.0f, 1.0f);
  const float shadows = 1.0f - smoothstep(0.0f, 0.5f, value);
  const float mid = smoothstep(0.15f, 0.45f, value) * (1.0f - smoothstep(0.55f, 0.85f, value));
  const float hi = smoothstep(0.5f, 1.0f, value);
  float target[3];
  for (int i = 0; i < 3; ++i) {
    const float grade = gr[0][i] * shadows + gr[1][i] * mid + gr[2][i] * hi;
    target[i] = p[i] * (1.0f + 0.25f * grade);
  }
  if (!std::isfinite(target[0]) || !std::isfinite(target[1]) || !std::isfinite(target[2])) return;
  const float sl = luminance(p), tl = luminance(target);
  if (std::fabs(sl) > 1.0e-6f && std::isfinite(sl) && std::fabs(tl) > 1.0e-6f && std::isfinite(tl) &&
      signum(sl) == signum(tl)) {
    const float scale = sl / tl;
    const float gd[3] = {target[0] * scale, target[1] * scale, target[2] * scale};
    if (std::isfinite(gd[0]) && std::isfinite(gd[1]) && std::isfinite(gd[2])) std::memcpy(p, gd, sizeof(gd));
  } else {
    std::memcpy(p, target, sizeof(target));
  }
}
float color_saturation(const float* p, float lum) {
  float chroma = 0.0f;
  for (int c = 0; c < 3; ++c) chroma = rmax(chroma, std::fabs(p[c] - lum));
  return rclamp(chroma / rmax(std::fabs(lum), 1.0e-6f), 0.0f, 1.0f);
}
float srgb_encode(float v) { return v <= 0.0031308f ? 12.92f * v : 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f; }
float sanitize_clip(float v) {
  if (std::isnan(v) || v == -INFINITY) return 0.0f;
  if (v == INFINITY) return 1.0f;
  return rclamp(v, 0.0f, 1.0f);
}
}  // namespace

extern "C" void ro_white_balance(float* rgb, size_t pixels, const float g[3]) {
  for (size_t i = 0; i < pixels; ++i) {
    rgb[3 * i] *= g[0];
    rgb[3 * i + 1] *= g[1];
    rgb[3 * i + 2] *= g[2];
  }
}

extern "C" void ro_camera_matrix(float* rgb, size_t pixels, const float m[9]) {
  for (size_t i = 0; i < pixels; ++i) {
    float* p = rgb + 3 * i;
    const float v[3] = {p[0], p[1], p[2]};
    for (int r = 0; r < 3; ++r) p[r] = m[3 * r] * v[0] + m[3 * r + 1] * v[1] + m[3 * r + 2] * v[2];
  }
}

extern "C" void ro_standard_base_lut(float* lut) {
  const float anchor = std::pow(0.18f, 1.45f - 1.0f) * (1.0f - 0.18f);
  for (int i = 0; i < 4096; ++i) {
    if (i == 4095) { lut[i] = 1.0f; continue; }
    const float coordinate = (float)i / 4095.0f;
    const float input = coordinate / (1.0f - coordinate);
    if (input == 0.0f) { lut[i] = 0.0f; continue; }
    const float numerator = std::pow(input, 1.45f);
    lut[i] = numerator / (numerator + anchor);
  }
}

// LightToneLut::new (light.rs:27-47): evaluate_light_tone at index/4095 for
// every index, then the running-maximum projection.
namespace {
float lt_smoothstep(float edge0, float edge1, float value) {
  const float normalized = rclamp((value - edge0) / (edge1 - edge0), 0.0f, 1.0f);
  return normalized * normalized * (3.0f - 2.0f * normalized);
}
// bounded_move (light.rs:131-137)
float lt_move(float value, float amount, float weight) {
  if (amount >= 0.0f) return value + (1.0f - value) * amount * weight;
  return value + value * amount * weight;
}
// protected_contrast (light.rs:119-129), pivot 0.18
float lt_contrast(float input, float contrast) {
  if (contrast == 0.0f) return input;
  const float exponent = std::exp2(contrast);
  const float pivot = 0.18f;
  if (input <= pivot) return pivot * std::pow(input / pivot, exponent);
  return 1.0f - (1.0f - pivot) * std::pow((1.0f - input) / (1.0f - pivot), exponent);
}
// evaluate_light_tone (light.rs:90-117): strengths 0.45 shadows/highlights, 0.25 blacks/whites
float lt_evaluate(float input, float contrast, float highlights, float shadows, float whites, float blacks) {
  float output = lt_contrast(input, contrast);
  const float shadow_weight = lt_smoothstep(0.0f, 0.16f, input) * (1.0f - lt_smoothstep(0.38f, 0.68f, input));
  const float highlight_weight = lt_smoothstep(0.32f, 0.62f, input) * (1.0f - lt_smoothstep(0.84f, 1.0f, input));
  output = lt_move(output, shadows, 0.45f * shadow_weight);
  output = lt_move(output, highlights, 0.45f * highlight_weight);
  const float black_weight = 1.0f - lt_smoothstep(0.0f, 0.32f, input);
  const float white_weight = lt_smoothstep(0.68f, 1.0f, input);
  output = lt_move(output, blacks, 0.25f * black_weight);
  output = lt_move(output, whites, 0.25f * white_weight);
  return rclamp(output, 0.0f, 1.0f);
}
// apply_light_tone (stages.rs:631-645) with LightToneLut::sample / sample_extended (light.rs:49-64).
void apply_light_tone(float* p, const float* lut, bool extended) {
  const float current = luminance(p);
  const float target = (extended && std::isfinite(current) && current > 1.0f) ? current + lut[4095] - 1.0f
                                                                               : lut_sample(lut, current);
  if (!std::isfinite(target) || std::fabs(target - current) <= F32_EPSILON) return;
  apply_luminance_delta(p, current, target);
}
}  // namespace

extern "C" void ro_light_tone_lut(float contrast, float highlights, float shadows, float whites, float blacks,
                                  float* lut) {
  for (int index = 0; index < 4096; ++index)
    lut[index] = lt_evaluate((float)index / 4095.0f, contrast, highlights, shadows, whites, blacks);
  float previous = lut[0];
  for (int index = 1; index < 4096; ++index) {
    lut[index] = rmax(lut[index], previous);
    previous = lut[index];
  }
}

// apply_adjustments_with_local, stages.rs:380-528, for the global (no local mask) path.
extern "C" void ro_adjust_apply(float* rgb, size_t pixels, const ro_adjust* a) {
  const float gain = std::exp2(a->exposure_ev);
  const bool has_sat = std::fabs(a->saturation - 1.0f) > F32_EPSILON || a->vibrance != 0.0f;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < pixels; ++i) {
    float* p = rgb + 3 * i;
    if (a->exposure_ev != 0.0f)
      for (int c = 0; c < 3; ++c) p[c] *= gain;
    if (a->base_lut) apply_lut_tone(p, a->base_lut, true);
    if (a->light_lut) apply_light_tone(p, a->light_lut, a->extended != 0);
    if (a->tone_lut) apply_lut_tone(p, a->tone_lut, false);
    if (has_sat) {
      const float lum = luminance(p);
      const float sat = a->saturation * (1.0f + a->vibrance * (1.0f - color_saturation(p, lum)));
      if (std::fabs(sat - 1.0f) > F32_EPSILON)
        for (int c = 0; c < 3; ++c) p[c] = lum + sat * (p[c] - lum);
    }
    if (a->has_hsl) apply_hsl(p, a->hsl);
    if (a->has_grading) apply_grading(p, a->grading);
  }
}

extern "C" void ro_display_srgb8(const float* rgb, size_t pixels, uint8_t* out) {
  // Matrix3::then (matrix.rs:51-61): Iterator::sum starts at -0.0.
  float m[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      float s = -0.0f;
      for (int k = 0; k < 3; ++k) s += XYZ_TO_SRGB[r][k] * REC2020_TO_XYZ[k][c];
      m[r][c] = s;
    }
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < pixels; ++i) {
    const float* p = rgb + 3 * i;
    for (int r = 0; r < 3; ++r) {
      const float lin = m[r][0] * p[0] + m[r][1] * p[1] + m[r][2] * p[2];
      const float enc = srgb_encode(sanitize_clip(lin));
      out[3 * i + r] = (uint8_t)rclamp(std::round(enc * 255.0f + 0.0f), 0.0f, 255.0f);
    }
  }
}

extern "C" void ro_histogram(const uint8_t* rgb8, size_t pixels, uint64_t hist[4 * 256], uint64_t clipped[6]) {
  std::memset(hist, 0, sizeof(uint64_t) * 4 * 256);
  for (size_t i = 0; i < pixels; ++i) {
    const uint32_t r = rgb8[3 * i], g = rgb8[3 * i + 1], b = rgb8[3 * i + 2];
    hist[r]++;
    hist[256 + g]++;
    hist[512 + b]++;
    hist[768 + (2126 * r + 7152 * g + 722 * b + 5000) / 10000]++;
  }
  for (int c = 0; c < 3; ++c) {
    clipped[c] = hist[256 * c];
    clipped[3 + c] = hist[256 * c + 255];
  }
}
