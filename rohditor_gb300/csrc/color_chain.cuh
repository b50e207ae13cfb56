// The global adjustment chain of the colour stage, shared by the preview
// render (k_color.cu) and the display / extended-range output (k_output.cu).
//
//  exposure, base rendering LUT, Light tone LUT, tone curve LUT, saturation /
//  vibrance, 8-band HSL and 3-way grading: crates/core/src/cpu/stages.rs:380-528
//  and helpers :605-901 (local masks are not part of this path); Light tone
//  sampling crates/edit/src/light.rs:49-88. Every operation is a
//  separately rounded f32 operation in the reference's order (the library is
//  compiled without FMA contraction).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr float F32_EPS = 1.1920929e-7f;
constexpr float TRANSITION = 0.02f;
__constant__ float HSL_CENTERS[8] = {0.0f, 30.0f / 360.0f, 60.0f / 360.0f, 120.0f / 360.0f,
                                     180.0f / 360.0f, 240.0f / 360.0f, 270.0f / 360.0f, 300.0f / 360.0f};

__device__ __forceinline__ float luminance(const float* p) {
  return p[0] * 0.2627f + p[1] * 0.6780f + p[2] * 0.0593f;
}
__device__ __forceinline__ float sstep(float e0, float e1, float v) {
  float n = (v - e0) / (e1 - e0);
  n = n < 0.0f ? 0.0f : (n > 1.0f ? 1.0f : n);
  return n * n * (3.0f - 2.0f * n);
}
// f32::rem_euclid. fmod(x, m) is x itself when |x| < |m| (the common case
// for hues), so fmodf runs only outside that range.
__device__ __forceinline__ float rem_euclid(float x, float m) {
  const float r = fabsf(x) < fabsf(m) ? x : fmodf(x, m);
  return r < 0.0f ? r + fabsf(m) : r;
}
__device__ __forceinline__ float rmax(float a, float b) {
  if (isnan(a)) return b;
  if (isnan(b)) return a;
  return a > b ? a : b;
}
__device__ __forceinline__ float rmin(float a, float b) {
  if (isnan(a)) return b;
  if (isnan(b)) return a;
  return a < b ? a : b;
}
__device__ __forceinline__ float rclamp(float v, float lo, float hi) {
  if (v < lo) v = lo;
  if (v > hi) v = hi;
  return v;
}
__device__ __forceinline__ float sgn(float v) { return signbit(v) ? -1.0f : 1.0f; }
__device__ __forceinline__ bool fin3(const float* p) { return isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]); }

__device__ __forceinline__ float base_sample(const float* __restrict__ values, float input) {
  if (!isfinite(input) || input <= 0.0f) return input;
  const float coordinate = input / (1.0f + input);
  const float position = coordinate * 4095.0f;
  unsigned lower = (unsigned)floorf(position);
  if (lower > 4095u) lower = 4095u;
  const unsigned upper = lower + 1 > 4095u ? 4095u : lower + 1;
  const float fraction = position - (float)lower;
  const float a = __ldg(values + lower);
  return a + (__ldg(values + upper) - a) * fraction;
}
__device__ __forceinline__ float lut_sample(const float* __restrict__ values, float input) {
  if (!(input >= 0.0f && input <= 1.0f)) return input;
  const float position = input * 4095.0f;
  const unsigned lower = (unsigned)floorf(position);
  const unsigned upper = lower + 1 > 4095u ? 4095u : lower + 1;
  const float fraction = position - (float)lower;
  const float a = __ldg(values + lower);
  return a + (__ldg(values + upper) - a) * fraction;
}

// stages.rs:657-701
__device__ void luminance_delta(float* p, float current, float target) {
  if (!isfinite(current) || !isfinite(target)) return;
  if ((current > 1.0e-6f && target >= TRANSITION) || (current < -1.0e-6f && target <= -TRANSITION)) {
    const float s = target / current;
    const float u[3] = {p[0] * s, p[1] * s, p[2] * s};
    if (fin3(u)) {
      p[0] = u[0]; p[1] = u[1]; p[2] = u[2];
      return;
    }
  }
  const float delta = target - current;
  if (!isfinite(delta)) return;
  const float add[3] = {p[0] + delta, p[1] + delta, p[2] + delta};
  if (!fin3(add)) return;
  if (fabsf(current) <= 1.0e-6f || sgn(current) != sgn(target)) {
    p[0] = add[0]; p[1] = add[1]; p[2] = add[2];
    return;
  }
  const float rw = sstep(0.0f, TRANSITION, fabsf(target));
  if (rw <= F32_EPS) {
    p[0] = add[0]; p[1] = add[1]; p[2] = add[2];
    return;
  }
  const float s = target / current;
  const float sc[3] = {p[0] * s, p[1] * s, p[2] * s};
  const float u[3] = {add[0] + (sc[0] - add[0]) * rw, add[1] + (sc[1] - add[1]) * rw, add[2] + (sc[2] - add[2]) * rw};
  if (fin3(u)) {
    p[0] = u[0]; p[1] = u[1]; p[2] = u[2];
  }
}

__device__ void rgb_to_hsl(const float* c, float* out) {
  const float mx = rmax(rmax(c[0], c[1]), c[2]);
  const float mn = rmin(rmin(c[0], c[1]), c[2]);
  const float l = (mx + mn) * 0.5f;
  const float chroma = mx - mn;
  if (chroma <= F32_EPS) { out[0] = 0.0f; out[1] = 0.0f; out[2] = l; return; }
  const float s = chroma / (1.0f - fabsf(2.0f * l - 1.0f));
  float hue;
  if (mx == c[0]) hue = rem_euclid((c[1] - c[2]) / chroma, 6.0f) / 6.0f;
  else if (mx == c[1]) hue = ((c[2] - c[0]) / chroma + 2.0f) / 6.0f;
  else hue = ((c[0] - c[1]) / chroma + 4.0f) / 6.0f;
  out[0] = hue; out[1] = s; out[2] = l;
}
__device__ void hsl_to_rgb(float h, float s, float l, float* out) {
  if (s <= F32_EPS) { out[0] = out[1] = out[2] = l; return; }
  const float chroma = (1.0f - fabsf(2.0f * l - 1.0f)) * s;
  const float hp = h * 6.0f;
  // rem_euclid(hp, 2): for hp in [0, 6) the remainder hp - 2k is exact
  // (Sterbenz), as fmodf's is.
  const float rem = (hp >= 0.0f && hp < 6.0f) ? (hp < 2.0f ? hp : (hp < 4.0f ? hp - 2.0f : hp - 4.0f))
                                              : rem_euclid(hp, 2.0f);
  const float sec = chroma * (1.0f - fabsf(rem - 1.0f));
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
// stages.rs:703-784
__device__ void apply_hsl(float* p, const float (*hsl)[3]) {
  const float r = p[0], g = p[1], b = p[2];
  if (!fin3(p)) return;
  const float offset = rmax(-rmin(rmin(r, g), b), 0.0f);
  const float sh[3] = {r + offset, g + offset, b + offset};
  if (!fin3(sh)) return;
  float scale = 0.0f;
  scale = rmax(scale, sh[0]);
  scale = rmax(scale, sh[1]);
  scale = rmax(scale, sh[2]);
  if (!isfinite(scale) || scale <= F32_EPS) return;
  const float norm[3] = {sh[0] / scale, sh[1] / scale, sh[2] / scale};
  float hv[3];
  rgb_to_hsl(norm, hv);
  float hue = hv[0], sat = hv[1], light = hv[2];
  const float cw = sstep(0.0f, 0.05f, sat);
  if (cw <= F32_EPS) return;
  // The two bands around the hue get weights 1 - f and f, every other band 0
  // (selected per band, so the weights stay in registers).
  int left = -1, right = -1;
  float fraction = 0.0f;
  if (isfinite(hue)) {
    const float hh = rem_euclid(hue, 1.0f);
    left = 7;
    right = 0;
    float start = HSL_CENTERS[7], end = 1.0f;
    for (int k = 0; k < 7; ++k)
      if (hh >= HSL_CENTERS[k] && hh < HSL_CENTERS[k + 1]) {
        left = k; right = k + 1; start = HSL_CENTERS[k]; end = HSL_CENTERS[k + 1];
        break;
      }
    fraction = rclamp((hh - start) / (end - start), 0.0f, 1.0f);
  }
  float hs = 0.0f, ss = 0.0f, ls = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const float wk = k == left ? 1.0f - fraction : (k == right ? fraction : 0.0f);
    const float wt = wk * cw;
    hs += hsl[k][0] * 0.125f * wt;
    ss += hsl[k][1] * 0.5f * wt;
    ls += hsl[k][2] * 0.25f * wt;
  }
  if (hs == 0.0f && ss == 0.0f && ls == 0.0f) return;
  hue = rem_euclid(hue + hs, 1.0f);
  sat = rclamp(sat + ss, 0.0f, 1.0f);
  light = rclamp(light + ls, 0.0f, 1.0f);
  float conv[3];
  hsl_to_rgb(hue, sat, light, conv);
  const float rest[3] = {conv[0] * scale - offset, conv[1] * scale - offset, conv[2] * scale - offset};
  if (fin3(rest)) {
    p[0] = rest[0]; p[1] = rest[1]; p[2] = rest[2];
  }
}
// stages.rs:805-844
__device__ void apply_grading(float* p, const float (*gr)[3]) {
  const float value = rclamp(luminance(p), 0.0f, 1.0f);
  const float shadows = 1.0f - sstep(0.0f, 0.5f, value);
  const float mid = sstep(0.15f, 0.45f, value) * (1.0f - sstep(0.55f, 0.85f, value));
  const float hi = sstep(0.5f, 1.0f, value);
  float target[3];
  for (int i = 0; i < 3; ++i) {
    const float grade = gr[0][i] * shadows + gr[1][i] * mid + gr[2][i] * hi;
    target[i] = p[i] * (1.0f + 0.25f * grade);
  }
  if (!fin3(target)) return;
  const float sl = luminance(p), tl = luminance(target);
  if (fabsf(sl) > 1.0e-6f && isfinite(sl) && fabsf(tl) > 1.0e-6f && isfinite(tl) && sgn(sl) == sgn(tl)) {
    const float s = sl / tl;
    const float gd[3] = {target[0] * s, target[1] * s, target[2] * s};
    if (fin3(gd)) {
      p[0] = gd[0]; p[1] = gd[1]; p[2] = gd[2];
    }
  } else {
    p[0] = target[0]; p[1] = target[1]; p[2] = target[2];
  }
}

// Parameters of the adjustment chain; LUT pointers are device addresses.
struct AdjustParams {
  float exposure_gain;
  int has_exposure;
  int extended;               // 1: extended-range rendition (Light tone continues above 1)
  const float* base_lut;
  const float* light_lut;
  const float* tone_lut;
  int has_sat;
  float saturation, vibrance;
  int has_hsl;
  float hsl[8][3];
  int has_grading;
  float grading[3][3];
};

// apply_adjustments_with_local for the global path (stages.rs:380-528): the
// working pixel is linear Rec.2020.
__device__ __forceinline__ void apply_adjustments(const AdjustParams& a, float* v) {
  if (a.has_exposure) {
    v[0] *= a.exposure_gain;
    v[1] *= a.exposure_gain;
    v[2] *= a.exposure_gain;
  }
  if (a.base_lut) {
    const float cur = luminance(v);
    const float tgt = base_sample(a.base_lut, cur);
    if (isfinite(tgt) && fabsf(tgt - cur) > F32_EPS) luminance_delta(v, cur, tgt);
  }
  if (a.light_lut) {
    // apply_light_tone (stages.rs:631-645): LightToneLut::sample, or
    // sample_extended (light.rs:59-64) for an extended rendition, where a
    // finite luminance above 1 continues from the table's last value with
    // unit slope.
    const float cur = luminance(v);
    const float tgt = (a.extended && isfinite(cur) && cur > 1.0f) ? (cur + __ldg(a.light_lut + 4095)) - 1.0f
                                                                  : lut_sample(a.light_lut, cur);
    if (isfinite(tgt) && fabsf(tgt - cur) > F32_EPS) luminance_delta(v, cur, tgt);
  }
  if (a.tone_lut) {
    const float cur = luminance(v);
    const float tgt = lut_sample(a.tone_lut, cur);
    if (isfinite(tgt) && fabsf(tgt - cur) > F32_EPS) luminance_delta(v, cur, tgt);
  }
  if (a.has_sat) {
    const float lum = luminance(v);
    float chroma = 0.0f;
    for (int c = 0; c < 3; ++c) chroma = rmax(chroma, fabsf(v[c] - lum));
    const float cs = rclamp(chroma / rmax(fabsf(lum), 1.0e-6f), 0.0f, 1.0f);
    const float sat = a.saturation * (1.0f + a.vibrance * (1.0f - cs));
    if (fabsf(sat - 1.0f) > F32_EPS)
      for (int c = 0; c < 3; ++c) v[c] = lum + sat * (v[c] - lum);
  }
  if (a.has_hsl) apply_hsl(v, a.hsl);
  if (a.has_grading) apply_grading(v, a.grading);
}

// ---- float-float arithmetic (error-free transformations) -------------------
// A pair (hi, lo) stands for hi + lo with |lo| <= ulp(hi) / 2. two_prod is
// exact (Dekker / FMA); the products below lose at most a few units of 2^-48
// relative. The library is compiled without FMA contraction, so every fmaf
// here is explicit and every other product is rounded on its own.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF two_prod(float a, float b) {
  const float p = a * b;
  return FF{p, fmaf(a, b, -p)};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {
  const float s = a + b;
  return FF{s, b - (s - a)};
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const FF p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
  const FF p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, p.lo + a.lo * b);
}
__device__ __forceinline__ float next_up(float r) { return __int_as_float(__float_as_int(r) + 1); }
__device__ __forceinline__ float next_down(float r) { return __int_as_float(__float_as_int(r) - 1); }

// ---- correctly rounded sRGB transfer power -----------------------------------
// Largest distance, in ulps, of powf(x, 1/2.4) from the correctly rounded
// power over the transfer's domain (0.0031308, 1]; the exhaustive device check
// of the library (rd_check_math) asserts it.
constexpr int TRANSFER_POW_ULPS = 1;

// Which side of m = r + h does x^e lie on, e = 1/2.4 rounded to f32?
// e = 5/12 - 2^-23/12 exactly, so x^e > m  <=>  x^5 > m^12 * x^(2^-23), and
// x^(2^-23) = 1 + w + w^2/2 + O(w^3) with w = 2^-23 ln x, |w| < 7e-7. Both
// sides are formed in float-float; their relative error stays below 2^-41, so
// a difference above 2^-38 decides. Returns +1 (above), -1 (below) or 0 (too
// close to call: the true power is within about 2^-41 of the midpoint).
__device__ __forceinline__ int transfer_side(float x, float r, float h) {
  const FF x2 = two_prod(x, x);
  const FF q = ff_mul_f(ff_mul(x2, x2), x);
  const FF m{r, h};
  const FF m2 = ff_mul(m, m);
  const FF m4 = ff_mul(m2, m2);
  const FF m12 = ff_mul(ff_mul(m4, m4), m4);
  const float w = logf(x) * 1.1920928955078125e-7f;  // exact scaling by 2^-23
  const float c = w + 0.5f * w * w;
  const FF p = fast_two_sum(m12.hi, m12.lo + m12.hi * c);
  const float d = (q.hi - p.hi) + (q.lo - p.lo);  // q.hi - p.hi is exact (Sterbenz)
  const float eps = q.hi * 3.637978807091713e-12f;  // 2^-38
  return d > eps ? 1 : (d < -eps ? -1 : 0);
}

// x^e for x in (0.0031308, 1] correctly rounded to f32: powf, moved by one ulp
// where the exact midpoint test says so, in double where it cannot tell.
__device__ __forceinline__ float transfer_pow_rn(float x) {
  const float e = 1.0f / 2.4f;
  const float r = powf(x, e);
  const float up = next_up(r), down = next_down(r);
  const int above = transfer_side(x, r, (up - r) * 0.5f);
  if (above > 0) return up;
  if (above == 0) return (float)pow((double)x, (double)e);
  const int below = transfer_side(x, r, (down - r) * 0.5f);
  if (below < 0) return down;
  if (below == 0) return (float)pow((double)x, (double)e);
  return r;
}

__device__ __forceinline__ float transfer_code(float r, float scale, float dither) {
  return roundf((1.055f * r - 0.055f) * scale + dither);
}

// linear_srgb_to_srgb (crates/color/src/transfer.rs:5-11) followed by the
// quantisation (encoded * scale + dither).round().clamp(0, scale) of
// stages.rs:1085-1087 and :1181-1183, for the three channels of a pixel
// already in [0, 1], with the power correctly rounded.
//
// The code is a monotone function of the power r, and powf is within one ulp
// of the correctly rounded power. When the codes of powf's result one ulp
// down and one ulp up agree, that is the code. Otherwise one boundary lies
// between them, and the side of the midpoint on that boundary's side decides
// between two codes (transfer_side, double only when it cannot tell). The
// pixel's undecided channels are resolved in one loop, so a warp pays the
// decision once per pixel, not once per channel.
__device__ __forceinline__ void quantize_srgb3(const float* lin, float scale, float dither, float* code) {
  const float e = 1.0f / 2.4f;
  float r[3];
  unsigned undecided = 0, upward = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (lin[c] <= 0.0031308f) {
      code[c] = roundf(12.92f * lin[c] * scale + dither);
      r[c] = 0.0f;
    } else {
      r[c] = powf(lin[c], e);
      const float q = (1.055f * r[c] - 0.055f) * scale + dither;
      code[c] = roundf(q);
      // One ulp of r moves q by at most 1.055 * scale * 2^-23 plus the
      // rounding of the three operations, under scale * 4e-7 together; only a
      // q within twice that of a rounding boundary can change code.
      if (fabsf((q - floorf(q)) - 0.5f) < scale * 7.5e-7f) {
        const float lo = transfer_code(next_down(r[c]), scale, dither);
        const float hi = transfer_code(next_up(r[c]), scale, dither);
        if (lo != hi) {
          undecided |= 1u << c;
          if (code[c] == lo) upward |= 1u << c;  // the boundary is above r
        }
      }
    }
  }
  while (undecided) {
    const int c = __ffs(undecided) - 1;
    undecided &= undecided - 1;
    const float x = c == 0 ? lin[0] : (c == 1 ? lin[1] : lin[2]);
    const float rc = c == 0 ? r[0] : (c == 1 ? r[1] : r[2]);
    const bool up = (upward >> c) & 1u;
    const float nb = up ? next_up(rc) : next_down(rc);
    const int side = transfer_side(x, rc, (nb - rc) * 0.5f);
    float rr = rc;
    if (side == 0) rr = (float)pow((double)x, (double)e);
    else if (up ? side > 0 : side < 0) rr = nb;
    const float q = transfer_code(rr, scale, dither);
    if (c == 0) code[0] = q;
    else if (c == 1) code[1] = q;
    else code[2] = q;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) code[c] = rclamp(code[c], 0.0f, scale);
}

// The LUTs of one colour description are staged together on the device:
// base rendering at [0, 4096), Light tone at [4096, 8192), tone curve at
// [8192, 12288).
constexpr int LUT_ENTRIES = 4096;
constexpr int LUT_SET_ENTRIES = 3 * LUT_ENTRIES;
constexpr size_t LUT_SET_BYTES = sizeof(float) * LUT_SET_ENTRIES;

inline bool has_any_lut(const rd_color_desc& c) { return c.has_base_lut || c.has_light_tone_lut || c.has_tone_lut; }

// Copies the description's LUTs into a host staging set laid out as above.
inline void stage_luts(const rd_color_desc& c, float* host_set) {
  if (c.has_base_lut) std::memcpy(host_set, c.base_lut, sizeof(float) * LUT_ENTRIES);
  if (c.has_light_tone_lut) std::memcpy(host_set + LUT_ENTRIES, c.light_tone_lut, sizeof(float) * LUT_ENTRIES);
  if (c.has_tone_lut) std::memcpy(host_set + 2 * LUT_ENTRIES, c.tone_lut, sizeof(float) * LUT_ENTRIES);
}

// Points the chain at a device LUT set laid out as above (null for an absent LUT).
inline void set_lut_pointers(AdjustParams& a, const rd_color_desc& c, const float* device_set) {
  a.base_lut = c.has_base_lut ? device_set : nullptr;
  a.light_lut = c.has_light_tone_lut ? device_set + LUT_ENTRIES : nullptr;
  a.tone_lut = c.has_tone_lut ? device_set + 2 * LUT_ENTRIES : nullptr;
}

// Scalar adjustment parameters of a colour description; the caller stages the
// LUTs and sets their device addresses.
inline AdjustParams adjust_params(const rd_color_desc& c) {
  AdjustParams a{};
  a.has_exposure = c.exposure_ev != 0.0f;
  a.exposure_gain = std::exp2(c.exposure_ev);
  a.has_sat = std::fabs(c.saturation - 1.0f) > F32_EPS || c.vibrance != 0.0f;
  a.saturation = c.saturation;
  a.vibrance = c.vibrance;
  a.has_hsl = c.has_hsl;
  for (int k = 0; k < 8; ++k)
    for (int j = 0; j < 3; ++j) a.hsl[k][j] = c.hsl[k][j];
  a.has_grading = c.has_grading;
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j) a.grading[k][j] = c.grading[k][j];
  return a;
}

// LINEAR_REC2020_TO_XYZ_D65.then(to_display) (display_output.rs:27-34,
// matrix.rs:51-61): Iterator::sum starts at -0.0.
inline void rec2020_to_display(const float to_display[3][3], float out[9]) {
  const float A[3][3] = {{0.63695806f, 0.1446169f, 0.16888097f},
                         {0.2627002f, 0.67799807f, 0.059301715f},
                         {0.0f, 0.028072694f, 1.0609851f}};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      float s = -0.0f;
      for (int k = 0; k < 3; ++k) s += to_display[r][k] * A[k][c];
      out[3 * r + c] = s;
    }
}
// XYZ_D65_TO_LINEAR_SRGB and XYZ_D65_TO_LINEAR_DISPLAY_P3 (matrix.rs:110-128).
constexpr float XYZ_TO_SRGB[3][3] = {{3.24097f, -1.5373832f, -0.49861076f},
                                     {-0.96924365f, 1.8759675f, 0.04155506f},
                                     {0.05563008f, -0.20397696f, 1.0569715f}};
constexpr float XYZ_TO_DISPLAY_P3[3][3] = {{2.493497f, -0.9313836f, -0.4027108f},
                                           {-0.829489f, 1.7626641f, 0.0236247f},
                                           {0.0358458f, -0.0761724f, 0.9568845f}};

}  // namespace
}  // namespace rd
