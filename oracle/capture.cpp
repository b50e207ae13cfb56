// CPU oracle: masked Richardson-Lucy capture sharpening, restated from
// crates/core/src/sharpening.rs:87-389 and the Gaussian kernel of
// crates/detail/src/gaussian.rs:9-17. The reference fixes the iteration count
// at CAPTURE_SHARPENING_ITERATIONS = 8 (sharpening.rs:13); here it is a
// parameter so 10- and 20-iteration workloads can be checked too.
// Test infrastructure only (see oracle_common.h).
#include <algorithm>
#include <cmath>
#include <vector>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

namespace {
constexpr float FLOOR = 1.0e-6f;

float smoothstep(float low, float high, float value) {
  const float t = rclamp((value - low) / (high - low), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

// sharpening.rs:318-326: reflect about the outer pixel boundary.
std::size_t mirror_half(long index, std::size_t length) {
  const long period = (long)length * 2;
  long folded = index % period;
  if (folded < 0) folded += period;
  return folded < (long)length ? (std::size_t)folded : (std::size_t)(2 * (long)length - 1 - folded);
}

// sharpening.rs:328-389
void blur(const std::vector<float>& input, std::vector<float>& temp, std::vector<float>& output, int width,
          int height, const std::vector<float>& kernel) {
  const int r = (int)kernel.size() / 2;
  const int taps = (int)kernel.size();
#pragma omp parallel for schedule(static)
  for (int y = 0; y < height; ++y) {
    float* row = temp.data() + (std::size_t)y * width;
    const float* in = input.data() + (std::size_t)y * width;
    for (int x = 0; x < width; ++x) row[x] = 0.0f;
    if (width > 2 * r) {
      for (int k = 0; k < taps; ++k)
        for (int x = r; x < width - r; ++x) row[x] += in[x - r + k] * kernel[k];
    }
    for (int x = 0; x < width; ++x) {
      if (width <= 2 * r || x < r || x >= width - r) {
        float sum = -0.0f;  // Iterator::sum for f32 starts at -0.0
        for (int k = 0; k < taps; ++k) sum += in[mirror_half((long)x + k - r, width)] * kernel[k];
        row[x] = sum;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int y = 0; y < height; ++y) {
    float* row = output.data() + (std::size_t)y * width;
    for (int x = 0; x < width; ++x) row[x] = 0.0f;
    for (int k = 0; k < taps; ++k) {
      const float* src = temp.data() + mirror_half((long)y + k - r, height) * (std::size_t)width;
      for (int x = 0; x < width; ++x) row[x] += src[x] * kernel[k];
    }
  }
}
}  // namespace

extern "C" int ro_gaussian_kernel(float sigma, float* weights, int max_taps) {
  const int radius = (int)std::ceil(3.0f * sigma);
  const int taps = 2 * radius + 1;
  if (taps > max_taps) return -1;
  float sum = -0.0f;
  for (int i = 0; i < taps; ++i) {
    const float t = (float)(i - radius) / sigma;
    weights[i] = std::exp(-0.5f * (t * t));
    sum += weights[i];
  }
  for (int i = 0; i < taps; ++i) weights[i] /= sum;
  return taps;
}

extern "C" int ro_capture_sharpen(float* rgb, int w, int h, float amount, float radius, float noise,
                                  const float ceilings[3], int iterations) {
  if (!(amount > 0.0f)) return 0;
  float kbuf[64];
  const int taps = ro_gaussian_kernel(radius, kbuf, 64);
  if (taps < 0) return -1;
  const std::vector<float> kernel(kbuf, kbuf + taps);
  const std::size_t n = (std::size_t)w * h;
  std::vector<float> guide(n), mask(n), temp(n), blurred(n), ratio(n);
  for (std::size_t i = 0; i < n; ++i) {
    const float* p = rgb + 3 * i;
    if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2])) return -2;
    float g = -0.0f;
    for (int c = 0; c < 3; ++c) g += rmax(p[c], 0.0f) / 3.0f;
    guide[i] = rmax(g, FLOOR);
    float peak = 0.0f;
    for (int c = 0; c < 3; ++c) peak = rmax(peak, p[c] / ceilings[c]);
    mask[i] = 1.0f - smoothstep(0.85f, 0.98f, peak);
  }
  std::vector<float> estimate = guide;
  blur(mask, temp, blurred, w, h, kernel);
  for (std::size_t i = 0; i < n; ++i) {
    const float b2 = blurred[i] * blurred[i];
    mask[i] = rmin(mask[i], b2 * b2);
  }
  blur(guide, temp, blurred, w, h, kernel);
  for (std::size_t i = 0; i < n; ++i) {
    const float threshold = 0.0005f + noise * 0.008f + blurred[i] * noise * 0.02f;
    const float detail = std::fabs(guide[i] - blurred[i]);
    mask[i] *= smoothstep(threshold, threshold * 3.0f, detail) * smoothstep(0.001f, 0.01f, guide[i]);
  }
  for (int it = 0; it < iterations; ++it) {
    blur(estimate, temp, blurred, w, h, kernel);
    for (std::size_t i = 0; i < n; ++i) ratio[i] = guide[i] / rmax(blurred[i], FLOOR);
    blur(ratio, temp, blurred, w, h, kernel);
    for (std::size_t i = 0; i < n; ++i)
      estimate[i] = rclamp(estimate[i] * blurred[i], guide[i] * 0.5f, guide[i] * 2.0f);
  }
  for (std::size_t i = 0; i < n; ++i) {
    const float gain = 1.0f + amount * mask[i] * (estimate[i] / guide[i] - 1.0f);
    float* p = rgb + 3 * i;
    if (gain != 1.0f && std::isfinite(p[0] * gain) && std::isfinite(p[1] * gain) && std::isfinite(p[2] * gain)) {
      p[0] *= gain;
      p[1] *= gain;
      p[2] *= gain;
    }
  }
  return 0;
}
