// CPU restatement of the library's seeded synthetic Bayer scene generator
// (test and benchmark infrastructure).
//
// The reference has no scene generator of its own: its benches read files.
// The workloads here are seeded synthetic mosaics, and the CPU arm of the
// benchmark must develop the very same mosaic the GPU arm develops without
// loading the GPU library. This file restates the generator step by step
// from its description:
//   * counter-based draws: SplitMix64 of (seed xor SplitMix64(index * 0x100000001B3 + draw));
//   * uniforms (k + 1/2) / 2^23 from 23-bit fields of a draw;
//   * normal deviates as the Irwin-Hall sum of twelve uniforms minus 6;
//   * e^-x as 2^-trunc(x/ln2) times the 12-term Taylor series of e^-r (Horner);
//   * scene: per-channel gradients, 64 rectangles, 48 one-pixel lines, 48 or
//     96 Gaussian highlight blobs sized for the clip fraction;
//   * photon noise (Poisson at 0.5 e-/DN: normal approximation above 30 e-,
//     Knuth's product method below), read noise sigma 3 DN, hot pixels,
//     quantised as clamp(rint(black + DN), 0, white).
// Every step is an integer operation or an IEEE f32 +, -, *, / or sqrt,
// rounded on its own (built with -ffp-contract=off), so the result equals the
// device generator's bit for bit; a GPU test checks that.
#include <cmath>
#include <cstdint>
#include <vector>

#include "rd_oracle.h"

namespace {

uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
uint64_t bits_of(uint64_t seed, uint64_t index, unsigned draw) {
  return mix64(seed ^ mix64(index * 0x100000001B3ull + draw));
}
float unit(uint64_t field) { return ((float)(field & 0x7FFFFFull) + 0.5f) * 1.1920928955078125e-7f; }
float uniform_at(uint64_t seed, uint64_t index, unsigned draw) { return unit(bits_of(seed, index, draw) >> 41); }
float normal_at(uint64_t seed, uint64_t index, unsigned draw) {
  float sum = 0.0f;
  for (unsigned j = 0; j < 6; ++j) {
    const uint64_t h = bits_of(seed, index, draw + j);
    sum += unit(h >> 41);
    sum += unit(h >> 18);
  }
  return sum - 6.0f;
}
float exp_minus(float x) {
  const float ln2 = 0.693147182f;
  const int k = (int)(x / ln2);
  const float r = x - (float)k * ln2;
  float t = 1.0f;
  for (int n = 12; n >= 1; --n) t = 1.0f - r * t / (float)n;
  for (int i = 0; i < k; ++i) t *= 0.5f;
  return t;
}
int cfa_color(int pattern, int x, int y) {
  static const int colors[4][4] = {{0, 1, 1, 2}, {2, 1, 1, 0}, {1, 0, 2, 1}, {1, 2, 0, 1}};
  return colors[pattern][((y & 1) << 1) | (x & 1)];
}

struct Rect {
  float x0, y0, x1, y1, rgb[3];
};
struct Line {
  int vertical, pos;
  float rgb[3];
};
struct Blob {
  float x, y, inv2s2, amp;
};

}  // namespace

extern "C" int ro_synth_mosaic(const ro_synth* d, uint16_t* out) {
  if (d->width < 2 || d->height < 2) return -1;
  const int W = (int)d->width, H = (int)d->height;
  const float span = d->white - d->black;
  const uint64_t seed = d->seed;
  // Scene layout: draws 1000, 1001, ... at index 0xFFFFFFFF.
  unsigned draw = 1000;
  auto U = [&]() { return uniform_at(seed, 0xFFFFFFFFull, draw++); };
  std::vector<Rect> rects(64);
  for (Rect& r : rects) {
    const float w = (0.02f + 0.12f * U()) * W, h = (0.02f + 0.12f * U()) * H;
    r.x0 = std::floor(U() * (W - w));
    r.y0 = std::floor(U() * (H - h));
    r.x1 = r.x0 + std::floor(w);
    r.y1 = r.y0 + std::floor(h);
    for (int c = 0; c < 3; ++c) r.rgb[c] = 0.05f + 0.75f * U();
  }
  std::vector<Line> lines(48);
  for (size_t k = 0; k < lines.size(); ++k) {
    Line& l = lines[k];
    l.vertical = (int)(k & 1);
    l.pos = (int)(U() * (l.vertical ? W : H));
    for (int c = 0; c < 3; ++c) l.rgb[c] = 0.05f + 0.8f * U();
  }
  std::vector<Blob> blobs;
  if (d->clip_fraction > 0.0f) {
    const int n = d->highlight_blobs ? 48 : 96;
    const float amp = 3.0f;
    const float area_per = 1.6964493f * 3.14159265f;  // ln(3 / 0.55) * pi
    const float s2 = d->clip_fraction * (float)W * (float)H / (n * area_per);
    blobs.resize(n);
    for (Blob& b : blobs) {
      b.x = U() * W;
      b.y = U() * H;
      const float s2k = s2 * (0.5f + U());
      b.inv2s2 = 1.0f / s2k;
      b.amp = amp;
    }
  }
#pragma omp parallel for schedule(static)
  for (int y = 0; y < H; ++y) {
    for (int x = 0; x < W; ++x) {
      const int ch = cfa_color(d->cfa, x, y);
      const float u = (float)x / (float)W, v = (float)y / (float)H;
      float refl;
      if (ch == 0) refl = 0.18f + 0.35f * u * (1.0f - 0.4f * v);
      else if (ch == 1) refl = 0.22f + 0.30f * v + 0.10f * u * v;
      else refl = 0.15f + 0.30f * (1.0f - u) * (0.5f + 0.5f * v);
      for (const Rect& r : rects)
        if (x >= r.x0 && x < r.x1 && y >= r.y0 && y < r.y1) refl = r.rgb[ch];
      for (const Line& l : lines)
        if ((l.vertical && x == l.pos) || (!l.vertical && y == l.pos)) refl = l.rgb[ch];
      for (const Blob& b : blobs) {
        const float dx = (float)x - b.x, dy = (float)y - b.y;
        const float e = (dx * dx + dy * dy) * b.inv2s2;
        if (e < 12.0f) refl += b.amp * exp_minus(e);
      }
      const float signal = std::fmax(refl * d->gains[ch] * span, 0.0f);
      const uint64_t index = (uint64_t)y * W + x;
      const float mean = 0.5f * signal;
      float electrons;
      if (mean > 30.0f) {
        electrons = mean + std::sqrt(mean) * normal_at(seed, index, 0);
      } else {
        const float limit = exp_minus(mean);
        float prod = uniform_at(seed, index, 16);
        int k = 0;
        while (prod > limit && k < 200) {
          ++k;
          prod *= uniform_at(seed, index, 16 + k);
        }
        electrons = (float)k;
      }
      float dn = electrons / 0.5f + 3.0f * normal_at(seed, index, 8);
      if (d->hot_pixel_fraction > 0.0f && uniform_at(seed, index, 300) < d->hot_pixel_fraction) dn = span * 2.0f;
      float value = std::rint(d->black + dn);
      value = std::fmin(std::fmax(value, 0.0f), d->white);
      out[index] = (uint16_t)value;
    }
  }
  return 0;
}
