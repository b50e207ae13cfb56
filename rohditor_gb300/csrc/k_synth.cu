// Seeded synthetic Bayer scenes for tests and benchmarks.
//
// A counter-based generator (SplitMix64 keyed by seed, pixel index and draw
// number) makes every sample a pure function of its coordinates, so a mosaic
// of any size is produced in one parallel pass and is identical run to run.
// The per-pixel arithmetic uses no library function whose last bit differs
// between host and device, so a host build of the same steps (the CPU oracle
// has one) reproduces the mosaic bit for bit.
// Scene: smooth colour gradients, random sharp-edged rectangles and 1-pixel
// lines, optional Gaussian highlight blobs whose cores clip, then photon
// (Poisson, 0.5 e-/DN) and Gaussian read noise (sigma 3 DN), quantised to u16
// as clamp(black + DN, 0, white).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr int MAX_RECTS = 64, MAX_LINES = 48, MAX_BLOBS = 128;

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

struct SynthParams {
  int W, H, cfa;
  float black, white, span;   // span = white - black (DN at reflectance 1)
  float gains[3];
  unsigned long long seed;
  int nrects, nlines, nblobs;
  Rect rects[MAX_RECTS];
  Line lines[MAX_LINES];
  Blob blobs[MAX_BLOBS];
  float hot_fraction;
};

__host__ __device__ inline unsigned long long splitmix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__host__ __device__ inline unsigned long long draw_bits(unsigned long long seed, unsigned long long index,
                                                        unsigned draw) {
  return splitmix(seed ^ splitmix(index * 0x100000001B3ull + draw));
}
// Every value below is built from integer operations and IEEE f32 +, -, *, /
// and sqrt, each rounded on its own (no contraction on either side), so the
// host and the device give the same bits.
//
// A uniform in (0, 1) from 23 bits of a draw: (k + 1/2) / 2^23, exact.
__host__ __device__ inline float unit_from(unsigned long long bits) {
  return ((float)(bits & 0x7FFFFFull) + 0.5f) * 1.1920928955078125e-7f;
}
__host__ __device__ inline float uniform(unsigned long long seed, unsigned long long index, unsigned draw) {
  return unit_from(draw_bits(seed, index, draw) >> 41);
}
// A standard normal deviate as the Irwin-Hall sum of twelve uniforms minus 6
// (mean 0, variance 1, support [-6, 6]); two uniforms per draw, from bits
// 41..63 and 18..40.
__host__ __device__ inline float normal(unsigned long long seed, unsigned long long index, unsigned draw) {
  float sum = 0.0f;
  for (unsigned j = 0; j < 6; ++j) {
    const unsigned long long h = draw_bits(seed, index, draw + j);
    sum += unit_from(h >> 41);
    sum += unit_from(h >> 18);
  }
  return sum - 6.0f;
}
// e^-x for 0 <= x < 80: x = k ln2 + r with k = trunc(x / ln2), then
// 2^-k (exact halvings) times the Taylor series of e^-r to the r^12 term,
// evaluated by Horner's rule.
__host__ __device__ inline float exp_neg(float x) {
  const float ln2 = 0.693147182f;
  const int k = (int)(x / ln2);
  const float r = x - (float)k * ln2;
  float t = 1.0f;
  for (int n = 12; n >= 1; --n) t = 1.0f - r * t / (float)n;
  for (int i = 0; i < k; ++i) t *= 0.5f;
  return t;
}

// Draw numbers of one pixel: photon noise 0..5 (normal) or 16.. (Poisson
// products), read noise 8..13, hot pixel 300.
__global__ void synth_kernel(const SynthParams* __restrict__ pp, uint16_t* __restrict__ out) {
  const SynthParams& p = *pp;
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= p.W) return;
  const int ch = color_at(p.cfa, x, y);
  const float u = (float)x / (float)p.W, v = (float)y / (float)p.H;
  // Smooth gradients (reflectance), different per channel.
  float refl;
  if (ch == 0) refl = 0.18f + 0.35f * u * (1.0f - 0.4f * v);
  else if (ch == 1) refl = 0.22f + 0.30f * v + 0.10f * u * v;
  else refl = 0.15f + 0.30f * (1.0f - u) * (0.5f + 0.5f * v);
  for (int k = 0; k < p.nrects; ++k) {
    const Rect& r = p.rects[k];
    if (x >= r.x0 && x < r.x1 && y >= r.y0 && y < r.y1) refl = r.rgb[ch];
  }
  for (int k = 0; k < p.nlines; ++k) {
    const Line& l = p.lines[k];
    if ((l.vertical && x == l.pos) || (!l.vertical && y == l.pos)) refl = l.rgb[ch];
  }
  for (int k = 0; k < p.nblobs; ++k) {
    const Blob& b = p.blobs[k];
    const float dx = (float)x - b.x, dy = (float)y - b.y;
    const float d2 = dx * dx + dy * dy;
    const float e = d2 * b.inv2s2;
    if (e < 12.0f) refl += b.amp * exp_neg(e);
  }
  // Camera response of this channel, in DN above black.
  const float signal = fmaxf(refl * p.gains[ch] * p.span, 0.0f);
  const unsigned long long index = (unsigned long long)y * p.W + x;
  // Shot noise: electrons = 0.5 * DN ~ Poisson, normal approximation above 30 e-.
  const float electrons_mean = 0.5f * signal;
  float electrons;
  if (electrons_mean > 30.0f) {
    electrons = electrons_mean + sqrtf(electrons_mean) * normal(p.seed, index, 0);
  } else {
    // Knuth's product method for small means.
    const float limit = exp_neg(electrons_mean);
    float prod = uniform(p.seed, index, 16);
    int k = 0;
    while (prod > limit && k < 200) {
      ++k;
      prod *= uniform(p.seed, index, 16 + k);
    }
    electrons = (float)k;
  }
  float dn = electrons / 0.5f + 3.0f * normal(p.seed, index, 8);
  if (p.hot_fraction > 0.0f && uniform(p.seed, index, 300) < p.hot_fraction) dn = p.span * 2.0f;
  float value = rintf(p.black + dn);
  value = fminf(fmaxf(value, 0.0f), p.white);
  out[index] = (uint16_t)value;
}

}  // namespace

Status run_synth(Context& ctx, const rd_synth_desc& d, uint16_t* out) {
  if (d.width < 2 || d.height < 2) return Status{RD_INVALID_DIMENSIONS, "synthetic mosaic must be at least 2x2"};
  SynthParams p{};
  p.W = (int)d.width;
  p.H = (int)d.height;
  p.cfa = d.cfa;
  p.black = d.black;
  p.white = d.white;
  p.span = d.white - d.black;
  for (int c = 0; c < 3; ++c) p.gains[c] = d.gains[c];
  p.seed = d.seed;
  p.hot_fraction = d.hot_pixel_fraction;
  // Scene layout from host draws of the same generator.
  unsigned draw = 1000;
  auto U = [&]() { return uniform(d.seed, 0xFFFFFFFFull, draw++); };
  p.nrects = MAX_RECTS;
  for (int k = 0; k < p.nrects; ++k) {
    Rect& r = p.rects[k];
    const float w = (0.02f + 0.12f * U()) * p.W, h = (0.02f + 0.12f * U()) * p.H;
    r.x0 = std::floor(U() * (p.W - w));
    r.y0 = std::floor(U() * (p.H - h));
    r.x1 = r.x0 + std::floor(w);
    r.y1 = r.y0 + std::floor(h);
    for (int c = 0; c < 3; ++c) r.rgb[c] = 0.05f + 0.75f * U();
  }
  p.nlines = MAX_LINES;
  for (int k = 0; k < p.nlines; ++k) {
    Line& l = p.lines[k];
    l.vertical = k & 1;
    l.pos = (int)(U() * (l.vertical ? p.W : p.H));
    for (int c = 0; c < 3; ++c) l.rgb[c] = 0.05f + 0.8f * U();
  }
  // Highlight blobs: the clipped core of a blob of amplitude A and width s is a
  // disc of radius s*sqrt(ln(A/(1-b))) where b ~ 0.45 is the local scene level,
  // so N blobs of radius s clip about N*pi*s^2*ln(A/0.55) pixels.
  if (d.clip_fraction > 0.0f) {
    const int n = d.highlight_blobs ? 48 : 96;
    const float amp = 3.0f;
    const float area_per = 1.6964493f * 3.14159265f;  // ln(3 / 0.55) * pi
    const float s2 = d.clip_fraction * (float)p.W * (float)p.H / (n * area_per);
    p.nblobs = n;
    for (int k = 0; k < n; ++k) {
      Blob& b = p.blobs[k];
      b.x = U() * p.W;
      b.y = U() * p.H;
      const float s2k = s2 * (0.5f + U());  // varied sizes, same mean area
      b.inv2s2 = 1.0f / s2k;
      b.amp = amp;
    }
  }
  void* dp = nullptr;
  RD_TRY(device_alloc(ctx, sizeof(SynthParams), &dp));
  RD_CUDA_TRY(cudaMemcpyAsync(dp, &p, sizeof(SynthParams), cudaMemcpyHostToDevice, ctx.stream));
  dim3 grid((p.W + 255) / 256, p.H);
  RD_LAUNCH(ctx, K_SYNTH, synth_kernel<<<grid, 256, 0, ctx.stream>>>(static_cast<const SynthParams*>(dp), out));
  const cudaError_t launch = cudaGetLastError();
  device_free(ctx, dp, sizeof(SynthParams));
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

}  // namespace rd
