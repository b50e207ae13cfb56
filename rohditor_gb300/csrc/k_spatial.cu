// Lens distortion / TCA gather (crates/optics/src/{plan,resample}.rs) and
// exact separable area reduction (crates/core/src/resample.rs) on sm_103a.
//
// Optics: the per-column and per-row halves of the pre-transform
// (plan.rs:448-455 and correction.rs input_coordinate_x/y) are resolved on the
// host in f64 and uploaded as f32 tables, so a pixel starts from two loads.
// The inverse distortion runs the lensfun Newton iteration in f64 from the f32
// coordinates (radius sqrt(f64(x*x + y*y)), <= 7 steps, |F| < 1e-5, input kept
// on non-convergence; Poly3 returns NaN), TCA is applied in f32 and the
// post-transform back to pixels is f64 narrowed once, as in
// plan.rs:466-483. Each channel is a 4x4 Catmull-Rom gather with the
// reference's tap order (resample.rs:21-33); a footprint outside [1, W-2]
// sets the error word, which the host turns into RD_INVALID_INPUT.
//
// Area reduction: the host builds the overlap tables exactly as
// AreaReductionAxis::new (f64 overlaps narrowed to f32); the horizontal and
// vertical passes accumulate taps in table order from 0, as the reference.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "lens_model.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

struct FastOptics {
  float cxh, cxl, cyh, cyl, uh, ul;  // f64 constants split into FP32 pairs
};

struct OpticsParams {
  const float* in;   // planar RGB
  const float* mult; // vignetting multipliers, or null
  float* out;
  int W, H;
  const float* ix;   // per-column input x (f32, lens units)
  const float* iy;   // per-row input y
  double cx, cy, unscale;
  int dist_model;
  float d0, d1, d2;
  int tca_model;
  float tr[3], tb[3];
  unsigned* error;
  FastOptics fast;
};

__device__ __forceinline__ void undistort(const OpticsParams& p, float x, float y, float& ox, float& oy) {
  lens_undistort(p.dist_model, p.d0, p.d1, p.d2, x, y, ox, oy);
}

__device__ __forceinline__ void tca_poly3(const float* ch, float x, float y, float& ox, float& oy) {
  lens_tca_poly3(ch, x, y, ox, oy);
}

// ---- exact FP32 fast path -------------------------------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, so the per-pixel f64
// arithmetic of the reference (lensfun's Newton inversion, the f64 pixel
// transform) is evaluated in double-float FP32 arithmetic (~44-bit accuracy).
// The f64 result is then rounded to f32 exactly as the reference does; when
// the double-float value lies so close to an f32 rounding midpoint (or to the
// Newton break threshold) that the two could disagree, the pixel takes the
// f64 path instead. The output is therefore the f64 path's, bit for bit.
struct df {
  float h, l;
};
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = a * b;
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, s.l + x.l + y.l);
}
__device__ __forceinline__ df df_mul(df x, df y) {
  df p = two_prod(x.h, y.h);
  p.l = p.l + (x.h * y.l + x.l * y.h);
  return fast_two_sum(p.h, p.l);
}
__device__ __forceinline__ df df_mul_f(df x, float b) {
  df p = two_prod(x.h, b);
  p.l = p.l + x.l * b;
  return fast_two_sum(p.h, p.l);
}
__device__ __forceinline__ df df_div(df x, df y) {
  const float q1 = x.h / y.h;
  const df r = df_add(x, df_mul_f({-y.h, -y.l}, q1));
  const float q2 = r.h / y.h;
  return fast_two_sum(q1, q2);
}
// Nearest f32 of a normalised double-float value (|l| <= ulp(h)/2). The
// rounding midpoints next to h sit at h +- ulp(h)/2, so `amb` is set when |l|
// lies within a relative 2^-40 of ulp(h)/2, and also whenever the gaps around
// h are uneven or tiny (h a power of two, zero, subnormal-adjacent or not
// finite); the caller then takes the f64 path.
__device__ __forceinline__ float df_round(df v, bool& amb) {
  const float r = v.h + v.l;
  const unsigned bits = __float_as_uint(v.h) & 0x7fffffffu;
  const unsigned expo = bits >> 23;
  if (expo <= 25u || expo == 255u || (bits & 0x7fffffu) == 0u) {
    amb = true;
    return r;
  }
  const float half_ulp = __uint_as_float((expo - 24u) << 23);
  if (!(fabsf(fabsf(v.l) - half_ulp) > fabsf(v.h) * 9.094947e-13f)) amb = true;  // 2^-40
  return r;
}

// (n + c) * unscale in f64, narrowed to f32 (plan.rs:476-478).
__device__ __forceinline__ float post_transform(float n, float ch, float cl, const FastOptics& f, double c64,
                                                double unscale, bool& fell_back) {
  df t = two_sum(n, ch);
  t = fast_two_sum(t.h, t.l + cl);
  bool amb = false;
  const float r = df_round(df_mul(t, {f.uh, f.ul}), amb);
  if (!amb) return r;
  fell_back = true;
  return (float)(((double)n + c64) * unscale);
}

// Poly5 inverse from f32 (x, y): the f64 Newton result, computed through the
// one-step closed form when that is what the iteration does (break at step 0:
// ratio 1; break at step 1: ratio = 1 - g/d with g = k1 u + k2 u^2 and
// d = 1 + 3 k1 u + 5 k2 u^2 for u = x^2 + y^2), else through f64.
__device__ __forceinline__ void undistort_poly5_fast(float x, float y, float a, float b, float& ox, float& oy,
                                                     bool& need_f64) {
  ox = x;
  oy = y;
  const float s = x * x + y * y;
  if (s == 0.0f) return;
  const float g32 = a * s + b * (s * s);
  const float sq = sqrtf(s);
  const float f0 = sq * g32;
  const float thr = 1.0e-5f;
  if (fabsf(f0) < thr * (1.0f - 1.0e-5f)) return;  // |F(rd)| < 1e-5: frozen at the input
  if (fabsf(f0) <= thr * (1.0f + 1.0e-5f)) {
    need_f64 = true;
    return;
  }
  const float d32 = 1.0f + 3.0f * a * s + 5.0f * b * (s * s);
  const float q32 = f0 / d32;
  const float f1 = (3.0f * a * sq + 10.0f * b * sq * s) * q32 * q32;  // F(ru1) ~ F''/2 (F/F')^2
  if (!(fabsf(f1) < 1.0e-6f) || !(d32 > 0.0f)) {
    need_f64 = true;
    return;
  }
  const df as = two_prod(a, s);
  const df ss = two_prod(s, s);
  const df bss = df_mul_f(ss, b);
  const df g = df_add(as, bss);
  const df d = df_add(df_add({1.0f, 0.0f}, df_mul_f(as, 3.0f)), df_mul_f(bss, 5.0f));
  const df q = df_div(g, d);
  const df ratio = fast_two_sum(1.0f, -q.h);
  const df rr = {ratio.h, ratio.l - q.l};
  if (!(rr.h > 0.0f)) {
    need_f64 = true;
    return;
  }
  bool amb = false;
  const float rx = df_round(df_mul_f(rr, x), amb);
  const float ry = df_round(df_mul_f(rr, y), amb);
  if (amb) {
    need_f64 = true;
    return;
  }
  ox = rx;
  oy = ry;
}

// cubic_weight (resample.rs) at the four distances x - (fx - 1) .. x - (fx + 2)
// of a footprint with fx = floor(x) >= 1. Those differences are exact and lie
// in [1, 2), [0, 1), [-1, 0) and [-2, -1), so each weight takes one fixed
// branch: |d| <= 1 for the middle two, 1 < |d| < 2 for the outer two. The
// outer distances reach 1 or 2 only when x is an integer, where the
// reference's branch and this one both give +0.0.
__device__ __forceinline__ void cubic_weights(float x, int fx, float (&w)[4]) {
  const float a0 = fabsf(x - (float)(fx - 1));
  const float a1 = fabsf(x - (float)fx);
  const float a2 = fabsf(x - (float)(fx + 1));
  const float a3 = fabsf(x - (float)(fx + 2));
  w[0] = -0.5f * a0 * a0 * a0 + 2.5f * a0 * a0 - 4.0f * a0 + 2.0f;
  w[1] = 1.5f * a1 * a1 * a1 - 2.5f * a1 * a1 + 1.0f;
  w[2] = 1.5f * a2 * a2 * a2 - 2.5f * a2 * a2 + 1.0f;
  w[3] = -0.5f * a3 * a3 * a3 + 2.5f * a3 * a3 - 4.0f * a3 + 2.0f;
}

// resample.rs:3-41. Returns false for a non-finite coordinate or a footprint
// that leaves the image.
template <bool VIG>
__device__ __forceinline__ bool cubic_sample(const float* __restrict__ plane, const float* __restrict__ mult, int W,
                                             int H, float x, float y, float& out) {
  if (!isfinite(x) || !isfinite(y)) return false;
  const int fx = (int)floorf(x), fy = (int)floorf(y);
  if (fx - 1 < 0 || fy - 1 < 0 || fx + 2 >= W || fy + 2 >= H) return false;
  float value = 0.0f;
  float wx[4], wys[4];
  cubic_weights(x, fx, wx);  // same for every row
  cubic_weights(y, fy, wys);
#pragma unroll
  for (int oy = -1; oy <= 2; ++oy) {
    const float wy = wys[oy + 1];
    const float* row = plane + (long long)(fy + oy) * W;
    const float* mrow = VIG ? mult + (long long)(fy + oy) * W : nullptr;
#pragma unroll
    for (int ox = -1; ox <= 2; ++ox) {
      const float weight = wy * wx[ox + 1];
      float sample = __ldg(row + fx + ox);
      if (VIG) sample = sample * __ldg(mrow + fx + ox);  // the vignetted source value
      value += sample * weight;
    }
  }
  if (!isfinite(value)) return false;
  out = value;
  return true;
}

template <bool VIG>
__global__ void __launch_bounds__(512) optics_kernel(const OpticsParams p) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (x >= p.W || y >= p.H) return;
  float gx, gy;
  const float ix = p.ix[x], iy = p.iy[y];
  if (p.dist_model == RD_DISTORTION_POLY5) {
    bool need_f64 = false;
    undistort_poly5_fast(ix, iy, p.d0, p.d1, gx, gy, need_f64);
    if (need_f64) undistort(p, ix, iy, gx, gy);
  } else {
    undistort(p, ix, iy, gx, gy);
  }
  bool bad = !isfinite(gx) || !isfinite(gy);
  float n[6] = {gx, gy, gx, gy, gx, gy};
  if (p.tca_model == RD_TCA_LINEAR) {
    n[0] = gx * p.tr[0];
    n[1] = gy * p.tr[0];
    n[4] = gx * p.tb[0];
    n[5] = gy * p.tb[0];
  } else if (p.tca_model == RD_TCA_POLY3) {
    tca_poly3(p.tr, gx, gy, n[0], n[1]);
    tca_poly3(p.tb, gx, gy, n[4], n[5]);
  }
  const long long plane = (long long)p.W * p.H;
  const long long o = (long long)y * p.W + x;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    bool fell_back = false;
    const float sx = post_transform(n[2 * c], p.fast.cxh, p.fast.cxl, p.fast, p.cx, p.unscale, fell_back);
    const float sy = post_transform(n[2 * c + 1], p.fast.cyh, p.fast.cyl, p.fast, p.cy, p.unscale, fell_back);
    float v = 0.0f;
    if (!bad && !cubic_sample<VIG>(p.in + c * plane, p.mult, p.W, p.H, sx, sy, v)) bad = true;
    p.out[c * plane + o] = v;
  }
  if (bad) atomicOr(p.error, 8u);
}

// f32 hypot as the reference gets it (f32::hypot, glibc hypotf): the double
// sum of the two exact double squares, its double square root, narrowed once.
// Here the square root is taken in double-float from the exact FP32-pair sum
// of squares (one Newton correction of sqrtf); the rare result too close to
// an f32 rounding boundary (or zero, tiny, huge) is recomputed in f64.
__device__ __forceinline__ float hypot_f32(float x, float y) {
  const df s = df_add(two_prod(x, x), two_prod(y, y));
  const float r0 = sqrtf(s.h);
  const df r2 = two_prod(r0, r0);
  const float residual = ((s.h - r2.h) - r2.l) + s.l;  // s.h - r2.h is exact
  bool amb = false;
  const float r = df_round(fast_two_sum(r0, __fdividef(residual, 2.0f * r0)), amb);
  if (!amb) return r;
  return (float)sqrt((double)x * (double)x + (double)y * (double)y);
}

// Self-check of hypot_f32: x runs over every f32 in [first, last), y is a
// hashed f32 of either sign with |y| < 2; counts results that differ from the
// double computation.
__global__ void hypot_check_kernel(unsigned first, unsigned last, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  for (unsigned b = first + blockIdx.x * blockDim.x + threadIdx.x; b < last; b += gridDim.x * blockDim.x) {
    unsigned h = b * 2654435761u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const float x = __uint_as_float(b);
    const float y = __uint_as_float((h & 0x807fffffu) | ((109u + (h >> 23) % 19u) << 23));  // 2^-18 <= |y| < 2
    const float want = (float)sqrt((double)x * (double)x + (double)y * (double)y);
    if (__float_as_uint(hypot_f32(x, y)) != __float_as_uint(want)) ++bad;
    if (__float_as_uint(hypot_f32(x, 0.0f)) != __float_as_uint(x)) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}

// The radial-table branch of the remap (correction.rs:122-151): the three
// channel multipliers come from one lookup at the pixel's input radius
// (RadialMultipliers::lookup, radial.rs:212-229: nearest knot on the pixel's
// side of a pinned freeze boundary, else the linear blend of the two knots),
// then plan.rs:136-141's post-transform and the Catmull-Rom gather per
// channel. `knots` holds [m_r, m_g, m_b, pin] per knot; it is 16 KB and stays
// in L1.
template <bool VIG>
__global__ void __launch_bounds__(512) optics_lut_kernel(const OpticsParams p, const float4* __restrict__ knots,
                                                         float step) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (x >= p.W || y >= p.H) return;
  const float ix = p.ix[x], iy = p.iy[y];
  const float radius = hypot_f32(ix, iy);
  const float position = radius / step;
  const int index = position < (float)(RADIAL_KNOTS - 2) ? (int)position : RADIAL_KNOTS - 2;
  const float4 lo = __ldg(knots + index), hi = __ldg(knots + index + 1);
  float m[3];
  if (lo.w == lo.w) {  // pinned segment
    const float4 k = radius >= lo.w ? hi : lo;
    m[0] = k.x;
    m[1] = k.y;
    m[2] = k.z;
  } else {
    float blend = position - (float)index;
    if (blend > 1.0f) blend = 1.0f;
    m[0] = lo.x * (1.0f - blend) + hi.x * blend;
    m[1] = lo.y * (1.0f - blend) + hi.y * blend;
    m[2] = lo.z * (1.0f - blend) + hi.z * blend;
  }
  const long long plane = (long long)p.W * p.H;
  const long long o = (long long)y * p.W + x;
  bool bad = false;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    bool fell_back = false;
    const float sx = post_transform(ix * m[c], p.fast.cxh, p.fast.cxl, p.fast, p.cx, p.unscale, fell_back);
    const float sy = post_transform(iy * m[c], p.fast.cyh, p.fast.cyl, p.fast, p.cy, p.unscale, fell_back);
    float v = 0.0f;
    if (!bad && !cubic_sample<VIG>(p.in + c * plane, p.mult, p.W, p.H, sx, sy, v)) bad = true;
    p.out[c * plane + o] = v;
  }
  if (bad) atomicOr(p.error, 8u);
}

// Horizontal area pass: one thread per (row, target column, channel-plane).
template <bool VIG>
__device__ __forceinline__ float area_row(const float* __restrict__ row, const float* __restrict__ mrow,
                                          const float* __restrict__ hw, int hn) {
  float mid = 0.0f;
  for (int j = 0; j < hn; ++j) {
    float sample = __ldg(row + j);
    if (VIG) sample = sample * __ldg(mrow + j);
    mid += sample * __ldg(hw + j);
  }
  return mid;
}

// Exact separable area reduction in one pass: a thread owns one output
// column and channel of a tile of AREA_ROWS output rows and streams the
// tile's input rows in order. Each input row's horizontal sum is computed
// once and added to the vertical sum of every output row it belongs to (the
// row where two output rows meet goes to both), so neither pass stores the
// intermediate rows. Both sums accumulate their taps in table order from 0,
// as the two-pass form (and resample.rs) does, so the outputs are the same
// bit for bit.
constexpr int AREA_ROWS = 16;

template <bool VIG>
__global__ void __launch_bounds__(128) area_kernel(const float* __restrict__ in, const float* __restrict__ mult,
                                                   int W, int H, int tw, int th, const int* __restrict__ hfirst,
                                                   const int* __restrict__ hoffset, const int* __restrict__ hcount,
                                                   const float* __restrict__ hweights,
                                                   const int* __restrict__ vfirst, const int* __restrict__ voffset,
                                                   const int* __restrict__ vcount, const float* __restrict__ vweights,
                                                   float* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.z;
  if (s >= tw) return;
  const int t0 = blockIdx.y * AREA_ROWS, t1 = min(t0 + AREA_ROWS, th);
  const float* plane = in + (long long)c * W * H + hfirst[s];
  const float* mplane = VIG ? mult + hfirst[s] : nullptr;
  const float* hw = hweights + hoffset[s];
  const int hn = hcount[s];
  float* o = out + (long long)c * tw * th + s;
  int t = t0;
  int first = vfirst[t], end = first + vcount[t];
  const float* vw = vweights + voffset[t];
  float acc = 0.0f;
  const int r_end = vfirst[t1 - 1] + vcount[t1 - 1];
  // Adds one input row's horizontal sum to the vertical sum(s) it belongs to;
  // false once the tile's last output row is written.
  auto take = [&](int r, float mid) {
    acc += mid * __ldg(vw + (r - first));
    if (r == end - 1) {
      o[(long long)t * tw] = acc;
      if (++t == t1) return false;
      const int nf = vfirst[t];
      vw = vweights + voffset[t];
      // The next output row starts at or before this input row (they share
      // at most this one).
      acc = 0.0f;
      if (nf <= r) acc += mid * __ldg(vw + (r - nf));
      first = nf;
      end = nf + vcount[t];
    }
    return true;
  };
  if (hn <= 4) {
    // Up to four taps per row (reductions up to 3x): the samples of four rows
    // are loaded together before any of their sums, so their latencies
    // overlap; each sum still adds its taps in order from 0.
    float w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) w[j] = j < hn ? __ldg(hw + j) : 0.0f;
    for (int r0 = first; r0 < r_end; r0 += 4) {
      float smp[4][4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float* row = plane + (long long)(r0 + q) * W;
        const float* mrow = VIG ? mplane + (long long)(r0 + q) * W : nullptr;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float v = 0.0f;
          if (r0 + q < r_end && j < hn) {
            v = __ldg(row + j);
            if (VIG) v = v * __ldg(mrow + j);
          }
          smp[q][j] = v;
        }
      }
      bool more = true;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (!more || r0 + q >= r_end) break;
        float mid = 0.0f;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (j < hn) mid += smp[q][j] * w[j];
        more = take(r0 + q, mid);
      }
      if (!more) break;
    }
    return;
  }
  for (int r = first; r < r_end; ++r)
    if (!take(r, area_row<VIG>(plane + (long long)r * W, VIG ? mplane + (long long)r * W : nullptr, hw, hn))) break;
}

struct AxisTable {
  std::vector<int> first, offset, count;
  std::vector<float> weights;
};

// AreaReductionAxis::new (resample.rs:45-113).
AxisTable build_axis(int source, int target) {
  AxisTable a;
  const double scale = (double)source / (double)target;
  for (int t = 0; t < target; ++t) {
    const double left = (double)t * scale, right = (double)(t + 1) * scale;
    const int first = (int)std::floor(left);
    const int end = std::min((int)std::ceil(right), source);
    a.first.push_back(first);
    a.offset.push_back((int)a.weights.size());
    a.count.push_back(end - first);
    for (int s = first; s < end; ++s) {
      const double overlap = std::min(right, (double)(s + 1)) - std::max(left, (double)s);
      a.weights.push_back((float)(overlap / scale));
    }
  }
  return a;
}

}  // namespace

// Per-axis pre-transform, plan.rs:448-455 / correction.rs input_coordinate_x,y.
std::vector<float> optics_input_coordinates(const rd_optics_desc& o) {
  const int W = (int)o.width, H = (int)o.height;
  std::vector<float> tab((size_t)W + H);
  const double cpx = o.center_x * o.norm_unscale, cpy = o.center_y * o.norm_unscale;
  for (int x = 0; x < W; ++x) {
    const double mapped = cpx + ((double)x - cpx) / (double)o.scale;
    tab[x] = (float)(mapped * o.norm_scale - o.center_x);
  }
  for (int y = 0; y < H; ++y) {
    const double mapped = cpy + ((double)y - cpy) / (double)o.scale;
    tab[W + y] = (float)(mapped * o.norm_scale - o.center_y);
  }
  return tab;
}

Status run_optics_gather(Context& ctx, const rd_optics_desc& o, const float* rgb_in, const float* mult,
                         float* rgb_out) {
  const int W = (int)o.width, H = (int)o.height;
  const std::vector<float> tab = optics_input_coordinates(o);
  // The remap's branch is decided once per apply (correction.rs:110-121).
  const RadialTable radial = build_radial_table(o, tab.data(), tab.data() + W);
  const bool lut = radial.guard == RD_RADIAL_ACCEPTED;
  std::vector<float> staged = lut ? radial.knots : std::vector<float>();
  const size_t knot_floats = staged.size();  // a multiple of 4: the coordinate tables stay 16-byte aligned
  staged.insert(staged.end(), tab.begin(), tab.end());
  const size_t bytes = sizeof(float) * staged.size();
  void* d = nullptr;
  RD_TRY(device_alloc(ctx, bytes, &d));
  float* dbuf = static_cast<float*>(d);
  RD_TRY(upload(ctx, dbuf, staged.data(), bytes));
  const float* dtab = dbuf + knot_floats;
  OpticsParams p{};
  p.in = rgb_in;
  p.mult = mult;
  p.out = rgb_out;
  p.W = W;
  p.H = H;
  p.ix = dtab;
  p.iy = dtab + W;
  p.cx = o.center_x;
  p.cy = o.center_y;
  p.unscale = o.norm_unscale;
  p.dist_model = o.distortion_model;
  p.d0 = o.distortion[0];
  p.d1 = o.distortion[1];
  p.d2 = o.distortion[2];
  p.tca_model = o.tca_model;
  for (int c = 0; c < 3; ++c) {
    p.tr[c] = o.tca_red[c];
    p.tb[c] = o.tca_blue[c];
  }
  p.error = ctx.d_error;
  auto split = [](double v, float& h, float& l) {
    h = (float)v;
    l = (float)(v - (double)h);
  };
  split(o.center_x, p.fast.cxh, p.fast.cxl);
  split(o.center_y, p.fast.cyh, p.fast.cyl);
  split(o.norm_unscale, p.fast.uh, p.fast.ul);
  // Tiles of 32 columns and `rows` rows (one warp per row), tuned across
  // calls per image shape: the tile only decides which CTA takes which pixel.
  const ShapeKey key{TUNE_OPTICS, W, H, 0};
  const ShapePick pick = shape_begin(ctx, key, 8, {4, 16});
  const int rows = pick.value;
  const dim3 grid((W + 31) / 32, (H + rows - 1) / rows);
  const unsigned block = 32u * (unsigned)rows;
  const float4* knots = reinterpret_cast<const float4*>(dbuf);
  if (lut && p.mult) {
    RD_LAUNCH(ctx, K_OPTICS, optics_lut_kernel<true><<<grid, block, 0, ctx.stream>>>(p, knots, radial.step));
  } else if (lut) {
    RD_LAUNCH(ctx, K_OPTICS, optics_lut_kernel<false><<<grid, block, 0, ctx.stream>>>(p, knots, radial.step));
  } else if (p.mult) {
    RD_LAUNCH(ctx, K_OPTICS, optics_kernel<true><<<grid, block, 0, ctx.stream>>>(p));
  } else {
    RD_LAUNCH(ctx, K_OPTICS, optics_kernel<false><<<grid, block, 0, ctx.stream>>>(p));
  }
  shape_end(ctx, key, pick);
  const cudaError_t launch = cudaGetLastError();
  device_free(ctx, dbuf, bytes);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}


Status run_hypot_check(Context& ctx, uint64_t* result) {
  void* p = nullptr;
  RD_TRY(device_alloc(ctx, 16, &p));
  RD_CUDA_TRY(cudaMemsetAsync(p, 0, 16, ctx.stream));
  const float lo = 0x1p-12f, hi = 2.0f;
  unsigned first = 0, last = 0;
  std::memcpy(&first, &lo, 4);
  std::memcpy(&last, &hi, 4);
  const int grid = (ctx.sm_count > 0 ? ctx.sm_count : 152) * 8;
  RD_LAUNCH(ctx, K_OPTICS, (hypot_check_kernel<<<grid, 256, 0, ctx.stream>>>(
                               first, last, static_cast<unsigned long long*>(p))));
  Status st;
  uint64_t v = 0;
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&v, p, 8, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "hypot check failed"};
  device_free(ctx, p, 16);
  if (st.ok()) *result = v;
  return st;
}

Status run_area_reduce(Context& ctx, const float* rgb, const float* mult, int W, int H, int tw, int th, float* out) {
  const AxisTable ha = build_axis(W, tw), va = build_axis(H, th);
  const size_t ints = ha.first.size() * 3 + va.first.size() * 3;
  const size_t bytes = ints * sizeof(int) + (ha.weights.size() + va.weights.size()) * sizeof(float);
  std::vector<unsigned char> host(bytes);
  unsigned char* q = host.data();
  auto put = [&](const void* src, size_t n) {
    std::memcpy(q, src, n);
    q += n;
  };
  put(ha.first.data(), tw * sizeof(int));
  put(ha.offset.data(), tw * sizeof(int));
  put(ha.count.data(), tw * sizeof(int));
  put(va.first.data(), th * sizeof(int));
  put(va.offset.data(), th * sizeof(int));
  put(va.count.data(), th * sizeof(int));
  put(ha.weights.data(), ha.weights.size() * sizeof(float));
  put(va.weights.data(), va.weights.size() * sizeof(float));
  void* d = nullptr;
  RD_TRY(device_alloc(ctx, bytes, &d));
  unsigned char* b = static_cast<unsigned char*>(d);
  RD_TRY(upload(ctx, b, host.data(), bytes));
  const int* hf = reinterpret_cast<const int*>(b);
  const int* ho = hf + tw;
  const int* hc = ho + tw;
  const int* vf = hc + tw;
  const int* vo = vf + th;
  const int* vc = vo + th;
  const float* hw = reinterpret_cast<const float*>(vc + th);
  const float* vw = hw + ha.weights.size();
  const dim3 grid((tw + 127) / 128, (th + AREA_ROWS - 1) / AREA_ROWS, 3);
  if (mult) {
    RD_LAUNCH(ctx, K_AREA, area_kernel<true><<<grid, 128, 0, ctx.stream>>>(rgb, mult, W, H, tw, th, hf, ho, hc, hw,
                                                                               vf, vo, vc, vw, out));
  } else {
    RD_LAUNCH(ctx, K_AREA, area_kernel<false><<<grid, 128, 0, ctx.stream>>>(rgb, mult, W, H, tw, th, hf, ho, hc,
                                                                                hw, vf, vo, vc, vw, out));
  }
  const cudaError_t launch = cudaGetLastError();
  device_free(ctx, b, bytes);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

}  // namespace rd
