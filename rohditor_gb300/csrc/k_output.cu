// Display and extended-range output of a linear Rec.2020 base on sm_103a:
// the adjustment chain, orientation + crop, gamut mapping into sRGB or
// Display P3 primaries (hard clip or OKLCH chroma compression), and the output
// encoding (display 8-bit, 16-bit, or unquantised linear f32 / f16 up to a
// headroom).
//
//  geometry          OutputGeometry (crates/core/src/geometry.rs:36-121,166-184) and
//                    OrientationMap::source_coordinate_in_bounds
//                    (crates/image/src/orientation.rs:150-170)
//  output transform  DisplayOutputTransform (crates/core/src/color/display_output.rs:24-59)
//  gamut mapping     clip_linear_rgb, compress_chroma (crates/color/src/gamut.rs:100-222),
//                    OkLab (crates/color/src/oklab.rs:1-60)
//  8 / 16-bit        render_display8_cancellable, render_display_srgb16_with_geometry_and_diagnostics,
//                    quantization_dither (crates/core/src/cpu/stages.rs:1028-1214)
//  extended          render_extended_linear_with_geometry (crates/core/src/cpu/extended.rs:27-106)
//
// One kernel reads the planar base once and writes the interleaved output
// once. The output is cut into 32x32 tiles; for the four orientations that
// swap the axes a tile's source block is staged through shared memory so both
// the planar reads and the interleaved writes stay coalesced. Gamut statuses
// are counted per thread, reduced per warp and flushed once per CTA.
//
// The reference's cube root and transfer power come from the platform libm,
// which is not correctly rounded (glibc 2.39's cbrtf misses on about one f32
// in ten). This file computes both correctly rounded: the cube root by one
// Newton step in double from cbrtf followed by an exact midpoint test, the
// transfer through quantize_srgb3 (color_chain.cuh).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "color_chain.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

enum : int { FMT_U8 = RD_OUTPUT_SRGB8, FMT_U16 = RD_OUTPUT_SRGB16, FMT_F32 = RD_OUTPUT_EXTENDED_F32,
             FMT_F16 = RD_OUTPUT_EXTENDED_F16 };
// GamutMapStatus (gamut.rs:43-50), the order of the diagnostics counters.
enum : int { ST_IN_GAMUT = 0, ST_COMPRESSED = 1, ST_LIMITED = 2, ST_CLIPPED_FALLBACK = 3, ST_INVALID = 4 };

// ------------------------------------------------------------ cube root
// Correctly rounded cube root of an f32.
//
// cbrtf's estimate r is within an ulp. The side of the midpoint m = r +- ulp/2
// that the true root lies on is the sign of x - m^3, with m^3 formed in
// float-float (relative error below 2^-44): a difference above 2^-40 x
// decides, and r moves to its neighbour when the root lies beyond the
// midpoint. Inputs outside [2^-60, 2^60] are scaled by 2^-+90 first (exact,
// and the root scales by 2^-+30) so that no low part of the float-float
// arithmetic underflows. Only when the root is within about 2^-42 of a
// midpoint (about one input in 10^5) does the double method below decide.

// Double method: one Newton step for y^3 = x from cbrtf, then the exact sign
// of m^3 - x at the midpoint towards the double value (m*m is exact in double,
// the product with m splits into hi + lo by an FMA, and hi - x is exact
// because hi and x agree to within a factor of two). For positive finite x.
__device__ __noinline__ float cbrt_rn_double(float ax) {
  const double d = (double)ax;
  const float y0 = cbrtf(ax);
  const double y0d = (double)y0;
  const double residual = d - y0d * y0d * y0d;
  const float inv = 1.0f / (3.0f * y0 * y0);
  const double yd = y0d + residual * (double)inv;
  float r = (float)yd;
  if (yd != (double)r) {
    const bool up = yd > (double)r;
    const float nb = up ? next_up(r) : next_down(r);
    const double m = ((double)r + (double)nb) * 0.5;
    const double m2 = m * m;
    const double hi = m2 * m;
    const double lo = fma(m2, m, -hi);
    const double diff = (hi - d) + lo;  // sign of m^3 - x
    if (up ? diff < 0.0 : diff > 0.0) r = nb;
  }
  return r;
}

// +1 when cbrt(x) > r + h, -1 when below, 0 when too close to call.
__device__ __forceinline__ int cube_side(float x, float r, float h) {
  const FF m{r, h};
  const FF m3 = ff_mul(ff_mul(m, m), m);
  const float d = (x - m3.hi) - m3.lo;             // x - m3.hi is exact (Sterbenz)
  const float eps = x * 9.094947017729282e-13f;  // 2^-40
  return d > eps ? 1 : (d < -eps ? -1 : 0);
}

__device__ __forceinline__ float cbrt_rn(float x) {
  if (x == 0.0f || !isfinite(x)) return x;
  float ax = fabsf(x), post = 1.0f;
  if (ax < 0x1p-60f) {
    ax *= 0x1p90f;
    post = 0x1p-30f;
  } else if (ax > 0x1p60f) {
    ax *= 0x1p-90f;
    post = 0x1p30f;
  }
  float r = cbrtf(ax);
  for (int k = 0; k < 3; ++k) {
    const float up = next_up(r);
    const int above = cube_side(ax, r, (up - r) * 0.5f);
    if (above > 0) {
      r = up;
      continue;
    }
    if (above == 0) {
      r = cbrt_rn_double(ax);
      break;
    }
    const float down = next_down(r);
    const int below = cube_side(ax, r, (down - r) * 0.5f);
    if (below < 0) {
      r = down;
      continue;
    }
    if (below == 0) r = cbrt_rn_double(ax);
    break;
  }
  return copysignf(r * post, x);
}

// ------------------------------------------------------------ OkLab
// Ottosson's OkLab (oklab.rs:18-48) and the exact sRGB <-> Display P3
// conversions it is extended with (oklab.rs:5-16, 50-60). Matrix rows are
// applied as r0*v0 + r1*v1 + r2*v2, left to right (matrix.rs:173-175).
__device__ __forceinline__ void xform(const float (&m)[3][3], const float* v, float* out) {
  const float a = v[0], b = v[1], c = v[2];
#pragma unroll
  for (int r = 0; r < 3; ++r) out[r] = m[r][0] * a + m[r][1] * b + m[r][2] * c;
}
__constant__ float P3_TO_SRGB[3][3] = {{1.2249402f, -0.2249402f, 0.0f},
                                       {-0.042057f, 1.042057f, 0.0f},
                                       {-0.0196376f, -0.078636f, 1.0982736f}};
__constant__ float SRGB_TO_P3[3][3] = {{0.822462f, 0.177538f, 0.0f},
                                       {0.0331942f, 0.9668058f, 0.0f},
                                       {0.0170826f, 0.0723974f, 0.9105199f}};

__device__ __forceinline__ void to_oklab(int p3, const float* rgb, float* lab) {
  float c[3] = {rgb[0], rgb[1], rgb[2]};
  if (p3) xform(P3_TO_SRGB, rgb, c);
  const float l = 0.41222146f * c[0] + 0.53633255f * c[1] + 0.051445995f * c[2];
  const float m = 0.2119035f * c[0] + 0.6806995f * c[1] + 0.10739696f * c[2];
  const float s = 0.08830246f * c[0] + 0.28171885f * c[1] + 0.6299787f * c[2];
  const float lr = cbrt_rn(l), mr = cbrt_rn(m), sr = cbrt_rn(s);
  lab[0] = 0.21045426f * lr + 0.7936178f * mr - 0.004072047f * sr;
  lab[1] = 1.9779985f * lr - 2.4285922f * mr + 0.4505937f * sr;
  lab[2] = 0.025904037f * lr + 0.78277177f * mr - 0.80867577f * sr;
}
__device__ __forceinline__ void from_oklab(int p3, float L, float a, float b, float* rgb) {
  const float lr = L + 0.39633778f * a + 0.21580376f * b;
  const float mr = L - 0.105561346f * a - 0.06385417f * b;
  const float sr = L - 0.08948418f * a - 1.2914855f * b;
  const float l = lr * lr * lr, m = mr * mr * mr, s = sr * sr * sr;
  float c[3];
  c[0] = 4.0767417f * l - 3.3077116f * m + 0.23096994f * s;
  c[1] = -1.268438f * l + 2.6097574f * m - 0.34131938f * s;
  c[2] = -0.0041960863f * l - 0.7034186f * m + 1.7076147f * s;
  if (p3) {
    xform(SRGB_TO_P3, c, rgb);
  } else {
    rgb[0] = c[0];
    rgb[1] = c[1];
    rgb[2] = c[2];
  }
}

// ------------------------------------------------------------ gamut mapping
__device__ __forceinline__ bool in_gamut(const float* v, float ceiling) {
  return v[0] >= 0.0f && v[0] <= ceiling && v[1] >= 0.0f && v[1] <= ceiling && v[2] >= 0.0f && v[2] <= ceiling;
}
// sanitize_and_clip (gamut.rs:199-207).
__device__ __forceinline__ float sanitize(float v, float ceiling) {
  if (isnan(v) || v == -INFINITY) return 0.0f;
  if (v == INFINITY) return ceiling;
  return rclamp(v, 0.0f, ceiling);
}
__device__ __forceinline__ void sanitize3(const float* in, float ceiling, float* out) {
  out[0] = sanitize(in[0], ceiling);
  out[1] = sanitize(in[1], ceiling);
  out[2] = sanitize(in[2], ceiling);
}
// clip_linear_rgb (gamut.rs:110-122).
__device__ __forceinline__ int clip_rgb(const float* rgb, float ceiling, float* out) {
  const bool finite = fin3(rgb);
  const bool inside = finite && in_gamut(rgb, ceiling);
  sanitize3(rgb, ceiling, out);
  return !finite ? ST_INVALID : (inside ? ST_IN_GAMUT : ST_CLIPPED_FALLBACK);
}
// compress_chroma (gamut.rs:124-182): in-gamut pixels pass bit-exactly; the
// rest keep their OkLab hue and (limited) lightness and lose chroma, found by
// 16 bisection steps on the scale of the a/b pair. The front returns -1 for a
// pixel that needs the bisection (finite and out of gamut), which
// compress_out_of_gamut then maps.
__device__ __forceinline__ int compress_front(const float* rgb, float ceiling, float* out) {
  if (!fin3(rgb)) {
    sanitize3(rgb, ceiling, out);
    return ST_INVALID;
  }
  if (in_gamut(rgb, ceiling)) {
    out[0] = rgb[0];
    out[1] = rgb[1];
    out[2] = rgb[2];
    return ST_IN_GAMUT;
  }
  return -1;
}
__device__ int compress_out_of_gamut(const float* rgb, int p3, float ceiling, float lightness_ceiling, float* out) {
  float lab[3];
  to_oklab(p3, rgb, lab);
  if (!fin3(lab)) {
    sanitize3(rgb, ceiling, out);
    return ST_CLIPPED_FALLBACK;
  }
  const float limited = rclamp(lab[0], 0.0f, lightness_ceiling);
  const int status = limited != lab[0] ? ST_LIMITED : ST_COMPRESSED;
  // chroma = hypot(a, b) <= 1e-6 with the hypot correctly rounded, i.e.
  // a^2 + b^2 below (1e-6 + half an ulp)^2 = 1.0000001e-12. The f32 sum of
  // squares is within 2^-22 of the exact one, so it decides outside a 1e-5
  // band around the bound; inside it the squares are exact in double.
  const float a2f = lab[1] * lab[1] + lab[2] * lab[2];
  bool neutral;
  if (a2f < 0.99999e-12f) neutral = true;
  else if (a2f > 1.00001e-12f) neutral = false;
  else neutral = (float)sqrt((double)lab[1] * (double)lab[1] + (double)lab[2] * (double)lab[2]) <= 1.0e-6f;
  float c[3];
  if (neutral) {
    from_oklab(p3, limited, 0.0f, 0.0f, c);
    sanitize3(c, ceiling, out);
    return status;
  }
  float lower = 0.0f, upper = 1.0f;
  for (int k = 0; k < 16; ++k) {
    const float scale = (lower + upper) * 0.5f;
    from_oklab(p3, limited, lab[1] * scale, lab[2] * scale, c);
    // in_gamut is false for NaN and infinities, so it covers the finite test.
    if (in_gamut(c, ceiling)) lower = scale;
    else upper = scale;
  }
  from_oklab(p3, limited, lab[1] * lower, lab[2] * lower, c);
  if (!fin3(c)) {
    sanitize3(rgb, ceiling, out);
    return ST_CLIPPED_FALLBACK;
  }
  sanitize3(c, ceiling, out);
  return status;
}

// quantization_dither (stages.rs:1197-1214): the 8x8 Bayer threshold matrix,
// (b + 0.5) / 64 - 0.5 at the output coordinate.
__constant__ unsigned char BAYER8[8][8] = {
    {0, 32, 8, 40, 2, 34, 10, 42},  {48, 16, 56, 24, 50, 18, 58, 26}, {12, 44, 4, 36, 14, 46, 6, 38},
    {60, 28, 52, 20, 62, 30, 54, 22}, {3, 35, 11, 43, 1, 33, 9, 41},    {51, 19, 59, 27, 49, 17, 57, 25},
    {15, 47, 7, 39, 13, 45, 5, 37},  {63, 31, 55, 23, 61, 29, 53, 21}};

// ------------------------------------------------------------ kernel
struct OutputParams {
  const float* in;            // planar Rec.2020 [3][SH][SW]
  int SW, SH;
  AdjustParams adj;
  float m[9];                 // Rec.2020 -> linear display primaries
  int p3;                     // gamut of the chroma compression
  int compress;               // 1: compress_chroma, 0: clip_linear_rgb
  float ceiling;              // 1, or the headroom of an extended output
  float lightness_ceiling;    // correctly rounded cube root of the ceiling
  int dither;
  int flip_h, flip_v;         // mirror the source x / y after the axis swap
  int left, top, OW, OH;      // crop origin on the oriented canvas, output size
  void* out;                  // interleaved [OH][3*OW] of the format
  unsigned long long* hist;   // 1024 bins of the 8-bit output, or null
  unsigned long long* gamut;  // 5 status counters, or null
};

constexpr int TILE = 32;
constexpr int ROWS = 8;  // warps per CTA; each handles every 8th tile row

template <int FMT>
__device__ __forceinline__ void encode_pixel(const OutputParams& p, int ox, int oy, const float* mapped,
                                             unsigned int* bins) {
  const long long o = ((long long)oy * p.OW + ox) * 3;
  if (FMT == FMT_F32) {
    float* d = static_cast<float*>(p.out) + o;
    d[0] = mapped[0];
    d[1] = mapped[1];
    d[2] = mapped[2];
  } else if (FMT == FMT_F16) {
    unsigned short* d = static_cast<unsigned short*>(p.out) + o;
    d[0] = __half_as_ushort(__float2half_rn(mapped[0]));
    d[1] = __half_as_ushort(__float2half_rn(mapped[1]));
    d[2] = __half_as_ushort(__float2half_rn(mapped[2]));
  } else {
    const float scale = FMT == FMT_U16 ? 65535.0f : 255.0f;
    const float dz = p.dither ? ((float)BAYER8[oy & 7][ox & 7] + 0.5f) / 64.0f - 0.5f : 0.0f;
    float code[3];
    quantize_srgb3(mapped, scale, dz, code);
    const float q0 = code[0], q1 = code[1], q2 = code[2];
    if (FMT == FMT_U16) {
      unsigned short* d = static_cast<unsigned short*>(p.out) + o;
      d[0] = (unsigned short)q0;
      d[1] = (unsigned short)q1;
      d[2] = (unsigned short)q2;
    } else {
      const unsigned r = (unsigned)q0, g = (unsigned)q1, b = (unsigned)q2;
      unsigned char* d = static_cast<unsigned char*>(p.out) + o;
      d[0] = (unsigned char)r;
      d[1] = (unsigned char)g;
      d[2] = (unsigned char)b;
      if (p.hist) {
        atomicAdd(&bins[r], 1u);
        atomicAdd(&bins[256 + g], 1u);
        atomicAdd(&bins[512 + b], 1u);
        atomicAdd(&bins[768 + (2126u * r + 7152u * g + 722u * b + 5000u) / 10000u], 1u);
      }
    }
  }
}

// One CTA walks 32x32 output tiles. With chroma compression, a tile's
// out-of-gamut pixels (which need the 16-step bisection, the bulk of the work)
// are queued in shared memory by warp-aggregated appends and mapped in a
// second pass over the queue, so every warp of that pass is full instead of
// carrying the in-gamut lanes of a divergent branch.
struct Deferred {
  float r, g, b;
  int xy;  // local tile coordinate: y * TILE + x
};

template <int FMT, bool SWAP, bool COMPRESS>
__global__ void __launch_bounds__(TILE * ROWS) output_kernel(const OutputParams p) {
  __shared__ unsigned int bins[FMT == FMT_U8 ? 1024 : 1];
  __shared__ unsigned int diag[5];
  __shared__ float stage[SWAP ? 3 : 1][TILE][TILE + 1];
  __shared__ Deferred queue[COMPRESS ? TILE * TILE : 1];
  __shared__ int queued;
  const int tid = threadIdx.x, lane = tid & 31, row = tid >> 5;
  if (FMT == FMT_U8)
    for (int k = tid; k < 1024; k += TILE * ROWS) bins[k] = 0;
  if (tid < 5) diag[tid] = 0;
  unsigned int n_in = 0, n_comp = 0, n_lim = 0, n_clip = 0, n_inv = 0;
  auto count = [&](int st) {
    n_in += st == ST_IN_GAMUT;
    n_comp += st == ST_COMPRESSED;
    n_lim += st == ST_LIMITED;
    n_clip += st == ST_CLIPPED_FALLBACK;
    n_inv += st == ST_INVALID;
  };
  const int tiles_x = (p.OW + TILE - 1) / TILE;
  const long long ntiles = (long long)tiles_x * ((p.OH + TILE - 1) / TILE);
  const long long plane = (long long)p.SW * p.SH;
  for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int ox0 = (int)(t % tiles_x) * TILE, oy0 = (int)(t / tiles_x) * TILE;
    // The previous tile's staged samples and queue are consumed.
    __syncthreads();
    if (COMPRESS && tid == 0) queued = 0;
    if (SWAP) {
      // Output (ox, oy) reads source column top+oy of source row left+ox (both
      // mirrored as the orientation says): stage[c][ox - ox0][oy - oy0], loaded
      // with oy fastest so a warp reads along one source row.
      for (int k = row; k < TILE; k += ROWS) {
        const int ox = ox0 + k, oy = oy0 + lane;
        if (ox < p.OW && oy < p.OH) {
          const int X = p.left + ox, Y = p.top + oy;
          const int sx = p.flip_h ? p.SW - 1 - Y : Y;
          const int sy = p.flip_v ? p.SH - 1 - X : X;
          const long long i = (long long)sy * p.SW + sx;
          stage[0][k][lane] = __ldg(p.in + i);
          stage[1][k][lane] = __ldg(p.in + plane + i);
          stage[2][k][lane] = __ldg(p.in + 2 * plane + i);
        }
      }
    }
    if (SWAP || COMPRESS) __syncthreads();
    for (int k = row; k < TILE; k += ROWS) {
      const int ox = ox0 + lane, oy = oy0 + k;
      const bool valid = ox < p.OW && oy < p.OH;
      float lin[3] = {0.0f, 0.0f, 0.0f}, mapped[3];
      int st = ST_IN_GAMUT;
      if (valid) {
        float v[3];
        if (SWAP) {
          v[0] = stage[0][lane][k];
          v[1] = stage[1][lane][k];
          v[2] = stage[2][lane][k];
        } else {
          const int X = p.left + ox, Y = p.top + oy;
          const int sx = p.flip_h ? p.SW - 1 - X : X;
          const int sy = p.flip_v ? p.SH - 1 - Y : Y;
          const long long i = (long long)sy * p.SW + sx;
          v[0] = __ldg(p.in + i);
          v[1] = __ldg(p.in + plane + i);
          v[2] = __ldg(p.in + 2 * plane + i);
        }
        apply_adjustments(p.adj, v);
#pragma unroll
        for (int r = 0; r < 3; ++r) lin[r] = p.m[3 * r] * v[0] + p.m[3 * r + 1] * v[1] + p.m[3 * r + 2] * v[2];
        st = COMPRESS ? compress_front(lin, p.ceiling, mapped) : clip_rgb(lin, p.ceiling, mapped);
      }
      const bool defer = COMPRESS && valid && st < 0;
      if (COMPRESS) {
        const unsigned int ballot = __ballot_sync(0xffffffffu, defer);
        if (ballot) {
          int base = 0;
          if (lane == 0) base = atomicAdd(&queued, __popc(ballot));
          base = __shfl_sync(0xffffffffu, base, 0);
          if (defer)
            queue[base + __popc(ballot & ((1u << lane) - 1u))] = Deferred{lin[0], lin[1], lin[2], k * TILE + lane};
        }
      }
      if (valid && !defer) {
        count(st);
        encode_pixel<FMT>(p, ox, oy, mapped, bins);
      }
    }
    if (COMPRESS) {
      __syncthreads();
      const int n = queued;
      for (int j = tid; j < n; j += TILE * ROWS) {
        const Deferred d = queue[j];
        const float lin[3] = {d.r, d.g, d.b};
        float mapped[3];
        const int st = compress_out_of_gamut(lin, p.p3, p.ceiling, p.lightness_ceiling, mapped);
        count(st);
        encode_pixel<FMT>(p, ox0 + d.xy % TILE, oy0 + d.xy / TILE, mapped, bins);
      }
    }
  }
  const unsigned int counts[5] = {__reduce_add_sync(0xffffffffu, n_in), __reduce_add_sync(0xffffffffu, n_comp),
                                  __reduce_add_sync(0xffffffffu, n_lim), __reduce_add_sync(0xffffffffu, n_clip),
                                  __reduce_add_sync(0xffffffffu, n_inv)};
  __syncthreads();
  if (lane == 0)
    for (int s = 0; s < 5; ++s)
      if (counts[s]) atomicAdd(&diag[s], counts[s]);
  __syncthreads();
  if (p.gamut && tid < 5 && diag[tid]) atomicAdd(&p.gamut[tid], (unsigned long long)diag[tid]);
  if (FMT == FMT_U8 && p.hist)
    for (int k = tid; k < 1024; k += TILE * ROWS)
      if (bins[k]) atomicAdd(&p.hist[k], (unsigned long long)bins[k]);
}

// ------------------------------------------------------------ self-checks
// Exact sign of (a * 2^ea)^3 - b * 2^eb for a < 2^26 and b < 2^24.
__device__ int compare_cube_exact(unsigned long long a, int ea, unsigned long long b, int eb) {
  unsigned __int128 A = (unsigned __int128)a * a * a, B = b;
  int e1 = 3 * ea, e2 = eb;
  while (e1 > e2) {
    if (A >= ((unsigned __int128)1 << 125)) return 1;
    A <<= 1;
    --e1;
  }
  while (e2 > e1) {
    if (B >= ((unsigned __int128)1 << 125)) return -1;
    B <<= 1;
    --e2;
  }
  return A < B ? -1 : (A > B ? 1 : 0);
}
__device__ void decompose_f32(unsigned int u, unsigned long long* M, int* E) {
  const int ex = (u >> 23) & 255;
  const unsigned int m = u & 0x7fffffu;
  *M = ex == 0 ? m : (m | 0x800000u);
  *E = ex == 0 ? -149 : ex - 150;
}
// Every positive finite f32: is cbrt_rn(x) between the cubes of its two
// neighbouring midpoints? Counts the results that are not.
__global__ void cbrt_check_kernel(unsigned long long* failures) {
  unsigned int bad = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  for (unsigned int u = 1 + blockIdx.x * blockDim.x + threadIdx.x; u < 0x7f800000u; u += stride) {
    const float x = __uint_as_float(u);
    const float y = cbrt_rn(x);
    unsigned long long X, Y;
    int F, E;
    decompose_f32(u, &X, &F);
    decompose_f32(__float_as_uint(y), &Y, &E);
    const bool power_of_two = Y == 0x800000ull && E > -149;
    const int lower = power_of_two ? compare_cube_exact(4 * Y - 1, E - 2, X, F)
                                   : compare_cube_exact(2 * Y - 1, E - 1, X, F);
    const int upper = compare_cube_exact(2 * Y + 1, E - 1, X, F);
    const float neg = cbrt_rn(-x);
    bad += !(lower < 0 && upper > 0) || neg != -y;
  }
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(failures, (unsigned long long)bad);
}
// Largest distance in ulps between powf(x, 1/2.4) and the power computed in
// double and rounded once, over every f32 of (0.0031308, 1].
__global__ void transfer_pow_check_kernel(unsigned int first, unsigned int last, unsigned int* max_ulps) {
  unsigned int worst = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  const float e = 1.0f / 2.4f;
  for (unsigned int u = first + blockIdx.x * blockDim.x + threadIdx.x; u <= last; u += stride) {
    const float x = __uint_as_float(u);
    const int a = __float_as_int(powf(x, e));
    const int b = __float_as_int((float)pow((double)x, (double)e));
    worst = max(worst, (unsigned int)abs(a - b));
  }
  worst = __reduce_max_sync(0xffffffffu, worst);
  if ((threadIdx.x & 31) == 0) atomicMax(max_ulps, worst);
}

// Every f32 of (0.0031308, 1]: transfer_pow_rn against the power computed in
// double and rounded once. Counts the differences.
__global__ void transfer_rn_check_kernel(unsigned int first, unsigned int last, unsigned long long* failures) {
  unsigned int bad = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  const float e = 1.0f / 2.4f;
  for (unsigned int u = first + blockIdx.x * blockDim.x + threadIdx.x; u <= last; u += stride) {
    const float x = __uint_as_float(u);
    bad += transfer_pow_rn(x) != (float)pow((double)x, (double)e);
  }
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(failures, (unsigned long long)bad);
}

// Every f32 of (0.0031308, 1], 8- and 16-bit, with and without dither:
// quantize_srgb3's code against the code of the correctly rounded power.
__global__ void quantize_check_kernel(unsigned int first, unsigned int last, unsigned long long* failures) {
  unsigned int bad = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  const float dithers[3] = {0.0f, (0.0f + 0.5f) / 64.0f - 0.5f, (63.0f + 0.5f) / 64.0f - 0.5f};
  for (unsigned int u = first + blockIdx.x * blockDim.x + threadIdx.x; u <= last; u += stride) {
    const float x = __uint_as_float(u);
    const float r = transfer_pow_rn(x);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const float scale = s ? 65535.0f : 255.0f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float lin[3] = {x, 0.5f, 0.0f};
        float code[3];
        quantize_srgb3(lin, scale, dithers[d], code);
        bad += code[0] != rclamp(transfer_code(r, scale, dithers[d]), 0.0f, scale);
      }
    }
  }
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(failures, (unsigned long long)bad);
}

// Host copy of cbrt_rn's method (std::cbrt in double as the estimate).
float cbrt_rn_host(float x) {
  if (x == 0.0f || !std::isfinite(x)) return x;
  const float ax = std::fabs(x);
  const double d = ax;
  const double yd = std::cbrt(d);
  float r = (float)yd;
  if (yd != (double)r) {
    const bool up = yd > (double)r;
    const float nb = std::nextafter(r, up ? INFINITY : 0.0f);
    const double m = ((double)r + (double)nb) * 0.5;
    const double m2 = m * m;
    const double hi = m2 * m;
    const double lo = std::fma(m2, m, -hi);
    const double diff = (hi - d) + lo;
    if (up ? diff < 0.0 : diff > 0.0) r = nb;
  }
  return std::signbit(x) ? -r : r;
}

// resolve_edge (geometry.rs:180-184).
long long resolve_edge(double normalized, long long dimension) {
  double v = std::round(std::fma(normalized, (double)dimension, 0.0));
  v = std::min(std::max(v, 0.0), (double)dimension);
  return (long long)v;
}

}  // namespace

size_t output_bytes_per_pixel(int format) {
  switch (format) {
    case RD_OUTPUT_SRGB8: return 3;
    case RD_OUTPUT_SRGB16: return 6;
    case RD_OUTPUT_EXTENDED_F32: return 12;
    case RD_OUTPUT_EXTENDED_F16: return 6;
    default: return 0;
  }
}

Status resolve_output_geometry(int W, int H, const rd_output_desc& o, OutputGeometry* g) {
  if (W <= 0 || H <= 0) return Status{RD_INVALID_DIMENSIONS, "empty image"};
  if (output_bytes_per_pixel(o.format) == 0) return Status{RD_INVALID_INPUT, "unknown output format"};
  if (o.primaries != RD_PRIMARIES_SRGB && o.primaries != RD_PRIMARIES_DISPLAY_P3)
    return Status{RD_INVALID_INPUT, "unknown output primaries"};
  if (o.policy != RD_POLICY_CLIP && o.policy != RD_POLICY_CHROMA_COMPRESS)
    return Status{RD_INVALID_INPUT, "unknown output policy"};
  if (o.dither != RD_DITHER_NONE && o.dither != RD_DITHER_ORDERED_8X8)
    return Status{RD_INVALID_INPUT, "unknown dither mode"};
  if (o.orientation < RD_ORIENTATION_NORMAL || o.orientation > RD_ORIENTATION_UNKNOWN)
    return Status{RD_INVALID_INPUT, "unknown orientation"};
  const bool extended = o.format == RD_OUTPUT_EXTENDED_F32 || o.format == RD_OUTPUT_EXTENDED_F16;
  // validate_headroom (rendering.rs:188-194).
  if (extended && !(std::isfinite(o.headroom) && o.headroom >= 1.0f))
    return Status{RD_INVALID_INPUT, "headroom must be finite and at least 1"};
  // Orientation::axes (orientation.rs:41-52): (swap, mirror x, mirror y).
  static const int axes[9][3] = {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {0, 0, 1}, {1, 0, 0},
                                 {1, 0, 1}, {1, 1, 1}, {1, 1, 0}, {0, 0, 0}};
  g->swap = axes[o.orientation][0];
  g->flip_h = axes[o.orientation][1];
  g->flip_v = axes[o.orientation][2];
  g->src_w = W;
  g->src_h = H;
  const long long cw = g->swap ? H : W, ch = g->swap ? W : H;
  long long l = 0, t = 0, r = cw, b = ch;
  if (o.has_crop) {
    // validate_normalized_crop (geometry.rs:166-178).
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(o.crop[k]) || !(o.crop[k] >= 0.0 && o.crop[k] <= 1.0))
        return Status{RD_INVALID_INPUT, "crop edges must be finite and within 0..1"};
    if (!(o.crop[0] < o.crop[2] && o.crop[1] < o.crop[3]))
      return Status{RD_INVALID_INPUT, "crop edges must be ordered"};
    l = resolve_edge(o.crop[0], cw);
    t = resolve_edge(o.crop[1], ch);
    r = resolve_edge(o.crop[2], cw);
    b = resolve_edge(o.crop[3], ch);
    if (l >= r || t >= b) return Status{RD_INVALID_INPUT, "crop resolves below one pixel"};
  }
  g->left = (int)l;
  g->top = (int)t;
  g->width = (int)(r - l);
  g->height = (int)(b - t);
  return Status{};
}

Status run_display_output(Context& ctx, const float* rgb, const rd_color_desc& c, const rd_output_desc& o,
                          const OutputGeometry& g, void* d_out, unsigned long long* d_hist,
                          unsigned long long* d_gamut) {
  OutputParams p{};
  p.in = rgb;
  p.SW = g.src_w;
  p.SH = g.src_h;
  p.adj = adjust_params(c);
  const bool p3 = o.primaries == RD_PRIMARIES_DISPLAY_P3;
  rec2020_to_display(p3 ? XYZ_TO_DISPLAY_P3 : XYZ_TO_SRGB, p.m);
  p.p3 = p3 ? 1 : 0;
  p.compress = o.policy == RD_POLICY_CHROMA_COMPRESS ? 1 : 0;
  const bool extended = o.format == RD_OUTPUT_EXTENDED_F32 || o.format == RD_OUTPUT_EXTENDED_F16;
  p.ceiling = extended ? o.headroom : 1.0f;
  p.lightness_ceiling = cbrt_rn_host(p.ceiling);
  p.dither = !extended && o.dither == RD_DITHER_ORDERED_8X8;
  p.flip_h = g.flip_h;
  p.flip_v = g.flip_v;
  p.left = g.left;
  p.top = g.top;
  p.OW = g.width;
  p.OH = g.height;
  p.out = d_out;
  p.hist = o.format == RD_OUTPUT_SRGB8 ? d_hist : nullptr;
  p.gamut = d_gamut;
  p.adj.extended = extended ? 1 : 0;
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
  if (p.hist) RD_CUDA_TRY(cudaMemsetAsync(p.hist, 0, 1024 * sizeof(unsigned long long), ctx.stream));
  if (p.gamut) RD_CUDA_TRY(cudaMemsetAsync(p.gamut, 0, 5 * sizeof(unsigned long long), ctx.stream));
  const long long tiles = (long long)((g.width + TILE - 1) / TILE) * ((g.height + TILE - 1) / TILE);
  const int grid = (int)std::min<long long>(tiles, (long long)(ctx.sm_count > 0 ? ctx.sm_count : 152) * 8);
  const dim3 block(TILE * ROWS);
#define RD_OUTPUT_LAUNCH(F)                                                                                   \
  if (g.swap && p.compress) RD_LAUNCH(ctx, K_OUTPUT, (output_kernel<F, true, true><<<grid, block, 0, ctx.stream>>>(p)));  \
  else if (g.swap) RD_LAUNCH(ctx, K_OUTPUT, (output_kernel<F, true, false><<<grid, block, 0, ctx.stream>>>(p)));    \
  else if (p.compress) RD_LAUNCH(ctx, K_OUTPUT, (output_kernel<F, false, true><<<grid, block, 0, ctx.stream>>>(p))); \
  else RD_LAUNCH(ctx, K_OUTPUT, (output_kernel<F, false, false><<<grid, block, 0, ctx.stream>>>(p)))
  switch (o.format) {
    case RD_OUTPUT_SRGB8: RD_OUTPUT_LAUNCH(FMT_U8); break;
    case RD_OUTPUT_SRGB16: RD_OUTPUT_LAUNCH(FMT_U16); break;
    case RD_OUTPUT_EXTENDED_F32: RD_OUTPUT_LAUNCH(FMT_F32); break;
    default: RD_OUTPUT_LAUNCH(FMT_F16); break;
  }
#undef RD_OUTPUT_LAUNCH
  const cudaError_t launch = cudaGetLastError();
  if (luts) device_free(ctx, luts, LUT_SET_BYTES);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

Status run_math_check(Context& ctx, int which, uint64_t* result) {
  void* p = nullptr;
  RD_TRY(device_alloc(ctx, 16, &p));
  RD_CUDA_TRY(cudaMemsetAsync(p, 0, 16, ctx.stream));
  const int grid = (ctx.sm_count > 0 ? ctx.sm_count : 152) * 8;
  const float lo = 0.0031308f, one = 1.0f;
  unsigned int first = 0, last = 0;
  std::memcpy(&first, &lo, 4);
  std::memcpy(&last, &one, 4);
  if (which == 0) {
    RD_LAUNCH(ctx, K_OUTPUT, (cbrt_check_kernel<<<grid, 256, 0, ctx.stream>>>(static_cast<unsigned long long*>(p))));
  } else if (which == 1) {
    RD_LAUNCH(ctx, K_OUTPUT,
              (transfer_pow_check_kernel<<<grid, 256, 0, ctx.stream>>>(first + 1, last, static_cast<unsigned int*>(p))));
  } else if (which == 2) {
    RD_LAUNCH(ctx, K_OUTPUT, (transfer_rn_check_kernel<<<grid, 256, 0, ctx.stream>>>(
                                 first + 1, last, static_cast<unsigned long long*>(p))));
  } else {
    RD_LAUNCH(ctx, K_OUTPUT, (quantize_check_kernel<<<grid, 256, 0, ctx.stream>>>(
                                 first + 1, last, static_cast<unsigned long long*>(p))));
  }
  Status st;
  uint64_t v = 0;
  if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&v, p, 8, cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
      cudaStreamSynchronize(ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "math check failed"};
  device_free(ctx, p, 16);
  if (st.ok()) *result = which == 1 ? (v & 0xffffffffull) : v;
  return st;
}

}  // namespace rd
