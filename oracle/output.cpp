// CPU oracle: display and extended-range output of an adjusted linear
// Rec.2020 image. Orientation + crop geometry, clip or OKLCH chroma
// compression into sRGB / Display P3 primaries, the sRGB transfer, 8- and
// 16-bit quantisation with the optional ordered dither, and the gamut-mapping
// diagnostics. Test infrastructure only.
//
//  geometry          crates/core/src/geometry.rs:36-121,166-184;
//                    crates/image/src/orientation.rs:78-170
//  gamut mapping     crates/color/src/gamut.rs:100-222 (clip_linear_rgb,
//                    compress_chroma, sanitize_and_clip, is_in_gamut)
//  OkLab             crates/color/src/oklab.rs:1-60
//  matrices          crates/color/src/matrix.rs:45-61,103-135
//  output transform  crates/core/src/color/display_output.rs:24-59
//  8 / 16-bit        crates/core/src/cpu/stages.rs:1028-1214 (render_display8_cancellable,
//                    render_display_srgb16_with_geometry_and_diagnostics, quantization_dither)
//  extended          crates/core/src/cpu/extended.rs:27-106
//
// The reference takes its cube root and its transfer power from the platform
// libm (f32::cbrt, f32::powf). `ro_set_exact_math(1)` replaces both with the
// correctly rounded functions, the platform-independent definition; the CUDA
// library implements that definition.
#include <cmath>
#include <cstring>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

namespace {

bool g_exact_math = false;

// Correctly rounded f32 cube root: the double cube root rounded to f32, then
// corrected by comparing the cube of the nearest f32 midpoint with x in exact
// integer arithmetic.
typedef unsigned __int128 u128;

// f = M * 2^E with integer M, for a positive finite f32.
void decompose(float f, uint64_t* M, int* E) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  const int ex = (u >> 23) & 255;
  const uint32_t m = u & 0x7fffff;
  if (ex == 0) {
    *M = m;
    *E = -149;
  } else {
    *M = m | 0x800000u;
    *E = ex - 150;
  }
}
// Sign of (a * 2^ea)^3 - b * 2^eb, for a < 2^26 and b < 2^24.
int compare_cube(uint64_t a, int ea, uint64_t b, int eb) {
  u128 A = (u128)a * a * a, B = b;
  int e1 = 3 * ea, e2 = eb;
  while (e1 > e2) {
    if (A >= ((u128)1 << 125)) return 1;
    A <<= 1;
    --e1;
  }
  while (e2 > e1) {
    if (B >= ((u128)1 << 125)) return -1;
    B <<= 1;
    --e2;
  }
  return A < B ? -1 : (A > B ? 1 : 0);
}
float cbrt_correctly_rounded(float x) {
  if (x == 0.0f || !std::isfinite(x)) return x;
  const float ax = std::fabs(x);
  float y = (float)std::cbrt((double)ax);
  uint64_t X, Y;
  int F, E;
  decompose(ax, &X, &F);
  for (int guard = 0; guard < 4; ++guard) {
    decompose(y, &Y, &E);
    // The true root must lie between the midpoints below and above y.
    const bool power_of_two = Y == 0x800000u && E > -149;
    const int lower = power_of_two ? compare_cube(4 * Y - 1, E - 2, X, F) : compare_cube(2 * Y - 1, E - 1, X, F);
    const int upper = compare_cube(2 * Y + 1, E - 1, X, F);
    if (lower >= 0) y = std::nextafter(y, 0.0f);
    else if (upper <= 0) y = std::nextafter(y, INFINITY);
    else break;
  }
  return std::signbit(x) ? -y : y;
}

float cbrt_f(float x) { return g_exact_math ? cbrt_correctly_rounded(x) : std::cbrt(x); }
float transfer_pow(float v) {
  const float e = 1.0f / 2.4f;
  return g_exact_math ? (float)std::pow((double)v, (double)e) : std::pow(v, e);
}

// linear_srgb_to_srgb (crates/color/src/transfer.rs:5-11).
float srgb_encode(float v) { return v <= 0.0031308f ? 12.92f * v : 1.055f * transfer_pow(v) - 0.055f; }

// Matrix3::transform: dot(row, v) = r0*v0 + r1*v1 + r2*v2, left to right.
void transform(const float m[3][3], const float v[3], float out[3]) {
  const float a = v[0], b = v[1], c = v[2];
  for (int r = 0; r < 3; ++r) out[r] = m[r][0] * a + m[r][1] * b + m[r][2] * c;
}

constexpr float REC2020_TO_XYZ[3][3] = {{0.63695806f, 0.1446169f, 0.16888097f},
                                        {0.2627002f, 0.67799807f, 0.059301715f},
                                        {0.0f, 0.028072694f, 1.0609851f}};
constexpr float XYZ_TO_SRGB[3][3] = {{3.24097f, -1.5373832f, -0.49861076f},
                                     {-0.96924365f, 1.8759675f, 0.04155506f},
                                     {0.05563008f, -0.20397696f, 1.0569715f}};
constexpr float XYZ_TO_P3[3][3] = {{2.493497f, -0.9313836f, -0.4027108f},
                                   {-0.829489f, 1.7626641f, 0.0236247f},
                                   {0.0358458f, -0.0761724f, 0.9568845f}};
// Exact conversions between the sRGB and Display P3 primaries (oklab.rs:5-16).
constexpr float P3_TO_SRGB[3][3] = {{1.2249402f, -0.2249402f, 0.0f},
                                    {-0.042057f, 1.042057f, 0.0f},
                                    {-0.0196376f, -0.078636f, 1.0982736f}};
constexpr float SRGB_TO_P3[3][3] = {{0.822462f, 0.177538f, 0.0f},
                                    {0.0331942f, 0.9668058f, 0.0f},
                                    {0.0170826f, 0.0723974f, 0.9105199f}};

// Matrix3::then (matrix.rs:51-61): Iterator::sum starts at -0.0.
void then(const float first[3][3], const float next[3][3], float out[3][3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      float s = -0.0f;
      for (int k = 0; k < 3; ++k) s += next[r][k] * first[k][c];
      out[r][c] = s;
    }
}

// Ottosson's OkLab from linear sRGB and back (oklab.rs:18-48).
void srgb_to_oklab(const float c[3], float lab[3]) {
  const float r = c[0], g = c[1], b = c[2];
  const float l = 0.41222146f * r + 0.53633255f * g + 0.051445995f * b;
  const float m = 0.2119035f * r + 0.6806995f * g + 0.10739696f * b;
  const float s = 0.08830246f * r + 0.28171885f * g + 0.6299787f * b;
  const float lr = cbrt_f(l), mr = cbrt_f(m), sr = cbrt_f(s);
  lab[0] = 0.21045426f * lr + 0.7936178f * mr - 0.004072047f * sr;
  lab[1] = 1.9779985f * lr - 2.4285922f * mr + 0.4505937f * sr;
  lab[2] = 0.025904037f * lr + 0.78277177f * mr - 0.80867577f * sr;
}
void oklab_to_srgb(const float lab[3], float out[3]) {
  const float L = lab[0], a = lab[1], b = lab[2];
  const float lr = L + 0.39633778f * a + 0.21580376f * b;
  const float mr = L - 0.105561346f * a - 0.06385417f * b;
  const float sr = L - 0.08948418f * a - 1.2914855f * b;
  const float l = lr * lr * lr, m = mr * mr * mr, s = sr * sr * sr;
  out[0] = 4.0767417f * l - 3.3077116f * m + 0.23096994f * s;
  out[1] = -1.268438f * l + 2.6097574f * m - 0.34131938f * s;
  out[2] = -0.0041960863f * l - 0.7034186f * m + 1.7076147f * s;
}
// OutputGamut::rgb_to_oklab / oklab_to_rgb (gamut.rs:27-41).
void gamut_to_oklab(bool p3, const float rgb[3], float lab[3]) {
  if (!p3) return srgb_to_oklab(rgb, lab);
  float s[3];
  transform(P3_TO_SRGB, rgb, s);
  srgb_to_oklab(s, lab);
}
void oklab_to_gamut(bool p3, const float lab[3], float rgb[3]) {
  if (!p3) return oklab_to_srgb(lab, rgb);
  float s[3];
  oklab_to_srgb(lab, s);
  transform(SRGB_TO_P3, s, rgb);
}

enum Status { IN_GAMUT = 0, COMPRESSED = 1, LIMITED = 2, CLIPPED_FALLBACK = 3, INVALID = 4 };

bool finite3(const float v[3]) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }
bool in_gamut(const float v[3], float ceiling) {
  for (int c = 0; c < 3; ++c)
    if (!(v[c] >= 0.0f && v[c] <= ceiling)) return false;
  return true;
}
float sanitize_and_clip(float v, float ceiling) {
  if (std::isnan(v) || v == -INFINITY) return 0.0f;
  if (v == INFINITY) return ceiling;
  return rclamp(v, 0.0f, ceiling);
}
void sanitize3(const float in[3], float ceiling, float out[3]) {
  for (int c = 0; c < 3; ++c) out[c] = sanitize_and_clip(in[c], ceiling);
}

// clip_linear_rgb (gamut.rs:110-122).
int clip_rgb(const float rgb[3], float ceiling, float out[3]) {
  const bool finite = finite3(rgb);
  const bool inside = finite && in_gamut(rgb, ceiling);
  sanitize3(rgb, ceiling, out);
  return !finite ? INVALID : (inside ? IN_GAMUT : CLIPPED_FALLBACK);
}

// compress_chroma (gamut.rs:124-182), 16 bisection steps on the a/b scale.
int compress_chroma(const float rgb[3], bool p3, float ceiling, float out[3]) {
  if (!finite3(rgb)) {
    sanitize3(rgb, ceiling, out);
    return INVALID;
  }
  if (in_gamut(rgb, ceiling)) {
    std::memcpy(out, rgb, sizeof(float) * 3);
    return IN_GAMUT;
  }
  float lab[3];
  gamut_to_oklab(p3, rgb, lab);
  if (!finite3(lab)) {
    sanitize3(rgb, ceiling, out);
    return CLIPPED_FALLBACK;
  }
  const float limited = rclamp(lab[0], 0.0f, cbrt_f(ceiling));
  const bool was_limited = limited != lab[0];
  const float chroma = std::hypot(lab[1], lab[2]);
  const int status = was_limited ? LIMITED : COMPRESSED;
  if (chroma <= 1.0e-6f) {
    const float grey[3] = {limited, 0.0f, 0.0f};
    float g[3];
    oklab_to_gamut(p3, grey, g);
    sanitize3(g, ceiling, out);
    return status;
  }
  float lower = 0.0f, upper = 1.0f;
  for (int k = 0; k < 16; ++k) {
    const float scale = (lower + upper) * 0.5f;
    const float cand_lab[3] = {limited, lab[1] * scale, lab[2] * scale};
    float cand[3];
    oklab_to_gamut(p3, cand_lab, cand);
    if (finite3(cand) && in_gamut(cand, ceiling)) lower = scale;
    else upper = scale;
  }
  const float mapped_lab[3] = {limited, lab[1] * lower, lab[2] * lower};
  float mapped[3];
  oklab_to_gamut(p3, mapped_lab, mapped);
  if (!finite3(mapped)) {
    sanitize3(rgb, ceiling, out);
    return CLIPPED_FALLBACK;
  }
  sanitize3(mapped, ceiling, out);
  return status;
}

// quantization_dither (stages.rs:1197-1214): the 8x8 Bayer threshold matrix.
float dither_at(int mode, int x, int y) {
  static const unsigned char bayer[8][8] = {
      {0, 32, 8, 40, 2, 34, 10, 42},  {48, 16, 56, 24, 50, 18, 58, 26}, {12, 44, 4, 36, 14, 46, 6, 38},
      {60, 28, 52, 20, 62, 30, 54, 22}, {3, 35, 11, 43, 1, 33, 9, 41},    {51, 19, 59, 27, 49, 17, 57, 25},
      {15, 47, 7, 39, 13, 45, 5, 37},  {63, 31, 55, 23, 61, 29, 53, 21}};
  if (mode == 0) return 0.0f;
  return ((float)bayer[y & 7][x & 7] + 0.5f) / 64.0f - 0.5f;
}

// resolve_edge (geometry.rs:180-184).
long long resolve_edge(double normalized, long long dimension) {
  double v = std::round(std::fma(normalized, (double)dimension, 0.0));
  if (v < 0.0) v = 0.0;
  if (v > (double)dimension) v = (double)dimension;
  return (long long)v;
}

}  // namespace

extern "C" void ro_set_exact_math(int on) { g_exact_math = on != 0; }
extern "C" float ro_cbrt(float x) { return cbrt_f(x); }
extern "C" float ro_cbrt_correctly_rounded(float x) { return cbrt_correctly_rounded(x); }

// Gamut mapping of one linear pixel in the target primaries (gamut.rs:110-182).
extern "C" int ro_gamut_map(const float rgb[3], int p3, int policy, float ceiling, float out[3]) {
  return policy == 1 ? compress_chroma(rgb, p3 != 0, ceiling, out) : clip_rgb(rgb, ceiling, out);
}
extern "C" void ro_oklab(int p3, const float rgb[3], float lab[3]) { gamut_to_oklab(p3 != 0, rgb, lab); }
extern "C" void ro_oklab_inverse(int p3, const float lab[3], float rgb[3]) { oklab_to_gamut(p3 != 0, lab, rgb); }

extern "C" int ro_output_geometry(int w, int h, const ro_output* o, int* out_w, int* out_h, int crop[4]) {
  if (w <= 0 || h <= 0 || o->orientation < 0 || o->orientation > 8) return -1;
  // OrientationMap::new: Transpose, Rotate90, Transverse and Rotate270 swap the axes.
  const bool swap = o->orientation >= 4 && o->orientation <= 7;
  const long long W = swap ? h : w, H = swap ? w : h;
  long long l = 0, t = 0, r = W, b = H;
  if (o->has_crop) {
    // validate_normalized_crop (geometry.rs:166-178).
    for (int k = 0; k < 4; ++k)
      if (!std::isfinite(o->crop[k]) || !(o->crop[k] >= 0.0 && o->crop[k] <= 1.0)) return -1;
    if (!(o->crop[0] < o->crop[2] && o->crop[1] < o->crop[3])) return -1;
    l = resolve_edge(o->crop[0], W);
    t = resolve_edge(o->crop[1], H);
    r = resolve_edge(o->crop[2], W);
    b = resolve_edge(o->crop[3], H);
    if (l >= r || t >= b) return -1;
  }
  *out_w = (int)(r - l);
  *out_h = (int)(b - t);
  if (crop) {
    crop[0] = (int)l;
    crop[1] = (int)t;
    crop[2] = (int)r;
    crop[3] = (int)b;
  }
  return 0;
}

// OrientationMap::source_coordinate_in_bounds (orientation.rs:150-170) after
// the crop offset (geometry.rs:116-121).
extern "C" void ro_source_coordinate(int w, int h, int orientation, int x, int y, int* sx, int* sy) {
  switch (orientation) {
    case 1: *sx = w - 1 - x; *sy = y; break;               // HorizontalFlip
    case 2: *sx = w - 1 - x; *sy = h - 1 - y; break;       // Rotate180
    case 3: *sx = x; *sy = h - 1 - y; break;               // VerticalFlip
    case 4: *sx = y; *sy = x; break;                       // Transpose
    case 5: *sx = y; *sy = h - 1 - x; break;               // Rotate90
    case 6: *sx = w - 1 - y; *sy = h - 1 - x; break;       // Transverse
    case 7: *sx = w - 1 - y; *sy = x; break;               // Rotate270
    default: *sx = x; *sy = y; break;                      // Normal, Unknown
  }
}

// format 0: display u8 [oh][3*ow]; 1: sRGB u16 [oh][3*ow]; 2: extended linear
// f32 [oh][3*ow] (headroom >= 1). gamut = {in_gamut, compressed, limited,
// clipped_fallback, invalid}. Returns 0, or -1 for invalid geometry/headroom.
extern "C" int ro_render_output(const float* rgb, int w, int h, const ro_output* o, void* out, uint64_t gamut[5]) {
  int ow = 0, oh = 0, crop[4];
  if (ro_output_geometry(w, h, o, &ow, &oh, crop) != 0) return -1;
  const bool extended = o->format == 2;
  // validate_headroom (rendering.rs:188-194).
  if (extended && !(std::isfinite(o->headroom) && o->headroom >= 1.0f)) return -1;
  const float ceiling = extended ? o->headroom : 1.0f;
  const bool p3 = o->primaries == 1;
  float m[3][3];
  then(REC2020_TO_XYZ, p3 ? XYZ_TO_P3 : XYZ_TO_SRGB, m);
  uint64_t counts[5] = {0, 0, 0, 0, 0};
  for (int y = 0; y < oh; ++y)
    for (int x = 0; x < ow; ++x) {
      int sx, sy;
      ro_source_coordinate(w, h, o->orientation, crop[0] + x, crop[1] + y, &sx, &sy);
      const float* s = rgb + ((size_t)sy * w + sx) * 3;
      float lin[3], mapped[3];
      transform(m, s, lin);
      const int status = o->policy == 1 ? compress_chroma(lin, p3, ceiling, mapped) : clip_rgb(lin, ceiling, mapped);
      counts[status]++;
      const size_t i = ((size_t)y * ow + x) * 3;
      if (extended) {
        float* d = static_cast<float*>(out) + i;
        d[0] = mapped[0];
        d[1] = mapped[1];
        d[2] = mapped[2];
        continue;
      }
      const float scale = o->format == 1 ? 65535.0f : 255.0f;
      for (int c = 0; c < 3; ++c) {
        const float enc = srgb_encode(mapped[c]);
        const float q = rclamp(std::round(enc * scale + dither_at(o->dither, x, y)), 0.0f, scale);
        if (o->format == 1) static_cast<uint16_t*>(out)[i + c] = (uint16_t)q;
        else static_cast<uint8_t*>(out)[i + c] = (uint8_t)q;
      }
    }
  if (gamut) std::memcpy(gamut, counts, sizeof(counts));
  return 0;
}
