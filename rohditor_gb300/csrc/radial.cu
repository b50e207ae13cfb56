// Radial multiplier table of the optics remap (RadialMultipliers,
// crates/optics/src/radial.rs:157-491), built on the host once per apply.
//
// Every inverse kernel of the lens model maps (x, y) to (x, y) * f(|(x, y)|),
// so each channel's source coordinate is the input coordinate times a
// multiplier that depends on the input radius only. The reference tabulates
// the multipliers at 1024 uniform radii from the centre to the farthest
// mapped corner and, when the table passes its guards, remaps every pixel
// through a lookup instead of the per-pixel Newton solves. This file
// restates the build: the knots (radial.rs:172-208, 272-307), the step-0
// freeze boundaries located by f64 bisection and pinned (radial.rs:315-394,
// 400-453), and the five refusal rules (non-finite knot, radiality tripwire,
// two flips in one segment, ambiguous freeze band, unexplained jump;
// radial.rs:141-156, 453-491, 521-600). A refused table leaves the apply on
// the Newton path, as correction.rs:110-121 does.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "lens_model.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr float TRIPWIRE_TOLERANCE = 1e-4f;   // radial.rs:98
constexpr float JUMP_LIMIT = 1e-3f;           // radial.rs:102
constexpr int BISECTION_STEPS = 30;           // radial.rs:105
constexpr float FREEZE_NOISE_ULPS = 8.0f;     // radial.rs:111
constexpr float AMBIGUOUS_BAND_ULPS = 16.0f;  // radial.rs:121
constexpr float DIAGONAL = 0.70710677f;       // FRAC_1_SQRT_2 as f32: knots sit on the 45 degree ray

enum BreakKernel { BREAK_DISTORTION = 0, BREAK_TCA_RED = 1, BREAK_TCA_BLUE = 2 };

struct Flip {
  int segment;
  BreakKernel kernel;
  float radius;
};

void distort(const rd_optics_desc& o, float x, float y, float& gx, float& gy) {
  lens_undistort(o.distortion_model, o.distortion[0], o.distortion[1], o.distortion[2], x, y, gx, gy);
}

// The exact per-channel multiplier at one input coordinate (radial.rs:272-307).
void knot(const rd_optics_desc& o, float x, float y, float m[3]) {
  float gx, gy;
  distort(o, x, y, gx, gy);
  const float in_sq = x * x + y * y;
  const float s = in_sq > 0.0f ? (gx * x + gy * y) / in_sq : 1.0f;
  m[0] = m[1] = m[2] = s;
  if (o.tca_model == RD_TCA_LINEAR) {
    m[0] = s * o.tca_red[0];
    m[2] = s * o.tca_blue[0];
  } else if (o.tca_model == RD_TCA_POLY3) {
    float rx, ry, bx, by;
    lens_tca_poly3(o.tca_red, gx, gy, rx, ry);
    lens_tca_poly3(o.tca_blue, gx, gy, bx, by);
    const float g_sq = gx * gx + gy * gy;
    if (g_sq > 0.0f) {
      m[0] *= (rx * gx + ry * gy) / g_sq;
      m[2] *= (bx * gx + by * gy) / g_sq;
    }
  }
}

// Does the kernel break before its first Newton step at this coordinate
// (radial.rs:315-350)? The multiplier is then exactly 1.
bool distortion_frozen(const rd_optics_desc& o, float x, float y) {
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return true;
  const double a = o.distortion[0], b = o.distortion[1], c = o.distortion[2];
  double residual;
  switch (o.distortion_model) {
    case RD_DISTORTION_POLY3: {
      const double inv_k1 = (double)(1.0f / o.distortion[0]);
      const double rd_div_k1 = (double)(float)(rd * inv_k1);
      residual = rd * rd * rd + rd * inv_k1 - rd_div_k1;
      break;
    }
    case RD_DISTORTION_POLY5: {
      const double rs = rd * rd;
      residual = rd * (1.0 + a * rs + b * rs * rs) - rd;
      break;
    }
    case RD_DISTORTION_PTLENS:
      residual = rd * (a * rd * rd * rd + b * rd * rd + c * rd + 1.0) - rd;
      break;
    default:
      return false;
  }
  return std::fabs(residual) < LENS_NEWTON_EPS;
}

bool tca_frozen(const float ch[3], float gx, float gy) {
  const double rd = std::sqrt((double)(gx * gx + gy * gy));
  if (rd == 0.0) return true;
  const double v = ch[0], c = ch[1], b = ch[2];
  return std::fabs(b * rd * rd * rd + c * rd * rd + v * rd - rd) < LENS_NEWTON_EPS;
}

// The step-0 state on the 45 degree ray at an f64 radius (radial.rs:352-376).
bool frozen_at(const rd_optics_desc& o, BreakKernel k, double radius) {
  const float r = (float)radius;
  const float x = r * DIAGONAL, y = r * DIAGONAL;
  if (k == BREAK_DISTORTION) return distortion_frozen(o, x, y);
  float gx, gy;
  distort(o, x, y, gx, gy);
  if (o.tca_model != RD_TCA_POLY3) return false;
  return tca_frozen(k == BREAK_TCA_RED ? o.tca_red : o.tca_blue, gx, gy);
}

// radial.rs:381-394: the flip's radius on the side opposite the low end.
double bisect(const rd_optics_desc& o, BreakKernel k, double low, double high) {
  const bool low_state = frozen_at(o, k, low);
  for (int i = 0; i < BISECTION_STEPS; ++i) {
    const double middle = (low + high) * 0.5;
    if (frozen_at(o, k, middle) == low_state) low = middle;
    else high = middle;
  }
  return high;
}

// Gap to the next f32 below (radial.rs:494-496).
float ulp_below(float v) { return std::fabs(v - std::nextafter(v, -INFINITY)); }

double radius_band(double kernel_radius, double slope, double truncation) {
  return (double)FREEZE_NOISE_ULPS * (double)ulp_below((float)kernel_radius) + truncation / slope;
}
float narrow_band(double band) { return band > (double)FLT_MAX ? INFINITY : (float)band; }

// Input-radius band around a pinned break inside which a pixel's own step-0
// decision may differ from the bisection's (radial.rs:521-581).
float freeze_band(const rd_optics_desc& o, BreakKernel k, float br) {
  if (k == BREAK_DISTORTION) {
    const float x = br * DIAGONAL, y = br * DIAGONAL;
    const double r = std::sqrt((double)(x * x + y * y));
    const double a = o.distortion[0], b = o.distortion[1], c = o.distortion[2];
    double slope = 0.0, truncation = 0.0;
    if (o.distortion_model == RD_DISTORTION_POLY3) {
      slope = 3.0 * r * r;
      truncation = (double)ulp_below((float)(r * (double)(1.0f / o.distortion[0])));
    } else if (o.distortion_model == RD_DISTORTION_POLY5) {
      slope = std::fabs(3.0 * a * r * r + 5.0 * b * ((r * r) * (r * r)));
    } else if (o.distortion_model == RD_DISTORTION_PTLENS) {
      slope = std::fabs(4.0 * a * ((r * r) * r) + 3.0 * b * r * r + 2.0 * c * r);
    }
    return narrow_band(radius_band(r, slope, truncation));
  }
  if (o.tca_model != RD_TCA_POLY3) return INFINITY;
  const float x = br * DIAGONAL;
  float gx, gy;
  distort(o, x, x, gx, gy);
  const double gr = std::sqrt((double)(gx * gx + gy * gy));
  const float* ch = k == BREAK_TCA_RED ? o.tca_red : o.tca_blue;
  const double v = ch[0], c = ch[1], b = ch[2];
  const double slope = std::fabs(3.0 * b * gr * gr + 2.0 * c * gr + v - 1.0);
  const double h = (double)br * 1e-4;
  const float high = (float)((double)br + h) * DIAGONAL;
  const float low = (float)((double)br - h) * DIAGONAL;
  float hx, hy, lx, ly;
  distort(o, high, high, hx, hy);
  distort(o, low, low, lx, ly);
  const double high_r = std::sqrt((double)(hx * hx + hy * hy));
  const double low_r = std::sqrt((double)(lx * lx + ly * ly));
  const double scale = std::fabs((high_r - low_r) / (2.0 * h));
  return narrow_band(radius_band(gr, slope, 0.0) / scale);
}

}  // namespace

RadialTable build_radial_table(const rd_optics_desc& o, const float* input_x, const float* input_y) {
  RadialTable t;
  if (o.distortion_model == RD_DISTORTION_NONE && o.tca_model == RD_TCA_NONE) return t;
  const int W = (int)o.width, H = (int)o.height;
  float corner = 0.0f;  // radial.rs:232-246; f32::max keeps the non-NaN side
  for (int cy : {0, H - 1})
    for (int cx : {0, W - 1}) corner = std::fmax(corner, std::hypot(input_x[cx], input_y[cy]));
  if (!(std::isfinite(corner) && corner > 0.0f)) return t;
  t.step = corner / (float)(RADIAL_KNOTS - 1);
  std::vector<float> m(3 * RADIAL_KNOTS);
  bool radial = true;
  for (int i = 0; i < RADIAL_KNOTS; ++i) {
    const float r = (float)i * t.step;
    float diag[3], axis[3];
    knot(o, r * DIAGONAL, r * DIAGONAL, diag);
    knot(o, r, 0.0f, axis);
    for (int c = 0; c < 3; ++c) {
      const float margin = std::fabs(diag[c] - axis[c]) / std::fmax(std::fabs(diag[c]), 1e-3f);
      if (std::isnan(margin) || margin > TRIPWIRE_TOLERANCE) radial = false;
      m[3 * i + c] = diag[c];
    }
  }
  int guard = RD_RADIAL_ACCEPTED;
  auto refuse = [&](int rule) {
    if (guard == RD_RADIAL_ACCEPTED) guard = rule;
  };
  for (float v : m)
    if (!std::isfinite(v)) refuse(RD_RADIAL_NON_FINITE);
  std::vector<BreakKernel> kernels;
  if (o.distortion_model != RD_DISTORTION_NONE) kernels.push_back(BREAK_DISTORTION);
  if (o.tca_model == RD_TCA_POLY3) {
    kernels.push_back(BREAK_TCA_RED);
    kernels.push_back(BREAK_TCA_BLUE);
  }
  std::vector<Flip> flips;
  for (BreakKernel k : kernels) {
    bool previous = frozen_at(o, k, 0.0);
    for (int i = 1; i < RADIAL_KNOTS; ++i) {
      const double r = (double)((float)i * t.step);
      const bool current = frozen_at(o, k, r);
      if (current != previous) flips.push_back({i - 1, k, (float)bisect(o, k, (double)((float)(i - 1) * t.step), r)});
      previous = current;
    }
  }
  std::stable_sort(flips.begin(), flips.end(), [](const Flip& a, const Flip& b) {
    return a.segment != b.segment ? a.segment < b.segment : (int)a.kernel < (int)b.kernel;
  });
  std::vector<float> pin(RADIAL_KNOTS, NAN);
  int last = -1;
  for (const Flip& f : flips) {
    if (f.segment == last) {
      refuse(RD_RADIAL_BREAK_COLLISION);
      continue;
    }
    pin[f.segment] = f.radius;
    last = f.segment;
  }
  if (guard == RD_RADIAL_ACCEPTED)
    for (const Flip& f : flips) {
      const float band = freeze_band(o, f.kernel, f.radius);
      if (std::isnan(band) || band > AMBIGUOUS_BAND_ULPS * ulp_below(f.radius)) {
        guard = RD_RADIAL_FREEZE_AMBIGUITY;
        break;
      }
    }
  for (int i = 0; i + 1 < RADIAL_KNOTS; ++i)
    for (int c = 0; c < 3; ++c) {
      if (!(std::fabs(m[3 * (i + 1) + c] - m[3 * i + c]) > JUMP_LIMIT)) continue;
      bool explained = false;  // green follows the distortion flip only, red / blue also their own channel
      for (const Flip& f : flips)
        if (f.segment == i && (f.kernel == BREAK_DISTORTION || (c == 0 && f.kernel == BREAK_TCA_RED) ||
                               (c == 2 && f.kernel == BREAK_TCA_BLUE)))
          explained = true;
      if (!explained) refuse(RD_RADIAL_UNEXPLAINED_JUMP);
    }
  if (guard == RD_RADIAL_ACCEPTED && !radial) guard = RD_RADIAL_TRIPWIRE;
  t.guard = guard;
  t.knots.resize(4 * RADIAL_KNOTS);
  for (int i = 0; i < RADIAL_KNOTS; ++i) {
    for (int c = 0; c < 3; ++c) t.knots[4 * i + c] = m[3 * i + c];
    t.knots[4 * i + 3] = pin[i];
  }
  return t;
}

}  // namespace rd
