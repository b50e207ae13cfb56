// CPU oracle: lens optics execution, restated from crates/optics/src/
// {plan,correction,resample}.rs. Test infrastructure only.
//
// The inverse distortion/TCA kernels live in the un-vendored crate
// `lensfun = "=0.7.0"` (Cargo.toml:35). They are restated from the published
// Newton-inversion algorithm as the reference documents it
// (crates/optics/src/radial.rs:5-35, 311-351) and as its in-tree WGSL port
// runs it (crates/gpu/src/spatial/spatial.wgsl:91-178): radius
// rd = sqrt(f64(x*x + y*y)), up to 7 Newton steps in f64, break once
// |F(ru)| < 1e-5, and on non-convergence Poly3 returns NaN while Poly5,
// PTLens and TCA-Poly3 return the input unchanged. Bit parity with the crate
// itself is unpinned.
//
// The remap takes one of two branches per apply, as correction.rs:110-181
// decides it: the radial multiplier table of crates/optics/src/radial.rs
// (1024 knots, pinned freeze boundaries, five refusal guards) when its build
// accepts it, else the per-pixel Newton path.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

namespace {
constexpr double NEWTON_EPS = 0.00001;

void undist(const ro_optics* p, float x, float y, float* ox, float* oy) {
  *ox = x;
  *oy = y;
  if (p->distortion_model == 0) return;
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double a = p->distortion[0], b = p->distortion[1], c = p->distortion[2];
  double ru = rd;
  bool converged = false;
  if (p->distortion_model == 1) {  // Poly3
    const double inv_k1 = (double)(1.0f / p->distortion[0]);
    const double rd_div_k1 = (double)(float)(rd * inv_k1);
    for (int step = 0; step < 7; ++step) {
      const double f = ru * ru * ru + ru * inv_k1 - rd_div_k1;
      if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
      ru -= f / (3.0 * ru * ru + inv_k1);
    }
    if (!converged || ru < 0.0) { *ox = NAN; *oy = NAN; return; }
  } else if (p->distortion_model == 2) {  // Poly5
    for (int step = 0; step < 7; ++step) {
      const double ru2 = ru * ru;
      const double f = ru * (1.0 + a * ru2 + b * ru2 * ru2) - rd;
      if (std::fabs(f) < NEWTON_EPS) { converged = true; break; }
      ru -= f / (1.0 + 3.0 * a * ru2 + 5.0 * b * ru2 * ru2);
    }
    if (!converged || ru < 0.0) return;
  } else {  // PTLens
    for (int step = 0; step < 7; ++step) {
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

void tca_poly3(const float ch[3], float x, float y, float* ox, float* oy) {
  *ox = x;
  *oy = y;
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double v = ch[0], c = ch[1], b = ch[2];
  double ru = rd;
  bool converged = false;
  for (int step = 0; step < 7; ++step) {
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

// plan.rs:448-486 (map_coordinates_values), with scale from the plan.
bool map_coords(const ro_optics* p, double x, double y, float scale, float out[6]) {
  const double cpx = p->center_x * p->norm_unscale, cpy = p->center_y * p->norm_unscale;
  const double mx = cpx + (x - cpx) / (double)scale;
  const double my = cpy + (y - cpy) / (double)scale;
  const double ix = mx * p->norm_scale - p->center_x;
  const double iy = my * p->norm_scale - p->center_y;
  float gx, gy;
  undist(p, (float)ix, (float)iy, &gx, &gy);
  if (!std::isfinite(gx) || !std::isfinite(gy)) return false;
  float n[6] = {gx, gy, gx, gy, gx, gy};
  if (p->tca_model == 1) {
    n[0] = gx * p->tca_red[0];
    n[1] = gy * p->tca_red[0];
    n[4] = gx * p->tca_blue[0];
    n[5] = gy * p->tca_blue[0];
  } else if (p->tca_model == 2) {
    tca_poly3(p->tca_red, gx, gy, &n[0], &n[1]);
    tca_poly3(p->tca_blue, gx, gy, &n[4], &n[5]);
  }
  for (int c = 0; c < 3; ++c) {
    out[2 * c] = (float)(((double)n[2 * c] + p->center_x) * p->norm_unscale);
    out[2 * c + 1] = (float)(((double)n[2 * c + 1] + p->center_y) * p->norm_unscale);
    if (!std::isfinite(out[2 * c]) || !std::isfinite(out[2 * c + 1])) return false;
  }
  return true;
}

// plan.rs:537-559
bool perimeter_is_safe(const ro_optics* p, float scale) {
  const int max_x = p->width - 1, max_y = p->height - 1;
  for (int index = 0; index < 64; ++index) {
    const float t = (float)index / 63.0f;
    const float pts[4][2] = {{t * (float)max_x, 0.0f},
                             {t * (float)max_x, (float)max_y},
                             {0.0f, t * (float)max_y},
                             {(float)max_x, t * (float)max_y}};
    for (auto& pt : pts) {
      float c[6];
      // `x as usize` truncates the f32 perimeter coordinate.
      if (!map_coords(p, (double)(std::size_t)pt[0], (double)(std::size_t)pt[1], scale, c)) return false;
      for (int k = 0; k < 3; ++k)
        if (!(c[2 * k] >= 1.0f && c[2 * k + 1] >= 1.0f && c[2 * k] <= (float)(p->width - 2) &&
              c[2 * k + 1] <= (float)(p->height - 2)))
          return false;
    }
  }
  return true;
}

// resample.rs:43-54
float cubic_weight(float distance) {
  const float a = std::fabs(distance);
  if (a <= 1.0f) return 1.5f * a * a * a - 2.5f * a * a + 1.0f;
  if (a < 2.0f) return -0.5f * a * a * a + 2.5f * a * a - 4.0f * a + 2.0f;
  return 0.0f;
}

// resample.rs:3-41
bool cubic_sample(const float* data, int w, int h, int channel, float x, float y, float* out) {
  if (!std::isfinite(x) || !std::isfinite(y)) return false;
  const long fx = (long)std::floor(x), fy = (long)std::floor(y);
  if (fx - 1 < 0 || fy - 1 < 0 || fx + 2 >= w || fy + 2 >= h) return false;
  float value = 0.0f;
  for (int oy = -1; oy <= 2; ++oy) {
    const float wy = cubic_weight(y - (float)(fy + oy));
    const long sy = fy + oy;
    for (int ox = -1; ox <= 2; ++ox) {
      const float weight = wy * cubic_weight(x - (float)(fx + ox));
      value += data[(std::size_t)sy * 3 * w + 3 * (std::size_t)(fx + ox) + channel] * weight;
    }
  }
  if (!std::isfinite(value)) return false;
  *out = value;
  return true;
}

// ---- radial multiplier table (crates/optics/src/radial.rs) ----------------
constexpr int KNOTS = 1024;                    // radial.rs:85
constexpr float TRIPWIRE_TOLERANCE = 1e-4f;    // radial.rs:98
constexpr float JUMP_LIMIT = 1e-3f;            // radial.rs:102
constexpr int BISECTION_STEPS = 30;            // radial.rs:105
constexpr float FREEZE_NOISE_ULPS = 8.0f;      // radial.rs:111
constexpr float AMBIGUOUS_BAND_ULPS = 16.0f;   // radial.rs:121
constexpr float DIRECTION = 0.70710677f;       // FRAC_1_SQRT_2 as f32
enum Kernel { DISTORTION = 0, TCA_RED = 1, TCA_BLUE = 2 };

struct Flip {
  int index;
  Kernel kernel;
  float radius;
};

struct Radial {
  int guard = -1;  // -1 no table, 0 accepted, 1..5 the refusal (RD_RADIAL_* order)
  float step = 0.0f;
  std::vector<float> table;  // [KNOTS][3]
  std::vector<std::pair<int, float>> segments;
};

// plan.rs:119-130, narrowed where the branch narrows.
float input_x(const ro_optics* p, int x) {
  const double cpx = p->center_x * p->norm_unscale;
  return (float)((cpx + ((double)x - cpx) / (double)p->scale) * p->norm_scale - p->center_x);
}
float input_y(const ro_optics* p, int y) {
  const double cpy = p->center_y * p->norm_unscale;
  return (float)((cpy + ((double)y - cpy) / (double)p->scale) * p->norm_scale - p->center_y);
}

// radial.rs:272-307
void knot_multipliers(const ro_optics* p, float x, float y, float m[3]) {
  float gx, gy;
  undist(p, x, y, &gx, &gy);
  const float in_sq = x * x + y * y;
  const float sf = in_sq > 0.0f ? (gx * x + gy * y) / in_sq : 1.0f;
  m[0] = m[1] = m[2] = sf;
  if (p->tca_model == 1) {
    m[0] = sf * p->tca_red[0];
    m[2] = sf * p->tca_blue[0];
  } else if (p->tca_model == 2) {
    float rx, ry, bx, by;
    tca_poly3(p->tca_red, gx, gy, &rx, &ry);
    tca_poly3(p->tca_blue, gx, gy, &bx, &by);
    const float g_sq = gx * gx + gy * gy;
    if (g_sq > 0.0f) {
      m[0] *= (rx * gx + ry * gy) / g_sq;
      m[2] *= (bx * gx + by * gy) / g_sq;
    }
  }
}

// radial.rs:315-338
bool step0_break_distortion(const ro_optics* p, float x, float y) {
  const double rd = std::sqrt((double)(x * x + y * y));
  if (rd == 0.0) return true;
  double residual;
  if (p->distortion_model == 1) {
    const double inv_k1 = (double)(1.0f / p->distortion[0]);
    const double rd_div_k1 = (double)(float)(rd * inv_k1);
    residual = rd * rd * rd + rd * inv_k1 - rd_div_k1;
  } else if (p->distortion_model == 2) {
    const double rs = rd * rd;
    residual = rd * (1.0 + (double)p->distortion[0] * rs + (double)p->distortion[1] * rs * rs) - rd;
  } else if (p->distortion_model == 3) {
    const double a = p->distortion[0], b = p->distortion[1], c = p->distortion[2];
    residual = rd * (a * rd * rd * rd + b * rd * rd + c * rd + 1.0) - rd;
  } else {
    return false;
  }
  return std::fabs(residual) < NEWTON_EPS;
}

// radial.rs:342-350
bool step0_break_tca(const float ch[3], float gx, float gy) {
  const double rd = std::sqrt((double)(gx * gx + gy * gy));
  if (rd == 0.0) return true;
  const double v = ch[0], c = ch[1], b = ch[2];
  const double residual = b * rd * rd * rd + c * rd * rd + v * rd - rd;
  return std::fabs(residual) < NEWTON_EPS;
}

// radial.rs:352-376
bool break_predicate(const ro_optics* p, Kernel k, double radius) {
  const float r = (float)radius;
  const float x = r * DIRECTION, y = r * DIRECTION;
  if (k == DISTORTION) return step0_break_distortion(p, x, y);
  float gx, gy;
  undist(p, x, y, &gx, &gy);
  if (p->tca_model != 2) return false;
  return step0_break_tca(k == TCA_RED ? p->tca_red : p->tca_blue, gx, gy);
}

// radial.rs:381-394
double bisect_break(const ro_optics* p, Kernel k, double low, double high) {
  const bool low_state = break_predicate(p, k, low);
  for (int i = 0; i < BISECTION_STEPS; ++i) {
    const double middle = (low + high) * 0.5;
    if (break_predicate(p, k, middle) == low_state) low = middle;
    else high = middle;
  }
  return high;
}

// radial.rs:494-496 (ulp from the wider side of a binade boundary).
float ulp32(float v) { return std::fabs(v - std::nextafter(v, -INFINITY)); }

// radial.rs:585-600
double radius_band(double kernel_radius, double slope, double truncation) {
  return (double)FREEZE_NOISE_ULPS * (double)ulp32((float)kernel_radius) + truncation / slope;
}
float band_to_f32(double band) { return band > (double)FLT_MAX ? INFINITY : (float)band; }

// radial.rs:521-581
float freeze_ambiguity_band(const ro_optics* p, Kernel k, float br) {
  if (k == DISTORTION) {
    const float x = br * DIRECTION, y = br * DIRECTION;
    const double r = std::sqrt((double)(x * x + y * y));
    double slope = 0.0, truncation = 0.0;
    if (p->distortion_model == 1) {
      slope = 3.0 * r * r;
      truncation = (double)ulp32((float)(r * (double)(1.0f / p->distortion[0])));
    } else if (p->distortion_model == 2) {
      const double r4 = (r * r) * (r * r);
      slope = std::fabs(3.0 * (double)p->distortion[0] * r * r + 5.0 * (double)p->distortion[1] * r4);
    } else if (p->distortion_model == 3) {
      const double r3 = (r * r) * r;
      slope = std::fabs(4.0 * (double)p->distortion[0] * r3 + 3.0 * (double)p->distortion[1] * r * r +
                        2.0 * (double)p->distortion[2] * r);
    }
    return band_to_f32(radius_band(r, slope, truncation));
  }
  const float x = br * DIRECTION;
  float gx, gy;
  undist(p, x, x, &gx, &gy);
  const double gr = std::sqrt((double)(gx * gx + gy * gy));
  if (p->tca_model != 2) return INFINITY;
  const float* ch = k == TCA_RED ? p->tca_red : p->tca_blue;
  const double v = ch[0], c = ch[1], b = ch[2];
  const double slope = std::fabs(3.0 * b * gr * gr + 2.0 * c * gr + v - 1.0);
  const double h = (double)br * 1e-4;
  const float high = (float)((double)br + h) * DIRECTION;
  const float low = (float)((double)br - h) * DIRECTION;
  float hx, hy, lx, ly;
  undist(p, high, high, &hx, &hy);
  undist(p, low, low, &lx, &ly);
  const double high_r = std::sqrt((double)(hx * hx + hy * hy));
  const double low_r = std::sqrt((double)(lx * lx + ly * ly));
  const double scale = std::fabs((high_r - low_r) / (2.0 * h));
  return band_to_f32(radius_band(gr, slope, 0.0) / scale);
}

// radial.rs:232-246: hypot of the four mapped corners.
float corner_input_radius(const ro_optics* p) {
  float radius = 0.0f;
  const int xs[2] = {0, p->width - 1}, ys[2] = {0, p->height - 1};
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 2; ++i) {
      const float h = std::hypot(input_x(p, xs[i]), input_y(p, ys[j]));
      radius = std::fmax(radius, h);  // f32::max ignores NaN
    }
  return radius;
}

// RadialMultipliers::build + assess (radial.rs:172-208, 400-491).
Radial build_radial(const ro_optics* p) {
  Radial t;
  if (p->distortion_model == 0 && p->tca_model == 0) return t;
  const float corner = corner_input_radius(p);
  if (!(std::isfinite(corner) && corner > 0.0f)) return t;
  t.step = corner / (float)(KNOTS - 1);
  t.table.resize(3 * KNOTS);
  bool tripwire_ok = true;
  for (int i = 0; i < KNOTS; ++i) {
    const float radius = (float)i * t.step;
    float m[3], straight[3];
    knot_multipliers(p, radius * DIRECTION, radius * DIRECTION, m);
    knot_multipliers(p, radius, 0.0f, straight);
    for (int c = 0; c < 3; ++c) {
      const float margin = std::fabs(m[c] - straight[c]) / std::fmax(std::fabs(m[c]), 1e-3f);
      if (std::isnan(margin) || margin > TRIPWIRE_TOLERANCE) tripwire_ok = false;
      t.table[3 * i + c] = m[c];
    }
  }
  int guard = 0;
  auto refuse = [&](int g) {
    if (guard == 0) guard = g;
  };
  for (float v : t.table)
    if (!std::isfinite(v)) refuse(1);
  std::vector<Kernel> kernels;
  if (p->distortion_model != 0) kernels.push_back(DISTORTION);
  if (p->tca_model == 2) {
    kernels.push_back(TCA_RED);
    kernels.push_back(TCA_BLUE);
  }
  std::vector<Flip> flips;
  for (Kernel k : kernels) {
    bool previous = break_predicate(p, k, 0.0);
    for (int i = 1; i < KNOTS; ++i) {
      const double radius = (double)((float)i * t.step);
      const bool current = break_predicate(p, k, radius);
      if (current != previous) {
        const double low = (double)((float)(i - 1) * t.step);
        flips.push_back({i - 1, k, (float)bisect_break(p, k, low, radius)});
      }
      previous = current;
    }
  }
  std::stable_sort(flips.begin(), flips.end(), [](const Flip& a, const Flip& b) {
    return a.index != b.index ? a.index < b.index : (int)a.kernel < (int)b.kernel;
  });
  for (const Flip& f : flips) {
    if (!t.segments.empty() && t.segments.back().first == f.index) refuse(3);
    else t.segments.push_back({f.index, f.radius});
  }
  if (guard == 0) {
    for (const Flip& f : flips) {
      const float band = freeze_ambiguity_band(p, f.kernel, f.radius);
      if (std::isnan(band) || band > AMBIGUOUS_BAND_ULPS * ulp32(f.radius)) {
        guard = 4;
        break;
      }
    }
  }
  for (int i = 0; i + 1 < KNOTS; ++i)
    for (int c = 0; c < 3; ++c) {
      bool attributed = false;
      for (const Flip& f : flips)
        if (f.index == i && (f.kernel == DISTORTION || (c == 0 && f.kernel == TCA_RED) ||
                             (c == 2 && f.kernel == TCA_BLUE)))
          attributed = true;
      if (std::fabs(t.table[3 * (i + 1) + c] - t.table[3 * i + c]) > JUMP_LIMIT && !attributed) refuse(5);
    }
  if (guard == 0 && !tripwire_ok) guard = 2;
  t.guard = guard;
  return t;
}

// RadialMultipliers::lookup (radial.rs:212-229).
void radial_lookup(const Radial& t, float radius, float m[3]) {
  const float position = radius / t.step;
  const int index = std::min((int)position, KNOTS - 2);
  for (const auto& s : t.segments)
    if (s.first == index) {
      const int k = index + (radius >= s.second ? 1 : 0);
      for (int c = 0; c < 3; ++c) m[c] = t.table[3 * k + c];
      return;
    }
  float blend = position - (float)index;
  if (blend > 1.0f) blend = 1.0f;
  for (int c = 0; c < 3; ++c) m[c] = t.table[3 * index + c] * (1.0f - blend) + t.table[3 * (index + 1) + c] * blend;
}

// The table branch's coordinates (correction.rs:122-151): one lookup at the
// pixel's input radius, then plan.rs:136-141 per channel.
bool map_coords_lut(const ro_optics* p, const Radial& t, int x, int y, float out[6]) {
  const float ix = input_x(p, x), iy = input_y(p, y);
  float m[3];
  radial_lookup(t, std::hypot(ix, iy), m);
  for (int c = 0; c < 3; ++c) {
    out[2 * c] = (float)(((double)(ix * m[c]) + p->center_x) * p->norm_unscale);
    out[2 * c + 1] = (float)(((double)(iy * m[c]) + p->center_y) * p->norm_unscale);
  }
  return true;
}
}  // namespace

// plan.rs:173-231 (geometry constants) and :521-535 (find_scale).
extern "C" int ro_optics_plan(ro_optics* p, float crop, float real_focal, float lens_cx, float lens_cy) {
  const double wf = p->width >= 2 ? (double)(p->width - 1) : 1.0;
  const double hf = p->height >= 2 ? (double)(p->height - 1) : 1.0;
  p->norm_scale = std::hypot(36.0, 24.0) / (double)crop / std::hypot(wf + 1.0, hf + 1.0) / (double)real_focal;
  p->norm_unscale = 1.0 / p->norm_scale;
  const double lens_size = std::min(wf, hf);
  p->center_x = (wf / 2.0 + lens_size / 2.0 * (double)lens_cx) * p->norm_scale;
  p->center_y = (hf / 2.0 + lens_size / 2.0 * (double)lens_cy) * p->norm_scale;
  p->scale = 1.0f;
  if (p->distortion_model == 0 && p->tca_model == 0) return 0;
  float scale = 1.0f;
  for (int i = 0; i < 160; ++i) {
    if (perimeter_is_safe(p, scale)) {
      p->scale = scale;
      return 0;
    }
    scale *= 1.025f;
  }
  return -1;
}

extern "C" int ro_optics_map(const ro_optics* p, int x, int y, float coords[6]) {
  return map_coords(p, (double)x, (double)y, p->scale, coords) ? 0 : -1;
}

extern "C" int ro_optics_apply(const ro_optics* p, const float* rgb_in, float* rgb_out) {
  const int w = p->width, h = p->height;
  std::vector<float> img(rgb_in, rgb_in + (std::size_t)w * h * 3);
  // apply_vignetting, correction.rs:213-267 (incremental radius, f32).
  if (p->vignetting_model == 1) {
    const float k1 = p->vignetting[0], k2 = p->vignetting[1], k3 = p->vignetting[2];
    const float ns = (float)p->norm_scale;
    const float step = 2.0f * ns, step_sq = ns * ns;
    const float start_x = (float)(-p->center_x), start_y = (float)(-p->center_y);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int row = 0; row < h; ++row) {
      const float y = start_y + ns * (float)row;
      float x = start_x;
      float r2 = x * x + y * y;
      for (int col = 0; col < w; ++col) {
        const float r4 = r2 * r2, r6 = r4 * r2;
        const float gain = 1.0f + k1 * r2 + k2 * r4 + k3 * r6;
        if (!std::isfinite(gain) || gain == 0.0f) { bad |= 1; break; }
        const float mult = 1.0f / gain;
        float* px = img.data() + ((std::size_t)row * w + col) * 3;
        for (int c = 0; c < 3; ++c) px[c] *= mult;
        r2 += step * x + step_sq;
        x += ns;
      }
    }
    if (bad) return -2;
  }
  if (p->distortion_model == 0 && p->tca_model == 0) {
    std::copy(img.begin(), img.end(), rgb_out);
    return 0;
  }
  const Radial table = build_radial(p);
  const bool lut = table.guard == 0;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float c[6];
      const bool mapped = lut ? map_coords_lut(p, table, x, y, c) : map_coords(p, (double)x, (double)y, p->scale, c);
      if (!mapped) { bad |= 1; continue; }
      for (int ch = 0; ch < 3; ++ch)
        if (!cubic_sample(img.data(), w, h, ch, c[2 * ch], c[2 * ch + 1], &rgb_out[((std::size_t)y * w + x) * 3 + ch]))
          bad |= 2;
    }
  return bad ? -3 : 0;
}

extern "C" int ro_optics_radial(const ro_optics* p, float* table, float* step, int* seg_index, float* seg_radius,
                                int max_segments, int* n_segments) {
  const Radial t = build_radial(p);
  if (t.guard >= 0) {
    if (table) std::copy(t.table.begin(), t.table.end(), table);
    if (step) *step = t.step;
    const int n = (int)t.segments.size();
    if (n_segments) *n_segments = n;
    for (int i = 0; i < n && i < max_segments; ++i) {
      seg_index[i] = t.segments[i].first;
      seg_radius[i] = t.segments[i].second;
    }
  }
  return t.guard;
}

extern "C" int ro_optics_map_lut(const ro_optics* p, int x, int y, float coords[6]) {
  const Radial t = build_radial(p);
  if (t.guard < 0) return -1;
  return map_coords_lut(p, t, x, y, coords) ? 0 : -1;
}
