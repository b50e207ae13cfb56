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
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float c[6];
      if (!map_coords(p, (double)x, (double)y, p->scale, c)) { bad |= 1; continue; }
      for (int ch = 0; ch < 3; ++ch)
        if (!cubic_sample(img.data(), w, h, ch, c[2 * ch], c[2 * ch + 1], &rgb_out[((std::size_t)y * w + x) * 3 + ch]))
          bad |= 2;
    }
  return bad ? -3 : 0;
}
