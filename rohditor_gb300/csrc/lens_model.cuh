// Inverse lens kernels shared by the optics gather (device) and the radial
// multiplier table build (host).
//
// They live in the un-vendored crate `lensfun = "=0.7.0"` (Cargo.toml:35) and
// are restated from its published Newton inversion as the reference documents
// and ports it (crates/optics/src/radial.rs:21-27,
// crates/gpu/src/spatial/spatial.wgsl:91-178): radius rd = sqrt(f64(x*x + y*y))
// from the f32 input, up to 7 Newton steps in f64 that break once
// |F(ru)| < 1e-5, the input scaled by ru / rd and narrowed once. On
// non-convergence Poly3 returns NaN; Poly5, PTLens and TCA-Poly3 return the
// input unchanged.
#pragma once

#include <cmath>

namespace rd {

constexpr double LENS_NEWTON_EPS = 0.00001;

// Inverse distortion (model 1 Poly3, 2 Poly5, 3 PTLens; 0 keeps the input).
__host__ __device__ inline void lens_undistort(int model, float k0, float k1, float k2, float x, float y, float& ox,
                                               float& oy) {
  ox = x;
  oy = y;
  if (model == 0) return;
  const double rd = sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double a = k0, b = k1, c = k2;
  double ru = rd;
  bool converged = false;
  if (model == 1) {
    const double inv_k1 = (double)(1.0f / k0);
    const double rd_div_k1 = (double)(float)(rd * inv_k1);
    for (int s = 0; s < 7; ++s) {
      const double f = ru * ru * ru + ru * inv_k1 - rd_div_k1;
      if (fabs(f) < LENS_NEWTON_EPS) { converged = true; break; }
      ru -= f / (3.0 * ru * ru + inv_k1);
    }
    if (!converged || ru < 0.0) { ox = nanf(""); oy = nanf(""); return; }
  } else if (model == 2) {
    for (int s = 0; s < 7; ++s) {
      const double ru2 = ru * ru;
      const double f = ru * (1.0 + a * ru2 + b * ru2 * ru2) - rd;
      if (fabs(f) < LENS_NEWTON_EPS) { converged = true; break; }
      ru -= f / (1.0 + 3.0 * a * ru2 + 5.0 * b * ru2 * ru2);
    }
    if (!converged || ru < 0.0) return;
  } else {
    for (int s = 0; s < 7; ++s) {
      const double f = ru * (a * ru * ru * ru + b * ru * ru + c * ru + 1.0) - rd;
      if (fabs(f) < LENS_NEWTON_EPS) { converged = true; break; }
      ru -= f / (4.0 * a * ru * ru * ru + 3.0 * b * ru * ru + 2.0 * c * ru + 1.0);
    }
    if (!converged || ru < 0.0) return;
  }
  const double ratio = ru / rd;
  ox = (float)((double)x * ratio);
  oy = (float)((double)y * ratio);
}

// Reverse TCA Poly3 of one channel, coefficients (v, c, b).
__host__ __device__ inline void lens_tca_poly3(const float* ch, float x, float y, float& ox, float& oy) {
  ox = x;
  oy = y;
  const double rd = sqrt((double)(x * x + y * y));
  if (rd == 0.0) return;
  const double v = ch[0], c = ch[1], b = ch[2];
  double ru = rd;
  bool converged = false;
  for (int s = 0; s < 7; ++s) {
    const double ru2 = ru * ru;
    const double f = b * ru2 * ru + c * ru2 + v * ru - rd;
    if (fabs(f) < LENS_NEWTON_EPS) { converged = true; break; }
    ru -= f / (3.0 * b * ru2 + 2.0 * c * ru + v);
  }
  if (!converged || ru <= 0.0) return;
  const double ratio = ru / rd;
  ox = (float)((double)x * ratio);
  oy = (float)((double)y * ratio);
}

}  // namespace rd
