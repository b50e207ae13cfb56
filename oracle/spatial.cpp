// CPU oracle: exact separable pixel-area reduction, restated from
// crates/core/src/resample.rs:45-113 (axis tables) and :235-324 (horizontal
// then vertical accumulation). Test infrastructure only.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rd_oracle.h"

namespace {
struct Axis {
  std::vector<int> first, offset, count;
  std::vector<float> weights;
};
Axis build_axis(int source, int target) {
  Axis a;
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

extern "C" int ro_area_reduce(const float* rgb, int w, int h, int tw, int th, float* out) {
  if (tw <= 0 || th <= 0 || tw > w || th > h) return -1;
  if (tw == w && th == h) {
    std::copy(rgb, rgb + (std::size_t)w * h * 3, out);
    return 0;
  }
  const Axis ha = build_axis(w, tw), va = build_axis(h, th);
  std::vector<float> mid((std::size_t)h * tw * 3, 0.0f);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int t = 0; t < tw; ++t) {
      float* d = &mid[((std::size_t)y * tw + t) * 3];
      for (int k = 0; k < ha.count[t]; ++k) {
        const float wgt = ha.weights[ha.offset[t] + k];
        const float* s = rgb + ((std::size_t)y * w + ha.first[t] + k) * 3;
        for (int c = 0; c < 3; ++c) d[c] += s[c] * wgt;
      }
    }
#pragma omp parallel for schedule(static)
  for (int t = 0; t < th; ++t) {
    float* row = out + (std::size_t)t * tw * 3;
    for (int i = 0; i < tw * 3; ++i) row[i] = 0.0f;
    for (int k = 0; k < va.count[t]; ++k) {
      const float wgt = va.weights[va.offset[t] + k];
      const float* src = mid.data() + (std::size_t)(va.first[t] + k) * tw * 3;
      for (int i = 0; i < tw * 3; ++i) row[i] += src[i] * wgt;
    }
  }
  return 0;
}
