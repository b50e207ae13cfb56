// CPU oracle: bilinear, Malvar-He-Cutler and RCD demosaic plus the channel
// balance wrapper, restated from crates/demosaic/src/{lib,balance,bilinear,
// malvar_he_cutler,rcd,rcd_stages,rcd_geometry}.rs. Test infrastructure only.
#include <algorithm>
#include <cstring>
#include <vector>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

namespace {

// bilinear.rs:95-113: average of the in-bounds offsets, in offset order.
float average_offsets(const float* m, int w, int h, int stride, int x, int y, const int (*off)[2], int n) {
  float sum = 0.0f;
  int count = 0;
  for (int k = 0; k < n; ++k) {
    const int nx = x + off[k][0], ny = y + off[k][1];
    if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
    sum += m[(std::size_t)ny * stride + nx];
    count += 1;
  }
  return count == 0 ? m[(std::size_t)y * stride + x] : sum / (float)count;
}

const int CROSS[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
const int DIAG[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
const int HORIZ[2][2] = {{-1, 0}, {1, 0}};
const int VERT[2][2] = {{0, -1}, {0, 1}};

// bilinear.rs:68-93
void bilinear_pixel(const float* m, int w, int h, int stride, int pattern, int x, int y, float rgb[3]) {
  const float s = m[(std::size_t)y * stride + x];
  switch (color_at(pattern, x, y)) {
    case 0:
      rgb[0] = s;
      rgb[1] = average_offsets(m, w, h, stride, x, y, CROSS, 4);
      rgb[2] = average_offsets(m, w, h, stride, x, y, DIAG, 4);
      break;
    case 2:
      rgb[0] = average_offsets(m, w, h, stride, x, y, DIAG, 4);
      rgb[1] = average_offsets(m, w, h, stride, x, y, CROSS, 4);
      rgb[2] = s;
      break;
    default: {
      const bool red_h = color_at(pattern, (std::size_t)x + 1, y) == 0;
      rgb[0] = average_offsets(m, w, h, stride, x, y, red_h ? HORIZ : VERT, 2);
      rgb[1] = s;
      rgb[2] = average_offsets(m, w, h, stride, x, y, red_h ? VERT : HORIZ, 2);
    }
  }
}

// malvar_he_cutler.rs:16-38
const int8_t G_AT_RB[5][5] = {{0, 0, -2, 0, 0}, {0, 0, 4, 0, 0}, {-2, 4, 8, 4, -2}, {0, 0, 4, 0, 0}, {0, 0, -2, 0, 0}};
const int8_t C_AT_G_ROW[5][5] = {{0, 0, 1, 0, 0}, {0, -2, 0, -2, 0}, {-2, 8, 10, 8, -2}, {0, -2, 0, -2, 0}, {0, 0, 1, 0, 0}};
const int8_t R_AT_B[5][5] = {{0, 0, -3, 0, 0}, {0, 4, 0, 4, 0}, {-3, 0, 12, 0, -3}, {0, 4, 0, 4, 0}, {0, 0, -3, 0, 0}};

// malvar_he_cutler.rs:100-122: row-major taps, zeros skipped, sum * (1/16).
float mhc_kernel(const float* m, int stride, int x, int y, const int8_t (*k)[5], bool transpose) {
  float sum = 0.0f;
  for (int ky = 0; ky < 5; ++ky)
    for (int kx = 0; kx < 5; ++kx) {
      const int c = transpose ? k[kx][ky] : k[ky][kx];
      if (c != 0) sum += (float)c * m[(std::size_t)(y + ky - 2) * stride + (x + kx - 2)];
    }
  return sum * (1.0f / 16.0f);
}

}  // namespace

extern "C" void ro_bilinear_reconstruct(const float* mosaic, int w, int h, int stride, int pattern,
                                        const float gains[3], float* out, int out_stride) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float rgb[3];
      bilinear_pixel(mosaic, w, h, stride, pattern, x, y, rgb);
      float* o = out + (std::size_t)y * out_stride + 3 * (std::size_t)x;
      o[0] = rgb[0] * gains[0];
      o[1] = rgb[1] * gains[1];
      o[2] = rgb[2] * gains[2];
    }
}

extern "C" void ro_mhc_reconstruct(const float* m, int w, int h, int stride, int pattern, const float gains[3],
                                   float* out, int out_stride) {
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float rgb[3];
      const bool border = x < 2 || y < 2 || x >= std::max(w - 2, 0) || y >= std::max(h - 2, 0);
      if (border) {
        bilinear_pixel(m, w, h, stride, pattern, x, y, rgb);
      } else {
        const float measured = m[(std::size_t)y * stride + x];
        switch (color_at(pattern, x, y)) {
          case 0:
            rgb[0] = measured;
            rgb[1] = mhc_kernel(m, stride, x, y, G_AT_RB, false);
            rgb[2] = mhc_kernel(m, stride, x, y, R_AT_B, false);
            break;
          case 2:
            rgb[0] = mhc_kernel(m, stride, x, y, R_AT_B, false);
            rgb[1] = mhc_kernel(m, stride, x, y, G_AT_RB, false);
            rgb[2] = measured;
            break;
          default: {
            const bool red_h = color_at(pattern, (std::size_t)x + 1, y) == 0;
            rgb[0] = mhc_kernel(m, stride, x, y, C_AT_G_ROW, !red_h);
            rgb[1] = measured;
            rgb[2] = mhc_kernel(m, stride, x, y, C_AT_G_ROW, red_h);
          }
        }
      }
      float* o = out + (std::size_t)y * out_stride + 3 * (std::size_t)x;
      o[0] = rgb[0] * gains[0];
      o[1] = rgb[1] * gains[1];
      o[2] = rgb[2] * gains[2];
    }
}

// ---------------------------------------------------------------- RCD
namespace rcd {
constexpr int TS = 194, BORDER = 10, STEP = TS - 2 * BORDER, MIN_DIM = 2 * BORDER + 4;
constexpr float EPSILON = 1.0e-5f, EPSILON_SQUARED = 1.0e-10f;

struct Scratch {
  std::vector<float> cfa, rgb[3], vh, pq, pcd, qcd, vbuf[3], hbuf;
  Scratch() {
    cfa.assign(TS * TS, 0.0f);
    for (auto& c : rgb) c.assign(TS * TS, 0.0f);
    vh.assign(TS * TS, 0.0f);
    pq.assign(TS * TS / 2, 0.0f);
    pcd.assign(TS * TS / 2, 0.0f);
    qcd.assign(TS * TS / 2, 0.0f);
    for (auto& b : vbuf) b.assign(TS, 0.0f);
    hbuf.assign(TS, 0.0f);
  }
  void clear() {
    std::fill(cfa.begin(), cfa.end(), 0.0f);
    for (auto& c : rgb) std::fill(c.begin(), c.end(), 0.0f);
    std::fill(vh.begin(), vh.end(), 0.0f);
    std::fill(pq.begin(), pq.end(), 0.0f);
    std::fill(pcd.begin(), pcd.end(), 0.0f);
    std::fill(qcd.begin(), qcd.end(), 0.0f);
    for (auto& b : vbuf) std::fill(b.begin(), b.end(), 0.0f);
    std::fill(hbuf.begin(), hbuf.end(), 0.0f);
  }
};

inline float sq(float v) { return v * v; }
// rcd_stages.rs:417-427
inline float vhp(const float* v, int i) {
  return (v[i - 3 * TS] - v[i - TS] - v[i + TS] + v[i + 3 * TS]) - 3.0f * (v[i - 2 * TS] + v[i + 2 * TS]) + 6.0f * v[i];
}
inline float hhp(const float* v, int i) {
  return (v[i - 3] - v[i - 1] - v[i + 1] + v[i + 3]) - 3.0f * (v[i - 2] + v[i + 2]) + 6.0f * v[i];
}
// rcd_stages.rs:433-460
inline float nonzero(float v) {
  if (std::fabs(v) >= EPSILON) return v;
  return std::signbit(v) ? -EPSILON : EPSILON;
}
inline float ratio_estimate(float sample, float lp, float nlp) {
  const float d = nonzero(EPSILON + lp + nlp);
  return sample * (2.0f * lp) / d;
}
inline float weighted_pair(float w1, float v1, float w2, float v2) {
  return (w1 * v1 + w2 * v2) / nonzero(w1 + w2);
}
inline float refined_direction(float c, float nw, float ne, float sw, float se) {
  const float n = 0.25f * (nw + ne + sw + se);
  const float sel = std::fabs(0.5f - c) < std::fabs(0.5f - n) ? n : c;
  return rclamp(sel, 0.0f, 1.0f);
}
// rcd_stages.rs:462-464: an explicit fused multiply-add.
inline float interpolate(float d, float h, float v) { return std::fmaf(d, h, (1.0f - d) * v); }
inline int off(int i, int dx, int dy) { return i + dy * TS + dx; }
// rcd_stages.rs:368-381
inline float cardinal_gradient(const float* v, int i, int dx, int dy) {
  const int one = off(i, dx, dy), opp = off(i, -dx, -dy), two = off(i, 2 * dx, 2 * dy);
  const int three = off(i, 3 * dx, 3 * dy), four = off(i, 4 * dx, 4 * dy);
  return EPSILON + std::fabs(v[one] - v[opp]) + std::fabs(v[i] - v[two]) + std::fabs(v[one] - v[three]) +
         std::fabs(v[two] - v[four]);
}
// rcd_stages.rs:383-398
inline float diagonal_gradient(const float* v, const float* g, int i, int dx, int dy) {
  const int near_ = off(i, dx, dy), opp = off(i, -dx, -dy), far_ = off(i, 3 * dx, 3 * dy), g2 = off(i, 2 * dx, 2 * dy);
  return EPSILON + std::fabs(v[near_] - v[opp]) + std::fabs(v[near_] - v[far_]) + std::fabs(g[i] - g[g2]);
}

void run_tile(Scratch& s, int tp) {
  float* cfa = s.cfa.data();
  // find_directions, rcd_stages.rs:8-48
  const int initial_end = std::min(TS - 3, 5);
  for (int row = 3; row < initial_end; ++row)
    for (int col = 4; col < TS - 4; ++col) s.vbuf[row - 3][col - 4] = sq(vhp(cfa, row * TS + col));
  int v0 = 0, v1 = 1, v2 = 2;
  for (int row = 4; row < TS - 4; ++row) {
    for (int col = 3; col < TS - 3; ++col) s.hbuf[col - 3] = sq(hhp(cfa, row * TS + col));
    for (int col = 4; col < TS - 4; ++col) s.vbuf[v2][col - 4] = sq(vhp(cfa, (row + 1) * TS + col));
    for (int col = 4; col < TS - 4; ++col) {
      const float vs = rmax(s.vbuf[v0][col - 4] + s.vbuf[v1][col - 4] + s.vbuf[v2][col - 4], EPSILON_SQUARED);
      const float hs = rmax(s.hbuf[col - 4] + s.hbuf[col - 3] + s.hbuf[col - 2], EPSILON_SQUARED);
      s.vh[row * TS + col] = vs / (vs + hs);
    }
    const int t = v0; v0 = v1; v1 = v2; v2 = t;
  }
  // calculate_low_pass, rcd_stages.rs:50-77
  for (int row = 2; row < TS - 2; ++row) {
    const int start = 2 + (color_at(tp, 0, row) & 1);
    for (int col = start; col < TS - 2; col += 2) {
      const int i = row * TS + col;
      s.pq[i / 2] = cfa[i] + 0.5f * (cfa[i - TS] + cfa[i + TS] + cfa[i - 1] + cfa[i + 1]) +
                    0.25f * (cfa[i - TS - 1] + cfa[i - TS + 1] + cfa[i + TS - 1] + cfa[i + TS + 1]);
    }
  }
  // interpolate_green, rcd_stages.rs:79-142
  for (int row = 4; row < TS - 4; ++row) {
    const int start = 4 + (color_at(tp, 0, row) & 1);
    for (int col = start; col < TS - 4; col += 2) {
      const int i = row * TS + col;
      const float ng = cardinal_gradient(cfa, i, 0, -1), sg = cardinal_gradient(cfa, i, 0, 1);
      const float wg = cardinal_gradient(cfa, i, -1, 0), eg = cardinal_gradient(cfa, i, 1, 0);
      const int li = i / 2;
      const float lp = s.pq[li];
      const float ne = ratio_estimate(cfa[i - TS], lp, s.pq[li - TS]);
      const float se = ratio_estimate(cfa[i + TS], lp, s.pq[li + TS]);
      const float we = ratio_estimate(cfa[i - 1], lp, s.pq[li - 1]);
      const float ee = ratio_estimate(cfa[i + 1], lp, s.pq[li + 1]);
      const float ve = weighted_pair(sg, ne, ng, se);
      const float he = weighted_pair(wg, ee, eg, we);
      const float dir = refined_direction(s.vh[i], s.vh[i - TS - 1], s.vh[i - TS + 1], s.vh[i + TS - 1], s.vh[i + TS + 1]);
      s.rgb[1][i] = interpolate(dir, he, ve);
    }
  }
  // calculate_diagonal_high_pass, rcd_stages.rs:160-199
  for (int row = 3; row < TS - 3; ++row)
    for (int col = 3; col < TS - 3; col += 2) {
      const int i = row * TS + col;
      s.pcd[i / 2] = sq((cfa[i - 3 * TS - 3] - cfa[i - TS - 1] - cfa[i + TS + 1] + cfa[i + 3 * TS + 3]) -
                        3.0f * (cfa[i - 2 * TS - 2] + cfa[i + 2 * TS + 2]) + 6.0f * cfa[i]);
      s.qcd[i / 2] = sq((cfa[i - 3 * TS + 3] - cfa[i - TS + 1] - cfa[i + TS - 1] + cfa[i + 3 * TS - 3]) -
                        3.0f * (cfa[i - 2 * TS + 2] + cfa[i + 2 * TS - 2]) + 6.0f * cfa[i]);
    }
  // calculate_diagonal_directions, rcd_stages.rs:201-229
  for (int row = 4; row < TS - 4; ++row) {
    const int start = 4 + (color_at(tp, 0, row) & 1);
    for (int col = start; col < TS - 4; col += 2) {
      const int i = row * TS + col;
      const int hi = i / 2, pr = (i - TS - 1) / 2, nr = (i + TS - 1) / 2;
      const float ps = rmax(s.pcd[pr] + s.pcd[hi] + s.pcd[nr + 1], EPSILON_SQUARED);
      const float qs = rmax(s.qcd[pr + 1] + s.qcd[hi] + s.qcd[nr], EPSILON_SQUARED);
      s.pq[hi] = ps / (ps + qs);
    }
  }
  // interpolate_opposite_color, rcd_stages.rs:231-288
  for (int row = 4; row < TS - 4; ++row) {
    const int start = 4 + (color_at(tp, 0, row) & 1);
    for (int col = start; col < TS - 4; col += 2) {
      const int i = row * TS + col;
      const int ch = 2 - color_at(tp, col, row);
      const int hi = i / 2, pr = (i - TS - 1) / 2, nr = (i + TS - 1) / 2;
      const float dir = refined_direction(s.pq[hi], s.pq[pr], s.pq[pr + 1], s.pq[nr], s.pq[nr + 1]);
      const float* c = s.rgb[ch].data();
      const float* g = s.rgb[1].data();
      const float nwg = diagonal_gradient(c, g, i, -1, -1), neg = diagonal_gradient(c, g, i, 1, -1);
      const float swg = diagonal_gradient(c, g, i, -1, 1), seg = diagonal_gradient(c, g, i, 1, 1);
      const float nwe = c[i - TS - 1] - g[i - TS - 1], nee = c[i - TS + 1] - g[i - TS + 1];
      const float swe = c[i + TS - 1] - g[i + TS - 1], see = c[i + TS + 1] - g[i + TS + 1];
      const float dp = weighted_pair(nwg, see, seg, nwe);
      const float dq = weighted_pair(neg, swe, swg, nee);
      s.rgb[ch][i] = g[i] + interpolate(dir, dq, dp);
    }
  }
  // interpolate_at_green, rcd_stages.rs:290-366
  for (int row = 4; row < TS - 4; ++row) {
    const int start = 4 + (color_at(tp, 1, row) & 1);
    for (int col = start; col < TS - 4; col += 2) {
      const int i = row * TS + col;
      const float dir = refined_direction(s.vh[i], s.vh[i - TS - 1], s.vh[i - TS + 1], s.vh[i + TS - 1], s.vh[i + TS + 1]);
      const float* g = s.rgb[1].data();
      const float green = g[i];
      const float n1 = EPSILON + std::fabs(green - g[i - 2 * TS]);
      const float s1 = EPSILON + std::fabs(green - g[i + 2 * TS]);
      const float w1 = EPSILON + std::fabs(green - g[i - 2]);
      const float e1 = EPSILON + std::fabs(green - g[i + 2]);
      const float gn = g[i - TS], gs = g[i + TS], gw = g[i - 1], ge = g[i + 1];
      for (int ch = 0; ch <= 2; ch += 2) {
        float* c = s.rgb[ch].data();
        const float nsa = std::fabs(c[i - TS] - c[i + TS]);
        const float ewa = std::fabs(c[i - 1] - c[i + 1]);
        const float ngr = n1 + nsa + std::fabs(c[i - TS] - c[i - 3 * TS]);
        const float sgr = s1 + nsa + std::fabs(c[i + TS] - c[i + 3 * TS]);
        const float wgr = w1 + ewa + std::fabs(c[i - 1] - c[i - 3]);
        const float egr = e1 + ewa + std::fabs(c[i + 1] - c[i + 3]);
        const float ne = c[i - TS] - gn, se = c[i + TS] - gs, we = c[i - 1] - gw, ee = c[i + 1] - ge;
        const float vert = weighted_pair(ngr, se, sgr, ne);
        const float horiz = weighted_pair(egr, we, wgr, ee);
        c[i] = green + interpolate(dir, horiz, vert);
      }
    }
  }
}
}  // namespace rcd

extern "C" int ro_rcd_reconstruct(const float* m, int w, int h, int stride, int pattern, const float gains[3],
                                  float* out, int out_stride) {
  using namespace rcd;
  if (w <= MIN_DIM || h <= MIN_DIM) {
    ro_bilinear_reconstruct(m, w, h, stride, pattern, gains, out, out_stride);
    return 0;
  }
  const int cols = (w + STEP - 1) / STEP, rows = (h + STEP - 1) / STEP;
#pragma omp parallel
  {
    Scratch s;
#pragma omp for schedule(dynamic)
    for (int t = 0; t < cols * rows; ++t) {
      const int ox = (t % cols) * STEP, oy = (t / cols) * STEP;
      const int tp = shifted(pattern, ox, oy);
      s.clear();
      // populate, rcd.rs:226-271
      const long wx = (long)ox - BORDER, wy = (long)oy - BORDER;
      for (int row = 0; row < TS; ++row) {
        const int c0 = color_at(tp, 0, row), c1 = color_at(tp, 1, row);
        const std::size_t sy = mirror_coordinate(wy + row, h);
        for (int col = 0; col < TS; ++col) {
          const float v = m[sy * stride + mirror_coordinate(wx + col, w)];
          s.cfa[row * TS + col] = v;
          s.rgb[c0][row * TS + col] = v;
        }
        std::memcpy(&s.rgb[c1][row * TS], &s.cfa[row * TS], sizeof(float) * TS);
      }
      run_tile(s, tp);
      // write_tile, rcd.rs:275-308
      const int xe = std::min(ox + STEP, w), ye = std::min(oy + STEP, h);
      for (int gy = oy; gy < ye; ++gy)
        for (int gx = ox; gx < xe; ++gx) {
          const int idx = (gy - oy + BORDER) * TS + (gx - ox) + BORDER;
          float rgb[3] = {s.rgb[0][idx], s.rgb[1][idx], s.rgb[2][idx]};
          rgb[color_at(pattern, gx, gy)] = m[(std::size_t)gy * stride + gx];
          float* o = out + (std::size_t)gy * out_stride + 3 * (std::size_t)gx;
          o[0] = rgb[0] * gains[0];
          o[1] = rgb[1] * gains[1];
          o[2] = rgb[2] * gains[2];
        }
    }
  }
  return 0;
}

// demosaic_cancellable, crates/demosaic/src/lib.rs:302-370, with ChannelBalance
// (crates/demosaic/src/balance.rs:30-93). algorithm: 0 bilinear, 1 MHC, 2 RCD, 3 AMaZE.
extern "C" int ro_demosaic(const float* mosaic, int w, int h, int pattern, const float balance[3], int algorithm,
                           float* out) {
  if (w < 2 || h < 2) return -1;
  for (int c = 0; c < 3; ++c)
    if (!std::isfinite(balance[c]) || !(balance[c] > 0.0f)) return -2;
  const float largest = rmax(rmax(balance[0], balance[1]), balance[2]);
  const float fwd[3] = {balance[0] / largest, balance[1] / largest, balance[2] / largest};
  const bool identity = fwd[0] == 1.0f && fwd[1] == 1.0f && fwd[2] == 1.0f;
  std::vector<float> scaled;
  const float* src = mosaic;
  float gains[3] = {1.0f, 1.0f, 1.0f};
  float clip_point = 1.0f;
  if ((algorithm == 2 || algorithm == 3) && !identity) {
    scaled.resize((std::size_t)w * h);
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < w; ++x)
        scaled[(std::size_t)y * w + x] = mosaic[(std::size_t)y * w + x] * fwd[color_at(pattern, x, y)];
    src = scaled.data();
    for (int c = 0; c < 3; ++c) gains[c] = 1.0f / fwd[c];
    clip_point = rmin(rmin(fwd[0], fwd[1]), fwd[2]);
  }
  switch (algorithm) {
    case 0: ro_bilinear_reconstruct(src, w, h, w, pattern, gains, out, 3 * w); return 0;
    case 1: ro_mhc_reconstruct(src, w, h, w, pattern, gains, out, 3 * w); return 0;
    case 2: return ro_rcd_reconstruct(src, w, h, w, pattern, gains, out, 3 * w);
    case 3: return ro_amaze_reconstruct(src, w, h, w, pattern, gains, clip_point, out, 3 * w);
    default: return -3;
  }
}
