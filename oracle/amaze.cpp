// CPU oracle: tiled AMaZE demosaic, restated from the reference's Rust port of
// RawTherapee's amaze_demosaic_RT.cc (crates/demosaic/src/amaze/*.rs).
//
// Test infrastructure only (see oracle_common.h). Every stage keeps the
// reference's loop bounds, in-place raster-order updates and operation order so
// the output is bit-identical; the reference's golden FNV-1a hashes
// (crates/demosaic/tests/amaze_golden.rs:54-86) and stage probes
// (crates/demosaic/src/amaze/mod.rs:336-393) pin it in tests/test_oracle.py.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "oracle_common.h"
#include "rd_oracle.h"

namespace oracle {
namespace amaze {

// Geometry: crates/demosaic/src/amaze_geometry.rs:13-15.
constexpr int TS = 256;
constexpr int TSH = TS / 2;
constexpr int BORDER = 16;
constexpr int VALID = TS - 2 * BORDER;
// Neighbour offsets: crates/demosaic/src/amaze/math.rs:14-22.
constexpr long V1 = TS, V2 = 2 * TS, P1 = -TS + 1, P2 = -2 * TS + 2, M1 = TS + 1, M2 = 2 * TS + 2;
// Constants: crates/demosaic/src/amaze/math.rs:24-60.
constexpr float EPS = 1.0e-5f;
constexpr float EPSSQ = 1.0e-10f;
constexpr float ARTHRESH = 0.75f;
constexpr float GAUSSODD[4] = {0.14659727707323927f, 0.103592713382435f, 0.0732036125103057f,
                               0.0365543548389495f};
constexpr float NYQTHRESH = 0.5f;
constexpr float GAUSSGRAD[6] = {NYQTHRESH * 0.07384411893421103f, NYQTHRESH * 0.06207511968171489f,
                                NYQTHRESH * 0.0521818194747806f,  NYQTHRESH * 0.03687419286733595f,
                                NYQTHRESH * 0.03099732204057846f, NYQTHRESH * 0.018413194161458882f};
constexpr float GAUSSEVEN[2] = {0.13719494435797422f, 0.05640252782101291f};
constexpr float GQUINC[4] = {0.169917f, 0.108947f, 0.069855f, 0.0287182f};

inline float sqr(float x) { return x * x; }
inline float fmin_(float a, float b) { return a < b ? a : b; }
inline float fmax_(float a, float b) { return a > b ? a : b; }
inline float median(float a, float b, float c) { return fmax_(fmin_(a, b), fmin_(fmax_(b, a), c)); }
inline float intp(float a, float b, float c) { return a * (b - c) + c; }
inline int fc(int pattern, int row, int col) { return color_at(pattern, col, row); }
inline int green_at_even(int pattern, int row) { return fc(pattern, row, 2) & 1; }

// Per-tile planes (crates/demosaic/src/amaze/scratch.rs:17-75).
struct Scratch {
  std::vector<float> cfa, green, delhvsqsum, dirwts0, dirwts1, vcd, hcd, vcdalt, hcdalt, cddiffsq,
      dgintv, dginth, hvwt, dgrb0, dgrb1, dgrb2_h, dgrb2_v, delp, delm, sq1m, sq1p, nyqutest, pmwt,
      rbm, rbp, rbint, red, blue;
  std::vector<uint8_t> nyquist, nyquist2;
  Scratch() {
    for (auto* p : {&cfa, &green, &delhvsqsum, &dirwts0, &dirwts1, &vcd, &hcd, &vcdalt, &hcdalt,
                    &cddiffsq, &dgintv, &dginth, &red, &blue})
      p->assign(TS * TS, 0.0f);
    for (auto* p : {&hvwt, &dgrb0, &dgrb1, &dgrb2_h, &dgrb2_v, &delp, &delm, &sq1m, &sq1p,
                    &nyqutest, &pmwt, &rbm, &rbp, &rbint})
      p->assign(TS * TSH, 0.0f);
    nyquist.assign(TS * TSH, 0);
    nyquist2.assign(TS * TSH, 0);
  }
  // scratch.rs:105-111: only these planes are reset per tile.
  void clear() {
    std::fill(nyquist.begin(), nyquist.end(), 0);
    std::fill(nyquist2.begin(), nyquist2.end(), 0);
    std::fill(dgrb2_h.begin(), dgrb2_h.end(), 0.0f);
    std::fill(dgrb2_v.begin(), dgrb2_v.end(), 0.0f);
  }
};

// green.rs:13-29
static void gradients(Scratch& s) {
  const float* cfa = s.cfa.data();
  for (int rr = 2; rr < TS - 2; ++rr) {
    for (int cc = 2; cc < TS - 2; ++cc) {
      const int i = rr * TS + cc;
      const float delh = std::fabs(cfa[i + 1] - cfa[i - 1]);
      const float delv = std::fabs(cfa[i + TS] - cfa[i - TS]);
      s.dirwts0[i] = EPS + std::fabs(cfa[i + 2 * TS] - cfa[i]) + std::fabs(cfa[i] - cfa[i - 2 * TS]) + delv;
      s.dirwts1[i] = EPS + std::fabs(cfa[i + 2] - cfa[i]) + std::fabs(cfa[i] - cfa[i - 2]) + delh;
      s.delhvsqsum[i] = sqr(delh) + sqr(delv);
    }
  }
}

inline float adaptive_or(float ratio, float centre, float fallback) {
  return std::fabs(1.0f - ratio) < ARTHRESH ? centre * ratio : fallback;
}

// green.rs:46-139
static void colour_differences(Scratch& s, int pattern, float clip_pt8) {
  const float* cfa = s.cfa.data();
  const float* w0 = s.dirwts0.data();
  const float* w1 = s.dirwts1.data();
  for (int rr = 4; rr < TS - 4; ++rr) {
    const bool green_first = (fc(pattern, rr, 4) & 1) == 1;
    for (int cc = 4; cc < TS - 4; ++cc) {
      const int i = rr * TS + cc;
      const bool fcswitch = green_first == ((cc & 1) == 0);
      const float cur = cfa[i];
      const float up = cfa[i - TS], up2 = cfa[i - 2 * TS], down = cfa[i + TS], down2 = cfa[i + 2 * TS];
      const float left = cfa[i - 1], left2 = cfa[i - 2], right = cfa[i + 1], right2 = cfa[i + 2];
      const float cru = up * (w0[i - 2 * TS] + w0[i]) / (w0[i - 2 * TS] * (EPS + cur) + w0[i] * (EPS + up2));
      const float crd = down * (w0[i + 2 * TS] + w0[i]) / (w0[i + 2 * TS] * (EPS + cur) + w0[i] * (EPS + down2));
      const float crl = left * (w1[i - 2] + w1[i]) / (w1[i - 2] * (EPS + cur) + w1[i] * (EPS + left2));
      const float crr = right * (w1[i + 2] + w1[i]) / (w1[i + 2] * (EPS + cur) + w1[i] * (EPS + right2));
      const float guha = up + 0.5f * (cur - up2);
      const float gdha = down + 0.5f * (cur - down2);
      const float glha = left + 0.5f * (cur - left2);
      const float grha = right + 0.5f * (cur - right2);
      float guar = adaptive_or(cru, cur, guha);
      float gdar = adaptive_or(crd, cur, gdha);
      float glar = adaptive_or(crl, cur, glha);
      float grar = adaptive_or(crr, cur, grha);
      const float hwt = w1[i - 1] / (w1[i - 1] + w1[i + 1]);
      const float vwt = w0[i - TS] / (w0[i + TS] + w0[i - TS]);
      const float gintvha = vwt * gdha + (1.0f - vwt) * guha;
      const float ginthha = hwt * grha + (1.0f - hwt) * glha;
      float vcd, hcd, vcdalt, hcdalt;
      if (fcswitch) {
        vcd = cur - (vwt * gdar + (1.0f - vwt) * guar);
        hcd = cur - (hwt * grar + (1.0f - hwt) * glar);
        vcdalt = cur - gintvha;
        hcdalt = cur - ginthha;
      } else {
        vcd = (vwt * gdar + (1.0f - vwt) * guar) - cur;
        hcd = (hwt * grar + (1.0f - hwt) * glar) - cur;
        vcdalt = gintvha - cur;
        hcdalt = ginthha - cur;
      }
      const bool clipped = (cur > clip_pt8) | (gintvha > clip_pt8) | (ginthha > clip_pt8);
      if (clipped) {
        guar = guha; gdar = gdha; glar = glha; grar = grha;
        vcd = vcdalt; hcd = hcdalt;
      }
      s.dgintv[i] = fmin_(sqr(guha - gdha), sqr(guar - gdar));
      s.dginth[i] = fmin_(sqr(glha - grha), sqr(glar - grar));
      s.vcd[i] = vcd;
      s.hcd[i] = hcd;
      s.vcdalt[i] = vcdalt;
      s.hcdalt[i] = hcdalt;
    }
  }
}

// green.rs:144-158
inline float bound_at_green(float d, float cur, float a, float b, float clip_pt) {
  const float g = -d + cur;
  const float alt = -median(g, a, b) + cur;
  float bounded = d;
  if (d > 0.0f) {
    if (3.0f * d > g + cur) {
      bounded = alt;
    } else {
      const float weight = 1.0f - 3.0f * d / (EPS + g + cur);
      bounded = weight * d + (1.0f - weight) * alt;
    }
  }
  return g > clip_pt ? alt : bounded;
}
// green.rs:163-177
inline float bound_at_red_blue(float d, float cur, float a, float b, float clip_pt) {
  const float g = d + cur;
  const float alt = median(g, a, b) - cur;
  float bounded = d;
  if (d < 0.0f) {
    if (3.0f * d < -(g + cur)) {
      bounded = alt;
    } else {
      const float weight = 1.0f + 3.0f * d / (EPS + g + cur);
      bounded = weight * d + (1.0f - weight) * alt;
    }
  }
  return g > clip_pt ? alt : bounded;
}
inline float spread(float a, float b, float c) {
  return 3.0f * (sqr(a) + sqr(b) + sqr(c)) - sqr(a + b + c);
}

// green.rs:187-222: in place, raster order. hcd[cc-2] and vcd[rr-2] are the
// already-bounded values of this pass.
static void bound_differences(Scratch& s, int pattern, float clip_pt) {
  float* vcd = s.vcd.data();
  float* hcd = s.hcd.data();
  const float* vcdalt = s.vcdalt.data();
  const float* hcdalt = s.hcdalt.data();
  const float* cfa = s.cfa.data();
  for (int rr = 4; rr < TS - 4; ++rr) {
    bool green = (fc(pattern, rr, 4) & 1) == 1;
    for (int cc = 4; cc < TS - 4; ++cc) {
      const int i = rr * TS + cc;
      const float hcdvar = spread(hcd[i - 2], hcd[i], hcd[i + 2]);
      const float hcdaltvar = spread(hcdalt[i - 2], hcdalt[i], hcdalt[i + 2]);
      const float vcdvar = spread(vcd[i - 2 * TS], vcd[i], vcd[i + 2 * TS]);
      const float vcdaltvar = spread(vcdalt[i - 2 * TS], vcdalt[i], vcdalt[i + 2 * TS]);
      const float h = hcdaltvar < hcdvar ? hcdalt[i] : hcd[i];
      const float v = vcdaltvar < vcdvar ? vcdalt[i] : vcd[i];
      const float cur = cfa[i];
      if (green) {
        hcd[i] = bound_at_green(h, cur, cfa[i - 1], cfa[i + 1], clip_pt);
        vcd[i] = bound_at_green(v, cur, cfa[i - TS], cfa[i + TS], clip_pt);
      } else {
        hcd[i] = bound_at_red_blue(h, cur, cfa[i - 1], cfa[i + 1], clip_pt);
        vcd[i] = bound_at_red_blue(v, cur, cfa[i - TS], cfa[i + TS], clip_pt);
        s.cddiffsq[i] = sqr(vcd[i] - hcd[i]);
      }
      green = !green;
    }
  }
}

// green.rs:225-292
static void direction_weights(Scratch& s, int pattern) {
  const float* vcd = s.vcd.data();
  const float* hcd = s.hcd.data();
  const float* dgintv = s.dgintv.data();
  const float* dginth = s.dginth.data();
  const float* w0 = s.dirwts0.data();
  const float* w1 = s.dirwts1.data();
  for (int rr = 6; rr < TS - 6; ++rr) {
    for (int cc = 6 + green_at_even(pattern, rr); cc < TS - 6; cc += 2) {
      const int i = rr * TS + cc;
      const float uave = vcd[i] + vcd[i - TS] + vcd[i - 2 * TS] + vcd[i - 3 * TS];
      const float dave = vcd[i] + vcd[i + TS] + vcd[i + 2 * TS] + vcd[i + 3 * TS];
      const float lave = hcd[i] + hcd[i - 1] + hcd[i - 2] + hcd[i - 3];
      const float rave = hcd[i] + hcd[i + 1] + hcd[i + 2] + hcd[i + 3];
      const float dgrbvvaru = sqr(vcd[i] - uave) + sqr(vcd[i - TS] - uave) + sqr(vcd[i - 2 * TS] - uave) + sqr(vcd[i - 3 * TS] - uave);
      const float dgrbvvard = sqr(vcd[i] - dave) + sqr(vcd[i + TS] - dave) + sqr(vcd[i + 2 * TS] - dave) + sqr(vcd[i + 3 * TS] - dave);
      const float dgrbhvarl = sqr(hcd[i] - lave) + sqr(hcd[i - 1] - lave) + sqr(hcd[i - 2] - lave) + sqr(hcd[i - 3] - lave);
      const float dgrbhvarr = sqr(hcd[i] - rave) + sqr(hcd[i + 1] - rave) + sqr(hcd[i + 2] - rave) + sqr(hcd[i + 3] - rave);
      const float hwt = w1[i - 1] / (w1[i - 1] + w1[i + 1]);
      const float vwt = w0[i - TS] / (w0[i + TS] + w0[i - TS]);
      const float vcdvar = EPSSQ + vwt * dgrbvvard + (1.0f - vwt) * dgrbvvaru;
      const float hcdvar = EPSSQ + hwt * dgrbhvarr + (1.0f - hwt) * dgrbhvarl;
      const float fluct_u = dgintv[i] + dgintv[i - TS] + dgintv[i - 2 * TS];
      const float fluct_d = dgintv[i] + dgintv[i + TS] + dgintv[i + 2 * TS];
      const float fluct_l = dginth[i] + dginth[i - 1] + dginth[i - 2];
      const float fluct_r = dginth[i] + dginth[i + 1] + dginth[i + 2];
      const float vcdvar1 = EPSSQ + vwt * fluct_d + (1.0f - vwt) * fluct_u;
      const float hcdvar1 = EPSSQ + hwt * fluct_r + (1.0f - hwt) * fluct_l;
      const float varwt = hcdvar / (vcdvar + hcdvar);
      const float diffwt = hcdvar1 / (vcdvar1 + hcdvar1);
      s.hvwt[i >> 1] = ((0.5f - varwt) * (0.5f - diffwt) > 0.0f &&
                        std::fabs(0.5f - diffwt) < std::fabs(0.5f - varwt))
                           ? varwt
                           : diffwt;
    }
  }
}

struct NyquistArea {
  int start_row, end_row, start_col, end_col;
};

// nyquist.rs:25-95
static bool detect(Scratch& s, int pattern, NyquistArea* area) {
  const float* c = s.cddiffsq.data();
  const float* d = s.delhvsqsum.data();
  for (int rr = 6; rr < TS - 6; ++rr) {
    for (int cc = 6 + green_at_even(pattern, rr); cc < TS - 6; cc += 2) {
      const int i = rr * TS + cc;
      s.nyqutest[i >> 1] =
          (GAUSSODD[0] * c[i] +
           GAUSSODD[1] * (c[i - TS - 1] + c[i - TS + 1] + c[i + TS - 1] + c[i + TS + 1]) +
           GAUSSODD[2] * (c[i - 2 * TS] + c[i - 2] + c[i + 2] + c[i + 2 * TS]) +
           GAUSSODD[3] * (c[i - 2 * TS - 2] + c[i - 2 * TS + 2] + c[i + 2 * TS - 2] + c[i + 2 * TS + 2])) -
          (GAUSSGRAD[0] * d[i] +
           GAUSSGRAD[1] * (d[i - TS] + d[i + 1] + d[i - 1] + d[i + TS]) +
           GAUSSGRAD[2] * (d[i - TS - 1] + d[i - TS + 1] + d[i + TS - 1] + d[i + TS + 1]) +
           GAUSSGRAD[3] * (d[i - 2 * TS] + d[i - 2] + d[i + 2] + d[i + 2 * TS]) +
           GAUSSGRAD[4] * (d[i - 2 * TS - 1] + d[i - 2 * TS + 1] + d[i - TS - 2] + d[i - TS + 2] +
                           d[i + TS - 2] + d[i + TS + 2] + d[i + 2 * TS - 1] + d[i + 2 * TS + 1]) +
           GAUSSGRAD[5] * (d[i - 2 * TS - 2] + d[i - 2 * TS + 2] + d[i + 2 * TS - 2] + d[i + 2 * TS + 2]));
    }
  }
  int start_row = 0, end_row = 0, start_col = TS + 1, end_col = 0;
  for (int rr = 6; rr < TS - 6; ++rr) {
    for (int cc = 6 + green_at_even(pattern, rr); cc < TS - 6; cc += 2) {
      const int i = rr * TS + cc;
      if (s.nyqutest[i >> 1] > 0.0f) {
        s.nyquist[i >> 1] = 1;
        if (start_row == 0) start_row = rr;
        end_row = rr;
        start_col = std::min(start_col, cc);
        end_col = std::max(end_col, cc);
      }
    }
  }
  if (start_row == end_row || start_col == end_col) return false;
  end_row += 1;
  end_col += 1;
  start_col -= start_col & 1;
  area->start_row = std::max(start_row, 8);
  area->end_row = std::min(end_row, TS - 8);
  area->start_col = std::max(start_col, 8);
  area->end_col = std::min(end_col, TS - 8);
  return true;
}

// nyquist.rs:108-170
static void area_interpolation(Scratch& s, int pattern, const NyquistArea& a) {
  const uint8_t* n = s.nyquist.data();
  for (int rr = a.start_row; rr < a.end_row; ++rr) {
    const long first = (long)rr * TS + a.start_col + green_at_even(pattern, rr);
    for (long i = first; i < (long)rr * TS + a.end_col; i += 2) {
      const unsigned votes = n[(i - V2) >> 1] + n[(i - M1) >> 1] + n[(i + P1) >> 1] + n[(i - 2) >> 1] +
                             n[(i + 2) >> 1] + n[(i - P1) >> 1] + n[(i + M1) >> 1] + n[(i + V2) >> 1];
      s.nyquist2[i >> 1] = votes >= 5 ? 1 : (votes == 4 ? n[i >> 1] : 0);
    }
  }
  const float* cfa = s.cfa.data();
  for (int rr = a.start_row; rr < a.end_row; ++rr) {
    const long first = (long)rr * TS + a.start_col + green_at_even(pattern, rr);
    for (long i = first; i < (long)rr * TS + a.end_col; i += 2) {
      if (s.nyquist2[i >> 1] == 0) continue;
      float sumcfa = 0.0f, sumh = 0.0f, sumv = 0.0f, sumsqh = 0.0f, sumsqv = 0.0f, areawt = 0.0f;
      for (int di = -6; di < 7; di += 2) {
        long i1 = i + di * V1 - 6;
        for (int dj = -6; dj < 7; dj += 2) {
          if (s.nyquist2[i1 >> 1] != 0) {
            const float c = cfa[i1];
            sumcfa += c;
            sumh += cfa[i1 - 1] + cfa[i1 + 1];
            sumv += cfa[i1 - V1] + cfa[i1 + V1];
            sumsqh += sqr(c - cfa[i1 - 1]) + sqr(c - cfa[i1 + 1]);
            sumsqv += sqr(c - cfa[i1 - V1]) + sqr(c - cfa[i1 + V1]);
            areawt += 1.0f;
          }
          i1 += 2;
        }
      }
      sumh = sumcfa - 0.5f * sumh;
      sumv = sumcfa - 0.5f * sumv;
      areawt *= 0.5f;
      const float hcdvar = EPSSQ + std::fabs(areawt * sumsqh - sumh * sumh);
      const float vcdvar = EPSSQ + std::fabs(areawt * sumsqv - sumv * sumv);
      s.hvwt[i >> 1] = hcdvar / (vcdvar + hcdvar);
    }
  }
}

// nyquist.rs:176-222: hvwt updated in place, rows in order.
static void populate_green(Scratch& s, int pattern) {
  float* hv = s.hvwt.data();
  float* green = s.green.data();
  for (int rr = 8; rr < TS - 8; ++rr) {
    for (int cc = 8 + green_at_even(pattern, rr); cc < TS - 8; cc += 2) {
      const int i = rr * TS + cc;
      const int i1 = i >> 1;
      const float alt = (hv[((rr - 1) * TS + cc - 1) >> 1] + hv[((rr - 1) * TS + cc + 1) >> 1] +
                         hv[((rr + 1) * TS + cc - 1) >> 1] + hv[((rr + 1) * TS + cc + 1) >> 1]) /
                        4.0f;
      if (std::fabs(0.5f - hv[i1]) < std::fabs(0.5f - alt)) hv[i1] = alt;
      s.dgrb0[i1] = intp(hv[i1], s.vcd[i], s.hcd[i]);
      green[i] = s.cfa[i] + s.dgrb0[i1];
      const bool flagged = s.nyquist2[i1] != 0;
      s.dgrb2_h[i1] = flagged ? sqr(green[i] - 0.5f * (green[i - 1] + green[i + 1])) : 0.0f;
      s.dgrb2_v[i1] = flagged ? sqr(green[i] - 0.5f * (green[i - TS] + green[i + TS])) : 0.0f;
    }
  }
}

// nyquist.rs:225-236
static void refine_green(Scratch& s, int pattern, const NyquistArea& a) {
  for (int rr = a.start_row; rr < a.end_row; ++rr) {
    const long first = (long)rr * TS + a.start_col + green_at_even(pattern, rr);
    for (long i = first; i < (long)rr * TS + a.end_col; i += 2) {
      if (s.nyquist2[i >> 1] == 0) continue;
      auto average = [&](const float* p) {
        return EPSSQ + (GQUINC[0] * p[i >> 1] +
                        GQUINC[1] * (p[(i - M1) >> 1] + p[(i + P1) >> 1] + p[(i - P1) >> 1] + p[(i + M1) >> 1]) +
                        GQUINC[2] * (p[(i - V2) >> 1] + p[(i - 2) >> 1] + p[(i + 2) >> 1] + p[(i + V2) >> 1]) +
                        GQUINC[3] * (p[(i - M2) >> 1] + p[(i + P2) >> 1] + p[(i - P2) >> 1] + p[(i + M2) >> 1]));
      };
      const float gvarh = average(s.dgrb2_h.data());
      const float gvarv = average(s.dgrb2_v.data());
      s.dgrb0[i >> 1] = (s.hcd[i] * gvarv + s.vcd[i] * gvarh) / (gvarv + gvarh);
      s.green[i] = s.cfa[i] + s.dgrb0[i >> 1];
    }
  }
}

// diagonal.rs:15-45
static void diagonal_gradients(Scratch& s, int pattern) {
  const float* cfa = s.cfa.data();
  for (int rr = 6; rr < TS - 6; ++rr) {
    const float* up = cfa + (rr - 1) * TS;
    const float* mid = cfa + rr * TS;
    const float* down = cfa + (rr + 1) * TS;
    float* delp = s.delp.data() + rr * TSH;
    float* delm = s.delm.data() + rr * TSH;
    float* sqp = s.sq1p.data() + rr * TSH;
    float* sqm = s.sq1m.data() + rr * TSH;
    if (green_at_even(pattern, rr) == 0) {
      for (int cc = 6; cc < TS - 6; cc += 2) {
        const int i1 = cc >> 1;
        delp[i1] = std::fabs(up[cc + 1] - down[cc - 1]);
        delm[i1] = std::fabs(down[cc + 1] - up[cc - 1]);
        const float g = mid[cc + 1];
        sqp[i1] = sqr(g - down[cc]) + sqr(g - up[cc + 2]);
        sqm[i1] = sqr(g - up[cc]) + sqr(g - down[cc + 2]);
      }
    } else {
      for (int cc = 6; cc < TS - 6; cc += 2) {
        const int i1 = cc >> 1;
        const float g = mid[cc];
        sqp[i1] = sqr(g - down[cc - 1]) + sqr(g - up[cc + 1]);
        sqm[i1] = sqr(g - up[cc - 1]) + sqr(g - down[cc + 1]);
        delp[i1] = std::fabs(up[cc + 2] - down[cc]);
        delm[i1] = std::fabs(down[cc + 2] - up[cc]);
      }
    }
  }
}

// diagonal.rs:49-62; rows[k] is the half row rr-2+k.
inline float even_kernel(const float* const rows[5], int cc) {
  return GAUSSEVEN[0] * (rows[1][cc >> 1] + rows[2][(cc - 1) >> 1] + rows[2][(cc + 1) >> 1] + rows[3][cc >> 1]) +
         GAUSSEVEN[1] * (rows[0][(cc - 1) >> 1] + rows[0][(cc + 1) >> 1] + rows[1][(cc - 2) >> 1] +
                         rows[1][(cc + 2) >> 1] + rows[3][(cc - 2) >> 1] + rows[3][(cc + 2) >> 1] +
                         rows[4][(cc - 1) >> 1] + rows[4][(cc + 1) >> 1]);
}
inline float diagonal_estimate(float centre, float near_, float far_) {
  const float ratio = 2.0f * near_ / (EPS + centre + far_);
  return std::fabs(1.0f - ratio) < ARTHRESH ? centre * ratio : near_ + 0.5f * (centre - far_);
}
inline float bound_diagonal(float estimate, float centre, float a, float b, float clip_pt) {
  float value = estimate;
  if (value < centre) {
    if (2.0f * value < centre) {
      value = median(value, a, b);
    } else {
      const float weight = 2.0f * (centre - value) / (EPS + value + centre);
      value = weight * value + (1.0f - weight) * median(value, a, b);
    }
  }
  return value > clip_pt ? median(value, a, b) : value;
}

// diagonal.rs:99-145
static void diagonal_estimates(Scratch& s, int pattern, float clip_pt) {
  const float* cfa = s.cfa.data();
  for (int rr = 8; rr < TS - 8; ++rr) {
    const float* delm[5];
    const float* delp[5];
    const float* sqm[5];
    const float* sqp[5];
    for (int k = 0; k < 5; ++k) {
      delm[k] = s.delm.data() + (rr + k - 2) * TSH;
      delp[k] = s.delp.data() + (rr + k - 2) * TSH;
      sqm[k] = s.sq1m.data() + (rr + k - 2) * TSH;
      sqp[k] = s.sq1p.data() + (rr + k - 2) * TSH;
    }
    for (int cc = 8 + green_at_even(pattern, rr); cc < TS - 8; cc += 2) {
      const int i = rr * TS + cc;
      const int i1 = cc >> 1;
      const float centre = cfa[i];
      const float se1 = cfa[i + TS + 1], se2 = cfa[i + 2 * TS + 2];
      const float nw1 = cfa[i - TS - 1], nw2 = cfa[i - 2 * TS - 2];
      const float ne1 = cfa[i - TS + 1], ne2 = cfa[i - 2 * TS + 2];
      const float sw1 = cfa[i + TS - 1], sw2 = cfa[i + 2 * TS - 2];
      const float rbse = diagonal_estimate(centre, se1, se2);
      const float rbnw = diagonal_estimate(centre, nw1, nw2);
      const float rbne = diagonal_estimate(centre, ne1, ne2);
      const float rbsw = diagonal_estimate(centre, sw1, sw2);
      const float wtse = EPS + delm[2][i1] + delm[3][(cc + 1) >> 1] + delm[4][(cc + 2) >> 1];
      const float wtnw = EPS + delm[2][i1] + delm[1][(cc - 1) >> 1] + delm[0][(cc - 2) >> 1];
      const float wtne = EPS + delp[2][i1] + delp[1][(cc + 1) >> 1] + delp[0][(cc + 2) >> 1];
      const float wtsw = EPS + delp[2][i1] + delp[3][(cc - 1) >> 1] + delp[4][(cc - 2) >> 1];
      const float rbm_est = (wtse * rbnw + wtnw * rbse) / (wtse + wtnw);
      const float rbp_est = (wtne * rbsw + wtsw * rbne) / (wtne + wtsw);
      const float rbvarm = EPSSQ + even_kernel(sqm, cc);
      s.pmwt[rr * TSH + i1] = rbvarm / ((EPSSQ + even_kernel(sqp, cc)) + rbvarm);
      s.rbp[rr * TSH + i1] = bound_diagonal(rbp_est, centre, sw1, ne1, clip_pt);
      s.rbm[rr * TSH + i1] = bound_diagonal(rbm_est, centre, nw1, se1, clip_pt);
    }
  }
}

// diagonal.rs:150-171: pmwt in place, rows in order.
static void combine_diagonals(Scratch& s, int pattern) {
  float* pm = s.pmwt.data();
  for (int rr = 10; rr < TS - 10; ++rr) {
    for (int cc = 10 + green_at_even(pattern, rr); cc < TS - 10; cc += 2) {
      const int i1 = cc >> 1;
      const float alt = (pm[(rr - 1) * TSH + ((cc - 1) >> 1)] + pm[(rr - 1) * TSH + ((cc + 1) >> 1)] +
                         pm[(rr + 1) * TSH + ((cc - 1) >> 1)] + pm[(rr + 1) * TSH + ((cc + 1) >> 1)]) /
                        4.0f;
      float& p = pm[rr * TSH + i1];
      if (std::fabs(0.5f - p) < std::fabs(0.5f - alt)) p = alt;
      s.rbint[rr * TSH + i1] = 0.5f * (s.cfa[rr * TS + cc] + s.rbm[rr * TSH + i1] * (1.0f - p) + s.rbp[rr * TSH + i1] * p);
    }
  }
}

inline float green_from_rb(float sample, float centre, float other) {
  const float ratio = sample * 2.0f / (EPS + centre + other);
  return std::fabs(1.0f - ratio) < ARTHRESH ? centre * ratio : sample + 0.5f * (centre - other);
}

// diagonal.rs:205-247
static void refine_green_with_rb(Scratch& s, int pattern, float clip_pt) {
  const float* cfa = s.cfa.data();
  const float* w0 = s.dirwts0.data();
  const float* w1 = s.dirwts1.data();
  for (int rr = 12; rr < TS - 12; ++rr) {
    const float* rb_up = s.rbint.data() + (rr - 2) * TSH;
    const float* rb = s.rbint.data() + rr * TSH;
    const float* rb_down = s.rbint.data() + (rr + 2) * TSH;
    for (int cc = 12 + green_at_even(pattern, rr); cc < TS - 12; cc += 2) {
      const int i = rr * TS + cc;
      const int i1 = cc >> 1;
      const float pmwt = s.pmwt[rr * TSH + i1];
      const float hvwt = s.hvwt[rr * TSH + i1];
      if (std::fabs(0.5f - pmwt) < std::fabs(0.5f - hvwt)) continue;
      const float centre = rb[i1];
      const float gu = green_from_rb(cfa[i - TS], centre, rb_up[i1]);
      const float gd = green_from_rb(cfa[i + TS], centre, rb_down[i1]);
      const float gl = green_from_rb(cfa[i - 1], centre, rb[i1 - 1]);
      const float gr = green_from_rb(cfa[i + 1], centre, rb[i1 + 1]);
      float gintv = (w0[i - TS] * gd + w0[i + TS] * gu) / (w0[i + TS] + w0[i - TS]);
      float ginth = (w1[i - 1] * gr + w1[i + 1] * gl) / (w1[i - 1] + w1[i + 1]);
      gintv = bound_diagonal(gintv, centre, cfa[i - TS], cfa[i + TS], clip_pt);
      ginth = bound_diagonal(ginth, centre, cfa[i - 1], cfa[i + 1], clip_pt);
      s.green[i] = ginth * (1.0f - hvwt) + gintv * hvwt;
      s.dgrb0[rr * TSH + i1] = s.green[i] - cfa[i];
    }
  }
}

// chroma.rs:11-19
static void red_offset(int pattern, int* ey, int* ex) {
  const int c00 = color_at(pattern, 0, 0), c10 = color_at(pattern, 1, 0);
  if (c00 == 1 && c10 == 0) { *ey = 0; *ex = 1; }
  else if (c00 == 1) { *ey = 1; *ex = 0; }
  else if (c00 == 0) { *ey = 0; *ex = 0; }
  else { *ey = 1; *ex = 1; }
}

// chroma.rs:23-91
static void interpolate_chroma(Scratch& s, int pattern) {
  int ey, ex;
  red_offset(pattern, &ey, &ex);
  for (int rr = 13 - ey; rr < TS - 12; rr += 2) {
    for (int i1 = (rr * TS + 13 - ex) >> 1; i1 < ((rr * TS + TS - 12) >> 1); ++i1) {
      s.dgrb1[i1] = s.dgrb0[i1];
      s.dgrb0[i1] = 0.0f;
    }
  }
  for (int rr = 14; rr < TS - 14; ++rr) {
    const int start = 14 + green_at_even(pattern, rr);
    const int plane = 1 - fc(pattern, rr, start) / 2;
    float* p = plane == 0 ? s.dgrb0.data() : s.dgrb1.data();
    auto d = [&](int dr, int cc, int dc) { return p[(rr + dr) * TSH + ((cc + dc) >> 1)]; };
    for (int cc = start; cc < TS - 14; cc += 2) {
      const float wtnw = 1.0f / (EPS + std::fabs(d(-1, cc, -1) - d(1, cc, 1)) +
                                 std::fabs(d(-1, cc, -1) - d(-3, cc, -3)) +
                                 std::fabs(d(1, cc, 1) - d(-3, cc, -3)));
      const float wtne = 1.0f / (EPS + std::fabs(d(-1, cc, 1) - d(1, cc, -1)) +
                                 std::fabs(d(-1, cc, 1) - d(-3, cc, 3)) +
                                 std::fabs(d(1, cc, -1) - d(-3, cc, 3)));
      const float wtsw = 1.0f / (EPS + std::fabs(d(1, cc, -1) - d(-1, cc, 1)) +
                                 std::fabs(d(1, cc, -1) - d(3, cc, 3)) +
                                 std::fabs(d(-1, cc, 1) - d(3, cc, -3)));
      const float wtse = 1.0f / (EPS + std::fabs(d(1, cc, 1) - d(-1, cc, -1)) +
                                 std::fabs(d(1, cc, 1) - d(3, cc, -3)) +
                                 std::fabs(d(-1, cc, -1) - d(3, cc, 3)));
      p[rr * TSH + (cc >> 1)] =
          (wtnw * (1.325f * d(-1, cc, -1) - 0.175f * d(-3, cc, -3) - 0.075f * d(-1, cc, -3) - 0.075f * d(-3, cc, -1)) +
           wtne * (1.325f * d(-1, cc, 1) - 0.175f * d(-3, cc, 3) - 0.075f * d(-1, cc, 3) - 0.075f * d(1, cc, 1)) +
           wtsw * (1.325f * d(1, cc, -1) - 0.175f * d(3, cc, -3) - 0.075f * d(1, cc, -3) - 0.075f * d(-1, cc, -1)) +
           wtse * (1.325f * d(1, cc, 1) - 0.175f * d(3, cc, 3) - 0.075f * d(1, cc, 3) - 0.075f * d(3, cc, 1))) /
          (wtnw + wtne + wtsw + wtse);
    }
  }
}

// chroma.rs:98-147
static void finish_planes(Scratch& s, int pattern) {
  for (int rr = 16; rr < TS - 16; ++rr) {
    const float* green = s.green.data() + rr * TS;
    const float* hv_up = s.hvwt.data() + (rr - 1) * TSH;
    const float* hv = s.hvwt.data() + rr * TSH;
    const float* hv_down = s.hvwt.data() + (rr + 1) * TSH;
    const float* gr_up = s.dgrb0.data() + (rr - 1) * TSH;
    const float* gr = s.dgrb0.data() + rr * TSH;
    const float* gr_down = s.dgrb0.data() + (rr + 1) * TSH;
    const float* gb_up = s.dgrb1.data() + (rr - 1) * TSH;
    const float* gb = s.dgrb1.data() + rr * TSH;
    const float* gb_down = s.dgrb1.data() + (rr + 1) * TSH;
    float* red = s.red.data() + rr * TS;
    float* blue = s.blue.data() + rr * TS;
    auto at_green = [&](int cc, float* r, float* b) {
      const float up = hv_up[cc >> 1], down = hv_down[cc >> 1];
      const float left = hv[(cc - 1) >> 1], right = hv[(cc + 1) >> 1];
      const float temp = 1.0f / (up + 2.0f - right - left + down);
      auto blend = [&](const float* d_up, const float* d, const float* d_down) {
        return (up * d_up[cc >> 1] + (1.0f - right) * d[(cc + 1) >> 1] + (1.0f - left) * d[(cc - 1) >> 1] +
                down * d_down[cc >> 1]) *
               temp;
      };
      *r = green[cc] - blend(gr_up, gr, gr_down);
      *b = green[cc] - blend(gb_up, gb, gb_down);
    };
    auto at_red_blue = [&](int cc, float* r, float* b) {
      *r = green[cc] - gr[cc >> 1];
      *b = green[cc] - gb[cc >> 1];
    };
    const bool green_first = fc(pattern, rr, 16) == 1;
    for (int cc = 16; cc < TS - 16; cc += 2) {
      float r0, b0, r1, b1;
      if (green_first) {
        at_green(cc, &r0, &b0);
        at_red_blue(cc + 1, &r1, &b1);
      } else {
        at_red_blue(cc, &r0, &b0);
        at_green(cc + 1, &r1, &b1);
      }
      red[cc] = fmax_(r0, 0.0f);
      blue[cc] = fmax_(b0, 0.0f);
      red[cc + 1] = fmax_(r1, 0.0f);
      blue[cc + 1] = fmax_(b1, 0.0f);
    }
  }
}

// mod.rs:136-164
static void reconstruct_tile(Scratch& s, int pattern, float clip_point) {
  const float clip_pt8 = 0.8f * clip_point;
  gradients(s);
  colour_differences(s, pattern, clip_pt8);
  bound_differences(s, pattern, clip_point);
  direction_weights(s, pattern);
  NyquistArea area;
  const bool has_area = detect(s, pattern, &area);
  if (has_area) area_interpolation(s, pattern, area);
  populate_green(s, pattern);
  if (has_area) refine_green(s, pattern, area);
  diagonal_gradients(s, pattern);
  diagonal_estimates(s, pattern, clip_point);
  combine_diagonals(s, pattern);
  refine_green_with_rb(s, pattern, clip_point);
  interpolate_chroma(s, pattern);
  finish_planes(s, pattern);
}

// mod.rs:175-194
static void populate(Scratch& s, const float* mosaic, int w, int h, int stride, int origin_x, int origin_y) {
  const long first_x = (long)origin_x - BORDER;
  for (int row = 0; row < TS; ++row) {
    const std::size_t sy = mirror_coordinate((long long)origin_y + row - BORDER, h);
    for (int col = 0; col < TS; ++col) {
      const std::size_t sx = mirror_coordinate(first_x + col, w);
      const float v = mosaic[sy * (std::size_t)stride + sx];
      s.cfa[row * TS + col] = v;
      s.green[row * TS + col] = v;
    }
  }
}

}  // namespace amaze
}  // namespace oracle

using namespace oracle;

extern "C" int ro_amaze_reconstruct(const float* mosaic, int w, int h, int stride, int pattern,
                                    const float gains[3], float clip_point, float* out, int out_stride) {
  using namespace oracle::amaze;
  if (w <= 2 * BORDER || h <= 2 * BORDER) {
    ro_bilinear_reconstruct(mosaic, w, h, stride, pattern, gains, out, out_stride);
    return 0;
  }
  const int cols = (w + VALID - 1) / VALID;
  const int rows = (h + VALID - 1) / VALID;
  int bad = 0;
#pragma omp parallel
  {
    Scratch s;
#pragma omp for schedule(dynamic) reduction(| : bad)
    for (int t = 0; t < cols * rows; ++t) {
      const int tx = t % cols, ty = t / cols;
      const int ox = tx * VALID, oy = ty * VALID;
      // mod.rs:122: the tile pattern is the image pattern shifted by the (even) origin.
      const int tpattern = shifted(pattern, 0, oy);
      s.clear();
      populate(s, mosaic, w, h, stride, ox, oy);
      reconstruct_tile(s, tpattern, clip_point);
      // write_tile, mod.rs:196-268
      const int x_end = std::min(ox + VALID, w), y_end = std::min(oy + VALID, h);
      for (int gy = oy; gy < y_end; ++gy) {
        const int ly = gy - oy + BORDER;
        for (int gx = ox; gx < x_end; ++gx) {
          const int lx = gx - ox + BORDER;
          const int at = ly * TS + lx;
          const float sample = mosaic[(std::size_t)gy * stride + gx];
          const int channel = color_at(pattern, gx, gy);
          float rgb[3] = {channel == 0 ? sample : s.red[at],
                          channel == 1 ? sample : amaze::fmax_(s.green[at], 0.0f),
                          channel == 2 ? sample : s.blue[at]};
          rgb[0] *= gains[0];
          rgb[1] *= gains[1];
          rgb[2] *= gains[2];
          if (!std::isfinite(rgb[0]) || !std::isfinite(rgb[1]) || !std::isfinite(rgb[2])) bad |= 1;
          float* o = out + (std::size_t)gy * out_stride + 3 * (std::size_t)gx;
          o[0] = rgb[0];
          o[1] = rgb[1];
          o[2] = rgb[2];
        }
      }
    }
  }
  return bad ? -1 : 0;
}

// Stage probes on one tile at origin (0, 0): runs every stage and copies the
// named plane out (full planes 256x256, half planes 256x128), for the
// reference's bit-exact stage snapshot (crates/demosaic/src/amaze/mod.rs:336-427).
extern "C" int ro_amaze_probe_tile(const float* mosaic, int w, int h, int stride, int pattern,
                                   float clip_point, const char* plane, float* out) {
  using namespace oracle::amaze;
  Scratch s;
  s.clear();
  populate(s, mosaic, w, h, stride, 0, 0);
  reconstruct_tile(s, pattern, clip_point);
  const std::vector<float>* full = nullptr;
  const std::vector<float>* half = nullptr;
  const std::vector<uint8_t>* flags = nullptr;
  const std::string name(plane);
  if (name == "cfa") full = &s.cfa; else if (name == "green") full = &s.green;
  else if (name == "delhvsqsum") full = &s.delhvsqsum; else if (name == "dirwts0") full = &s.dirwts0;
  else if (name == "dirwts1") full = &s.dirwts1; else if (name == "vcd") full = &s.vcd;
  else if (name == "hcd") full = &s.hcd; else if (name == "vcdalt") full = &s.vcdalt;
  else if (name == "hcdalt") full = &s.hcdalt; else if (name == "cddiffsq") full = &s.cddiffsq;
  else if (name == "dgintv") full = &s.dgintv; else if (name == "dginth") full = &s.dginth;
  else if (name == "hvwt") half = &s.hvwt; else if (name == "dgrb0") half = &s.dgrb0;
  else if (name == "dgrb1") half = &s.dgrb1; else if (name == "dgrb2_h") half = &s.dgrb2_h;
  else if (name == "dgrb2_v") half = &s.dgrb2_v; else if (name == "delp") half = &s.delp;
  else if (name == "delm") half = &s.delm; else if (name == "sq1m") half = &s.sq1m;
  else if (name == "sq1p") half = &s.sq1p; else if (name == "nyqutest") half = &s.nyqutest;
  else if (name == "pmwt") half = &s.pmwt; else if (name == "rbm") half = &s.rbm;
  else if (name == "rbp") half = &s.rbp; else if (name == "rbint") half = &s.rbint;
  else if (name == "nyquist") flags = &s.nyquist; else if (name == "nyquist2") flags = &s.nyquist2;
  else return -1;
  if (full) std::memcpy(out, full->data(), sizeof(float) * TS * TS);
  if (half) std::memcpy(out, half->data(), sizeof(float) * TS * TSH);
  if (flags)
    for (int k = 0; k < TS * TSH; ++k) out[k] = (*flags)[k];
  return 0;
}
