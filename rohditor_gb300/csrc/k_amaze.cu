// AMaZE demosaic on sm_103a.
//
// The reference reconstructs 256-pixel tiles with a 16-pixel mirrored halo
// (crates/demosaic/src/amaze_geometry.rs:13-15, amaze/mod.rs:60-214), and its
// result depends on that tile grid: each tile keeps its own Nyquist bounding
// box (amaze/nyquist.rs:25-95) and several stages are in-place raster-order
// recurrences whose start depends on the tile edge. This kernel keeps the grid
// and the arithmetic bit-identical and maps the work as follows:
//
//  * one persistent CTA (512 threads) per tile in flight; each CTA owns a
//    scratch slot of 12 full + 14 half planes (~5 MB) that stays hot in L2;
//  * the raw u16 samples are normalized, clipped and channel-balanced while
//    the tile is loaded (MosaicSource), so no f32 mosaic is written to HBM;
//  * the recurrences are restated exactly:
//      - bound_differences (green.rs:187-222): hcd is a recurrence along each
//        row with stride 2 and vcd along each column with stride 2; every
//        (row, parity) and (column, parity) chain runs in its own thread;
//      - populate_green / combine_diagonals (nyquist.rs:176-222,
//        diagonal.rs:150-171): the hvwt / pmwt updates read the already
//        updated row above, so rows are swept in order with a CTA barrier,
//        and the per-site products that only read the final weight run as a
//        separate parallel pass;
//  * everything else is a parallel sweep between CTA barriers;
//  * the tile core is written straight to the planar RGB output, with the
//    measured sample restored, green clamped at zero and the inverse balance
//    applied (amaze/mod.rs:196-268).
// The file is compiled with --fmad=false so no multiply-add is fused, as in
// the reference.
#include <cuda_runtime.h>

#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr int TS = 256, TSH = 128, BORDER = 16, VALID = TS - 2 * BORDER;
constexpr int FULL = TS * TS, HALFN = TS * TSH;
constexpr int THREADS = 512;

enum { P_CFA, P_GREEN, P_DELHV, P_W0, P_W1, P_VCD, P_HCD, P_VCDALT, P_HCDALT, P_CDD, P_DGINTV, P_DGINTH, N_FULL };
enum { H_HVWT, H_DGRB0, H_DGRB1, H_D2H, H_D2V, H_DELP, H_DELM, H_SQ1M, H_SQ1P, H_NYQT, H_PMWT, H_RBM, H_RBP,
       H_RBINT, N_HALF };
// Two u8 flag planes (nyquist, nyquist2) follow, HALFN bytes each.
constexpr size_t SLOT_FLOATS = (size_t)N_FULL * FULL + (size_t)N_HALF * HALFN + (2 * HALFN) / 4;

constexpr long V1 = TS, V2 = 2 * TS, P1 = -TS + 1, P2 = -2 * TS + 2, M1 = TS + 1, M2 = 2 * TS + 2;
constexpr float EPS = 1.0e-5f, EPSSQ = 1.0e-10f, ARTHRESH = 0.75f;
__constant__ float GAUSSODD[4] = {0.14659727707323927f, 0.103592713382435f, 0.0732036125103057f,
                                  0.0365543548389495f};
__constant__ float GAUSSGRAD[6] = {0.5f * 0.07384411893421103f, 0.5f * 0.06207511968171489f,
                                   0.5f * 0.0521818194747806f,  0.5f * 0.03687419286733595f,
                                   0.5f * 0.03099732204057846f, 0.5f * 0.018413194161458882f};
__constant__ float GAUSSEVEN[2] = {0.13719494435797422f, 0.05640252782101291f};
__constant__ float GQUINC[4] = {0.169917f, 0.108947f, 0.069855f, 0.0287182f};

__device__ __forceinline__ float sqr(float x) { return x * x; }
__device__ __forceinline__ float fmin_(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float fmax_(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float median(float a, float b, float c) {
  return fmax_(fmin_(a, b), fmin_(fmax_(b, a), c));
}
__device__ __forceinline__ float intp(float a, float b, float c) { return a * (b - c) + c; }
__device__ __forceinline__ int fc(int pattern, int row, int col) { return color_at(pattern, col, row); }
__device__ __forceinline__ int gae(int pattern, int row) { return fc(pattern, row, 2) & 1; }
__device__ __forceinline__ float adaptive_or(float ratio, float centre, float fallback) {
  return fabsf(1.0f - ratio) < ARTHRESH ? centre * ratio : fallback;
}
__device__ __forceinline__ float bound_at_green(float d, float cur, float a, float b, float clip_pt) {
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
__device__ __forceinline__ float bound_at_red_blue(float d, float cur, float a, float b, float clip_pt) {
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
__device__ __forceinline__ float spread(float a, float b, float c) {
  return 3.0f * (sqr(a) + sqr(b) + sqr(c)) - sqr(a + b + c);
}
__device__ __forceinline__ float diagonal_estimate(float centre, float n, float f) {
  const float ratio = 2.0f * n / (EPS + centre + f);
  return fabsf(1.0f - ratio) < ARTHRESH ? centre * ratio : n + 0.5f * (centre - f);
}
__device__ __forceinline__ float bound_diagonal(float estimate, float centre, float a, float b, float clip_pt) {
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
__device__ __forceinline__ float green_from_rb(float sample, float centre, float other) {
  const float ratio = sample * 2.0f / (EPS + centre + other);
  return fabsf(1.0f - ratio) < ARTHRESH ? centre * ratio : sample + 0.5f * (centre - other);
}

struct Planes {
  float* f[N_FULL];
  float* h[N_HALF];
  unsigned char* nyq;
  unsigned char* nyq2;
};

__device__ __forceinline__ Planes slot_planes(float* base) {
  Planes p;
  for (int k = 0; k < N_FULL; ++k) p.f[k] = base + (size_t)k * FULL;
  float* hb = base + (size_t)N_FULL * FULL;
  for (int k = 0; k < N_HALF; ++k) p.h[k] = hb + (size_t)k * HALFN;
  p.nyq = reinterpret_cast<unsigned char*>(hb + (size_t)N_HALF * HALFN);
  p.nyq2 = p.nyq + HALFN;
  return p;
}

// Number of red/blue sites in [c0 + gae, c1) with step 2.
__device__ __forceinline__ int site_count(int c0, int c1) { return (c1 - c0 + 1) / 2; }

struct AmazeParams {
  MosaicSource src;
  float* out;              // planar RGB, 3 * width * height
  float* scratch;          // SLOT_FLOATS per CTA
  int tiles_x, tiles_y;
  float clip_point;
  float gains[3];          // inverse balance applied to the output
  int count_clip;          // 1: accumulate Clip statistics of core pixels
  unsigned long long* clip_stats;
  unsigned int* error;
};

__global__ void __launch_bounds__(THREADS, 2) amaze_kernel(const AmazeParams prm) {
  const MosaicSource& src = prm.src;
  Planes P = slot_planes(prm.scratch + (size_t)blockIdx.x * SLOT_FLOATS);
  float* cfa = P.f[P_CFA];
  float* green = P.f[P_GREEN];
  float* w0 = P.f[P_W0];
  float* w1 = P.f[P_W1];
  float* vcd = P.f[P_VCD];
  float* hcd = P.f[P_HCD];
  float* vcdalt = P.f[P_VCDALT];
  float* hcdalt = P.f[P_HCDALT];
  float* cdd = P.f[P_CDD];
  float* delhv = P.f[P_DELHV];
  float* dgintv = P.f[P_DGINTV];
  float* dginth = P.f[P_DGINTH];
  float* hvwt = P.h[H_HVWT];
  float* dgrb0 = P.h[H_DGRB0];
  float* dgrb1 = P.h[H_DGRB1];
  float* d2h = P.h[H_D2H];
  float* d2v = P.h[H_D2V];
  float* pmwt = P.h[H_PMWT];
  const int t = threadIdx.x;
  const int pattern = src.cfa;
  const float clip_pt = prm.clip_point;
  const float clip_pt8 = 0.8f * clip_pt;
  const int W = src.width, H = src.height;
  const long long plane = (long long)W * H;
  __shared__ int s_box[4];
  __shared__ unsigned long long s_stats[6];
  __shared__ int s_bad;

  const int ntiles = prm.tiles_x * prm.tiles_y;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int ox = (tile % prm.tiles_x) * VALID, oy = (tile / prm.tiles_x) * VALID;

    // ---- populate (mod.rs:175-194) and per-tile clears (scratch.rs:105-111)
    for (int k = t; k < FULL; k += THREADS) {
      const int row = k >> 8, col = k & (TS - 1);
      const int sx = mirror_index(ox - BORDER + col, W), sy = mirror_index(oy - BORDER + row, H);
      const float v = source_balanced(src, sx, sy);
      cfa[k] = v;
      green[k] = v;
    }
    for (int k = t; k < HALFN; k += THREADS) {
      P.nyq[k] = 0;
      P.nyq2[k] = 0;
      d2h[k] = 0.0f;
      d2v[k] = 0.0f;
    }
    if (t < 6) s_stats[t] = 0;
    if (t == 0) {
      s_box[0] = TS; s_box[1] = 0; s_box[2] = TS + 1; s_box[3] = 0;
      s_bad = 0;
    }
    __syncthreads();

    // ---- gradients (green.rs:13-29)
    for (int k = t; k < (TS - 4) * (TS - 4); k += THREADS) {
      const int rr = 2 + k / (TS - 4), cc = 2 + k % (TS - 4);
      const int i = rr * TS + cc;
      const float delh = fabsf(cfa[i + 1] - cfa[i - 1]);
      const float delv = fabsf(cfa[i + TS] - cfa[i - TS]);
      w0[i] = EPS + fabsf(cfa[i + 2 * TS] - cfa[i]) + fabsf(cfa[i] - cfa[i - 2 * TS]) + delv;
      w1[i] = EPS + fabsf(cfa[i + 2] - cfa[i]) + fabsf(cfa[i] - cfa[i - 2]) + delh;
      delhv[i] = sqr(delh) + sqr(delv);
    }
    __syncthreads();

    // ---- colour differences (green.rs:46-139)
    for (int k = t; k < (TS - 8) * (TS - 8); k += THREADS) {
      const int rr = 4 + k / (TS - 8), cc = 4 + k % (TS - 8);
      const int i = rr * TS + cc;
      const bool green_first = (fc(pattern, rr, 4) & 1) == 1;
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
      float v, h, va, ha;
      if (fcswitch) {
        v = cur - (vwt * gdar + (1.0f - vwt) * guar);
        h = cur - (hwt * grar + (1.0f - hwt) * glar);
        va = cur - gintvha;
        ha = cur - ginthha;
      } else {
        v = (vwt * gdar + (1.0f - vwt) * guar) - cur;
        h = (hwt * grar + (1.0f - hwt) * glar) - cur;
        va = gintvha - cur;
        ha = ginthha - cur;
      }
      const bool clipped = (cur > clip_pt8) | (gintvha > clip_pt8) | (ginthha > clip_pt8);
      if (clipped) {
        guar = guha; gdar = gdha; glar = glha; grar = grha;
        v = va; h = ha;
      }
      dgintv[i] = fmin_(sqr(guha - gdha), sqr(guar - gdar));
      dginth[i] = fmin_(sqr(glha - grha), sqr(glar - grar));
      vcd[i] = v;
      hcd[i] = h;
      vcdalt[i] = va;
      hcdalt[i] = ha;
    }
    __syncthreads();

    // ---- bound_differences (green.rs:187-222): exact chain restatement.
    if (t < 2 * (TS - 8)) {
      const int line = 4 + (t >> 1), par = t & 1;
      // Horizontal chain: row `line`, columns 4+par, 6+par, ...
      const int hr = line;
      const bool hg4 = (fc(pattern, hr, 4) & 1) == 1;
      float prev_h = hcd[hr * TS + 2 + par];
      // Vertical chain: column `line`, rows 4+par, 6+par, ...
      const int vc = line;
      float prev_v = vcd[(2 + par) * TS + vc];
      for (int k = 0; k < (TS - 8) / 2; ++k) {
        {
          const int cc = 4 + par + 2 * k;
          const int i = hr * TS + cc;
          const float hcdvar = spread(prev_h, hcd[i], hcd[i + 2]);
          const float hcdaltvar = spread(hcdalt[i - 2], hcdalt[i], hcdalt[i + 2]);
          const float hsel = hcdaltvar < hcdvar ? hcdalt[i] : hcd[i];
          const bool g = hg4 != (((cc - 4) & 1) == 1);
          const float cur = cfa[i];
          const float b = g ? bound_at_green(hsel, cur, cfa[i - 1], cfa[i + 1], clip_pt)
                            : bound_at_red_blue(hsel, cur, cfa[i - 1], cfa[i + 1], clip_pt);
          hcd[i] = b;
          prev_h = b;
        }
        {
          const int rr = 4 + par + 2 * k;
          const int i = rr * TS + vc;
          const float vcdvar = spread(prev_v, vcd[i], vcd[i + 2 * TS]);
          const float vcdaltvar = spread(vcdalt[i - 2 * TS], vcdalt[i], vcdalt[i + 2 * TS]);
          const float vsel = vcdaltvar < vcdvar ? vcdalt[i] : vcd[i];
          const bool g = ((fc(pattern, rr, 4) & 1) == 1) != (((vc - 4) & 1) == 1);
          const float cur = cfa[i];
          const float b = g ? bound_at_green(vsel, cur, cfa[i - TS], cfa[i + TS], clip_pt)
                            : bound_at_red_blue(vsel, cur, cfa[i - TS], cfa[i + TS], clip_pt);
          vcd[i] = b;
          prev_v = b;
        }
      }
    }
    __syncthreads();
    for (int k = t; k < (TS - 8) * (TS - 8); k += THREADS) {
      const int rr = 4 + k / (TS - 8), cc = 4 + k % (TS - 8);
      const bool g = ((fc(pattern, rr, 4) & 1) == 1) != (((cc - 4) & 1) == 1);
      if (!g) {
        const int i = rr * TS + cc;
        cdd[i] = sqr(vcd[i] - hcd[i]);
      }
    }
    __syncthreads();

    // ---- direction_weights (green.rs:225-292)
    {
      const int per_row = site_count(6, TS - 6);
      for (int k = t; k < (TS - 12) * per_row; k += THREADS) {
        const int rr = 6 + k / per_row;
        const int cc = 6 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 6) continue;
        const int i = rr * TS + cc;
        const float uave = vcd[i] + vcd[i - TS] + vcd[i - 2 * TS] + vcd[i - 3 * TS];
        const float dave = vcd[i] + vcd[i + TS] + vcd[i + 2 * TS] + vcd[i + 3 * TS];
        const float lave = hcd[i] + hcd[i - 1] + hcd[i - 2] + hcd[i - 3];
        const float rave = hcd[i] + hcd[i + 1] + hcd[i + 2] + hcd[i + 3];
        const float vu = sqr(vcd[i] - uave) + sqr(vcd[i - TS] - uave) + sqr(vcd[i - 2 * TS] - uave) + sqr(vcd[i - 3 * TS] - uave);
        const float vd = sqr(vcd[i] - dave) + sqr(vcd[i + TS] - dave) + sqr(vcd[i + 2 * TS] - dave) + sqr(vcd[i + 3 * TS] - dave);
        const float hl = sqr(hcd[i] - lave) + sqr(hcd[i - 1] - lave) + sqr(hcd[i - 2] - lave) + sqr(hcd[i - 3] - lave);
        const float hrr = sqr(hcd[i] - rave) + sqr(hcd[i + 1] - rave) + sqr(hcd[i + 2] - rave) + sqr(hcd[i + 3] - rave);
        const float hwt = w1[i - 1] / (w1[i - 1] + w1[i + 1]);
        const float vwt = w0[i - TS] / (w0[i + TS] + w0[i - TS]);
        const float vcdvar = EPSSQ + vwt * vd + (1.0f - vwt) * vu;
        const float hcdvar = EPSSQ + hwt * hrr + (1.0f - hwt) * hl;
        const float fu = dgintv[i] + dgintv[i - TS] + dgintv[i - 2 * TS];
        const float fd = dgintv[i] + dgintv[i + TS] + dgintv[i + 2 * TS];
        const float fl = dginth[i] + dginth[i - 1] + dginth[i - 2];
        const float fr = dginth[i] + dginth[i + 1] + dginth[i + 2];
        const float vcdvar1 = EPSSQ + vwt * fd + (1.0f - vwt) * fu;
        const float hcdvar1 = EPSSQ + hwt * fr + (1.0f - hwt) * fl;
        const float varwt = hcdvar / (vcdvar + hcdvar);
        const float diffwt = hcdvar1 / (vcdvar1 + hcdvar1);
        hvwt[i >> 1] = ((0.5f - varwt) * (0.5f - diffwt) > 0.0f && fabsf(0.5f - diffwt) < fabsf(0.5f - varwt))
                           ? varwt
                           : diffwt;
      }
    }
    __syncthreads();

    // ---- Nyquist test (nyquist.rs:25-95)
    {
      float* nyqt = P.h[H_NYQT];
      const float* c = cdd;
      const float* d = delhv;
      const int per_row = site_count(6, TS - 6);
      for (int k = t; k < (TS - 12) * per_row; k += THREADS) {
        const int rr = 6 + k / per_row;
        const int cc = 6 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 6) continue;
        const int i = rr * TS + cc;
        const float v =
            (GAUSSODD[0] * c[i] + GAUSSODD[1] * (c[i - TS - 1] + c[i - TS + 1] + c[i + TS - 1] + c[i + TS + 1]) +
             GAUSSODD[2] * (c[i - 2 * TS] + c[i - 2] + c[i + 2] + c[i + 2 * TS]) +
             GAUSSODD[3] * (c[i - 2 * TS - 2] + c[i - 2 * TS + 2] + c[i + 2 * TS - 2] + c[i + 2 * TS + 2])) -
            (GAUSSGRAD[0] * d[i] + GAUSSGRAD[1] * (d[i - TS] + d[i + 1] + d[i - 1] + d[i + TS]) +
             GAUSSGRAD[2] * (d[i - TS - 1] + d[i - TS + 1] + d[i + TS - 1] + d[i + TS + 1]) +
             GAUSSGRAD[3] * (d[i - 2 * TS] + d[i - 2] + d[i + 2] + d[i + 2 * TS]) +
             GAUSSGRAD[4] * (d[i - 2 * TS - 1] + d[i - 2 * TS + 1] + d[i - TS - 2] + d[i - TS + 2] + d[i + TS - 2] +
                             d[i + TS + 2] + d[i + 2 * TS - 1] + d[i + 2 * TS + 1]) +
             GAUSSGRAD[5] * (d[i - 2 * TS - 2] + d[i - 2 * TS + 2] + d[i + 2 * TS - 2] + d[i + 2 * TS + 2]));
        nyqt[i >> 1] = v;
        if (v > 0.0f) {
          P.nyq[i >> 1] = 1;
          atomicMin(&s_box[0], rr);
          atomicMax(&s_box[1], rr);
          atomicMin(&s_box[2], cc);
          atomicMax(&s_box[3], cc);
        }
      }
    }
    __syncthreads();
    int start_row = s_box[0], end_row = s_box[1], start_col = s_box[2], end_col = s_box[3];
    if (start_row == TS) start_row = 0;  // no flagged site
    const bool has_area = !(start_row == end_row || start_col == end_col);
    if (has_area) {
      end_row += 1;
      end_col += 1;
      start_col -= start_col & 1;
      start_row = max(start_row, 8);
      end_row = min(end_row, TS - 8);
      start_col = max(start_col, 8);
      end_col = min(end_col, TS - 8);
    }
    const int area_rows = has_area ? max(end_row - start_row, 0) : 0;
    const int area_sites = has_area ? (end_col - start_col + 1) / 2 + 1 : 0;

    // ---- area interpolation (nyquist.rs:108-170)
    if (has_area) {
      for (int k = t; k < area_rows * area_sites; k += THREADS) {
        const int rr = start_row + k / area_sites;
        const long i = (long)rr * TS + start_col + gae(pattern, rr) + 2 * (k % area_sites);
        if (i >= (long)rr * TS + end_col) continue;
        const unsigned char* n = P.nyq;
        const unsigned votes = n[(i - V2) >> 1] + n[(i - M1) >> 1] + n[(i + P1) >> 1] + n[(i - 2) >> 1] +
                               n[(i + 2) >> 1] + n[(i - P1) >> 1] + n[(i + M1) >> 1] + n[(i + V2) >> 1];
        P.nyq2[i >> 1] = votes >= 5 ? 1 : (votes == 4 ? n[i >> 1] : 0);
      }
      __syncthreads();
      for (int k = t; k < area_rows * area_sites; k += THREADS) {
        const int rr = start_row + k / area_sites;
        const long i = (long)rr * TS + start_col + gae(pattern, rr) + 2 * (k % area_sites);
        if (i >= (long)rr * TS + end_col) continue;
        if (P.nyq2[i >> 1] == 0) continue;
        float sumcfa = 0.0f, sumh = 0.0f, sumv = 0.0f, sumsqh = 0.0f, sumsqv = 0.0f, areawt = 0.0f;
        for (int di = -6; di < 7; di += 2) {
          long i1 = i + di * V1 - 6;
          for (int dj = -6; dj < 7; dj += 2) {
            if (P.nyq2[i1 >> 1] != 0) {
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
        const float hcdvar = EPSSQ + fabsf(areawt * sumsqh - sumh * sumh);
        const float vcdvar = EPSSQ + fabsf(areawt * sumsqv - sumv * sumv);
        hvwt[i >> 1] = hcdvar / (vcdvar + hcdvar);
      }
    }
    __syncthreads();

    // ---- populate_green (nyquist.rs:176-222): row-ordered hvwt update ...
    for (int rr = 8; rr < TS - 8; ++rr) {
      const int cc = 8 + gae(pattern, rr) + 2 * t;
      if (t < site_count(8, TS - 8) && cc < TS - 8) {
        const int i1 = (rr * TS + cc) >> 1;
        const float alt = (hvwt[((rr - 1) * TS + cc - 1) >> 1] + hvwt[((rr - 1) * TS + cc + 1) >> 1] +
                           hvwt[((rr + 1) * TS + cc - 1) >> 1] + hvwt[((rr + 1) * TS + cc + 1) >> 1]) /
                          4.0f;
        if (fabsf(0.5f - hvwt[i1]) < fabsf(0.5f - alt)) hvwt[i1] = alt;
      }
      __syncthreads();
    }
    // ... then the per-site products, which read only final weights.
    {
      const int per_row = site_count(8, TS - 8);
      for (int k = t; k < (TS - 16) * per_row; k += THREADS) {
        const int rr = 8 + k / per_row;
        const int cc = 8 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 8) continue;
        const int i = rr * TS + cc, i1 = i >> 1;
        const float dg = intp(hvwt[i1], vcd[i], hcd[i]);
        dgrb0[i1] = dg;
        const float gv = cfa[i] + dg;
        green[i] = gv;
        const bool flagged = P.nyq2[i1] != 0;
        d2h[i1] = flagged ? sqr(gv - 0.5f * (green[i - 1] + green[i + 1])) : 0.0f;
        d2v[i1] = flagged ? sqr(gv - 0.5f * (green[i - TS] + green[i + TS])) : 0.0f;
      }
    }
    __syncthreads();

    // ---- refine_green (nyquist.rs:225-236)
    if (has_area) {
      for (int k = t; k < area_rows * area_sites; k += THREADS) {
        const int rr = start_row + k / area_sites;
        const long i = (long)rr * TS + start_col + gae(pattern, rr) + 2 * (k % area_sites);
        if (i >= (long)rr * TS + end_col) continue;
        if (P.nyq2[i >> 1] == 0) continue;
        const float gvarh = EPSSQ + (GQUINC[0] * d2h[i >> 1] +
                                     GQUINC[1] * (d2h[(i - M1) >> 1] + d2h[(i + P1) >> 1] + d2h[(i - P1) >> 1] + d2h[(i + M1) >> 1]) +
                                     GQUINC[2] * (d2h[(i - V2) >> 1] + d2h[(i - 2) >> 1] + d2h[(i + 2) >> 1] + d2h[(i + V2) >> 1]) +
                                     GQUINC[3] * (d2h[(i - M2) >> 1] + d2h[(i + P2) >> 1] + d2h[(i - P2) >> 1] + d2h[(i + M2) >> 1]));
        const float gvarv = EPSSQ + (GQUINC[0] * d2v[i >> 1] +
                                     GQUINC[1] * (d2v[(i - M1) >> 1] + d2v[(i + P1) >> 1] + d2v[(i - P1) >> 1] + d2v[(i + M1) >> 1]) +
                                     GQUINC[2] * (d2v[(i - V2) >> 1] + d2v[(i - 2) >> 1] + d2v[(i + 2) >> 1] + d2v[(i + V2) >> 1]) +
                                     GQUINC[3] * (d2v[(i - M2) >> 1] + d2v[(i + P2) >> 1] + d2v[(i - P2) >> 1] + d2v[(i + M2) >> 1]));
        const float dg = (hcd[i] * gvarv + vcd[i] * gvarh) / (gvarv + gvarh);
        dgrb0[i >> 1] = dg;
        green[i] = cfa[i] + dg;
      }
    }
    __syncthreads();

    // ---- diagonal_gradients (diagonal.rs:15-45)
    {
      float* delp = P.h[H_DELP];
      float* delm = P.h[H_DELM];
      float* sqp = P.h[H_SQ1P];
      float* sqm = P.h[H_SQ1M];
      const int per_row = site_count(6, TS - 6) ;
      for (int k = t; k < (TS - 12) * per_row; k += THREADS) {
        const int rr = 6 + k / per_row;
        const int cc = 6 + 2 * (k % per_row);
        if (cc >= TS - 6) continue;
        const float* up = cfa + (rr - 1) * TS;
        const float* mid = cfa + rr * TS;
        const float* down = cfa + (rr + 1) * TS;
        const int i1 = rr * TSH + (cc >> 1);
        if (gae(pattern, rr) == 0) {
          delp[i1] = fabsf(up[cc + 1] - down[cc - 1]);
          delm[i1] = fabsf(down[cc + 1] - up[cc - 1]);
          const float g = mid[cc + 1];
          sqp[i1] = sqr(g - down[cc]) + sqr(g - up[cc + 2]);
          sqm[i1] = sqr(g - up[cc]) + sqr(g - down[cc + 2]);
        } else {
          const float g = mid[cc];
          sqp[i1] = sqr(g - down[cc - 1]) + sqr(g - up[cc + 1]);
          sqm[i1] = sqr(g - up[cc - 1]) + sqr(g - down[cc + 1]);
          delp[i1] = fabsf(up[cc + 2] - down[cc]);
          delm[i1] = fabsf(down[cc + 2] - up[cc]);
        }
      }
    }
    __syncthreads();

    // ---- diagonal_estimates (diagonal.rs:99-145)
    {
      const float* delp = P.h[H_DELP];
      const float* delm = P.h[H_DELM];
      const float* sqp = P.h[H_SQ1P];
      const float* sqm = P.h[H_SQ1M];
      float* rbp = P.h[H_RBP];
      float* rbm = P.h[H_RBM];
      const int per_row = site_count(8, TS - 8);
      for (int k = t; k < (TS - 16) * per_row; k += THREADS) {
        const int rr = 8 + k / per_row;
        const int cc = 8 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 8) continue;
        const int i = rr * TS + cc, i1 = cc >> 1;
        const float centre = cfa[i];
        const float se1 = cfa[i + TS + 1], se2 = cfa[i + 2 * TS + 2];
        const float nw1 = cfa[i - TS - 1], nw2 = cfa[i - 2 * TS - 2];
        const float ne1 = cfa[i - TS + 1], ne2 = cfa[i - 2 * TS + 2];
        const float sw1 = cfa[i + TS - 1], sw2 = cfa[i + 2 * TS - 2];
        const float rbse = diagonal_estimate(centre, se1, se2);
        const float rbnw = diagonal_estimate(centre, nw1, nw2);
        const float rbne = diagonal_estimate(centre, ne1, ne2);
        const float rbsw = diagonal_estimate(centre, sw1, sw2);
        const int r0 = (rr - 2) * TSH, r1 = (rr - 1) * TSH, r2 = rr * TSH, r3 = (rr + 1) * TSH, r4 = (rr + 2) * TSH;
        const float wtse = EPS + delm[r2 + i1] + delm[r3 + ((cc + 1) >> 1)] + delm[r4 + ((cc + 2) >> 1)];
        const float wtnw = EPS + delm[r2 + i1] + delm[r1 + ((cc - 1) >> 1)] + delm[r0 + ((cc - 2) >> 1)];
        const float wtne = EPS + delp[r2 + i1] + delp[r1 + ((cc + 1) >> 1)] + delp[r0 + ((cc + 2) >> 1)];
        const float wtsw = EPS + delp[r2 + i1] + delp[r3 + ((cc - 1) >> 1)] + delp[r4 + ((cc - 2) >> 1)];
        const float rbm_est = (wtse * rbnw + wtnw * rbse) / (wtse + wtnw);
        const float rbp_est = (wtne * rbsw + wtsw * rbne) / (wtne + wtsw);
        const float em = GAUSSEVEN[0] * (sqm[r1 + (cc >> 1)] + sqm[r2 + ((cc - 1) >> 1)] + sqm[r2 + ((cc + 1) >> 1)] + sqm[r3 + (cc >> 1)]) +
                         GAUSSEVEN[1] * (sqm[r0 + ((cc - 1) >> 1)] + sqm[r0 + ((cc + 1) >> 1)] + sqm[r1 + ((cc - 2) >> 1)] +
                                         sqm[r1 + ((cc + 2) >> 1)] + sqm[r3 + ((cc - 2) >> 1)] + sqm[r3 + ((cc + 2) >> 1)] +
                                         sqm[r4 + ((cc - 1) >> 1)] + sqm[r4 + ((cc + 1) >> 1)]);
        const float ep = GAUSSEVEN[0] * (sqp[r1 + (cc >> 1)] + sqp[r2 + ((cc - 1) >> 1)] + sqp[r2 + ((cc + 1) >> 1)] + sqp[r3 + (cc >> 1)]) +
                         GAUSSEVEN[1] * (sqp[r0 + ((cc - 1) >> 1)] + sqp[r0 + ((cc + 1) >> 1)] + sqp[r1 + ((cc - 2) >> 1)] +
                                         sqp[r1 + ((cc + 2) >> 1)] + sqp[r3 + ((cc - 2) >> 1)] + sqp[r3 + ((cc + 2) >> 1)] +
                                         sqp[r4 + ((cc - 1) >> 1)] + sqp[r4 + ((cc + 1) >> 1)]);
        const float rbvarm = EPSSQ + em;
        pmwt[r2 + i1] = rbvarm / ((EPSSQ + ep) + rbvarm);
        rbp[r2 + i1] = bound_diagonal(rbp_est, centre, sw1, ne1, clip_pt);
        rbm[r2 + i1] = bound_diagonal(rbm_est, centre, nw1, se1, clip_pt);
      }
    }
    __syncthreads();

    // ---- combine_diagonals (diagonal.rs:150-171): row-ordered pmwt update ...
    for (int rr = 10; rr < TS - 10; ++rr) {
      const int cc = 10 + gae(pattern, rr) + 2 * t;
      if (t < site_count(10, TS - 10) && cc < TS - 10) {
        const float alt = (pmwt[(rr - 1) * TSH + ((cc - 1) >> 1)] + pmwt[(rr - 1) * TSH + ((cc + 1) >> 1)] +
                           pmwt[(rr + 1) * TSH + ((cc - 1) >> 1)] + pmwt[(rr + 1) * TSH + ((cc + 1) >> 1)]) /
                          4.0f;
        float* p = &pmwt[rr * TSH + (cc >> 1)];
        if (fabsf(0.5f - *p) < fabsf(0.5f - alt)) *p = alt;
      }
      __syncthreads();
    }
    // ... then R+B from the final weights.
    {
      const float* rbp = P.h[H_RBP];
      const float* rbm = P.h[H_RBM];
      float* rbint = P.h[H_RBINT];
      const int per_row = site_count(10, TS - 10);
      for (int k = t; k < (TS - 20) * per_row; k += THREADS) {
        const int rr = 10 + k / per_row;
        const int cc = 10 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 10) continue;
        const int j = rr * TSH + (cc >> 1);
        const float p = pmwt[j];
        rbint[j] = 0.5f * (cfa[rr * TS + cc] + rbm[j] * (1.0f - p) + rbp[j] * p);
      }
    }
    __syncthreads();

    // ---- refine_green_with_rb (diagonal.rs:205-247)
    {
      const float* rbint = P.h[H_RBINT];
      const int per_row = site_count(12, TS - 12);
      for (int k = t; k < (TS - 24) * per_row; k += THREADS) {
        const int rr = 12 + k / per_row;
        const int cc = 12 + gae(pattern, rr) + 2 * (k % per_row);
        if (cc >= TS - 12) continue;
        const int i = rr * TS + cc, i1 = cc >> 1;
        const float pm = pmwt[rr * TSH + i1];
        const float hv = hvwt[rr * TSH + i1];
        if (fabsf(0.5f - pm) < fabsf(0.5f - hv)) continue;
        const float* rb_up = rbint + (rr - 2) * TSH;
        const float* rb = rbint + rr * TSH;
        const float* rb_down = rbint + (rr + 2) * TSH;
        const float centre = rb[i1];
        const float gu = green_from_rb(cfa[i - TS], centre, rb_up[i1]);
        const float gd = green_from_rb(cfa[i + TS], centre, rb_down[i1]);
        const float gl = green_from_rb(cfa[i - 1], centre, rb[i1 - 1]);
        const float gr = green_from_rb(cfa[i + 1], centre, rb[i1 + 1]);
        float gintv = (w0[i - TS] * gd + w0[i + TS] * gu) / (w0[i + TS] + w0[i - TS]);
        float ginth = (w1[i - 1] * gr + w1[i + 1] * gl) / (w1[i - 1] + w1[i + 1]);
        gintv = bound_diagonal(gintv, centre, cfa[i - TS], cfa[i + TS], clip_pt);
        ginth = bound_diagonal(ginth, centre, cfa[i - 1], cfa[i + 1], clip_pt);
        const float gv = ginth * (1.0f - hv) + gintv * hv;
        green[i] = gv;
        dgrb0[rr * TSH + i1] = gv - cfa[i];
      }
    }
    __syncthreads();

    // ---- interpolate_chroma (chroma.rs:23-91). Reads and writes of each plane
    // fall on different Bayer cosets, so the sweep is order-free.
    {
      const int c00 = color_at(pattern, 0, 0), c10 = color_at(pattern, 1, 0);
      int ey, ex;
      if (c00 == 1 && c10 == 0) { ey = 0; ex = 1; }
      else if (c00 == 1) { ey = 1; ex = 0; }
      else if (c00 == 0) { ey = 0; ex = 0; }
      else { ey = 1; ex = 1; }
      const int first_row = 13 - ey;
      const int rows = (TS - 12 - first_row + 1) / 2;
      const int lo = (13 - ex) >> 1, hi = (TS - 12) >> 1;  // half-index range within the row
      for (int k = t; k < rows * (hi - lo); k += THREADS) {
        const int rr = first_row + 2 * (k / (hi - lo));
        const int i1 = rr * TSH + lo + k % (hi - lo);
        dgrb1[i1] = dgrb0[i1];
        dgrb0[i1] = 0.0f;
      }
    }
    __syncthreads();
    {
      const int per_row = site_count(14, TS - 14);
      for (int k = t; k < (TS - 28) * per_row; k += THREADS) {
        const int rr = 14 + k / per_row;
        const int start = 14 + gae(pattern, rr);
        const int cc = start + 2 * (k % per_row);
        if (cc >= TS - 14) continue;
        float* p = (1 - fc(pattern, rr, start) / 2) == 0 ? dgrb0 : dgrb1;
        auto d = [&](int dr, int dc) { return p[(rr + dr) * TSH + ((cc + dc) >> 1)]; };
        const float wtnw = 1.0f / (EPS + fabsf(d(-1, -1) - d(1, 1)) + fabsf(d(-1, -1) - d(-3, -3)) + fabsf(d(1, 1) - d(-3, -3)));
        const float wtne = 1.0f / (EPS + fabsf(d(-1, 1) - d(1, -1)) + fabsf(d(-1, 1) - d(-3, 3)) + fabsf(d(1, -1) - d(-3, 3)));
        const float wtsw = 1.0f / (EPS + fabsf(d(1, -1) - d(-1, 1)) + fabsf(d(1, -1) - d(3, 3)) + fabsf(d(-1, 1) - d(3, -3)));
        const float wtse = 1.0f / (EPS + fabsf(d(1, 1) - d(-1, -1)) + fabsf(d(1, 1) - d(3, -3)) + fabsf(d(-1, -1) - d(3, 3)));
        p[rr * TSH + (cc >> 1)] =
            (wtnw * (1.325f * d(-1, -1) - 0.175f * d(-3, -3) - 0.075f * d(-1, -3) - 0.075f * d(-3, -1)) +
             wtne * (1.325f * d(-1, 1) - 0.175f * d(-3, 3) - 0.075f * d(-1, 3) - 0.075f * d(1, 1)) +
             wtsw * (1.325f * d(1, -1) - 0.175f * d(3, -3) - 0.075f * d(1, -3) - 0.075f * d(-1, -1)) +
             wtse * (1.325f * d(1, 1) - 0.175f * d(3, 3) - 0.075f * d(1, 3) - 0.075f * d(3, 1))) /
            (wtnw + wtne + wtsw + wtse);
      }
    }
    __syncthreads();

    // ---- finish_planes (chroma.rs:98-147) + write_tile (mod.rs:196-268)
    {
      unsigned long long affected = 0, changed = 0, over = 0, ac[3] = {0, 0, 0};
      int bad = 0;
      for (int k = t; k < VALID * VALID; k += THREADS) {
        const int ly = k / VALID, lx = k % VALID;
        const int gx = ox + lx, gy = oy + ly;
        if (gx >= W || gy >= H) continue;
        const int rr = ly + BORDER, cc = lx + BORDER;
        const int i = rr * TS + cc;
        float r, b;
        const float gv = green[i];
        if (fc(pattern, rr, cc) == 1) {
          const float up = hvwt[(rr - 1) * TSH + (cc >> 1)], down = hvwt[(rr + 1) * TSH + (cc >> 1)];
          const float left = hvwt[rr * TSH + ((cc - 1) >> 1)], right = hvwt[rr * TSH + ((cc + 1) >> 1)];
          const float temp = 1.0f / (up + 2.0f - right - left + down);
          const float br = (up * dgrb0[(rr - 1) * TSH + (cc >> 1)] + (1.0f - right) * dgrb0[rr * TSH + ((cc + 1) >> 1)] +
                            (1.0f - left) * dgrb0[rr * TSH + ((cc - 1) >> 1)] + down * dgrb0[(rr + 1) * TSH + (cc >> 1)]) *
                           temp;
          const float bb = (up * dgrb1[(rr - 1) * TSH + (cc >> 1)] + (1.0f - right) * dgrb1[rr * TSH + ((cc + 1) >> 1)] +
                            (1.0f - left) * dgrb1[rr * TSH + ((cc - 1) >> 1)] + down * dgrb1[(rr + 1) * TSH + (cc >> 1)]) *
                           temp;
          r = gv - br;
          b = gv - bb;
        } else {
          r = gv - dgrb0[rr * TSH + (cc >> 1)];
          b = gv - dgrb1[rr * TSH + (cc >> 1)];
        }
        r = fmax_(r, 0.0f);
        b = fmax_(b, 0.0f);
        const float sample = source_balanced(src, gx, gy);
        const int ch = color_at(pattern, gx, gy);
        float rgb0 = ch == 0 ? sample : r;
        float rgb1 = ch == 1 ? sample : fmax_(gv, 0.0f);
        float rgb2 = ch == 2 ? sample : b;
        rgb0 = rgb0 * prm.gains[0];
        rgb1 = rgb1 * prm.gains[1];
        rgb2 = rgb2 * prm.gains[2];
        if (!isfinite(rgb0) || !isfinite(rgb1) || !isfinite(rgb2)) bad = 1;
        const long long o = (long long)gy * W + gx;
        prm.out[o] = rgb0;
        prm.out[plane + o] = rgb1;
        prm.out[2 * plane + o] = rgb2;
        if (prm.count_clip) {
          const float v = source_normalized(src, gx, gy);
          const float limit = src.clip_levels[ch];
          if (v >= limit) { affected++; ac[ch]++; }
          if (v > 1.0f) over++;
          if (v > limit) changed++;
        }
      }
      if (prm.count_clip) {
        unsigned long long vals[6] = {affected, changed, over, ac[0], ac[1], ac[2]};
        for (int c = 0; c < 6; ++c) {
          unsigned long long v = vals[c];
          for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
          if ((t & 31) == 0 && v) atomicAdd(&s_stats[c], v);
        }
      }
      if (bad) atomicOr(&s_bad, 1);
    }
    __syncthreads();
    if (t == 0) {
      if (prm.count_clip)
        for (int c = 0; c < 6; ++c)
          if (s_stats[c]) atomicAdd(&prm.clip_stats[c], s_stats[c]);
      if (s_bad) atomicOr(prm.error, 1u);
    }
    __syncthreads();
  }
}

}  // namespace

size_t amaze_slot_floats() { return SLOT_FLOATS; }

Status run_amaze(Context& ctx, const MosaicSource& src, const float gains[3], float clip_point, float* rgb,
                 int count_clip, unsigned long long* clip_stats) {
  const int tiles_x = (src.width + VALID - 1) / VALID, tiles_y = (src.height + VALID - 1) / VALID;
  const int ntiles = tiles_x * tiles_y;
  // Two resident CTAs per SM; balance the waves so the last one is full.
  const int max_ctas = 2 * (ctx.sm_count > 0 ? ctx.sm_count : 152);
  const int waves = (ntiles + max_ctas - 1) / max_ctas;
  const int grid = (ntiles + waves - 1) / waves;
  if ((size_t)grid > ctx.amaze_slots) {
    // Slots are kept between calls and only grow, to the grid of the largest image seen.
    if (ctx.amaze_scratch) device_free(ctx, ctx.amaze_scratch, ctx.amaze_slots * SLOT_FLOATS * sizeof(float));
    ctx.amaze_scratch = nullptr;
    ctx.amaze_slots = 0;
    void* p = nullptr;
    RD_TRY(device_alloc(ctx, (size_t)grid * SLOT_FLOATS * sizeof(float), &p));
    // vcd/hcd/vcdalt/hcdalt are read outside the region the stages write and
    // must stay zero there (scratch.rs:95-104); nothing ever writes them.
    RD_CUDA_TRY(cudaMemsetAsync(p, 0, (size_t)grid * SLOT_FLOATS * sizeof(float), ctx.stream));
    ctx.amaze_scratch = static_cast<float*>(p);
    ctx.amaze_slots = grid;
  }
  AmazeParams prm;
  prm.src = src;
  prm.out = rgb;
  prm.scratch = ctx.amaze_scratch;
  prm.tiles_x = tiles_x;
  prm.tiles_y = tiles_y;
  prm.clip_point = clip_point;
  for (int c = 0; c < 3; ++c) prm.gains[c] = gains[c];
  prm.count_clip = count_clip;
  prm.clip_stats = clip_stats;
  prm.error = ctx.d_error;
  RD_LAUNCH(ctx, K_AMAZE, amaze_kernel<<<grid, THREADS, 0, ctx.stream>>>(prm));
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

}  // namespace rd
