// AMaZE demosaic on sm_103a: row-streamed tiles in shared memory.
//
// The reference reconstructs 256-pixel tiles with a 16-pixel mirrored halo
// (crates/demosaic/src/amaze_geometry.rs:13-15, amaze/mod.rs:60-214), and its
// result depends on that tile grid: several stages are in-place raster-order
// recurrences whose start depends on the tile edge. This kernel keeps the grid
// and the arithmetic bit-identical and maps one tile onto one SM:
//
//  * one persistent 1024-thread CTA per SM takes half-tile work items (phase
//    A or phase B of a tile, all phase-A items first) from a counter (or, on a
//    context that yields its SMs, one CTA per item); a phase is processed top
//    to bottom in steps of 8 rows. Every stage runs a fixed number of rows
//    behind the rows loaded so far (its lag is the sum of the stencil reaches
//    of the stages feeding it), and each plane lives in a shared-memory ring
//    that holds just the rows still to be read;
//  * phase A (gradients .. Nyquist test, green.rs + nyquist.rs:25-95) writes
//    four small planes per tile (direction weight, bounded vertical and
//    horizontal colour differences at red/blue sites, Nyquist flag: 416 KB)
//    to the tile's slab and publishes it with a release flag; phase B (Nyquist
//    area .. output, nyquist.rs:108-236, diagonal.rs, chroma.rs,
//    mod.rs:196-268), possibly on another SM, waits for the flag (bounded,
//    error word on timeout) and streams the slab back from L2 with the mosaic;
//  * the per-tile Nyquist bounding box (nyquist.rs:60-105) only prunes work:
//    a site outside it has at most three flagged voters and is never refined,
//    so the streamed stages evaluate every site of [8, 248)^2 and get the same
//    flags without a tile-wide barrier;
//  * recurrences, restated exactly:
//      - bound_differences (green.rs:187-222): each hcd row chain is a
//        two-state automaton (the bounded value is one of two candidates that
//        do not depend on the chain); one warp per chain evaluates both
//        candidates and the state transitions of 124 steps in parallel and
//        resolves the chain with a warp scan of the transition maps. The vcd
//        column chains run one per thread with the chain value held in a
//        register across steps;
//      - populate_green / combine_diagonals (nyquist.rs:176-222,
//        diagonal.rs:150-171): the hvwt / pmwt updates read the already
//        updated row above, so one warp sweeps each recurrence row by row;
//  * the raw u16 samples are normalized, clipped and channel-balanced while
//    rows are loaded (MosaicSource), so no f32 mosaic is written to HBM, and
//    the tile core is written straight to the planar RGB output with the
//    measured sample restored, green clamped at zero and the inverse balance
//    applied.
// The file is compiled with --fmad=false so no multiply-add is fused, as in
// the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "rd_internal.cuh"
#include "tma.cuh"

namespace rd {
namespace {

constexpr int TS = 256, TSH = 128, BORDER = 16, VALID = TS - 2 * BORDER;
constexpr int THREADS = 1024;
static_assert(THREADS == 512 || THREADS == 1024, "thread roles below");
// First thread of the vcd column chains: warps 16.. with 1024 threads, else
// the same threads as the hcd chains, after them.
constexpr int VCD_T0 = THREADS == 1024 ? 512 : 0;
constexpr int AREA_THREADS = THREADS - 64;  // warps 2.. in phase B
constexpr int BH = 8;  // rows per streaming step

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


// 64-bit shared-memory access of two adjacent floats (the address is 8-byte aligned).
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

// The colour differences of one pixel (green.rs:46-139), from its stencil:
// the mosaic at the pixel (cur), one and two rows up / down and columns left /
// right, the vertical gradient weights w0 at the pixel and two rows up / down
// (and one row up / down for the vertical weight), the horizontal weights w1
// at the pixel, two columns left / right and one column left / right.
struct ColourDiff {
  float dgv, dgh, v, h, va, ha;
};
__device__ __forceinline__ void colour_difference(float cur, float up, float up2, float down, float down2, float left,
                                                  float left2, float right, float right2, float w0c, float w0u2,
                                                  float w0d2, float w0u, float w0d, float w1c, float w1l2, float w1r2,
                                                  float w1l, float w1r, bool fcswitch, float clip_pt8,
                                                  ColourDiff& out) {
  const float cru = up * (w0u2 + w0c) / (w0u2 * (EPS + cur) + w0c * (EPS + up2));
  const float crd = down * (w0d2 + w0c) / (w0d2 * (EPS + cur) + w0c * (EPS + down2));
  const float crl = left * (w1l2 + w1c) / (w1l2 * (EPS + cur) + w1c * (EPS + left2));
  const float crr = right * (w1r2 + w1c) / (w1r2 * (EPS + cur) + w1c * (EPS + right2));
  const float guha = up + 0.5f * (cur - up2);
  const float gdha = down + 0.5f * (cur - down2);
  const float glha = left + 0.5f * (cur - left2);
  const float grha = right + 0.5f * (cur - right2);
  float guar = adaptive_or(cru, cur, guha);
  float gdar = adaptive_or(crd, cur, gdha);
  float glar = adaptive_or(crl, cur, glha);
  float grar = adaptive_or(crr, cur, grha);
  const float hwt = w1l / (w1l + w1r);
  const float vwt = w0u / (w0d + w0u);
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
  out.dgv = fmin_(sqr(guha - gdha), sqr(guar - gdar));
  out.dgh = fmin_(sqr(glha - grha), sqr(glar - grar));
  out.v = v;
  out.h = h;
  out.va = va;
  out.ha = ha;
}

// A ring of RS rows (a power of two) of LEN elements; row r lives in slot r mod RS.
template <int RS, int LEN, typename T = float>
struct Ring {
  T* p;
  __device__ __forceinline__ T* row(int r) const { return p + (r & (RS - 1)) * LEN; }
};

// Shared-memory layout, in floats. Ring depths follow from the stage lags
// (depth >= consumer lag - producer lag + upward reach + BH).
// Phase A: nine 16-row full rings, an 8-row hcdalt ring, a 16-row cdd half ring.
enum { A_CFA, A_W0, A_W1, A_DELHV, A_VCD, A_HCD, A_VALT, A_DGV, A_DGH, A_N16 };
constexpr int A_HALT_OFF = A_N16 * 16 * TS;
constexpr int A_CDD_OFF = A_HALT_OFF + 8 * TS;
constexpr int A_FLOATS = A_CDD_OFF + 16 * TSH;
// Phase B: 32-row mosaic ring; 32-row half rings for the slab planes and for
// the diagonal weights / estimates (read two steps after they are made);
// 16-row half rings; u8 Nyquist flags (16 rows) and refined flags (32 rows).
constexpr int B_CFA_OFF = 0;
constexpr int B_HV_OFF = B_CFA_OFF + 32 * TS;
constexpr int B_VRB_OFF = B_HV_OFF + 32 * TSH;
constexpr int B_HRB_OFF = B_VRB_OFF + 32 * TSH;
enum { B_DGRB0, B_DGRB1, B_GREEN, B_D2H, B_D2V, B_DELP, B_DELM, B_SQP, B_SQM, B_RBINT, B_N16 };
enum { B_PMWT, B_RBP, B_RBM, B_N32 };
constexpr int B_H32_OFF = B_HRB_OFF + 32 * TSH;
constexpr int B_H16_OFF = B_H32_OFF + B_N32 * 32 * TSH;
constexpr int B_U8_OFF = B_H16_OFF + B_N16 * 16 * TSH;
constexpr int B_FLOATS = B_U8_OFF + (16 * TSH + 32 * TSH) / 4;
constexpr int SMEM_FLOATS = A_FLOATS > B_FLOATS ? A_FLOATS : B_FLOATS;
// After the rings: the staging block of the mosaic-row tensor copies (8 rows
// of 256 f32 or u16 samples), 128-byte aligned.
constexpr int STAGE_FLOATS = BH * TS;
constexpr size_t SMEM_BYTES = sizeof(float) * (SMEM_FLOATS + STAGE_FLOATS) + 128;

// Per-CTA slab in global memory: hvwt, vcd, hcd at red/blue sites (half
// planes) and the Nyquist flags (u8 half plane).
constexpr size_t SLAB_FLOATS = 3 * (size_t)TS * TSH + (size_t)TS * TSH / 4;

// One image of a launch: its mosaic source, output planes and balance, and
// the global index of its first tile (slabs and flags are per global tile).
struct AmazeImage {
  CUtensorMap map;         // the mosaic for 256 x 8 boxes (f32 mosaic or raw u16), when copy != 0
  MosaicSource src;
  float* out;              // planar RGB, 3 * width * height
  unsigned long long* clip_stats;
  int tiles_x, tiles_y;
  int tile0;               // global index of the image's tile 0
  int count_clip;          // 1: accumulate Clip statistics of core pixels
  float clip_point;
  float gains[3];          // inverse balance applied to the output
  int copy;                // AMAZE_COPY_*: how rows inside the image are staged
};
static_assert(sizeof(AmazeImage) % 64 == 0, "tensor maps in the image table stay 64-byte aligned");
enum { AMAZE_COPY_NONE = 0, AMAZE_COPY_F32 = 1, AMAZE_COPY_U16 = 2 };

// A run of consecutive work items: phase A or phase B of tiles
// [0, count) of one image, in the order the counter hands them out.
struct AmazeSegment {
  int first_item, count, image, phase_b;
};

struct AmazeParams {
  const AmazeImage* images;
  const AmazeSegment* segs;
  int nsegs;
  int total_items;
  float* slab;             // SLAB_FLOATS per global tile
  unsigned int* error;
  unsigned* flags;         // per global tile: 1 once its phase A is complete (zeroed per launch)
  unsigned* work;          // work-item counter (zeroed per launch)
  unsigned wait_tries;     // iteration limit of the phase-B wait
  int withhold_tile;       // a global tile whose phase A does not publish (tests of the bounded wait), or -1
  int withhold_copy;       // 1: no mosaic-row copy is issued, each is still waited for (tests of the bounded wait)
  int one_item;            // 1: one work item per CTA (grid = items), else CTAs loop over items
};

constexpr unsigned AMAZE_WAIT_TIMEOUT = 64u;
// Error-word bit of a mosaic-row copy whose wait ran out (shared with the
// other demosaic kernels' tile copies).
constexpr unsigned AMAZE_COPY_TIMEOUT = 128u;
__device__ __forceinline__ unsigned load_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Mosaic sample at image coordinates (x, y), mirrored into the image when outside it.
__device__ __forceinline__ float tile_sample(const MosaicSource& src, int x, int y, int W, int H) {
  const int sx = (unsigned)x < (unsigned)W ? x : mirror_index(x, W);
  const int sy = (unsigned)y < (unsigned)H ? y : mirror_index(y, H);
  return source_balanced(src, sx, sy);
}

// One warp sweeps rows [lo, hi) of a weight recurrence (populate_green's hvwt
// update with START = 8, combine_diagonals' pmwt update with START = 10): at
// each red/blue site cc = START + gae + 2k of [START, 256 - START), the weight
// w takes alt = (w'(r-1, cc-1) + w'(r-1, cc+1) + w(r+1, cc-1) + w(r+1, cc+1)) / 4
// when alt is further from 0.5, where w' is the already updated row above.
// Lane l owns half-indices 4l + START/2 .. +3 (site k = half-index - START/2);
// the updated row above stays in registers (`up`), so a row costs two
// shuffles and no barrier. The row below and the row itself are read from
// shared memory, the updated row is written back there.
template <int START, class RingT>
__device__ __forceinline__ void recurrence_rows(const RingT& ring, int lo, int hi, int g0, int lane,
                                                float (&up)[4]) {
  constexpr int J0 = START / 2;                // half-index of site k = 0
  constexpr int SITES = (TS - 2 * START) / 2;  // sites per row
  const unsigned FULL = 0xffffffffu;
  const int jb = J0 + 4 * lane;
  for (int rr = lo; rr < hi; ++rr) {
    if (rr == START) {
      // The row above the first updated row keeps its values.
      const float* a = ring.row(rr - 1);
#pragma unroll
      for (int q = 0; q < 4; ++q) up[q] = jb + q < TSH ? a[jb + q] : 0.0f;
    }
    const int g = g0 ^ (rr & 1);
    const float* down = ring.row(rr + 1);
    float* cur = ring.row(rr);
    // Updated row above at half-indices jb - 1 and jb + 4 (neighbouring lanes;
    // jb - 1 of lane 0 lies left of every site and was never updated).
    float left_in = __shfl_up_sync(FULL, up[3], 1);
    const float right_in = __shfl_down_sync(FULL, up[0], 1);
    if (lane == 0) left_in = ring.row(rr - 1)[J0 - 1];
    float nu[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = jb + q, k = 4 * lane + q;
      nu[q] = 0.0f;
      if (j < TSH) {
        const float w = cur[j];
        nu[q] = w;
        if (k < SITES) {
          const float ua = g == 0 ? (q == 0 ? left_in : up[q - 1]) : up[q];
          const float ub = g == 0 ? up[q] : (q == 3 ? right_in : up[q + 1]);
          // x * 0.25 and x / 4 are the same correctly rounded value for every x.
          const float alt = (ua + ub + down[j - 1 + g] + down[j + g]) * 0.25f;
          if (fabsf(0.5f - w) < fabsf(0.5f - alt)) {
            nu[q] = alt;
            cur[j] = alt;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) up[q] = nu[q];
  }
}

// Two-state transition maps: bit 0 = next state after state A, bit 1 = after
// state B (0 = A, 1 = B). compose(m, o) applies o first, then m.
__device__ __forceinline__ unsigned compose(unsigned m, unsigned o) {
  return ((m >> (o & 1u)) & 1u) | (((m >> ((o >> 1) & 1u)) & 1u) << 1);
}

__device__ __forceinline__ float bound_sel(bool green_site, float d, float cur, float a, float b, float clip_pt) {
  return green_site ? bound_at_green(d, cur, a, b, clip_pt) : bound_at_red_blue(d, cur, a, b, clip_pt);
}

__global__ void __launch_bounds__(THREADS, 1) amaze_kernel(const AmazeParams prm) {
  extern __shared__ __align__(128) float4 amaze_smem4[];
  float* sm = reinterpret_cast<float*>(amaze_smem4);
  // Staging block of the mosaic-row tensor copies, and their barrier.
  float* const stage =
      reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(sm + SMEM_FLOATS) + 127) & ~static_cast<uintptr_t>(127));
  __shared__ __align__(8) unsigned long long s_copy_bar;
  __shared__ unsigned long long s_stats[6];
  __shared__ int s_bad;
  // Refined Nyquist sites of a step (phase B), by step parity.
  __shared__ unsigned short s_nyq_queue[BH * (TS - 16) / 2];
  __shared__ int s_nyq_n[2];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const unsigned FULL = 0xffffffffu;
  // The image of the current item, copied from the launch's table when the
  // CTA moves to another image.
  __shared__ AmazeImage s_img;
  __shared__ int s_item, s_image, s_tile, s_phase;
  int loaded = -1;
  // Every thread's view of the copy barrier: the parity of its next
  // completion, whether a wait ran out (then no copy is issued again and rows
  // are loaded directly), and whether a copy is issued and not yet waited for.
  unsigned copy_parity = 0;
  bool copy_failed = false, copy_pending = false;
  if (t == 0) {
    mbar_init(&s_copy_bar);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }

  // Work items from the launch's counter, in the order of the segment table:
  // phase A of every tile of an image is handed out before any phase B of
  // that image (the table puts the images' phase-A runs one image ahead of
  // their phase-B runs), so a phase-B item only waits for a phase A that a
  // running CTA has taken, and phase A waits for nothing. The half-tile items
  // of all images fill the SMs far more evenly than whole tiles would. With
  // one_item each CTA ends after its item (the grid has one CTA per item), so
  // kernels of higher-priority streams get SMs within one item.
  do {
    __syncthreads();
    if (t == 0) {
      // The launch's last fetch resets the counter: with CTAs that loop, the
      // one past the items per CTA; with one item per CTA, the last item's.
      const unsigned v = atomicAdd(prm.work, 1u);
      if (v == (unsigned)prm.total_items + (prm.one_item ? 0u : gridDim.x) - 1u) atomicExch(prm.work, 0u);
      int image = -1, tile = 0, phase = 0;
      if ((int)v < prm.total_items) {
        int lo = 0, hi = prm.nsegs;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (prm.segs[mid].first_item <= (int)v) lo = mid;
          else hi = mid;
        }
        const AmazeSegment sg = prm.segs[lo];
        image = sg.image;
        tile = (int)v - sg.first_item;
        phase = sg.phase_b;
      }
      s_item = (int)v;
      s_image = image;
      s_tile = tile;
      s_phase = phase;
    }
    __syncthreads();
    if (s_item >= prm.total_items) break;
    const int tile = s_tile;
    const bool phase_b = s_phase != 0;
    if (s_image != loaded) {
      loaded = s_image;
      const int* from = reinterpret_cast<const int*>(prm.images + loaded);
      int* to = reinterpret_cast<int*>(&s_img);
      for (int k = t; k < (int)(sizeof(AmazeImage) / sizeof(int)); k += THREADS) to[k] = from[k];
      __syncthreads();
    }
    const AmazeImage& im = s_img;
    const MosaicSource& src = im.src;
    const int pattern = src.cfa;
    const float clip_pt = im.clip_point;
    const float clip_pt8 = 0.8f * clip_pt;
    const int W = src.width, H = src.height;
    const long long plane = (long long)W * H;
    // Rows holding blue sites: interpolate_chroma moves their differences to dgrb1 (chroma.rs:23-44).
    int ey;
    {
      const int c00 = color_at(pattern, 0, 0), c10 = color_at(pattern, 1, 0);
      if (c00 == 1 && c10 == 0) ey = 0;
      else if (c00 == 1) ey = 1;
      else if (c00 == 0) ey = 0;
      else ey = 1;
    }
    const int blue_par = (13 - ey) & 1;
    // Red/blue sites of row r sit at columns of parity g0 ^ (r & 1) (gae of the
    // reference); ctab is the packed 2x2 colour table of the pattern (color_at).
    const int g0 = gae(pattern, 0);
    const unsigned ctab = pattern == 0 ? 0x94u : pattern == 1 ? 0x16u : pattern == 2 ? 0x61u : 0x49u;
    const int ox = (tile % im.tiles_x) * VALID, oy = (tile / im.tiles_x) * VALID;
    const int gtile = im.tile0 + tile;
    // Per-tile slab: written by phase A, read by phase B (possibly on another SM).
    float* slab = prm.slab + (size_t)gtile * SLAB_FLOATS;
    float* g_hv = slab;
    float* g_vrb = slab + TS * TSH;
    float* g_hrb = slab + 2 * TS * TSH;
    unsigned char* g_nyq = reinterpret_cast<unsigned char*>(slab + 3 * TS * TSH);
    // Mosaic rows [lo, lo + 8) arrive by one tensor copy into the staging
    // block when they and the tile's columns lie inside the image; rows with
    // mirrored samples are loaded directly (tile_sample).
    const bool cols_inside = ox - BORDER >= 0 && ox - BORDER + TS <= W;
    auto copy_ok = [&](int lo) {
      const int y = oy - BORDER + lo;
      return im.copy != AMAZE_COPY_NONE && !copy_failed && cols_inside && y >= 0 && y + BH <= H;
    };
    // After a barrier that ended every read of the staging block.
    auto issue_copy = [&](int lo) {
      if (t == 0 && !prm.withhold_copy) {
        fence_proxy_async();
        const CUtensorMap* map = &prm.images[loaded].map;
        if (im.copy == AMAZE_COPY_F32) {
          mbar_expect_tx(&s_copy_bar, BH * TS * sizeof(float));
          tma_load_2d(stage, map, ox - BORDER, oy - BORDER + lo, &s_copy_bar);
        } else {
          mbar_expect_tx(&s_copy_bar, BH * TS * sizeof(uint16_t));
          tma_load_2d(stage, map, src.crop_x + ox - BORDER, src.crop_y + oy - BORDER + lo, &s_copy_bar);
        }
      }
      copy_pending = true;
    };
    // Bounded wait for the copy; false when it ran out (reported in the error
    // word; the caller then loads the rows directly).
    auto wait_copy = [&]() -> bool {
      bool done = false;
      for (unsigned i = 0; i < prm.wait_tries && !done; ++i) done = mbar_try_wait(&s_copy_bar, copy_parity);
      if (__syncthreads_or(!done)) {
        copy_failed = true;
        if (t == 0) atomicOr(prm.error, AMAZE_COPY_TIMEOUT);
        return false;
      }
      copy_parity ^= 1u;
      copy_pending = false;
      return true;
    };
    // Staged rows [lo, lo + 8) into a mosaic ring: normalized (raw samples),
    // Clip when selected, balanced (source_balanced of the same positions).
    auto convert_rows = [&](const auto& ring, int lo) {
      const uint16_t* raw = reinterpret_cast<const uint16_t*>(stage);
      for (int k = t; k < BH * TS; k += THREADS) {
        const int rr = lo + (k >> 8), cc = k & (TS - 1);
        const int x = ox - BORDER + cc, y = oy - BORDER + rr;
        const int ch = (ctab >> (2 * (((y & 1) << 1) | (x & 1)))) & 3;
        float v = im.copy == AMAZE_COPY_F32 ? stage[k]
                                            : normalize_raw(src, (float)raw[k], src.crop_x + x, src.crop_y + y);
        if (src.clip) {
          const float limit = src.clip_levels[ch];
          if (v > limit) v = limit;
        }
        ring.row(rr)[cc] = __fmul_rn(v, src.fwd[ch]);
      }
    };

    if (!phase_b) {
    // ================= phase A: green.rs:13-292, nyquist.rs:25-95 =================
    for (int k = t; k < A_FLOATS; k += THREADS) sm[k] = 0.0f;
    __syncthreads();
    {
      const Ring<16, TS> cfa{sm + A_CFA * 16 * TS}, w0{sm + A_W0 * 16 * TS}, w1{sm + A_W1 * 16 * TS},
          delhv{sm + A_DELHV * 16 * TS}, vcd{sm + A_VCD * 16 * TS}, hcd{sm + A_HCD * 16 * TS},
          valt{sm + A_VALT * 16 * TS}, dgv{sm + A_DGV * 16 * TS}, dgh{sm + A_DGH * 16 * TS};
      const Ring<8, TS> halt{sm + A_HALT_OFF};
      const Ring<16, TSH> cdd{sm + A_CDD_OFF};
      float vprev = 0.0f;  // vcd column chain value (threads 512..1007)
      // populate (mod.rs:175-194): rows [F, F+8) are loaded at the end of the
      // step before, while the last stage computes.
      auto load_rows = [&](int lo) {
        const int hi = min(lo + BH, TS);
        for (int k = t; k < (hi - lo) * TS; k += THREADS) {
          const int rr = lo + (k >> 8), cc = k & (TS - 1);
          cfa.row(rr)[cc] = tile_sample(src, ox - BORDER + cc, oy - BORDER + rr, W, H);
        }
      };
      load_rows(0);
      __syncthreads();
      for (int F = BH; F <= TS + 8; F += BH) {
        // -- gradients (green.rs:13-29), lag 2, rows/cols [2, 254)
        {
          const int lo = max(F - BH - 2, 2), hi = min(F - 2, TS - 2);
          for (int k = t; k < (hi - lo) * TS; k += THREADS) {
            const int rr = lo + (k >> 8), cc = 2 + (k & (TS - 1));
            if (cc >= TS - 2) continue;
            const float* c0 = cfa.row(rr);
            const float* cu = cfa.row(rr - 1);
            const float* cd = cfa.row(rr + 1);
            const float delh = fabsf(c0[cc + 1] - c0[cc - 1]);
            const float delv = fabsf(cd[cc] - cu[cc]);
            w0.row(rr)[cc] = EPS + fabsf(cfa.row(rr + 2)[cc] - c0[cc]) + fabsf(c0[cc] - cfa.row(rr - 2)[cc]) + delv;
            w1.row(rr)[cc] = EPS + fabsf(c0[cc + 2] - c0[cc]) + fabsf(c0[cc] - c0[cc - 2]) + delh;
            delhv.row(rr)[cc] = sqr(delh) + sqr(delv);
          }
        }
        __syncthreads();
        // -- colour differences (green.rs:46-139), lag 4, rows/cols [4, 252): a
        //    thread takes two horizontally adjacent pixels (an even column and
        //    the next), so their stencils come in 64-bit shared loads
        {
          const int lo = max(F - BH - 4, 4), hi = min(F - 4, TS - 4);
          for (int k = t; k < BH * 128; k += THREADS) {
            const int rr = lo + (k >> 7), pair = k & 127;
            if (rr >= hi || pair >= (TS - 8) / 2) continue;
            const int a = 4 + 2 * pair;
            const bool green_first = (g0 ^ (rr & 1)) == 1;
            const float* c0 = cfa.row(rr);
            const float2 cl = ld2(c0 + a - 2), cm = ld2(c0 + a), cr = ld2(c0 + a + 2);
            const float2 u1 = ld2(cfa.row(rr - 1) + a), u2 = ld2(cfa.row(rr - 2) + a);
            const float2 d1 = ld2(cfa.row(rr + 1) + a), d2 = ld2(cfa.row(rr + 2) + a);
            const float2 wc = ld2(w0.row(rr) + a), wu2 = ld2(w0.row(rr - 2) + a), wd2 = ld2(w0.row(rr + 2) + a);
            const float2 wu1 = ld2(w0.row(rr - 1) + a), wd1 = ld2(w0.row(rr + 1) + a);
            const float* w1r = w1.row(rr);
            const float2 hl = ld2(w1r + a - 2), hm = ld2(w1r + a), hr = ld2(w1r + a + 2);
            ColourDiff e, o;
            // Even column a: green_first decides the sign; the odd column a + 1 takes the other.
            colour_difference(cm.x, u1.x, u2.x, d1.x, d2.x, cl.y, cl.x, cm.y, cr.x, wc.x, wu2.x, wd2.x, wu1.x,
                              wd1.x, hm.x, hl.x, hr.x, hl.y, hm.y, green_first, clip_pt8, e);
            colour_difference(cm.y, u1.y, u2.y, d1.y, d2.y, cm.x, cl.y, cr.x, cr.y, wc.y, wu2.y, wd2.y, wu1.y,
                              wd1.y, hm.y, hl.y, hr.y, hm.x, hr.x, !green_first, clip_pt8, o);
            st2(dgv.row(rr) + a, e.dgv, o.dgv);
            st2(dgh.row(rr) + a, e.dgh, o.dgh);
            st2(vcd.row(rr) + a, e.v, o.v);
            st2(hcd.row(rr) + a, e.h, o.h);
            st2(valt.row(rr) + a, e.va, o.va);
            st2(halt.row(rr) + a, e.ha, o.ha);
          }
        }
        __syncthreads();
        // -- bound_differences (green.rs:187-222)
        if (warp < 16) {
          // hcd row chain of row F-12+warp/2, parity warp&1, lag 4: one warp per chain, in
          // four rounds of 32 consecutive steps (one step per lane).
          const int rr = F - 12 + (warp >> 1), par = warp & 1;
          if (rr >= 4 && rr < TS - 4) {
            float* hr = hcd.row(rr);
            const float* ha = halt.row(rr);
            const float* c0 = cfa.row(rr);
            const bool hg4 = (g0 ^ (rr & 1)) == 1;
            constexpr int STEPS = (TS - 8) / 2;  // 124 sites per chain
            unsigned s_in = 0;                   // chain state after the previous round
            float last_a = 0.0f, last_b = 0.0f;  // candidates of the previous round's last step
#pragma unroll
            for (int round = 0; round < 4; ++round) {
              const int k = 32 * round + lane;
              const int cc = 4 + par + 2 * k;
              const bool valid = k < STEPS;
              float ca = 0.0f, cb = 0.0f, hk = 0.0f, hk1 = 0.0f, av = 0.0f;
              if (valid) {
                const bool g = hg4 != (((cc - 4) & 1) == 1);
                const float cur = c0[cc];
                hk = hr[cc];
                hk1 = hr[cc + 2];
                av = spread(ha[cc - 2], ha[cc], ha[cc + 2]);
                ca = bound_sel(g, ha[cc], cur, c0[cc - 1], c0[cc + 1], clip_pt);
                cb = bound_sel(g, hk, cur, c0[cc - 1], c0[cc + 1], clip_pt);
              }
              float pa = __shfl_up_sync(FULL, ca, 1), pb = __shfl_up_sync(FULL, cb, 1);
              if (lane == 0) {
                pa = last_a;
                pb = last_b;
              }
              unsigned m;
              if (!valid) {
                m = 2u;  // identity
              } else if (k == 0) {
                // The chain starts from hcd at column 2 + par, which is zero.
                const unsigned s0 = av < spread(0.0f, hk, hk1) ? 0u : 1u;
                m = s0 | (s0 << 1);
              } else {
                const unsigned sa = av < spread(pa, hk, hk1) ? 0u : 1u;
                const unsigned sb = av < spread(pb, hk, hk1) ? 0u : 1u;
                m = sa | (sb << 1);
              }
#pragma unroll
              for (int d = 1; d < 32; d <<= 1) {
                const unsigned o = __shfl_up_sync(FULL, m, d);
                if (lane >= d) m = compose(m, o);
              }
              const unsigned st = (m >> s_in) & 1u;  // state after this lane's step
              __syncwarp();
              if (valid) hr[cc] = st ? cb : ca;
              s_in = __shfl_sync(FULL, st, 31);
              last_a = __shfl_sync(FULL, ca, 31);
              last_b = __shfl_sync(FULL, cb, 31);
            }
          }
        }
        if (t >= VCD_T0 && t < VCD_T0 + 2 * (TS - 8)) {
          // vcd column chains, lag 6: column vc, rows 4+par, 6+par, ... in order
          // (beside the hcd chains with 1024 threads, after them with fewer).
          const int u = t - VCD_T0, vc = 4 + u % (TS - 8), par = u / (TS - 8);
          const int lo = max(F - BH - 6, 4), hi = min(F - 6, TS - 4);
          const bool vg4 = ((vc - 4) & 1) == 1;
          for (int rr = lo + ((lo ^ par) & 1); rr < hi; rr += 2) {
            const float vcur = vcd.row(rr)[vc];
            const float vnext = rr + 2 < TS - 4 ? vcd.row(rr + 2)[vc] : 0.0f;
            const float aprev = rr - 2 >= 4 ? valt.row(rr - 2)[vc] : 0.0f;
            const float acur = valt.row(rr)[vc];
            const float anext = rr + 2 < TS - 4 ? valt.row(rr + 2)[vc] : 0.0f;
            const float vcdvar = spread(vprev, vcur, vnext);
            const float vcdaltvar = spread(aprev, acur, anext);
            const float vsel = vcdaltvar < vcdvar ? acur : vcur;
            const bool g = ((g0 ^ (rr & 1)) == 1) != vg4;
            const float b = bound_sel(g, vsel, cfa.row(rr)[vc], cfa.row(rr - 1)[vc], cfa.row(rr + 1)[vc], clip_pt);
            vcd.row(rr)[vc] = b;
            vprev = b;
          }
        }
        __syncthreads();
        // The next step's rows start arriving now (the staging block's last
        // reads ended with the step before).
        const bool copied = F < TS && copy_ok(F);
        if (copied) issue_copy(F);
        // -- cdd at red/blue sites (green.rs:187-222 tail), lag 6
        {
          const int lo = max(F - BH - 6, 4), hi = min(F - 6, TS - 4);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 4 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 4) continue;
            cdd.row(rr)[cc >> 1] = sqr(vcd.row(rr)[cc] - hcd.row(rr)[cc]);
          }
        }
        // -- direction_weights (green.rs:225-292), lag 9, red/blue sites of [6, 250)^2
        {
          const int lo = max(F - BH - 9, 6), hi = min(F - 9, TS - 6);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 6 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 6) continue;
            // vcd rows outside [4, 252) were never written: zero.
            float vv[7];
#pragma unroll
            for (int d = -3; d <= 3; ++d) {
              const int r = rr + d;
              vv[d + 3] = (r >= 4 && r < TS - 4) ? vcd.row(r)[cc] : 0.0f;
            }
            const float* hr = hcd.row(rr);
            const float uave = vv[3] + vv[2] + vv[1] + vv[0];
            const float dave = vv[3] + vv[4] + vv[5] + vv[6];
            const float lave = hr[cc] + hr[cc - 1] + hr[cc - 2] + hr[cc - 3];
            const float rave = hr[cc] + hr[cc + 1] + hr[cc + 2] + hr[cc + 3];
            const float vu = sqr(vv[3] - uave) + sqr(vv[2] - uave) + sqr(vv[1] - uave) + sqr(vv[0] - uave);
            const float vd = sqr(vv[3] - dave) + sqr(vv[4] - dave) + sqr(vv[5] - dave) + sqr(vv[6] - dave);
            const float hl = sqr(hr[cc] - lave) + sqr(hr[cc - 1] - lave) + sqr(hr[cc - 2] - lave) + sqr(hr[cc - 3] - lave);
            const float hrr = sqr(hr[cc] - rave) + sqr(hr[cc + 1] - rave) + sqr(hr[cc + 2] - rave) + sqr(hr[cc + 3] - rave);
            const float* w1r = w1.row(rr);
            const float hwt = w1r[cc - 1] / (w1r[cc - 1] + w1r[cc + 1]);
            const float w0u = w0.row(rr - 1)[cc], w0d = w0.row(rr + 1)[cc];
            const float vwt = w0u / (w0d + w0u);
            const float vcdvar = EPSSQ + vwt * vd + (1.0f - vwt) * vu;
            const float hcdvar = EPSSQ + hwt * hrr + (1.0f - hwt) * hl;
            const float dv0 = dgv.row(rr)[cc];
            const float fu = dv0 + dgv.row(rr - 1)[cc] + dgv.row(rr - 2)[cc];
            const float fd = dv0 + dgv.row(rr + 1)[cc] + dgv.row(rr + 2)[cc];
            const float* dhr = dgh.row(rr);
            const float fl = dhr[cc] + dhr[cc - 1] + dhr[cc - 2];
            const float fr = dhr[cc] + dhr[cc + 1] + dhr[cc + 2];
            const float vcdvar1 = EPSSQ + vwt * fd + (1.0f - vwt) * fu;
            const float hcdvar1 = EPSSQ + hwt * fr + (1.0f - hwt) * fl;
            const float varwt = hcdvar / (vcdvar + hcdvar);
            const float diffwt = hcdvar1 / (vcdvar1 + hcdvar1);
            const int o = rr * TSH + (cc >> 1);
            g_hv[o] = ((0.5f - varwt) * (0.5f - diffwt) > 0.0f && fabsf(0.5f - diffwt) < fabsf(0.5f - varwt))
                          ? varwt
                          : diffwt;
            g_vrb[o] = vv[3];
            g_hrb[o] = hr[cc];
          }
        }
        __syncthreads();
        // -- Nyquist test (nyquist.rs:25-95), lag 8, red/blue sites of [6, 250)^2
        {
          const int lo = max(F - BH - 8, 6), hi = min(F - 8, TS - 6);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 6 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 6) continue;
            const float* cm2 = cdd.row(rr - 2);
            const float* cm1 = cdd.row(rr - 1);
            const float* c0 = cdd.row(rr);
            const float* cp1 = cdd.row(rr + 1);
            const float* cp2 = cdd.row(rr + 2);
            const int j = cc >> 1, jm = (cc - 1) >> 1, jp = (cc + 1) >> 1;
            const float* dm2 = delhv.row(rr - 2);
            const float* dm1 = delhv.row(rr - 1);
            const float* d0 = delhv.row(rr);
            const float* dp1 = delhv.row(rr + 1);
            const float* dp2 = delhv.row(rr + 2);
            const float v =
                (GAUSSODD[0] * c0[j] + GAUSSODD[1] * (cm1[jm] + cm1[jp] + cp1[jm] + cp1[jp]) +
                 GAUSSODD[2] * (cm2[j] + c0[j - 1] + c0[j + 1] + cp2[j]) +
                 GAUSSODD[3] * (cm2[j - 1] + cm2[j + 1] + cp2[j - 1] + cp2[j + 1])) -
                (GAUSSGRAD[0] * d0[cc] + GAUSSGRAD[1] * (dm1[cc] + d0[cc + 1] + d0[cc - 1] + dp1[cc]) +
                 GAUSSGRAD[2] * (dm1[cc - 1] + dm1[cc + 1] + dp1[cc - 1] + dp1[cc + 1]) +
                 GAUSSGRAD[3] * (dm2[cc] + d0[cc - 2] + d0[cc + 2] + dp2[cc]) +
                 GAUSSGRAD[4] * (dm2[cc - 1] + dm2[cc + 1] + dm1[cc - 2] + dm1[cc + 2] + dp1[cc - 2] +
                                 dp1[cc + 2] + dp2[cc - 1] + dp2[cc + 1]) +
                 GAUSSGRAD[5] * (dm2[cc - 2] + dm2[cc + 2] + dp2[cc - 2] + dp2[cc + 2]));
            g_nyq[rr * TSH + j] = v > 0.0f ? 1 : 0;
          }
        }
        // -- rows of the next step (their ring slots held rows no stage reads any more)
        if (F < TS) {
          if (copied && wait_copy()) convert_rows(cfa, F);
          else load_rows(F);
        }
        __syncthreads();
      }
    }
    // Publish the slab: every thread's writes, then the tile's flag.
    __threadfence();
    __syncthreads();
    if (t == 0 && gtile != prm.withhold_tile) atomicExch(&prm.flags[gtile], 1u);
    continue;
    }

    // Phase B waits (bounded) until the tile's phase A has published its slab.
    if (t == 0) {
      unsigned tries = 0;
      while (load_acquire(&prm.flags[gtile]) == 0u) {
        if (++tries > prm.wait_tries) {
          atomicOr(prm.error, AMAZE_WAIT_TIMEOUT);
          break;
        }
        __nanosleep(128);
      }
      s_bad = 0;
    }
    if (t < 6) s_stats[t] = 0;

    // ================= phase B: nyquist.rs:108-236, diagonal.rs, chroma.rs, mod.rs:196-268 =================
    for (int k = t; k < B_FLOATS; k += THREADS) sm[k] = 0.0f;
    if (t < 2) s_nyq_n[t] = 0;
    __syncthreads();
    {
      const Ring<32, TS> cfa{sm + B_CFA_OFF};
      const Ring<32, TSH> hv{sm + B_HV_OFF}, vrb{sm + B_VRB_OFF}, hrb{sm + B_HRB_OFF};
      float* h16 = sm + B_H16_OFF;
      const Ring<16, TSH> dgrb0{h16 + B_DGRB0 * 16 * TSH}, dgrb1{h16 + B_DGRB1 * 16 * TSH},
          green{h16 + B_GREEN * 16 * TSH}, d2h{h16 + B_D2H * 16 * TSH}, d2v{h16 + B_D2V * 16 * TSH},
          delp{h16 + B_DELP * 16 * TSH}, delm{h16 + B_DELM * 16 * TSH}, sqp{h16 + B_SQP * 16 * TSH},
          sqm{h16 + B_SQM * 16 * TSH}, rbint{h16 + B_RBINT * 16 * TSH};
      float* h32 = sm + B_H32_OFF;
      const Ring<32, TSH> pmwt{h32 + B_PMWT * 32 * TSH}, rbp{h32 + B_RBP * 32 * TSH}, rbm{h32 + B_RBM * 32 * TSH};
      unsigned char* u8 = reinterpret_cast<unsigned char*>(sm + B_U8_OFF);
      const Ring<16, TSH, unsigned char> nyq{u8};
      const Ring<32, TSH, unsigned char> nyq2{u8 + 16 * TSH};
      unsigned long long affected = 0, changed = 0, over = 0, ac0 = 0, ac1 = 0, ac2 = 0;
      int bad = 0;
      // Updated weights of the row above, four half-indices per lane (warps 0 and 1).
      float hv_up[4] = {0.0f, 0.0f, 0.0f, 0.0f}, pm_up[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      // Rows [lo, lo+8) of the mosaic (staged by a tensor copy when one was
      // issued for them) and of the slab ([6, 250) only).
      bool copied = copy_ok(0);
      if (copied) issue_copy(0);
      auto load_rows = [&](int lo) {
        const bool staged = copied && wait_copy();
        if (staged) {
          convert_rows(cfa, lo);
        } else {
          for (int k = t; k < BH * TS; k += THREADS) {
            const int rr = lo + (k >> 8), cc = k & (TS - 1);
            cfa.row(rr)[cc] = tile_sample(src, ox - BORDER + cc, oy - BORDER + rr, W, H);
          }
        }
        for (int k = t; k < BH * TSH; k += THREADS) {
          const int rr = lo + (k >> 7), j = k & (TSH - 1);
          if (rr < 6 || rr >= TS - 6) continue;
          const int o = rr * TSH + j;
          // L2 reads: the slab may have been written by another SM.
          hv.row(rr)[j] = __ldcg(g_hv + o);
          vrb.row(rr)[j] = __ldcg(g_vrb + o);
          hrb.row(rr)[j] = __ldcg(g_hrb + o);
          nyq.row(rr)[j] = __ldcg(g_nyq + o);
        }
      };
      for (int F = BH; F <= TS + BH; F += BH) {
        if (F - BH < TS) load_rows(F - BH);
        __syncthreads();
        // The next step's rows start arriving now (the staging block was read above).
        copied = F < TS && copy_ok(F);
        if (copied) issue_copy(F);
        // -- Nyquist flag refinement (nyquist.rs:108-130), lag 2, red/blue sites of [8, 248)^2;
        //    diagonal_gradients (diagonal.rs:15-45), lag 6, rows [6, 250)
        {
          const int lo = max(F - BH - 2, 8), hi = min(F - 2, TS - 8);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 8) continue;
            const int j = cc >> 1, jm = (cc - 1) >> 1, jp = (cc + 1) >> 1;
            const unsigned char* nm2 = nyq.row(rr - 2);
            const unsigned char* nm1 = nyq.row(rr - 1);
            const unsigned char* n0 = nyq.row(rr);
            const unsigned char* np1 = nyq.row(rr + 1);
            const unsigned char* np2 = nyq.row(rr + 2);
            const unsigned votes = nm2[j] + nm1[jm] + nm1[jp] + n0[j - 1] + n0[j + 1] + np1[jm] + np1[jp] + np2[j];
            nyq2.row(rr)[j] = votes >= 5 ? 1 : (votes == 4 ? n0[j] : 0);
          }
        }
        {
          const int lo = max(F - BH - 6, 6), hi = min(F - 6, TS - 6);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 6 + 2 * (k & 127);
            if (cc >= TS - 6) continue;
            const float* up = cfa.row(rr - 1);
            const float* mid = cfa.row(rr);
            const float* down = cfa.row(rr + 1);
            const int j = cc >> 1;
            if ((g0 ^ (rr & 1)) == 0) {
              delp.row(rr)[j] = fabsf(up[cc + 1] - down[cc - 1]);
              delm.row(rr)[j] = fabsf(down[cc + 1] - up[cc - 1]);
              const float g = mid[cc + 1];
              sqp.row(rr)[j] = sqr(g - down[cc]) + sqr(g - up[cc + 2]);
              sqm.row(rr)[j] = sqr(g - up[cc]) + sqr(g - down[cc + 2]);
            } else {
              const float g = mid[cc];
              sqp.row(rr)[j] = sqr(g - down[cc - 1]) + sqr(g - up[cc + 1]);
              sqm.row(rr)[j] = sqr(g - up[cc - 1]) + sqr(g - down[cc + 1]);
              delp.row(rr)[j] = fabsf(up[cc + 2] - down[cc]);
              delm.row(rr)[j] = fabsf(down[cc + 2] - up[cc]);
            }
          }
        }
        __syncthreads();
        // -- warps 2-31: area interpolation and diagonal estimates (lag 8); warps 0-1:
        //    the row recurrences of populate_green's hvwt (nyquist.rs:176-222) and
        //    combine_diagonals' pmwt (diagonal.rs:150-171) one step behind (lag 17),
        //    so they read rows finished in the step before and overlap the others.
        if (warp >= 2) {
        // -- area interpolation at refined Nyquist sites (nyquist.rs:132-170), lag 8.
        //    The flagged sites of the step are queued in shared memory (warp-
        //    aggregated appends) and then taken by full warps; a neighbour's
        //    terms are added as +0.0 when it is not flagged, which leaves every
        //    sum unchanged (each starts at +0.0 and so can never be -0.0), so
        //    the 7x7 loop runs without divergence.
          {
            const int lo = max(F - BH - 8, 8), hi = min(F - 8, TS - 8);
            constexpr int per_row = (TS - 16) / 2;
            const int u = t - 64, par = (F / BH) & 1;
            // The step's sites are a multiple of 32 apart per pass, so every
            // lane of a warp takes the same number of passes.
            for (int k = u; k - (u & 31) < (hi - lo) * per_row; k += AREA_THREADS) {
              bool flagged = false;
              if (k < (hi - lo) * per_row) {
                const int rr = lo + k / per_row;
                const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k % per_row);
                flagged = nyq2.row(rr)[cc >> 1] != 0;
              }
              const unsigned ballot = __ballot_sync(FULL, flagged);
              if (ballot) {
                int base = 0;
                if (lane == 0) base = atomicAdd(&s_nyq_n[par], __popc(ballot));
                base = __shfl_sync(FULL, base, 0);
                if (flagged) s_nyq_queue[base + __popc(ballot & ((1u << lane) - 1u))] = (unsigned short)k;
              }
            }
            asm volatile("bar.sync 1, %0;" ::"n"(AREA_THREADS) : "memory");
            const int queued = s_nyq_n[par];
            for (int q = u; q < queued; q += AREA_THREADS) {
              const int k = s_nyq_queue[q];
              const int rr = lo + k / per_row;
              const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k % per_row);
              float sumcfa = 0.0f, sumh = 0.0f, sumv = 0.0f, sumsqh = 0.0f, sumsqv = 0.0f, areawt = 0.0f;
              for (int di = -6; di < 7; di += 2) {
                const int r1 = rr + di;
                // Refined flags outside [8, 248) were never set: zero.
                if (r1 < 8 || r1 >= TS - 8) continue;
                const unsigned char* f = nyq2.row(r1);
                const float* c0 = cfa.row(r1);
                const float* cu = cfa.row(r1 - 1);
                const float* cd = cfa.row(r1 + 1);
#pragma unroll
                for (int c1 = cc - 6; c1 < cc + 7; c1 += 2) {
                  const bool on = f[c1 >> 1] != 0;
                  const float c = c0[c1], l = c0[c1 - 1], r = c0[c1 + 1], up = cu[c1], dn = cd[c1];
                  sumcfa += on ? c : 0.0f;
                  sumh += on ? l + r : 0.0f;
                  sumv += on ? up + dn : 0.0f;
                  sumsqh += on ? sqr(c - l) + sqr(c - r) : 0.0f;
                  sumsqv += on ? sqr(c - up) + sqr(c - dn) : 0.0f;
                  areawt += on ? 1.0f : 0.0f;
                }
              }
              sumh = sumcfa - 0.5f * sumh;
              sumv = sumcfa - 0.5f * sumv;
              areawt *= 0.5f;
              const float hcdvar = EPSSQ + fabsf(areawt * sumsqh - sumh * sumh);
              const float vcdvar = EPSSQ + fabsf(areawt * sumsqv - sumv * sumv);
              hv.row(rr)[cc >> 1] = hcdvar / (vcdvar + hcdvar);
            }
            // The other parity's counter was last read in the step before.
            if (u == 0) s_nyq_n[par ^ 1] = 0;
          }
          // -- diagonal_estimates (diagonal.rs:99-145), lag 8, red/blue sites of [8, 248)^2
          {
            const int lo = max(F - BH - 8, 8), hi = min(F - 8, TS - 8);
            constexpr int per_row = (TS - 16) / 2;
            for (int k = t - 64; k < (hi - lo) * per_row; k += AREA_THREADS) {
              const int rr = lo + k / per_row;
              const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k % per_row);
              const int j = cc >> 1;
              const float* cm2 = cfa.row(rr - 2);
              const float* cm1 = cfa.row(rr - 1);
              const float* c0 = cfa.row(rr);
              const float* cp1 = cfa.row(rr + 1);
              const float* cp2 = cfa.row(rr + 2);
              const float centre = c0[cc];
              const float se1 = cp1[cc + 1], se2 = cp2[cc + 2];
              const float nw1 = cm1[cc - 1], nw2 = cm2[cc - 2];
              const float ne1 = cm1[cc + 1], ne2 = cm2[cc + 2];
              const float sw1 = cp1[cc - 1], sw2 = cp2[cc - 2];
              const float rbse = diagonal_estimate(centre, se1, se2);
              const float rbnw = diagonal_estimate(centre, nw1, nw2);
              const float rbne = diagonal_estimate(centre, ne1, ne2);
              const float rbsw = diagonal_estimate(centre, sw1, sw2);
              const float wtse = EPS + delm.row(rr)[j] + delm.row(rr + 1)[(cc + 1) >> 1] + delm.row(rr + 2)[(cc + 2) >> 1];
              const float wtnw = EPS + delm.row(rr)[j] + delm.row(rr - 1)[(cc - 1) >> 1] + delm.row(rr - 2)[(cc - 2) >> 1];
              const float wtne = EPS + delp.row(rr)[j] + delp.row(rr - 1)[(cc + 1) >> 1] + delp.row(rr - 2)[(cc + 2) >> 1];
              const float wtsw = EPS + delp.row(rr)[j] + delp.row(rr + 1)[(cc - 1) >> 1] + delp.row(rr + 2)[(cc - 2) >> 1];
              const float rbm_est = (wtse * rbnw + wtnw * rbse) / (wtse + wtnw);
              const float rbp_est = (wtne * rbsw + wtsw * rbne) / (wtne + wtsw);
              const float* qm0 = sqm.row(rr - 2);
              const float* qm1 = sqm.row(rr - 1);
              const float* qm2 = sqm.row(rr);
              const float* qm3 = sqm.row(rr + 1);
              const float* qm4 = sqm.row(rr + 2);
              const float em = GAUSSEVEN[0] * (qm1[cc >> 1] + qm2[(cc - 1) >> 1] + qm2[(cc + 1) >> 1] + qm3[cc >> 1]) +
                               GAUSSEVEN[1] * (qm0[(cc - 1) >> 1] + qm0[(cc + 1) >> 1] + qm1[(cc - 2) >> 1] +
                                               qm1[(cc + 2) >> 1] + qm3[(cc - 2) >> 1] + qm3[(cc + 2) >> 1] +
                                               qm4[(cc - 1) >> 1] + qm4[(cc + 1) >> 1]);
              const float* qp0 = sqp.row(rr - 2);
              const float* qp1 = sqp.row(rr - 1);
              const float* qp2 = sqp.row(rr);
              const float* qp3 = sqp.row(rr + 1);
              const float* qp4 = sqp.row(rr + 2);
              const float ep = GAUSSEVEN[0] * (qp1[cc >> 1] + qp2[(cc - 1) >> 1] + qp2[(cc + 1) >> 1] + qp3[cc >> 1]) +
                               GAUSSEVEN[1] * (qp0[(cc - 1) >> 1] + qp0[(cc + 1) >> 1] + qp1[(cc - 2) >> 1] +
                                               qp1[(cc + 2) >> 1] + qp3[(cc - 2) >> 1] + qp3[(cc + 2) >> 1] +
                                               qp4[(cc - 1) >> 1] + qp4[(cc + 1) >> 1]);
              const float rbvarm = EPSSQ + em;
              pmwt.row(rr)[j] = rbvarm / ((EPSSQ + ep) + rbvarm);
              rbp.row(rr)[j] = bound_diagonal(rbp_est, centre, sw1, ne1, clip_pt);
              rbm.row(rr)[j] = bound_diagonal(rbm_est, centre, nw1, se1, clip_pt);
            }
          }
        } else if (warp == 0) {
          recurrence_rows<8>(hv, max(F - BH - 17, 8), min(F - 17, TS - 8), g0, lane, hv_up);
        } else {
          recurrence_rows<10>(pmwt, max(F - BH - 17, 10), min(F - 17, TS - 10), g0, lane, pm_up);
        }
        __syncthreads();
        // -- per-site products of populate_green (lag 17, [8, 248)^2) and the R+B
        //    interpolation of combine_diagonals (lag 17, [10, 246)^2)
        {
          const int lo = max(F - BH - 17, 8), hi = min(F - 17, TS - 8);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 8) continue;
            const int j = cc >> 1;
            const float* c0 = cfa.row(rr);
            const float dg = intp(hv.row(rr)[j], vrb.row(rr)[j], hrb.row(rr)[j]);
            dgrb0.row(rr)[j] = dg;
            const float gv = c0[cc] + dg;
            green.row(rr)[j] = gv;
            const bool flagged = nyq2.row(rr)[j] != 0;
            d2h.row(rr)[j] = flagged ? sqr(gv - 0.5f * (c0[cc - 1] + c0[cc + 1])) : 0.0f;
            d2v.row(rr)[j] = flagged ? sqr(gv - 0.5f * (cfa.row(rr - 1)[cc] + cfa.row(rr + 1)[cc])) : 0.0f;
          }
        }
        {
          const int lo = max(F - BH - 17, 10), hi = min(F - 17, TS - 10);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 10 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 10) continue;
            const int j = cc >> 1;
            const float p = pmwt.row(rr)[j];
            rbint.row(rr)[j] = 0.5f * (cfa.row(rr)[cc] + rbm.row(rr)[j] * (1.0f - p) + rbp.row(rr)[j] * p);
          }
        }
        __syncthreads();
        // -- refine_green (nyquist.rs:225-236) at the refined Nyquist sites of
        //    [8, 248)^2, then refine_green_with_rb (diagonal.rs:205-247) and the
        //    move of blue-row differences to dgrb1 (chroma.rs:23-44) at the sites
        //    of [12, 244)^2, lag 19. The three run site by site in one pass: each
        //    writes only its own site's green / dgrb0 / dgrb1 and none reads
        //    what another writes at a different site, so every site sees the
        //    reference's stage order.
        {
          const int lo = max(F - BH - 19, 8), hi = min(F - 19, TS - 8);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int cc = 8 + (g0 ^ (rr & 1)) + 2 * (k & 127);
            if (cc >= TS - 8) continue;
            const int j = cc >> 1;
            if (nyq2.row(rr)[j] != 0) {
              // d2h / d2v rows outside [8, 248) were never written: zero.
              const float* hm2 = rr - 2 >= 8 ? d2h.row(rr - 2) : nullptr;
              const float* hp2 = rr + 2 < TS - 8 ? d2h.row(rr + 2) : nullptr;
              const float* hm1 = rr - 1 >= 8 ? d2h.row(rr - 1) : nullptr;
              const float* hp1 = rr + 1 < TS - 8 ? d2h.row(rr + 1) : nullptr;
              const float* vm2 = rr - 2 >= 8 ? d2v.row(rr - 2) : nullptr;
              const float* vp2 = rr + 2 < TS - 8 ? d2v.row(rr + 2) : nullptr;
              const float* vm1 = rr - 1 >= 8 ? d2v.row(rr - 1) : nullptr;
              const float* vp1 = rr + 1 < TS - 8 ? d2v.row(rr + 1) : nullptr;
              const float* h0 = d2h.row(rr);
              const float* v0 = d2v.row(rr);
              const int jm = (cc - 1) >> 1, jp = (cc + 1) >> 1;
              auto at = [](const float* r, int x) { return r ? r[x] : 0.0f; };
              const float gvarh = EPSSQ + (GQUINC[0] * h0[j] +
                                           GQUINC[1] * (at(hm1, jm) + at(hm1, jp) + at(hp1, jm) + at(hp1, jp)) +
                                           GQUINC[2] * (at(hm2, j) + h0[j - 1] + h0[j + 1] + at(hp2, j)) +
                                           GQUINC[3] * (at(hm2, j - 1) + at(hm2, j + 1) + at(hp2, j - 1) + at(hp2, j + 1)));
              const float gvarv = EPSSQ + (GQUINC[0] * v0[j] +
                                           GQUINC[1] * (at(vm1, jm) + at(vm1, jp) + at(vp1, jm) + at(vp1, jp)) +
                                           GQUINC[2] * (at(vm2, j) + v0[j - 1] + v0[j + 1] + at(vp2, j)) +
                                           GQUINC[3] * (at(vm2, j - 1) + at(vm2, j + 1) + at(vp2, j - 1) + at(vp2, j + 1)));
              const float dg = (hrb.row(rr)[j] * gvarv + vrb.row(rr)[j] * gvarh) / (gvarv + gvarh);
              dgrb0.row(rr)[j] = dg;
              green.row(rr)[j] = cfa.row(rr)[cc] + dg;
            }
            if (rr < 12 || rr >= TS - 12 || cc < 12 || cc >= TS - 12) continue;
            const float pm = pmwt.row(rr)[j];
            const float hvv = hv.row(rr)[j];
            if (!(fabsf(0.5f - pm) < fabsf(0.5f - hvv))) {
              const float* rb_up = rbint.row(rr - 2);
              const float* rb = rbint.row(rr);
              const float* rb_down = rbint.row(rr + 2);
              const float* c0 = cfa.row(rr);
              const float* cu = cfa.row(rr - 1);
              const float* cd = cfa.row(rr + 1);
              const float* cu2 = cfa.row(rr - 2);
              const float* cd2 = cfa.row(rr + 2);
              const float* cu3 = cfa.row(rr - 3);
              const float* cd3 = cfa.row(rr + 3);
              const float centre = rb[j];
              const float gu = green_from_rb(cu[cc], centre, rb_up[j]);
              const float gd = green_from_rb(cd[cc], centre, rb_down[j]);
              const float gl = green_from_rb(c0[cc - 1], centre, rb[j - 1]);
              const float gr = green_from_rb(c0[cc + 1], centre, rb[j + 1]);
              // Directional gradient weights (green.rs:13-29) at the four neighbours.
              const float w0u = EPS + fabsf(cd[cc] - cu[cc]) + fabsf(cu[cc] - cu3[cc]) + fabsf(c0[cc] - cu2[cc]);
              const float w0d = EPS + fabsf(cd3[cc] - cd[cc]) + fabsf(cd[cc] - cu[cc]) + fabsf(cd2[cc] - c0[cc]);
              const float w1l = EPS + fabsf(c0[cc + 1] - c0[cc - 1]) + fabsf(c0[cc - 1] - c0[cc - 3]) + fabsf(c0[cc] - c0[cc - 2]);
              const float w1r = EPS + fabsf(c0[cc + 3] - c0[cc + 1]) + fabsf(c0[cc + 1] - c0[cc - 1]) + fabsf(c0[cc + 2] - c0[cc]);
              float gintv = (w0u * gd + w0d * gu) / (w0d + w0u);
              float ginth = (w1l * gr + w1r * gl) / (w1l + w1r);
              gintv = bound_diagonal(gintv, centre, cu[cc], cd[cc], clip_pt);
              ginth = bound_diagonal(ginth, centre, c0[cc - 1], c0[cc + 1], clip_pt);
              const float gv = ginth * (1.0f - hvv) + gintv * hvv;
              green.row(rr)[j] = gv;
              dgrb0.row(rr)[j] = gv - c0[cc];
            }
            if ((rr & 1) == blue_par) {
              dgrb1.row(rr)[j] = dgrb0.row(rr)[j];
              dgrb0.row(rr)[j] = 0.0f;
            }
          }
        }
        __syncthreads();
        // -- interpolate_chroma (chroma.rs:46-91), lag 22, [14, 242)^2: reads and
        //    writes of each plane fall on different rows
        {
          const int lo = max(F - BH - 22, 14), hi = min(F - 22, TS - 14);
          constexpr int per_row = 128;  // site slots per row: 8 rows per step
          for (int k = t; k < (hi - lo) * per_row; k += THREADS) {
            const int rr = lo + (k >> 7);
            const int start = 14 + (g0 ^ (rr & 1));
            const int cc = start + 2 * (k & 127);
            if (cc >= TS - 14) continue;
            // A blue site interpolates the red difference (dgrb0), a red site the blue one.
            const Ring<16, TSH>& p = (rr & 1) == blue_par ? dgrb0 : dgrb1;
            auto d = [&](int dr, int dc) { return p.row(rr + dr)[(cc + dc) >> 1]; };
            const float wtnw = 1.0f / (EPS + fabsf(d(-1, -1) - d(1, 1)) + fabsf(d(-1, -1) - d(-3, -3)) + fabsf(d(1, 1) - d(-3, -3)));
            const float wtne = 1.0f / (EPS + fabsf(d(-1, 1) - d(1, -1)) + fabsf(d(-1, 1) - d(-3, 3)) + fabsf(d(1, -1) - d(-3, 3)));
            const float wtsw = 1.0f / (EPS + fabsf(d(1, -1) - d(-1, 1)) + fabsf(d(1, -1) - d(3, 3)) + fabsf(d(-1, 1) - d(3, -3)));
            const float wtse = 1.0f / (EPS + fabsf(d(1, 1) - d(-1, -1)) + fabsf(d(1, 1) - d(3, -3)) + fabsf(d(-1, -1) - d(3, 3)));
            p.row(rr)[cc >> 1] =
                (wtnw * (1.325f * d(-1, -1) - 0.175f * d(-3, -3) - 0.075f * d(-1, -3) - 0.075f * d(-3, -1)) +
                 wtne * (1.325f * d(-1, 1) - 0.175f * d(-3, 3) - 0.075f * d(-1, 3) - 0.075f * d(1, 1)) +
                 wtsw * (1.325f * d(1, -1) - 0.175f * d(3, -3) - 0.075f * d(1, -3) - 0.075f * d(-1, -1)) +
                 wtse * (1.325f * d(1, 1) - 0.175f * d(3, 3) - 0.075f * d(1, 3) - 0.075f * d(3, 1))) /
                (wtnw + wtne + wtsw + wtse);
          }
        }
        __syncthreads();
        // -- finish_planes (chroma.rs:98-147) + write_tile (mod.rs:196-268), lag 23, core rows
        {
          const int lo = max(F - BH - 23, BORDER), hi = min(F - 23, TS - BORDER);
          for (int k = t; k < (hi - lo) * TS; k += THREADS) {
            const int ly = lo - BORDER + (k >> 8), lx = k & (TS - 1);
            if (lx >= VALID) continue;
            const int gx = ox + lx, gy = oy + ly;
            if (gx >= W || gy >= H) continue;
            const int rr = ly + BORDER, cc = lx + BORDER;
            const float sample = cfa.row(rr)[cc];  // in-image core sample, not mirrored
            const int ch = (ctab >> (2 * (((gy & 1) << 1) | (gx & 1)))) & 3;
            float r, b, gv;
            if ((cc & 1) != (g0 ^ (rr & 1))) {  // green site
              gv = sample;
              const float* hvr = hv.row(rr);
              const float up = hv.row(rr - 1)[cc >> 1], down = hv.row(rr + 1)[cc >> 1];
              const float left = hvr[(cc - 1) >> 1], right = hvr[(cc + 1) >> 1];
              const float temp = 1.0f / (up + 2.0f - right - left + down);
              const float* a0 = dgrb0.row(rr);
              const float* b0 = dgrb1.row(rr);
              const float br = (up * dgrb0.row(rr - 1)[cc >> 1] + (1.0f - right) * a0[(cc + 1) >> 1] +
                                (1.0f - left) * a0[(cc - 1) >> 1] + down * dgrb0.row(rr + 1)[cc >> 1]) *
                               temp;
              const float bb = (up * dgrb1.row(rr - 1)[cc >> 1] + (1.0f - right) * b0[(cc + 1) >> 1] +
                                (1.0f - left) * b0[(cc - 1) >> 1] + down * dgrb1.row(rr + 1)[cc >> 1]) *
                               temp;
              r = gv - br;
              b = gv - bb;
            } else {
              gv = green.row(rr)[cc >> 1];
              r = gv - dgrb0.row(rr)[cc >> 1];
              b = gv - dgrb1.row(rr)[cc >> 1];
            }
            r = fmax_(r, 0.0f);
            b = fmax_(b, 0.0f);
            float rgb0 = ch == 0 ? sample : r;
            float rgb1 = ch == 1 ? sample : fmax_(gv, 0.0f);
            float rgb2 = ch == 2 ? sample : b;
            rgb0 = rgb0 * im.gains[0];
            rgb1 = rgb1 * im.gains[1];
            rgb2 = rgb2 * im.gains[2];
            if (!isfinite(rgb0) || !isfinite(rgb1) || !isfinite(rgb2)) bad = 1;
            const long long o = (long long)gy * W + gx;
            im.out[o] = rgb0;
            im.out[plane + o] = rgb1;
            im.out[2 * plane + o] = rgb2;
            if (im.count_clip) {
              const float v = source_normalized(src, gx, gy);
              const float limit = src.clip_levels[ch];
              if (v >= limit) {
                affected++;
                if (ch == 0) ac0++;
                else if (ch == 1) ac1++;
                else ac2++;
              }
              if (v > 1.0f) over++;
              if (v > limit) changed++;
            }
          }
        }
        __syncthreads();
      }
      if (im.count_clip) {
        unsigned long long vals[6] = {affected, changed, over, ac0, ac1, ac2};
        for (int c = 0; c < 6; ++c) {
          unsigned long long v = vals[c];
          for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(FULL, v, off);
          if (lane == 0 && v) atomicAdd(&s_stats[c], v);
        }
      }
      if (bad) atomicOr(&s_bad, 1);
    }
    __syncthreads();
    if (t == 0) {
      if (im.count_clip)
        for (int c = 0; c < 6; ++c)
          if (s_stats[c]) atomicAdd(&im.clip_stats[c], s_stats[c]);
      if (s_bad) atomicOr(prm.error, 1u);
    }
    __syncthreads();
  } while (!prm.one_item);
  // A copy whose wait ran out may still land: wait for it once more (bounded)
  // before the block's shared memory is released.
  if (copy_pending && t == 0)
    for (unsigned i = 0; i < prm.wait_tries && !mbar_try_wait(&s_copy_bar, copy_parity); ++i) {
    }
}

}  // namespace

// Per-tile slabs and tile flags for `tiles` tiles, kept between calls and only
// grown; reserved ahead of a graph capture so that launches never allocate.
Status reserve_amaze_scratch(Context& ctx, size_t tiles) {
  if (ctx.amaze_slots >= tiles) return Status{};
  if (ctx.amaze_scratch) device_free(ctx, ctx.amaze_scratch, ctx.amaze_bytes);
  ctx.amaze_scratch = nullptr;
  ctx.amaze_slots = 0;
  ctx.amaze_bytes = 0;
  const size_t bytes = tiles * SLAB_FLOATS * sizeof(float) + tiles * sizeof(unsigned);
  void* p = nullptr;
  RD_TRY(device_alloc(ctx, bytes, &p));
  ctx.amaze_scratch = static_cast<float*>(p);
  ctx.amaze_slots = tiles;
  ctx.amaze_bytes = bytes;
  return Status{};
}

size_t amaze_tiles(int width, int height) {
  return (size_t)((width + VALID - 1) / VALID) * (size_t)((height + VALID - 1) / VALID);
}

Status run_amaze_images(Context& ctx, const AmazeJob* jobs, int n) {
  if (n <= 0) return Status{};
  std::vector<AmazeImage> images((size_t)n);
  std::vector<AmazeSegment> segs;
  segs.reserve(2 * (size_t)n);
  size_t total_tiles = 0;
  for (int i = 0; i < n; ++i) {
    const AmazeJob& j = jobs[i];
    AmazeImage& im = images[i];
    im.src = j.src;
    im.out = j.rgb;
    im.clip_stats = j.clip_stats;
    im.tiles_x = (j.src.width + VALID - 1) / VALID;
    im.tiles_y = (j.src.height + VALID - 1) / VALID;
    im.tile0 = (int)total_tiles;
    im.count_clip = j.count_clip;
    im.clip_point = j.clip_point;
    for (int c = 0; c < 3; ++c) im.gains[c] = j.gains[c];
    // Rows of 256 samples by tensor copy: the f32 mosaic with a 16-byte row
    // pitch, or raw samples with a 16-byte pitch and a crop x on the 8-sample
    // grid (tile x starts 224 k - 16 then lie on the 16-byte grid).
    const MosaicSource& ms = j.src;
    im.copy = AMAZE_COPY_NONE;
    if (ms.f32) {
      if (make_tensor_map_2d(&im.map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, ms.f32, ms.width, ms.height,
                             (uint64_t)ms.width * sizeof(float), TS, BH))
        im.copy = AMAZE_COPY_F32;
    } else if (ms.crop_x % 8 == 0 &&
               make_tensor_map_2d(&im.map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, ms.raw, (uint64_t)ms.crop_x + ms.width,
                                  (uint64_t)ms.crop_y + ms.height, (uint64_t)ms.row_stride * sizeof(uint16_t), TS, BH)) {
      im.copy = AMAZE_COPY_U16;
    }
    total_tiles += (size_t)im.tiles_x * im.tiles_y;
  }
  if (total_tiles > (size_t)(INT32_MAX / 2)) return Status{RD_INVALID_DIMENSIONS, "too many demosaic tiles in one launch"};
  // Hand-out order: phase A of image 0; then, image after image, phase A of
  // image i followed by phase B of image i - 1; phase B of the last image.
  int item = 0;
  auto add = [&](int image, int phase_b) {
    const int count = images[image].tiles_x * images[image].tiles_y;
    segs.push_back(AmazeSegment{item, count, image, phase_b});
    item += count;
  };
  add(0, 0);
  for (int i = 1; i < n; ++i) {
    add(i, 0);
    add(i - 1, 1);
  }
  add(n - 1, 1);
  // One resident CTA per SM (shared memory); the CTAs take half-tile items
  // from the counter, looping over them, or one each when the context yields
  // its SMs between items.
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int grid = ctx.yield_sms ? item : std::min(item, sms);
  if (ctx.capturing && ctx.amaze_slots < total_tiles)
    return Status{RD_INVALID_INPUT, "demosaic scratch was not reserved before the capture"};
  RD_TRY(reserve_amaze_scratch(ctx, total_tiles));
  unsigned* flags = reinterpret_cast<unsigned*>(ctx.amaze_scratch + ctx.amaze_slots * SLAB_FLOATS);
  const size_t img_bytes = sizeof(AmazeImage) * (size_t)n;
  const size_t seg_off = (img_bytes + 255) & ~(size_t)255;
  const size_t table_bytes = seg_off + sizeof(AmazeSegment) * segs.size();
  // The image table starts on a 64-byte boundary (its tensor maps need it).
  void* table = nullptr;
  RD_TRY(device_alloc(ctx, table_bytes + 64, &table));
  unsigned char* tb =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(table) + 63) & ~static_cast<uintptr_t>(63));
  Status st = upload(ctx, tb, images.data(), img_bytes);
  if (st.ok()) st = upload(ctx, tb + seg_off, segs.data(), sizeof(AmazeSegment) * segs.size());
  if (st.ok() && cudaMemsetAsync(flags, 0, sizeof(unsigned) * total_tiles, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "demosaic flag reset failed"};
  if (st.ok() &&
      cudaFuncSetAttribute(amaze_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "demosaic shared-memory limit"};
  if (st.ok()) {
    AmazeParams prm;
    prm.images = reinterpret_cast<const AmazeImage*>(tb);
    prm.segs = reinterpret_cast<const AmazeSegment*>(tb + seg_off);
    prm.nsegs = (int)segs.size();
    prm.total_items = item;
    prm.slab = ctx.amaze_scratch;
    prm.error = ctx.d_error;
    prm.flags = flags;
    prm.work = ctx.d_work;
    prm.wait_tries = ctx.wait_limit ? ctx.wait_limit : AMAZE_DEFAULT_WAIT_TRIES;
    prm.withhold_tile = ctx.wait_withhold == RD_WAIT_AMAZE_TILE ? 0 : -1;
    prm.withhold_copy = ctx.wait_withhold == RD_WAIT_AMAZE_COPY ? 1 : 0;
    prm.one_item = ctx.yield_sms ? 1 : 0;
    RD_LAUNCH(ctx, K_AMAZE, amaze_kernel<<<grid, THREADS, SMEM_BYTES, ctx.stream>>>(prm));
    const cudaError_t launch = cudaGetLastError();
    if (launch != cudaSuccess) st = Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  }
  device_free(ctx, table, table_bytes + 64);
  return st;
}

Status run_amaze(Context& ctx, const MosaicSource& src, const float gains[3], float clip_point, float* rgb,
                 int count_clip, unsigned long long* clip_stats) {
  AmazeJob job;
  job.src = src;
  job.rgb = rgb;
  job.count_clip = count_clip;
  job.clip_stats = clip_stats;
  job.clip_point = clip_point;
  for (int c = 0; c < 3; ++c) job.gains[c] = gains[c];
  return run_amaze_images(ctx, &job, 1);
}

}  // namespace rd
