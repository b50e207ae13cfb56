// Bilinear / Malvar-He-Cutler and RCD demosaic on sm_103a, plus the
// demosaic dispatcher with the channel balance of crates/demosaic/src/
// {lib,balance}.rs:302-370, 30-93.
//
// Both kernels read the raw u16 sensor samples (normalize + Clip fused into the
// tile load through MosaicSource) or the f32 mosaic after Opposed, stage the
// tile with its halo in shared memory, and write planar f32 RGB with
// coalesced stores. Compiled with --fmad=false; RCD's one explicit
// multiply-add (rcd_stages.rs:462-464) is written as __fmaf_rn.
#include <cuda_runtime.h>

#include "rd_internal.cuh"

namespace rd {

Status run_amaze(Context& ctx, const MosaicSource& src, const float gains[3], float clip_point, float* rgb,
                 int count_clip, unsigned long long* clip_stats);

namespace {

// Warp-aggregated Clip statistics of one pixel: affected, changed, over white, affected per channel.
struct ClipTally {
  unsigned long long v[6] = {0, 0, 0, 0, 0, 0};
  __device__ void add(const MosaicSource& s, int x, int y) {
    const float value = source_normalized(s, x, y);
    const int ch = color_at(s.cfa, x, y);
    const float limit = s.clip_levels[ch];
    if (value >= limit) { v[0]++; v[3 + ch]++; }
    if (value > limit) v[1]++;
    if (value > 1.0f) v[2]++;
  }
  __device__ void flush(unsigned long long* out) {
    for (int c = 0; c < 6; ++c) {
      unsigned long long s = v[c];
      for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
      if ((threadIdx.x & 31) == 0 && s) atomicAdd(&out[c], s);
    }
  }
};

// ------------------------------------------------------------- bilinear / MHC
constexpr int MT = 32;            // output tile
constexpr int MH = 2;             // halo
constexpr int MW = MT + 2 * MH;   // staged tile

__constant__ signed char K_G_AT_RB[25] = {0, 0, -2, 0, 0, 0, 0, 4, 0, 0, -2, 4, 8, 4, -2, 0, 0, 4, 0, 0, 0, 0, -2, 0, 0};
__constant__ signed char K_C_AT_G[25] = {0, 0, 1, 0, 0, 0, -2, 0, -2, 0, -2, 8, 10, 8, -2, 0, -2, 0, -2, 0, 0, 0, 1, 0, 0};
__constant__ signed char K_R_AT_B[25] = {0, 0, -3, 0, 0, 0, 4, 0, 4, 0, -3, 0, 12, 0, -3, 0, 4, 0, 4, 0, 0, 0, -3, 0, 0};

// malvar_he_cutler.rs:100-122: row-major taps, zero taps skipped, then * (1/16).
__device__ __forceinline__ float mhc(const float (*tile)[MW + 1], int lx, int ly, const signed char* k, bool transpose) {
  float sum = 0.0f;
#pragma unroll
  for (int ky = 0; ky < 5; ++ky)
#pragma unroll
    for (int kx = 0; kx < 5; ++kx) {
      const int c = transpose ? k[kx * 5 + ky] : k[ky * 5 + kx];
      if (c != 0) sum += (float)c * tile[ly + ky - 2][lx + kx - 2];
    }
  return sum * (1.0f / 16.0f);
}

// bilinear.rs:95-113: mean of the in-image neighbours at the given offsets.
__device__ __forceinline__ float avg_offsets(const float (*tile)[MW + 1], int lx, int ly, int x, int y, int W, int H,
                                             const int (*off)[2], int n) {
  float sum = 0.0f;
  int count = 0;
  for (int k = 0; k < n; ++k) {
    const int nx = x + off[k][0], ny = y + off[k][1];
    if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
    sum += tile[ly + off[k][1]][lx + off[k][0]];
    count++;
  }
  return count == 0 ? tile[ly][lx] : sum / (float)count;
}

// Bilinear everywhere (mhc_interior = 0) or MHC with the bilinear 2-pixel
// border (malvar_he_cutler.rs:46-69). Reads the balanced mosaic and applies
// `gains`, which are 1 except for the bilinear fallback of RCD and AMaZE below
// their size gates (rcd.rs:49-51, amaze/mod.rs:73-75).
__global__ void __launch_bounds__(256) mhc_kernel(const MosaicSource src, int mhc_interior, float g0, float g1, float g2,
                                                  float* out, int count_clip, unsigned long long* clip_stats,
                                                  unsigned* error) {
  __shared__ float tile[MW][MW + 1];
  const int W = src.width, H = src.height;
  const int x0 = blockIdx.x * MT, y0 = blockIdx.y * MT;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  for (int k = tid; k < MW * MW; k += 256) {
    const int ly = k / MW, lx = k % MW;
    const int x = min(max(x0 + lx - MH, 0), W - 1), y = min(max(y0 + ly - MH, 0), H - 1);
    tile[ly][lx] = source_balanced(src, x, y);
  }
  __syncthreads();
  const int CROSS[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
  const int DIAG[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  const int HORIZ[2][2] = {{-1, 0}, {1, 0}};
  const int VERT[2][2] = {{0, -1}, {0, 1}};
  const long long plane = (long long)W * H;
  ClipTally tally;
  bool bad = false;
  for (int ry = threadIdx.y; ry < MT; ry += blockDim.y) {
    const int x = x0 + threadIdx.x, y = y0 + ry;
    if (x >= W || y >= H) continue;
    const int lx = threadIdx.x + MH, ly = ry + MH;
    const int ch = color_at(src.cfa, x, y);
    const float s = tile[ly][lx];
    float r, g, b;
    const bool border = !mhc_interior || x < 2 || y < 2 || x >= W - 2 || y >= H - 2;
    if (border) {
      if (ch == 0) {
        r = s; g = avg_offsets(tile, lx, ly, x, y, W, H, CROSS, 4); b = avg_offsets(tile, lx, ly, x, y, W, H, DIAG, 4);
      } else if (ch == 2) {
        r = avg_offsets(tile, lx, ly, x, y, W, H, DIAG, 4); g = avg_offsets(tile, lx, ly, x, y, W, H, CROSS, 4); b = s;
      } else {
        const bool red_h = color_at(src.cfa, x + 1, y) == 0;
        r = avg_offsets(tile, lx, ly, x, y, W, H, red_h ? HORIZ : VERT, 2);
        g = s;
        b = avg_offsets(tile, lx, ly, x, y, W, H, red_h ? VERT : HORIZ, 2);
      }
    } else {
      if (ch == 0) {
        r = s; g = mhc(tile, lx, ly, K_G_AT_RB, false); b = mhc(tile, lx, ly, K_R_AT_B, false);
      } else if (ch == 2) {
        r = mhc(tile, lx, ly, K_R_AT_B, false); g = mhc(tile, lx, ly, K_G_AT_RB, false); b = s;
      } else {
        const bool red_h = color_at(src.cfa, x + 1, y) == 0;
        r = mhc(tile, lx, ly, K_C_AT_G, !red_h);
        g = s;
        b = mhc(tile, lx, ly, K_C_AT_G, red_h);
      }
    }
    r = r * g0;
    g = g * g1;
    b = b * g2;
    if (!isfinite(r) || !isfinite(g) || !isfinite(b)) bad = true;
    const long long o = (long long)y * W + x;
    out[o] = r;
    out[plane + o] = g;
    out[2 * plane + o] = b;
    if (count_clip) tally.add(src, x, y);
  }
  if (count_clip) tally.flush(clip_stats);
  if (bad) atomicOr(error, 1u);
}

// ------------------------------------------------------------------------ RCD
// rcd_stages.rs, computed on a 52x52 window around a 32x32 core. The window
// origin is even in both axes like the reference's tile windows, so the pair
// layout of its half-resolution planes (index / 2) lines up with image columns.
constexpr int RT = 32, RB = 10, RW = RT + 2 * RB, RWH = RW / 2;
constexpr float REPS = 1.0e-5f, REPS2 = 1.0e-10f;

struct RcdSmem {
  float cfa[RW * RW];
  float rgb[3][RW * RW];
  float vh[RW * RW];
  float vhp[RW * RW];   // squared vertical high pass
  float hhp[RW * RW];   // squared horizontal high pass
  float pq[RW * RWH];
  float pcd[RW * RWH];
  float qcd[RW * RWH];
};

__device__ __forceinline__ float rsq(float v) { return v * v; }
__device__ __forceinline__ float nonzero(float v) {
  if (fabsf(v) >= REPS) return v;
  return signbit(v) ? -REPS : REPS;
}
__device__ __forceinline__ float ratio_estimate(float sample, float lp, float nlp) {
  const float d = nonzero(REPS + lp + nlp);
  return sample * (2.0f * lp) / d;
}
__device__ __forceinline__ float weighted_pair(float w1, float v1, float w2, float v2) {
  return (w1 * v1 + w2 * v2) / nonzero(w1 + w2);
}
__device__ __forceinline__ float refined_direction(float c, float nw, float ne, float sw, float se) {
  const float n = 0.25f * (nw + ne + sw + se);
  float sel = fabsf(0.5f - c) < fabsf(0.5f - n) ? n : c;
  if (sel < 0.0f) sel = 0.0f;
  if (sel > 1.0f) sel = 1.0f;
  return sel;
}
__device__ __forceinline__ float interpolate(float d, float h, float v) { return __fmaf_rn(d, h, (1.0f - d) * v); }
__device__ __forceinline__ float cardinal_gradient(const float* v, int i, int step) {
  return REPS + fabsf(v[i + step] - v[i - step]) + fabsf(v[i] - v[i + 2 * step]) + fabsf(v[i + step] - v[i + 3 * step]) +
         fabsf(v[i + 2 * step] - v[i + 4 * step]);
}
__device__ __forceinline__ float diagonal_gradient(const float* v, const float* g, int i, int step) {
  return REPS + fabsf(v[i + step] - v[i - step]) + fabsf(v[i + step] - v[i + 3 * step]) + fabsf(g[i] - g[i + 2 * step]);
}
__device__ __forceinline__ float rmaxf(float a, float b) {
  if (isnan(a)) return b;
  if (isnan(b)) return a;
  return a > b ? a : b;
}

__global__ void __launch_bounds__(256) rcd_kernel(const MosaicSource src, float gains0, float gains1, float gains2,
                                                  float* out, int count_clip, unsigned long long* clip_stats,
                                                  unsigned* error) {
  extern __shared__ float4 rcd_smem_raw[];
  RcdSmem& S = *reinterpret_cast<RcdSmem*>(rcd_smem_raw);
  const int W = src.width, H = src.height;
  const int wx = blockIdx.x * RT - RB, wy = blockIdx.y * RT - RB;  // window origin (even)
  const int tp = shifted_cfa(src.cfa, wx & 1, wy & 1);             // pattern at the window origin
  const int tid = threadIdx.x;
  // populate (rcd.rs:226-271): the two colours of each row get the CFA values.
  for (int k = tid; k < RW * RW; k += 256) {
    const int row = k / RW, col = k % RW;
    const float v = source_balanced(src, mirror_index(wx + col, W), mirror_index(wy + row, H));
    S.cfa[k] = v;
    const int c0 = color_at(tp, 0, row), c1 = color_at(tp, 1, row);
    S.rgb[0][k] = (c0 == 0 || c1 == 0) ? v : 0.0f;
    S.rgb[1][k] = v;  // every row holds green
    S.rgb[2][k] = (c0 == 2 || c1 == 2) ? v : 0.0f;
  }
  for (int k = tid; k < RW * RWH; k += 256) {
    S.pq[k] = 0.0f;
    S.pcd[k] = 0.0f;
    S.qcd[k] = 0.0f;
  }
  __syncthreads();
  const float* cfa = S.cfa;
  // Squared high passes (rcd_stages.rs:417-427), rows/cols with a 3-sample reach.
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (r >= 3 && r < RW - 3 && c >= 4 && c < RW - 4)
      S.vhp[k] = rsq((cfa[k - 3 * RW] - cfa[k - RW] - cfa[k + RW] + cfa[k + 3 * RW]) -
                     3.0f * (cfa[k - 2 * RW] + cfa[k + 2 * RW]) + 6.0f * cfa[k]);
    if (r >= 4 && r < RW - 4 && c >= 3 && c < RW - 3)
      S.hhp[k] = rsq((cfa[k - 3] - cfa[k - 1] - cfa[k + 1] + cfa[k + 3]) - 3.0f * (cfa[k - 2] + cfa[k + 2]) +
                     6.0f * cfa[k]);
  }
  __syncthreads();
  // find_directions (rcd_stages.rs:8-48) and the low pass (:50-77).
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (r >= 4 && r < RW - 4 && c >= 4 && c < RW - 4) {
      const float vs = rmaxf(S.vhp[k - RW] + S.vhp[k] + S.vhp[k + RW], REPS2);
      const float hs = rmaxf(S.hhp[k - 1] + S.hhp[k] + S.hhp[k + 1], REPS2);
      S.vh[k] = vs / (vs + hs);
    }
    if (r >= 2 && r < RW - 2 && c >= 2 && c < RW - 2 && (c & 1) == (color_at(tp, 0, r) & 1)) {
      S.pq[k / 2] = cfa[k] + 0.5f * (cfa[k - RW] + cfa[k + RW] + cfa[k - 1] + cfa[k + 1]) +
                    0.25f * (cfa[k - RW - 1] + cfa[k - RW + 1] + cfa[k + RW - 1] + cfa[k + RW + 1]);
    }
  }
  __syncthreads();
  // interpolate_green (rcd_stages.rs:79-142)
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (!(r >= 4 && r < RW - 4 && c >= 4 && c < RW - 4 && (c & 1) == (color_at(tp, 0, r) & 1))) continue;
    const float ng = cardinal_gradient(cfa, k, -RW), sg = cardinal_gradient(cfa, k, RW);
    const float wg = cardinal_gradient(cfa, k, -1), eg = cardinal_gradient(cfa, k, 1);
    const int li = k / 2;
    const float lp = S.pq[li];
    const float ne = ratio_estimate(cfa[k - RW], lp, S.pq[li - RW]);
    const float se = ratio_estimate(cfa[k + RW], lp, S.pq[li + RW]);
    const float we = ratio_estimate(cfa[k - 1], lp, S.pq[li - 1]);
    const float ee = ratio_estimate(cfa[k + 1], lp, S.pq[li + 1]);
    const float ve = weighted_pair(sg, ne, ng, se);
    const float he = weighted_pair(wg, ee, eg, we);
    const float dir = refined_direction(S.vh[k], S.vh[k - RW - 1], S.vh[k - RW + 1], S.vh[k + RW - 1], S.vh[k + RW + 1]);
    S.rgb[1][k] = interpolate(dir, he, ve);
  }
  // calculate_diagonal_high_pass (rcd_stages.rs:160-199): odd columns, all rows.
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (!(r >= 3 && r < RW - 3 && c >= 3 && c < RW - 3 && (c & 1) == 1)) continue;
    S.pcd[k / 2] = rsq((cfa[k - 3 * RW - 3] - cfa[k - RW - 1] - cfa[k + RW + 1] + cfa[k + 3 * RW + 3]) -
                       3.0f * (cfa[k - 2 * RW - 2] + cfa[k + 2 * RW + 2]) + 6.0f * cfa[k]);
    S.qcd[k / 2] = rsq((cfa[k - 3 * RW + 3] - cfa[k - RW + 1] - cfa[k + RW - 1] + cfa[k + 3 * RW - 3]) -
                       3.0f * (cfa[k - 2 * RW + 2] + cfa[k + 2 * RW - 2]) + 6.0f * cfa[k]);
  }
  __syncthreads();
  // calculate_diagonal_directions (rcd_stages.rs:201-229), into pq.
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (!(r >= 4 && r < RW - 4 && c >= 4 && c < RW - 4 && (c & 1) == (color_at(tp, 0, r) & 1))) continue;
    const int hi = k / 2, pr = (k - RW - 1) / 2, nr = (k + RW - 1) / 2;
    const float ps = rmaxf(S.pcd[pr] + S.pcd[hi] + S.pcd[nr + 1], REPS2);
    const float qs = rmaxf(S.qcd[pr + 1] + S.qcd[hi] + S.qcd[nr], REPS2);
    S.pq[hi] = ps / (ps + qs);
  }
  __syncthreads();
  // interpolate_opposite_color (rcd_stages.rs:231-288)
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (!(r >= 4 && r < RW - 4 && c >= 4 && c < RW - 4 && (c & 1) == (color_at(tp, 0, r) & 1))) continue;
    const int ch = 2 - color_at(tp, c, r);
    const int hi = k / 2, pr = (k - RW - 1) / 2, nr = (k + RW - 1) / 2;
    const float dir = refined_direction(S.pq[hi], S.pq[pr], S.pq[pr + 1], S.pq[nr], S.pq[nr + 1]);
    const float* v = S.rgb[ch];
    const float* g = S.rgb[1];
    const float nwg = diagonal_gradient(v, g, k, -RW - 1), neg = diagonal_gradient(v, g, k, -RW + 1);
    const float swg = diagonal_gradient(v, g, k, RW - 1), seg = diagonal_gradient(v, g, k, RW + 1);
    const float nwe = v[k - RW - 1] - g[k - RW - 1], nee = v[k - RW + 1] - g[k - RW + 1];
    const float swe = v[k + RW - 1] - g[k + RW - 1], see = v[k + RW + 1] - g[k + RW + 1];
    const float dp = weighted_pair(nwg, see, seg, nwe);
    const float dq = weighted_pair(neg, swe, swg, nee);
    S.rgb[ch][k] = g[k] + interpolate(dir, dq, dp);
  }
  __syncthreads();
  // interpolate_at_green (rcd_stages.rs:290-366)
  for (int k = tid; k < RW * RW; k += 256) {
    const int r = k / RW, c = k % RW;
    if (!(r >= 4 && r < RW - 4 && c >= 4 && c < RW - 4 && (c & 1) == (color_at(tp, 1, r) & 1))) continue;
    const float dir = refined_direction(S.vh[k], S.vh[k - RW - 1], S.vh[k - RW + 1], S.vh[k + RW - 1], S.vh[k + RW + 1]);
    const float* g = S.rgb[1];
    const float green = g[k];
    const float n1 = REPS + fabsf(green - g[k - 2 * RW]);
    const float s1 = REPS + fabsf(green - g[k + 2 * RW]);
    const float w1 = REPS + fabsf(green - g[k - 2]);
    const float e1 = REPS + fabsf(green - g[k + 2]);
    const float gn = g[k - RW], gs = g[k + RW], gw = g[k - 1], ge = g[k + 1];
    for (int ch = 0; ch <= 2; ch += 2) {
      float* v = S.rgb[ch];
      const float nsa = fabsf(v[k - RW] - v[k + RW]);
      const float ewa = fabsf(v[k - 1] - v[k + 1]);
      const float ngr = n1 + nsa + fabsf(v[k - RW] - v[k - 3 * RW]);
      const float sgr = s1 + nsa + fabsf(v[k + RW] - v[k + 3 * RW]);
      const float wgr = w1 + ewa + fabsf(v[k - 1] - v[k - 3]);
      const float egr = e1 + ewa + fabsf(v[k + 1] - v[k + 3]);
      const float ne = v[k - RW] - gn, se = v[k + RW] - gs, we = v[k - 1] - gw, ee = v[k + 1] - ge;
      const float vert = weighted_pair(ngr, se, sgr, ne);
      const float horiz = weighted_pair(egr, we, wgr, ee);
      v[k] = green + interpolate(dir, horiz, vert);
    }
  }
  __syncthreads();
  // write_tile (rcd.rs:275-308): the measured sample replaces its channel.
  const long long plane = (long long)W * H;
  ClipTally tally;
  bool bad = false;
  for (int k = tid; k < RT * RT; k += 256) {
    const int ly = k / RT, lx = k % RT;
    const int x = blockIdx.x * RT + lx, y = blockIdx.y * RT + ly;
    if (x >= W || y >= H) continue;
    const int idx = (ly + RB) * RW + lx + RB;
    float rgb[3] = {S.rgb[0][idx], S.rgb[1][idx], S.rgb[2][idx]};
    rgb[color_at(src.cfa, x, y)] = source_balanced(src, x, y);
    rgb[0] = rgb[0] * gains0;
    rgb[1] = rgb[1] * gains1;
    rgb[2] = rgb[2] * gains2;
    if (!isfinite(rgb[0]) || !isfinite(rgb[1]) || !isfinite(rgb[2])) bad = true;
    const long long o = (long long)y * W + x;
    out[o] = rgb[0];
    out[plane + o] = rgb[1];
    out[2 * plane + o] = rgb[2];
    if (count_clip) tally.add(src, x, y);
  }
  if (count_clip) tally.flush(clip_stats);
  if (bad) atomicOr(error, 1u);
}

// Normalize (+ Clip) into an f32 mosaic: the input of Opposed and of the
// stage entry point. Each sample is visited once, so Clip statistics are exact.
// Eight consecutive samples of a row per thread, loaded together (their
// latencies overlap), stored as two 16-byte stores when aligned.
constexpr int NPX = 8;

__global__ void __launch_bounds__(256) normalize_kernel(const MosaicSource src, float* out, int count_clip,
                                                        unsigned long long* clip_stats) {
  const int x0 = (blockIdx.x * blockDim.x + threadIdx.x) * NPX, y = blockIdx.y;
  ClipTally tally;
  if (x0 < src.width) {
    const int n = min(NPX, src.width - x0);
    float v[NPX];
#pragma unroll
    for (int j = 0; j < NPX; ++j) v[j] = j < n ? source_linear(src, x0 + j, y) : 0.0f;
    float* o = out + (long long)y * src.width + x0;
    if (n == NPX && (reinterpret_cast<uintptr_t>(o) & 15) == 0) {
      reinterpret_cast<float4*>(o)[0] = make_float4(v[0], v[1], v[2], v[3]);
      reinterpret_cast<float4*>(o)[1] = make_float4(v[4], v[5], v[6], v[7]);
    } else {
      for (int j = 0; j < n; ++j) o[j] = v[j];
    }
    if (count_clip)
      for (int j = 0; j < n; ++j) tally.add(src, x0 + j, y);
  }
  if (count_clip) tally.flush(clip_stats);
}

}  // namespace

Status launch_normalize(Context& ctx, const MosaicSource& src, float* out, unsigned long long* clip_stats) {
  dim3 grid((src.width + 256 * NPX - 1) / (256 * NPX), src.height);
  RD_LAUNCH(ctx, K_NORMALIZE, normalize_kernel<<<grid, 256, 0, ctx.stream>>>(src, out, src.clip, clip_stats));
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

// demosaic_cancellable (crates/demosaic/src/lib.rs:302-370): RCD and AMaZE run
// on the balanced mosaic (largest gain = 1) and undo it on the output.
// ChannelBalance (crates/demosaic/src/balance.rs:24-94): RCD and AMaZE scale
// the mosaic by gains / max(gains) and undo it on output; AMaZE's clip point
// is the smallest forward gain.
AmazeJob demosaic_job(const MosaicSource& src_in, int algorithm, float* rgb, unsigned long long* clip_stats) {
  AmazeJob job;
  job.src = src_in;
  job.rgb = rgb;
  job.clip_stats = clip_stats;
  job.count_clip = (src_in.f32 == nullptr && src_in.clip) ? 1 : 0;
  for (int c = 0; c < 3; ++c) job.gains[c] = 1.0f;
  job.clip_point = 1.0f;
  const float* bal = src_in.fwd;  // caller passes the as-shot balance in fwd
  float largest = bal[0] > bal[1] ? bal[0] : bal[1];
  largest = largest > bal[2] ? largest : bal[2];
  float fwd[3] = {bal[0] / largest, bal[1] / largest, bal[2] / largest};
  const bool identity = fwd[0] == 1.0f && fwd[1] == 1.0f && fwd[2] == 1.0f;
  const bool balanced = (algorithm == RD_DEMOSAIC_RCD || algorithm == RD_DEMOSAIC_AMAZE) && !identity;
  for (int c = 0; c < 3; ++c) job.src.fwd[c] = balanced ? fwd[c] : 1.0f;
  if (balanced) {
    for (int c = 0; c < 3; ++c) job.gains[c] = 1.0f / fwd[c];
    job.clip_point = fwd[0] < fwd[1] ? fwd[0] : fwd[1];
    job.clip_point = job.clip_point < fwd[2] ? job.clip_point : fwd[2];
  }
  return job;
}

Status run_demosaic(Context& ctx, const MosaicSource& src_in, int algorithm, float* rgb,
                    unsigned long long* clip_stats) {
  const int W = src_in.width, H = src_in.height;
  if (W < 2 || H < 2) return Status{RD_INVALID_DIMENSIONS, "demosaicing requires at least 2x2 samples"};
  const AmazeJob job = demosaic_job(src_in, algorithm, rgb, clip_stats);
  const MosaicSource& src = job.src;
  const int count_clip = job.count_clip;
  const float* gains = job.gains;
  const float clip_point = job.clip_point;
  switch (algorithm) {
    case RD_DEMOSAIC_BILINEAR:
    case RD_DEMOSAIC_MHC: {
      dim3 grid((W + MT - 1) / MT, (H + MT - 1) / MT);
      RD_LAUNCH(ctx, K_MHC, mhc_kernel<<<grid, dim3(32, 8), 0, ctx.stream>>>(src, algorithm == RD_DEMOSAIC_MHC ? 1 : 0, 1.0f, 1.0f, 1.0f,
                                                       rgb, count_clip, clip_stats, ctx.d_error));
      break;
    }
    case RD_DEMOSAIC_RCD: {
      if (W <= 2 * RB + 4 || H <= 2 * RB + 4) {  // rcd_tiles size gate: bilinear
        dim3 grid((W + MT - 1) / MT, (H + MT - 1) / MT);
        RD_LAUNCH(ctx, K_MHC, mhc_kernel<<<grid, dim3(32, 8), 0, ctx.stream>>>(src, 0, gains[0], gains[1], gains[2], rgb, count_clip,
                                                         clip_stats, ctx.d_error));
        break;
      }
      const size_t smem = sizeof(RcdSmem);
      RD_CUDA_TRY(cudaFuncSetAttribute(rcd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      dim3 grid((W + RT - 1) / RT, (H + RT - 1) / RT);
      RD_LAUNCH(ctx, K_RCD, rcd_kernel<<<grid, 256, smem, ctx.stream>>>(src, gains[0], gains[1], gains[2], rgb, count_clip, clip_stats,
                                                  ctx.d_error));
      break;
    }
    case RD_DEMOSAIC_AMAZE: {
      if (W <= 32 || H <= 32) {  // amaze_tiles size gate: bilinear
        dim3 grid((W + MT - 1) / MT, (H + MT - 1) / MT);
        RD_LAUNCH(ctx, K_MHC, mhc_kernel<<<grid, dim3(32, 8), 0, ctx.stream>>>(src, 0, gains[0], gains[1], gains[2], rgb, count_clip,
                                                         clip_stats, ctx.d_error));
        break;
      }
      RD_TRY(run_amaze(ctx, src, gains, clip_point, rgb, count_clip, clip_stats));
      break;
    }
    default:
      return Status{RD_UNSUPPORTED, "unknown demosaic algorithm"};
  }
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

}  // namespace rd
