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

#include <type_traits>

#include "rd_internal.cuh"
#include "tma.cuh"

namespace rd {

Status run_amaze(Context& ctx, const MosaicSource& src, const float gains[3], float clip_point, float* rgb,
                 int count_clip, unsigned long long* clip_stats);

namespace {

// Warp-aggregated Clip statistics of one pixel: affected, changed, over white, affected per channel.
struct ClipTally {
  unsigned long long v[6] = {0, 0, 0, 0, 0, 0};
  __device__ void add(const MosaicSource& s, int x, int y) {
    const int ch = color_at(s.cfa, x, y);
    add_value(source_normalized(s, x, y), ch, s.clip_levels[ch]);
  }
  // One normalized sample of channel ch against its Clip ceiling.
  __device__ void add_value(float value, int ch, float limit) {
    if (value >= limit) {
      v[0]++;
      // Constant indexes keep the counters in registers.
      if (ch == 0) v[3]++;
      else if (ch == 1) v[4]++;
      else v[5]++;
    }
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
// One CTA per 64x32 output tile whose origin is even in both axes. The tile's
// samples with their 2-pixel halo are staged in shared memory by one TMA
// tensor copy: the f32 mosaic (after Opposed) directly, or the raw u16
// samples, normalized, clipped and balanced in shared memory. Sources that
// TMA cannot address (a row pitch or crop offset off the 16-byte grid) are
// staged with plain loads. A thread then takes 2x2 quads, so the colour of
// each of its four pixels, and with it every kernel tap, is a compile-time
// constant (the CFA is a template parameter); a quad's 6x6 window comes from
// shared memory in 64-bit loads. Tiles within 2 pixels of the image edge run
// the per-pixel form with the in-image neighbour checks of bilinear.rs.
constexpr int QW = 64, QH = 32;            // output tile
constexpr int QFW = QW + 8, QFH = QH + 4;  // staged f32 tile: columns x0-4 .. x0+QW+3, rows y0-2 .. y0+QH+1
constexpr int QUW = QW + 16;               // staged u16 box: columns x0-8 .. x0+QW+7
enum { QUAD_PLAIN = 0, QUAD_TMA_F32 = 1, QUAD_TMA_U16 = 2 };
// Error-word bit of a tile copy whose wait ran out.
constexpr unsigned DEMOSAIC_COPY_TIMEOUT = 128u;

struct __align__(128) QuadSmem {
  float t[QFH][QFW];         // first: the f32 box lands 128-byte aligned
  uint16_t raw[QFH][QUW];    // 10368 bytes in: 128-byte aligned too
  unsigned long long bar;
};

// The three kernels of malvar_he_cutler.rs:15-37 (x16), row-major:
// 0 green at red/blue, 1 colour at green (same row), 2 red at blue / blue at red.
__host__ __device__ constexpr int mhc_coef(int kid, int ky, int kx) {
  constexpr signed char k[3][25] = {
      {0, 0, -2, 0, 0, 0, 0, 4, 0, 0, -2, 4, 8, 4, -2, 0, 0, 4, 0, 0, 0, 0, -2, 0, 0},
      {0, 0, 1, 0, 0, 0, -2, 0, -2, 0, -2, 8, 10, 8, -2, 0, -2, 0, -2, 0, 0, 0, 1, 0, 0},
      {0, 0, -3, 0, 0, 0, 4, 0, 4, 0, -3, 0, 12, 0, -3, 0, 4, 0, 4, 0, 0, 0, -3, 0, 0}};
  return k[kid][ky * 5 + kx];
}
__host__ __device__ constexpr int cfa_color(int pattern, int x, int y) {
  return ((pattern == 0 ? 0x94 : pattern == 1 ? 0x16 : pattern == 2 ? 0x61 : 0x49) >> (2 * (((y & 1) << 1) | (x & 1)))) &
         3;
}

// apply_kernel (malvar_he_cutler.rs:100-122): taps in row-major order of the
// (possibly transposed) kernel, zero taps skipped, from 0, then * (1/16).
// at(dy, dx) is the sample dy rows and dx columns from the pixel.
template <int KID, bool T, int I = 0, class At>
__device__ __forceinline__ void mhc_acc(float& sum, const At& at) {
  if constexpr (I < 25) {
    constexpr int ky = I / 5, kx = I % 5;
    constexpr int c = T ? mhc_coef(KID, kx, ky) : mhc_coef(KID, ky, kx);
    if constexpr (c != 0) sum += (float)c * at(ky - 2, kx - 2);
    mhc_acc<KID, T, I + 1>(sum, at);
  }
}
template <int KID, bool T, class At>
__device__ __forceinline__ float mhc_sum(const At& at) {
  float sum = 0.0f;
  mhc_acc<KID, T>(sum, at);
  return sum * (1.0f / 16.0f);
}

// reconstruct_interior_pixel (malvar_he_cutler.rs:73-97) or, with mhc false,
// bilinear::reconstruct_pixel (bilinear.rs:63-92) where every neighbour lies
// in the image (offsets summed in the reference's order, then / count).
template <int CH, bool RED_H, class At>
__device__ __forceinline__ void interior_pixel(const At& at, bool mhc, float& r, float& g, float& b) {
  const float s = at(0, 0);
  if (mhc) {
    if constexpr (CH == 0) {
      r = s; g = mhc_sum<0, false>(at); b = mhc_sum<2, false>(at);
    } else if constexpr (CH == 2) {
      r = mhc_sum<2, false>(at); g = mhc_sum<0, false>(at); b = s;
    } else {
      r = mhc_sum<1, !RED_H>(at); g = s; b = mhc_sum<1, RED_H>(at);
    }
  } else {
    // CROSS (-1,0),(1,0),(0,-1),(0,1); DIAGONAL (-1,-1),(1,-1),(-1,1),(1,1); offsets are (dx, dy).
    auto cross = [&] { float v = 0.0f; v += at(0, -1); v += at(0, 1); v += at(-1, 0); v += at(1, 0); return v / 4.0f; };
    auto diag = [&] { float v = 0.0f; v += at(-1, -1); v += at(-1, 1); v += at(1, -1); v += at(1, 1); return v / 4.0f; };
    auto horiz = [&] { float v = 0.0f; v += at(0, -1); v += at(0, 1); return v / 2.0f; };
    auto vert = [&] { float v = 0.0f; v += at(-1, 0); v += at(1, 0); return v / 2.0f; };
    if constexpr (CH == 0) {
      r = s; g = cross(); b = diag();
    } else if constexpr (CH == 2) {
      r = diag(); g = cross(); b = s;
    } else if constexpr (RED_H) {
      r = horiz(); g = s; b = vert();
    } else {
      r = vert(); g = s; b = horiz();
    }
  }
}

// bilinear.rs:95-113: mean of the in-image neighbours at the given offsets.
__device__ __forceinline__ float avg_offsets(const float* c, int x, int y, int W, int H, const int (*off)[2], int n) {
  float sum = 0.0f;
  int count = 0;
  for (int k = 0; k < n; ++k) {
    const int nx = x + off[k][0], ny = y + off[k][1];
    if (nx < 0 || ny < 0 || nx >= W || ny >= H) continue;
    sum += c[off[k][1] * QFW + off[k][0]];
    count++;
  }
  return count == 0 ? c[0] : sum / (float)count;
}

// Balanced value of one normalized sample (NormalizationContract output):
// Clip at the channel's ceiling when selected, then the demosaic balance.
__device__ __forceinline__ float staged_value(const MosaicSource& s, float v, int ch) {
  if (s.clip) {
    const float limit = s.clip_levels[ch];
    if (v > limit) v = limit;
  }
  return __fmul_rn(v, s.fwd[ch]);
}
__device__ __forceinline__ void tally_value(ClipTally& tally, const MosaicSource& s, float value, int ch) {
  tally.add_value(value, ch, s.clip_levels[ch]);
}

// `gains` are 1 except for the bilinear fallback of RCD and AMaZE below their
// size gates (rcd.rs:49-51, amaze/mod.rs:73-75). `convert`: the f32 box needs
// Clip or a balance applied in shared memory.
template <int CFA>
__global__ void __launch_bounds__(256) quad_kernel(const MosaicSource src, int mhc_interior, float g0, float g1,
                                                   float g2, float* out, int count_clip,
                                                   unsigned long long* clip_stats, unsigned* error,
                                                   const __grid_constant__ CUtensorMap map, int load, int convert,
                                                   unsigned wait_tries, int withhold) {
  __shared__ QuadSmem S;
  const int W = src.width, H = src.height;
  const int x0 = blockIdx.x * QW, y0 = blockIdx.y * QH;
  const int tid = threadIdx.x;
  ClipTally tally;
  // ---- stage the tile
  if (load != QUAD_PLAIN) {
    if (tid == 0) {
      mbar_init(&S.bar);
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid == 0 && !withhold) {
      if (load == QUAD_TMA_F32) {
        mbar_expect_tx(&S.bar, QFH * QFW * sizeof(float));
        tma_load_2d(&S.t[0][0], &map, x0 - 4, y0 - 2, &S.bar);
      } else {
        mbar_expect_tx(&S.bar, QFH * QUW * sizeof(uint16_t));
        tma_load_2d(&S.raw[0][0], &map, src.crop_x + x0 - 8, src.crop_y + y0 - 2, &S.bar);
      }
    }
    bool done = false;
    for (unsigned i = 0; i < wait_tries && !done; ++i) done = mbar_try_wait(&S.bar, 0);
    if (__syncthreads_or(!done)) {
      // The wait ran out: the block reads nothing, reports it and ends. A
      // copy that was issued may still land, so thread 0 waits for it once
      // more (bounded) while the block's shared memory is still held.
      if (tid == 0) {
        atomicOr(error, DEMOSAIC_COPY_TIMEOUT);
        if (!withhold)
          for (unsigned i = 0; i < wait_tries && !mbar_try_wait(&S.bar, 0); ++i) {
          }
      }
      return;
    }
    if (load == QUAD_TMA_U16 || convert) {
      for (int k = tid; k < QFH * QFW; k += 256) {
        const int r = k / QFW, c = k % QFW;
        const int x = x0 - 4 + c, y = y0 - 2 + r;
        const bool inside = (unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H;
        const int ch = cfa_color(CFA, x, y);
        float v = 0.0f;
        if (inside) {
          float n;
          if (load == QUAD_TMA_U16) {
            const int sx = src.crop_x + x, sy = src.crop_y + y;
            n = normalize_raw(src, (float)S.raw[r][c + 4], sx, sy);
          } else {
            n = S.t[r][c];
          }
          v = staged_value(src, n, ch);
          if (count_clip && r >= 2 && r < QH + 2 && c >= 4 && c < QW + 4) tally_value(tally, src, n, ch);
        }
        if (load == QUAD_TMA_U16) S.t[r][c] = v;
        else if (inside) S.t[r][c] = v;
      }
    }
  } else {
    for (int k = tid; k < QFH * QFW; k += 256) {
      const int r = k / QFW, c = k % QFW;
      const int x = x0 - 4 + c, y = y0 - 2 + r;
      const bool inside = (unsigned)x < (unsigned)W && (unsigned)y < (unsigned)H;
      float v = 0.0f;
      if (inside) {
        const int ch = cfa_color(CFA, x, y);
        const float n = source_normalized(src, x, y);
        v = staged_value(src, n, ch);
        if (count_clip && r >= 2 && r < QH + 2 && c >= 4 && c < QW + 4) tally_value(tally, src, n, ch);
      }
      S.t[r][c] = v;
    }
  }
  __syncthreads();
  // ---- reconstruct
  const long long plane = (long long)W * H;
  const bool mhc = mhc_interior != 0;
  bool bad = false;
  const bool edge = x0 < 2 || y0 < 2 || x0 + QW > W - 2 || y0 + QH > H - 2;
  if (!edge) {
    // Quads (2 * lane, 2 * qy) for qy = warp and warp + 8.
    const int lane = tid & 31, warp = tid >> 5;
    const bool pairs = (W & 1) == 0;  // rows start on 8-byte boundaries
#pragma unroll 1
    for (int qy = warp; qy < QH / 2; qy += 8) {
      float w[6][6];
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float2 v = *reinterpret_cast<const float2*>(&S.t[2 * qy + i][2 * lane + 2 + 2 * j]);
          w[i][2 * j] = v.x;
          w[i][2 * j + 1] = v.y;
        }
      float rgb[2][2][3];
      auto px = [&](auto dxc, auto dyc) {
        constexpr int DX = decltype(dxc)::value, DY = decltype(dyc)::value;
        constexpr int CH = cfa_color(CFA, DX, DY);
        constexpr bool RED_H = cfa_color(CFA, DX + 1, DY) == 0;
        auto at = [&](int dy, int dx) { return w[2 + DY + dy][2 + DX + dx]; };
        interior_pixel<CH, RED_H>(at, mhc, rgb[DY][DX][0], rgb[DY][DX][1], rgb[DY][DX][2]);
      };
      px(std::integral_constant<int, 0>{}, std::integral_constant<int, 0>{});
      px(std::integral_constant<int, 1>{}, std::integral_constant<int, 0>{});
      px(std::integral_constant<int, 0>{}, std::integral_constant<int, 1>{});
      px(std::integral_constant<int, 1>{}, std::integral_constant<int, 1>{});
      const int x = x0 + 2 * lane, y = y0 + 2 * qy;
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const long long o = (long long)(y + dy) * W + x;
        const float gains[3] = {g0, g1, g2};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float a = rgb[dy][0][c] * gains[c], b = rgb[dy][1][c] * gains[c];
          if (!isfinite(a) || !isfinite(b)) bad = true;
          float* p = out + c * plane + o;
          if (pairs) {
            *reinterpret_cast<float2*>(p) = make_float2(a, b);
          } else {
            p[0] = a;
            p[1] = b;
          }
        }
      }
    }
  } else {
    const int CROSS[4][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}};
    const int DIAG[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
    const int HORIZ[2][2] = {{-1, 0}, {1, 0}};
    const int VERT[2][2] = {{0, -1}, {0, 1}};
    for (int k = tid; k < QW * QH; k += 256) {
      const int x = x0 + (k % QW), y = y0 + k / QW;
      if (x >= W || y >= H) continue;
      const float* c = &S.t[y - y0 + 2][x - x0 + 4];
      auto at = [&](int dy, int dx) { return c[dy * QFW + dx]; };
      const int ch = cfa_color(CFA, x, y);
      const bool red_h = cfa_color(CFA, x + 1, y) == 0;
      float r, g, b;
      const bool border = !mhc || x < 2 || y < 2 || x >= W - 2 || y >= H - 2;
      if (border) {
        const float s = c[0];
        if (ch == 0) {
          r = s; g = avg_offsets(c, x, y, W, H, CROSS, 4); b = avg_offsets(c, x, y, W, H, DIAG, 4);
        } else if (ch == 2) {
          r = avg_offsets(c, x, y, W, H, DIAG, 4); g = avg_offsets(c, x, y, W, H, CROSS, 4); b = s;
        } else {
          r = avg_offsets(c, x, y, W, H, red_h ? HORIZ : VERT, 2);
          g = s;
          b = avg_offsets(c, x, y, W, H, red_h ? VERT : HORIZ, 2);
        }
      } else if (ch == 0) {
        interior_pixel<0, false>(at, true, r, g, b);
      } else if (ch == 2) {
        interior_pixel<2, false>(at, true, r, g, b);
      } else if (red_h) {
        interior_pixel<1, true>(at, true, r, g, b);
      } else {
        interior_pixel<1, false>(at, true, r, g, b);
      }
      r = r * g0;
      g = g * g1;
      b = b * g2;
      if (!isfinite(r) || !isfinite(g) || !isfinite(b)) bad = true;
      const long long o = (long long)y * W + x;
      out[o] = r;
      out[plane + o] = g;
      out[2 * plane + o] = b;
    }
  }
  if (count_clip) tally.flush(clip_stats);
  if (bad) atomicOr(error, 1u);
}

// ------------------------------------------------------------------------ RCD
// rcd_stages.rs on an 84x84 sample window around a 64x64 core, one CTA of
// 1024 threads per SM. RCD's core values never depend on where the core sits
// in its window (every stage leaves at least its stencil reach inside the
// 10-pixel halo), so the core size is free; 64x64 cores re-read 1.72 window
// samples per output pixel. The window origin is even in both axes like the
// reference's tile windows, so the pair layout of its half-resolution planes
// (index / 2 with an even row pitch) lines up with image columns. Windows
// inside the image arrive by one TMA tensor copy (the f32 mosaic, or the raw
// u16 samples normalized in shared memory); windows that cross the image
// edge are loaded with their mirrored samples. Each stage runs over exactly
// its sites (rows, and columns of one parity where the reference steps by
// two), so no thread spends issue slots on skipped positions.
constexpr int RT = 64, RB = 10, RW = RT + 2 * RB;  // core, halo, window
constexpr int RP = RW + 4;                        // plane row pitch: window column c sits at plane column c + 2
constexpr int RPH = RP / 2;                       // half-plane row pitch
constexpr int RU = RW + 12;                       // u16 box: columns wx - 6 .. wx + 89
constexpr int RTHREADS = 1024;
constexpr float REPS = 1.0e-5f, REPS2 = 1.0e-10f;

struct __align__(128) RcdSmem {
  float cfa[RW * RP];     // first: the f32 box lands 128-byte aligned
  float rgb[3][RW * RP];
  float vh[RW * RP];
  // The raw u16 window (before the high passes), then the squared vertical /
  // horizontal high passes, then the diagonal high passes (half planes).
  float hp[2][RW * RP];
  float pq[RW * RPH];     // low pass, then the diagonal directions
  unsigned long long bar;
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

// `load`: QUAD_PLAIN (mirrored plain loads), QUAD_TMA_F32 or QUAD_TMA_U16
// for windows inside the image; `convert`: the f32 box needs Clip or the
// balance applied in shared memory.
__global__ void __launch_bounds__(RTHREADS, 1) rcd_kernel(const MosaicSource src, float gains0, float gains1,
                                                          float gains2, float* out, int count_clip,
                                                          unsigned long long* clip_stats, unsigned* error,
                                                          const __grid_constant__ CUtensorMap map, int load,
                                                          int convert, unsigned wait_tries, int withhold) {
  extern __shared__ float4 rcd_smem_raw[];
  RcdSmem& S = *reinterpret_cast<RcdSmem*>(rcd_smem_raw);
  const int W = src.width, H = src.height;
  const int wx = blockIdx.x * RT - RB, wy = blockIdx.y * RT - RB;  // window origin (even)
  const int tp = shifted_cfa(src.cfa, wx & 1, wy & 1);             // pattern at the window origin
  const int tid = threadIdx.x;
  // Plane views: window (row, column) at index row * RP + column.
  float* const cfa = S.cfa + 2;
  float* const R0 = S.rgb[0] + 2;
  float* const G1 = S.rgb[1] + 2;
  float* const B2 = S.rgb[2] + 2;
  float* const vh = S.vh + 2;
  float* const vhp = S.hp[0] + 2;
  float* const hhp = S.hp[1] + 2;
  float* const pcd = S.hp[0];  // half planes (index / 2)
  float* const qcd = S.hp[1];
  float* const pq = S.pq;
  ClipTally tally;
  // ---- populate (rcd.rs:226-271): the window's balanced samples; the two
  //      colours of each row get the CFA values.
  const bool inside = wx >= 0 && wy >= 0 && wx + RW <= W && wy + RW <= H;
  const int mode = inside ? load : QUAD_PLAIN;
  if (mode != QUAD_PLAIN) {
    if (tid == 0) {
      mbar_init(&S.bar);
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    if (tid == 0 && !withhold) {
      if (mode == QUAD_TMA_F32) {
        mbar_expect_tx(&S.bar, RW * RP * sizeof(float));
        tma_load_2d(S.cfa, &map, wx - 2, wy, &S.bar);
      } else {
        mbar_expect_tx(&S.bar, RW * RU * sizeof(uint16_t));
        tma_load_2d(S.hp[0], &map, src.crop_x + wx - 6, src.crop_y + wy, &S.bar);
      }
    }
    bool done = false;
    for (unsigned i = 0; i < wait_tries && !done; ++i) done = mbar_try_wait(&S.bar, 0);
    if (__syncthreads_or(!done)) {
      // The wait ran out: report it and end the block; an issued copy may
      // still land, so thread 0 waits for it once more (bounded) first.
      if (tid == 0) {
        atomicOr(error, DEMOSAIC_COPY_TIMEOUT);
        if (!withhold)
          for (unsigned i = 0; i < wait_tries && !mbar_try_wait(&S.bar, 0); ++i) {
          }
      }
      return;
    }
  }
  const uint16_t* raw_win = reinterpret_cast<const uint16_t*>(S.hp[0]);
  for (int k = tid; k < RW * RW; k += RTHREADS) {
    const int row = k / RW, col = k - row * RW;
    const int i = row * RP + col;
    const int ch = color_at(tp, col, row);
    const bool core = row >= RB && row < RB + RT && col >= RB && col < RB + RT;
    float n;
    if (mode == QUAD_TMA_F32) {
      n = cfa[i];
    } else if (mode == QUAD_TMA_U16) {
      const int sx = src.crop_x + wx + col, sy = src.crop_y + wy + row;
      n = normalize_raw(src, (float)raw_win[row * RU + col + 6], sx, sy);
    } else {
      n = source_normalized(src, mirror_index(wx + col, W), mirror_index(wy + row, H));
    }
    float v = n;
    if (mode != QUAD_TMA_F32 || convert) v = staged_value(src, n, ch);
    if (count_clip && core && wx + col < W && wy + row < H) tally_value(tally, src, n, ch);
    const int c0 = color_at(tp, 0, row), c1 = color_at(tp, 1, row);
    cfa[i] = v;
    R0[i] = (c0 == 0 || c1 == 0) ? v : 0.0f;
    G1[i] = v;  // every row holds green
    B2[i] = (c0 == 2 || c1 == 2) ? v : 0.0f;
  }
  __syncthreads();
  // ---- squared high passes (rcd_stages.rs:8-48, 393-404): vertical at rows
  //      [3, RW-3) x cols [4, RW-4), horizontal at rows [4, RW-4) x cols [3, RW-3)
  for (int k = tid; k < (RW - 6) * (RW - 6); k += RTHREADS) {
    const int r = 3 + k / (RW - 6), c = 3 + k % (RW - 6);
    const int i = r * RP + c;
    if (c >= 4 && c < RW - 4)
      vhp[i] = rsq((cfa[i - 3 * RP] - cfa[i - RP] - cfa[i + RP] + cfa[i + 3 * RP]) -
                   3.0f * (cfa[i - 2 * RP] + cfa[i + 2 * RP]) + 6.0f * cfa[i]);
    if (r >= 4 && r < RW - 4)
      hhp[i] = rsq((cfa[i - 3] - cfa[i - 1] - cfa[i + 1] + cfa[i + 3]) - 3.0f * (cfa[i - 2] + cfa[i + 2]) + 6.0f * cfa[i]);
  }
  __syncthreads();
  // ---- find_directions (rcd_stages.rs:8-48) at [4, RW-4)^2 and the low pass
  //      (:55-82) at the red/blue sites of [2, RW-2)^2
  for (int k = tid; k < (RW - 8) * (RW - 8); k += RTHREADS) {
    const int r = 4 + k / (RW - 8), c = 4 + k % (RW - 8);
    const int i = r * RP + c;
    const float vs = rmaxf(vhp[i - RP] + vhp[i] + vhp[i + RP], REPS2);
    const float hs = rmaxf(hhp[i - 1] + hhp[i] + hhp[i + 1], REPS2);
    vh[i] = vs / (vs + hs);
  }
  for (int k = tid; k < (RW - 4) * ((RW - 4) / 2); k += RTHREADS) {
    const int r = 2 + k / ((RW - 4) / 2);
    const int c = 2 + (color_at(tp, 0, r) & 1) + 2 * (k % ((RW - 4) / 2));
    const int i = r * RP + c;
    pq[i / 2] = cfa[i] + 0.5f * (cfa[i - RP] + cfa[i + RP] + cfa[i - 1] + cfa[i + 1]) +
                0.25f * (cfa[i - RP - 1] + cfa[i - RP + 1] + cfa[i + RP - 1] + cfa[i + RP + 1]);
  }
  __syncthreads();
  // ---- interpolate_green (rcd_stages.rs:84-147) at the red/blue sites of
  //      [4, RW-4)^2; calculate_diagonal_high_pass (:162-196) at the odd
  //      columns of [3, RW-3)^2 (into the high-pass area, now free)
  constexpr int SITES4 = (RW - 8) / 2;  // red/blue sites per row of [4, RW-4)
  for (int k = tid; k < (RW - 8) * SITES4; k += RTHREADS) {
    const int r = 4 + k / SITES4;
    const int c = 4 + (color_at(tp, 0, r) & 1) + 2 * (k % SITES4);
    const int i = r * RP + c;
    const float ng = cardinal_gradient(cfa, i, -RP), sg = cardinal_gradient(cfa, i, RP);
    const float wg = cardinal_gradient(cfa, i, -1), eg = cardinal_gradient(cfa, i, 1);
    const int li = i / 2;
    const float lp = pq[li];
    const float ne = ratio_estimate(cfa[i - RP], lp, pq[li - RP]);
    const float se = ratio_estimate(cfa[i + RP], lp, pq[li + RP]);
    const float we = ratio_estimate(cfa[i - 1], lp, pq[li - 1]);
    const float ee = ratio_estimate(cfa[i + 1], lp, pq[li + 1]);
    const float ve = weighted_pair(sg, ne, ng, se);
    const float he = weighted_pair(wg, ee, eg, we);
    const float dir = refined_direction(vh[i], vh[i - RP - 1], vh[i - RP + 1], vh[i + RP - 1], vh[i + RP + 1]);
    G1[i] = interpolate(dir, he, ve);
  }
  constexpr int ODD3 = (RW - 6) / 2;  // odd columns of [3, RW-3)
  for (int k = tid; k < (RW - 6) * ODD3; k += RTHREADS) {
    const int r = 3 + k / ODD3, c = 3 + 2 * (k % ODD3);
    const int i = r * RP + c;
    pcd[i / 2] = rsq((cfa[i - 3 * RP - 3] - cfa[i - RP - 1] - cfa[i + RP + 1] + cfa[i + 3 * RP + 3]) -
                     3.0f * (cfa[i - 2 * RP - 2] + cfa[i + 2 * RP + 2]) + 6.0f * cfa[i]);
    qcd[i / 2] = rsq((cfa[i - 3 * RP + 3] - cfa[i - RP + 1] - cfa[i + RP - 1] + cfa[i + 3 * RP - 3]) -
                     3.0f * (cfa[i - 2 * RP + 2] + cfa[i + 2 * RP - 2]) + 6.0f * cfa[i]);
  }
  __syncthreads();
  // ---- calculate_diagonal_directions (rcd_stages.rs:198-225), into pq
  for (int k = tid; k < (RW - 8) * SITES4; k += RTHREADS) {
    const int r = 4 + k / SITES4;
    const int c = 4 + (color_at(tp, 0, r) & 1) + 2 * (k % SITES4);
    const int i = r * RP + c;
    const int hi = i / 2, pr = (i - RP - 1) / 2, nr = (i + RP - 1) / 2;
    const float ps = rmaxf(pcd[pr] + pcd[hi] + pcd[nr + 1], REPS2);
    const float qs = rmaxf(qcd[pr + 1] + qcd[hi] + qcd[nr], REPS2);
    pq[hi] = ps / (ps + qs);
  }
  __syncthreads();
  // ---- interpolate_opposite_color (rcd_stages.rs:227-285)
  for (int k = tid; k < (RW - 8) * SITES4; k += RTHREADS) {
    const int r = 4 + k / SITES4;
    const int c = 4 + (color_at(tp, 0, r) & 1) + 2 * (k % SITES4);
    const int i = r * RP + c;
    const int ch = 2 - color_at(tp, c, r);
    const int hi = i / 2, pr = (i - RP - 1) / 2, nr = (i + RP - 1) / 2;
    const float dir = refined_direction(pq[hi], pq[pr], pq[pr + 1], pq[nr], pq[nr + 1]);
    float* const v = ch == 0 ? R0 : B2;
    const float* g = G1;
    const float nwg = diagonal_gradient(v, g, i, -RP - 1), neg = diagonal_gradient(v, g, i, -RP + 1);
    const float swg = diagonal_gradient(v, g, i, RP - 1), seg = diagonal_gradient(v, g, i, RP + 1);
    const float nwe = v[i - RP - 1] - g[i - RP - 1], nee = v[i - RP + 1] - g[i - RP + 1];
    const float swe = v[i + RP - 1] - g[i + RP - 1], see = v[i + RP + 1] - g[i + RP + 1];
    const float dp = weighted_pair(nwg, see, seg, nwe);
    const float dq = weighted_pair(neg, swe, swg, nee);
    v[i] = g[i] + interpolate(dir, dq, dp);
  }
  __syncthreads();
  // ---- interpolate_at_green (rcd_stages.rs:287-355) at the green sites of [4, RW-4)^2
  for (int k = tid; k < (RW - 8) * SITES4; k += RTHREADS) {
    const int r = 4 + k / SITES4;
    const int c = 4 + (color_at(tp, 1, r) & 1) + 2 * (k % SITES4);
    const int i = r * RP + c;
    const float dir = refined_direction(vh[i], vh[i - RP - 1], vh[i - RP + 1], vh[i + RP - 1], vh[i + RP + 1]);
    const float* g = G1;
    const float green = g[i];
    const float n1 = REPS + fabsf(green - g[i - 2 * RP]);
    const float s1 = REPS + fabsf(green - g[i + 2 * RP]);
    const float w1 = REPS + fabsf(green - g[i - 2]);
    const float e1 = REPS + fabsf(green - g[i + 2]);
    const float gn = g[i - RP], gs = g[i + RP], gw = g[i - 1], ge = g[i + 1];
#pragma unroll
    for (int chn = 0; chn <= 2; chn += 2) {
      float* v = chn == 0 ? R0 : B2;
      const float nsa = fabsf(v[i - RP] - v[i + RP]);
      const float ewa = fabsf(v[i - 1] - v[i + 1]);
      const float ngr = n1 + nsa + fabsf(v[i - RP] - v[i - 3 * RP]);
      const float sgr = s1 + nsa + fabsf(v[i + RP] - v[i + 3 * RP]);
      const float wgr = w1 + ewa + fabsf(v[i - 1] - v[i - 3]);
      const float egr = e1 + ewa + fabsf(v[i + 1] - v[i + 3]);
      const float ne = v[i - RP] - gn, se = v[i + RP] - gs, we = v[i - 1] - gw, ee = v[i + 1] - ge;
      const float vert = weighted_pair(ngr, se, sgr, ne);
      const float horiz = weighted_pair(egr, we, wgr, ee);
      v[i] = green + interpolate(dir, horiz, vert);
    }
  }
  __syncthreads();
  // ---- write_tile (rcd.rs:275-308): the measured sample replaces its channel.
  const long long plane = (long long)W * H;
  bool bad = false;
  for (int k = tid; k < RT * RT; k += RTHREADS) {
    const int ly = k / RT, lx = k % RT;
    const int x = wx + RB + lx, y = wy + RB + ly;
    if (x >= W || y >= H) continue;
    const int i = (ly + RB) * RP + lx + RB;
    const int measured = color_at(tp, lx + RB, ly + RB);
    const float r = (measured == 0 ? cfa[i] : R0[i]) * gains0;
    const float g = (measured == 1 ? cfa[i] : G1[i]) * gains1;
    const float b = (measured == 2 ? cfa[i] : B2[i]) * gains2;
    if (!isfinite(r) || !isfinite(g) || !isfinite(b)) bad = true;
    const long long o = (long long)y * W + x;
    out[o] = r;
    out[plane + o] = g;
    out[2 * plane + o] = b;
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

// Bilinear (mhc = 0) or MHC over the whole image: one 64x32 tile per CTA,
// staged by a tensor copy of the f32 mosaic or of the raw u16 samples when
// TMA can address the source (16-byte row pitch, and a crop x on the 8-sample
// grid for raw samples), else by plain loads.
static Status launch_quad(Context& ctx, const MosaicSource& src, int mhc, const float gains[3], float* rgb,
                          int count_clip, unsigned long long* clip_stats) {
  const int W = src.width, H = src.height;
  CUtensorMap map{};
  int load = QUAD_PLAIN;
  if (src.f32) {
    if (make_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src.f32, W, H, (uint64_t)W * sizeof(float), QFW,
                           QFH))
      load = QUAD_TMA_F32;
  } else if (src.crop_x % 8 == 0 &&
             make_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, src.raw, (uint64_t)src.crop_x + W,
                                (uint64_t)src.crop_y + H, (uint64_t)src.row_stride * sizeof(uint16_t), QUW, QFH)) {
    load = QUAD_TMA_U16;
  }
  const int convert = load == QUAD_TMA_F32 && (src.clip || src.fwd[0] != 1.0f || src.fwd[1] != 1.0f || src.fwd[2] != 1.0f);
  const unsigned tries = ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES;
  const int withhold = load != QUAD_PLAIN && ctx.wait_withhold == RD_WAIT_DEMOSAIC_COPY ? 1 : 0;
  const dim3 grid((W + QW - 1) / QW, (H + QH - 1) / QH);
#define RD_QUAD(P)                                                                                                   \
  RD_LAUNCH(ctx, K_MHC,                                                                                              \
            quad_kernel<P><<<grid, 256, 0, ctx.stream>>>(src, mhc, gains[0], gains[1], gains[2], rgb, count_clip,    \
                                                         clip_stats, ctx.d_error, map, load, convert, tries, withhold))
  switch (src.cfa) {
    case 0: RD_QUAD(0); break;
    case 1: RD_QUAD(1); break;
    case 2: RD_QUAD(2); break;
    default: RD_QUAD(3); break;
  }
#undef RD_QUAD
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}

// RCD over the whole image: one 64x64 core per CTA; windows inside the image
// arrive by a tensor copy when TMA can address the source (as for the
// bilinear / MHC tiles), the others with their mirrored samples.
static Status launch_rcd(Context& ctx, const MosaicSource& src, const float gains[3], float* rgb, int count_clip,
                         unsigned long long* clip_stats) {
  const int W = src.width, H = src.height;
  CUtensorMap map{};
  int load = QUAD_PLAIN;
  if (src.f32) {
    if (make_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src.f32, W, H, (uint64_t)W * sizeof(float), RP, RW))
      load = QUAD_TMA_F32;
  } else if (src.crop_x % 8 == 0 &&
             make_tensor_map_2d(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, src.raw, (uint64_t)src.crop_x + W,
                                (uint64_t)src.crop_y + H, (uint64_t)src.row_stride * sizeof(uint16_t), RU, RW)) {
    load = QUAD_TMA_U16;
  }
  const int convert = load == QUAD_TMA_F32 && (src.clip || src.fwd[0] != 1.0f || src.fwd[1] != 1.0f || src.fwd[2] != 1.0f);
  const unsigned tries = ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES;
  const int withhold = load != QUAD_PLAIN && ctx.wait_withhold == RD_WAIT_DEMOSAIC_COPY ? 1 : 0;
  const size_t smem = sizeof(RcdSmem);
  RD_CUDA_TRY(cudaFuncSetAttribute(rcd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const dim3 grid((W + RT - 1) / RT, (H + RT - 1) / RT);
  RD_LAUNCH(ctx, K_RCD,
            rcd_kernel<<<grid, RTHREADS, smem, ctx.stream>>>(src, gains[0], gains[1], gains[2], rgb, count_clip,
                                                             clip_stats, ctx.d_error, map, load, convert, tries,
                                                             withhold));
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
      const float ones[3] = {1.0f, 1.0f, 1.0f};
      RD_TRY(launch_quad(ctx, src, algorithm == RD_DEMOSAIC_MHC ? 1 : 0, ones, rgb, count_clip, clip_stats));
      break;
    }
    case RD_DEMOSAIC_RCD: {
      if (W <= 2 * RB + 4 || H <= 2 * RB + 4) {  // rcd_tiles size gate: bilinear
        RD_TRY(launch_quad(ctx, src, 0, gains, rgb, count_clip, clip_stats));
        break;
      }
      RD_TRY(launch_rcd(ctx, src, gains, rgb, count_clip, clip_stats));
      break;
    }
    case RD_DEMOSAIC_AMAZE: {
      if (W <= 32 || H <= 32) {  // amaze_tiles size gate: bilinear
        RD_TRY(launch_quad(ctx, src, 0, gains, rgb, count_clip, clip_stats));
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
