// Masked Richardson-Lucy capture sharpening (crates/core/src/sharpening.rs:
// 87-389) and lens vignetting (crates/optics/src/correction.rs:213-267) on
// sm_103a.
//
// Data layout: planar RGB plus four full-resolution f32 planes (guide, mask,
// and a ping-pong pair for the estimate; the guide is the first estimate).
// Kernels:
//   rl_prep      guide = max(sum max(c,0)/3, 1e-6), mask = 1 - smoothstep(peak),
//                then blur(mask) and blur(guide) refine the mask, streamed
//                down column strips;
//   rl_stream    one whole RL iteration streamed down column strips:
//                blur(estimate) -> ratio = guide / max(b, 1e-6) -> blur(ratio)
//                -> estimate = clamp(estimate * b, guide/2, 2 guide)
//                so an iteration reads the estimate and guide once and writes
//                the estimate once (12 bytes per pixel of compulsory traffic);
//   rl_step      the same iteration with constant row lags for images of at
//                least 256 x 64 (fewer instructions per row, see below);
//   rl_apply     the bounded common RGB gain;
//   vignette_scan / vignette_plane  the exact incremental radius scan and the
//                vignetting multiplier plane the optics gather reads.
// Every blur keeps the reference's tap order (horizontal pass, then vertical,
// each tap added in kernel order from 0; border columns start from -0.0 as
// Iterator::sum does) and its half-sample mirror at the image edges. Field
// values outside the image are filled from their mirror position, so every
// stencil read equals the reference's mirrored read bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "rd_internal.cuh"
#include "tma.cuh"

namespace rd {
namespace {

constexpr float FLOOR = 1.0e-6f;
constexpr int MAX_TAPS = 9;  // radius <= 4 for sigma <= 1.2 (CAPTURE_RADIUS_RANGE)
// The Gaussian taps travel with each launch (by value), so concurrent develops
// with different radii never share them.
struct Taps {
  float w[MAX_TAPS];
  // -0.0f, the addend of the packed products below. As a launch argument the
  // compiler cannot fold it, so a packed product is never contracted with the
  // packed sum that takes it.
  float neg_zero;
};

// Packed FP32 (two lanes per instruction): the product x * w rounded once,
// as fma(x, w, -0.0) (x * w + -0.0 is x * w for every x * w, signed zeros
// included), and the sum a + p rounded once. A tap sum built from these is
// the scalar sum of separate multiplies and adds bit for bit.
__device__ __forceinline__ float2 pmul(float2 x, float2 w, float2 z) { return __ffma2_rn(x, w, z); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }

__device__ __forceinline__ float smoothstep(float low, float high, float value) {
  float t = (value - low) / (high - low);
  t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
  return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ float rmax(float a, float b) {
  if (isnan(a)) return b;
  if (isnan(b)) return a;
  return a > b ? a : b;
}
__device__ __forceinline__ float rmin(float a, float b) {
  if (isnan(a)) return b;
  if (isnan(b)) return a;
  return a < b ? a : b;
}
// sharpening.rs:318-326: reflect about the outer pixel boundary.
__device__ __forceinline__ int mirror_half(int index, int length) {
  const int period = 2 * length;
  int f = index % period;
  if (f < 0) f += period;
  return f < length ? f : 2 * length - 1 - f;
}



// ---- one RL iteration, streamed down column strips --------------------------
// A CTA owns a strip of SW = 128 - 2R output columns and a segment of rows and
// walks the segment top to bottom in steps of BH rows:
//   * estimate rows arrive one step ahead into a 24-row ring (the guide is
//     read from L2 where it is used): on interior strips one thread loads each
//     8-row block with a TMA tensor copy (cp.async.bulk.tensor, completion on
//     an mbarrier, the block's x start rounded down to 16 bytes and the
//     remainder applied when reading); strips at the image edge, whose
//     columns are mirrored, and images whose rows are not a multiple of 16
//     bytes copy 4-byte elements with cp.async;
//   * the horizontal pass of blur #1 runs on every arriving row; the vertical
//     pass and the ratio run R rows behind, the horizontal pass of blur #2 on
//     the same rows, and the vertical pass of blur #2 with the bounded update
//     2R rows behind, each from a 16-row ring;
//   * rows above or below the image are never computed: a vertical pass reads
//     the mirrored row instead, which holds the same values (a horizontal pass
//     commutes with a row reflection, and the ratio of a mirrored position is
//     its mirror's ratio), so only the 2R columns at each strip edge are
//     recomputed.
// Runs of RUN outputs per thread come from a register window, so shared
// memory is read about once per output; every output still sums its taps in
// kernel order from 0 (or -0.0 on horizontal border columns).
template <int R>
struct StreamGeom {
  static constexpr int T = 2 * R + 1;
  static constexpr int QW = 128;         // columns [x0 - R, x0 + SW + R): one per thread
  static constexpr int SW = QW - 2 * R;  // output columns of a strip
  static constexpr int EW = QW + 2 * R;  // estimate columns [x0 - 2R, x0 + SW + 2R)
  static constexpr int BH = 8, RIN = 24, RS = 16;  // RIN >= 2 BH + 2R: rows in use plus rows in flight
  // Estimate row stride in smem: EW columns plus up to 3 of TMA alignment
  // remainder, a multiple of 16 bytes; an 8-row block is 35 x 128 bytes.
  static constexpr int EWP = 140;
  static_assert(EW + 3 <= EWP && (EWP * 4) % 16 == 0 && (BH * EWP * 4) % 128 == 0, "estimate ring layout");
  static constexpr int H1_RUNS = 15, H1_RUN = (QW + H1_RUNS - 1) / H1_RUNS;
  static constexpr int H2_RUN = 8, H2_RUNS = (SW + H2_RUN - 1) / H2_RUN;
};

template <int R>
struct __align__(128) StreamSmem {
  using G = StreamGeom<R>;
  float e[G::RIN][G::EWP];  // estimate rows (first: 128-byte aligned TMA blocks)
  float t1[G::RS][G::QW];   // horizontal pass of blur #1
  float q[G::BH][G::QW];    // ratio rows of the current step
  float t2[G::RS][G::QW];   // horizontal pass of blur #2 (first SW columns)
  unsigned long long bar[3];  // one mbarrier per 8-row block of the estimate ring
};

// Every thread's view of a kernel's tensor-copy barriers: the parity of each
// barrier's next completion, which blocks have a copy issued and not yet
// waited for, and whether a wait gave up. Each wait is bounded: after `tries`
// polls it sets `failed` and the error word instead of spinning forever.
// From then on no copy is issued, and before the block exits `drain` waits
// (bounded again) for the copies still in flight, so no copy lands in shared
// memory the block has released. All threads call issue_block / wait / drain
// at the same points, so their views agree. `withhold` (tests of the bounded
// wait) makes every block skip its first copy while still waiting for it.
constexpr unsigned RL_TMA_TIMEOUT = 32u;
struct CopyWaits {
  unsigned phases = 0, pending = 0, tries;
  bool failed = false, withhold;
  unsigned* error;
  __device__ CopyWaits(unsigned tries_, bool withhold_, unsigned* error_)
      : tries(tries_), withhold(withhold_), error(error_) {}
  // Whether block b's copy is issued now (thread 0 then issues it).
  __device__ __forceinline__ bool issue_block(int b) {
    if (failed) return false;
    if (withhold) {
      withhold = false;
      return false;
    }
    pending |= 1u << b;
    return true;
  }
  __device__ __forceinline__ bool poll(unsigned long long* bar, int b) {
    const unsigned parity = (phases >> b) & 1u;
    for (unsigned i = 0; i < tries; ++i)
      if (mbar_try_wait(bar, parity)) {
        phases ^= 1u << b;
        pending &= ~(1u << b);
        return true;
      }
    return false;
  }
  __device__ __forceinline__ void wait(unsigned long long* bar, int b) {
    if (failed) return;
    if (!poll(bar, b)) {
      failed = true;
      atomicOr(error, RL_TMA_TIMEOUT);
    }
  }
  // After a failed wait: the copies still in flight, each waited for (bounded).
  __device__ __forceinline__ void drain(unsigned long long* bars, int n) {
    if (!failed) return;
    for (int b = 0; b < n; ++b)
      if (pending & (1u << b)) poll(&bars[b], b);
  }
};

__device__ __forceinline__ void cp_async4(float* smem, const float* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

__device__ __forceinline__ int mirror_row(int y, int H) { return (unsigned)y < (unsigned)H ? y : mirror_half(y, H); }

// Horizontal run: `n` (<= RUN) outputs starting at window column `c0` of
// `row`, written to `out`; `x0img` is the image column of the first output.
template <int R, int RUN>
__device__ __forceinline__ void hrun(const float* __restrict__ row, int c0, int n, float* __restrict__ out, int x0img,
                                     int W, const float (&w)[2 * R + 1]) {
  constexpr int T = 2 * R + 1;
  if (n == RUN && x0img >= R && x0img + RUN <= W - R) {
    // Whole run of interior columns: every sum starts at +0.0.
    float win[RUN + 2 * R];
#pragma unroll
    for (int k = 0; k < RUN + 2 * R; ++k) win[k] = row[c0 - R + k];
#pragma unroll
    for (int j = 0; j < RUN; ++j) {
      float v = 0.0f;
#pragma unroll
      for (int k = 0; k < T; ++k) v += win[j + k] * w[k];
      out[j] = v;
    }
    return;
  }
  float win[RUN + 2 * R];
#pragma unroll
  for (int k = 0; k < RUN + 2 * R; ++k) win[k] = (k < n + 2 * R) ? row[c0 - R + k] : 0.0f;
#pragma unroll
  for (int j = 0; j < RUN; ++j) {
    if (j < n) {
      const int x = x0img + j;
      float v = (W <= 2 * R || x < R || x >= W - R) ? -0.0f : 0.0f;
#pragma unroll
      for (int k = 0; k < T; ++k) v += win[j + k] * w[k];
      out[j] = v;
    }
  }
}

template <int R>
__global__ void __launch_bounds__(128) rl_stream_kernel(const float* __restrict__ est_in,
                                                        const float* __restrict__ guide,
                                                        float* __restrict__ est_out, int W, int H, int strips,
                                                        int seg_h, int items, const Taps taps,
                                                        const __grid_constant__ CUtensorMap est_map, int use_tma,
                                                        unsigned* error, unsigned wait_tries, int withhold) {
  using G = StreamGeom<R>;
  constexpr int T = G::T, SW = G::SW, QW = G::QW, EW = G::EW, BH = G::BH;
  extern __shared__ __align__(128) float4 rl_smem_raw[];
  StreamSmem<R>& S = *reinterpret_cast<StreamSmem<R>*>(rl_smem_raw);
  float w[T];
#pragma unroll
  for (int k = 0; k < T; ++k) w[k] = taps.w[k];
  const int tid = threadIdx.x;
  if (use_tma) {
    if (tid == 0) {
      for (int b = 0; b < 3; ++b) mbar_init(&S.bar[b]);
      asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
  }
  CopyWaits cw(wait_tries, withhold != 0, error);
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int x0 = (item % strips) * SW, y0 = (item / strips) * seg_h;
    const int y1 = min(y0 + seg_h, H);
    const int e_end = min(y1 + 2 * R, H), q_end = min(y1 + R, H);
    int e_next = max(y0 - 2 * R, 0), q_next = max(y0 - R, 0), o_next = y0;
    const bool edge = x0 - 2 * R < 0 || x0 + SW + 2 * R > W;
    const bool tma = use_tma && !edge;
    // Row r of the segment lives in ring slot (r - ebase) % RIN, so each step's
    // 8 rows fill one contiguous block of the ring.
    const int ebase = e_next;
    // Column c of the window [x0 - 2R, x0 + SW + 2R) sits at c + rem of its row.
    const int xal = (x0 - 2 * R) & ~3;
    const int rem = tma ? (x0 - 2 * R) - xal : 0;
    // Estimate rows [r0, r1) into the input ring: with TMA one block by thread
    // 0; else this thread copies window columns tid and tid + 128 (mirrored
    // into the image).
    const int xa = x0 - 2 * R + tid, xb = xa + 128;
    const int sxa = (unsigned)xa < (unsigned)W ? xa : mirror_half(xa, W);
    const bool has_b = tid + 128 < EW;
    const int sxb = has_b ? ((unsigned)xb < (unsigned)W ? xb : mirror_half(xb, W)) : 0;
    auto issue = [&](int r0, int r1) {
      if (r0 >= r1) return;
      if (tma) {
        const int b = ((r0 - ebase) / BH) % 3;
        if (cw.issue_block(b) && tid == 0) {
          fence_proxy_async();
          mbar_expect_tx(&S.bar[b], BH * G::EWP * sizeof(float));
          tma_load_2d(S.e[b * BH], &est_map, xal, r0, &S.bar[b]);
        }
        return;
      }
      int slot = (r0 - ebase) % G::RIN;
      const float* src = est_in + (long long)r0 * W;
      for (int r = r0; r < r1; ++r) {
        float* dst = S.e[slot];
        cp_async4(dst + tid, src + sxa);
        if (has_b) cp_async4(dst + tid + 128, src + sxb);
        src += W;
        slot = slot + 1 == G::RIN ? 0 : slot + 1;
      }
    };
    issue(e_next, min(e_next + BH, e_end));
    cp_async_commit();
    while (o_next < y1) {
      const int e_hi = min(e_next + BH, e_end);
      // Rows each later stage of this step will produce (availability of their inputs).
      const int q_avail = e_hi >= H ? q_end : e_hi - R;
      const int q_hi = max(q_next, min(min(q_next + BH, q_end), q_avail));
      const int o_avail = q_hi >= H ? y1 : q_hi - R;
      const int o_hi = max(o_next, min(min(o_next + BH, y1), o_avail));
      // Guide values of those rows, loaded now so their latency overlaps the copy wait
      // and the horizontal pass.
      float gq[BH], go[BH];
      {
        const int xq = x0 - R + tid, xo = x0 + tid;
        const bool okq = (unsigned)xq < (unsigned)W, oko = tid < SW && xo < W;
        const float* pq = guide + (long long)q_next * W + xq;
        const float* po = guide + (long long)o_next * W + xo;
#pragma unroll
        for (int j = 0; j < BH; ++j) {
          gq[j] = okq && j < q_hi - q_next ? __ldg(pq + (long long)j * W) : 0.0f;
          go[j] = oko && j < o_hi - o_next ? __ldg(po + (long long)j * W) : 0.0f;
        }
      }
      issue(e_hi, min(e_hi + BH, e_end));
      cp_async_commit();
      cp_async_wait1();
      if (tma && e_hi > e_next) cw.wait(&S.bar[((e_next - ebase) / BH) % 3], ((e_next - ebase) / BH) % 3);
      __syncthreads();
      // 1. horizontal pass of blur #1 on rows [e_next, e_hi)
      const int eslot = (e_next - ebase) % G::RIN;  // first slot of this step's block
      for (int k = tid; k < (e_hi - e_next) * G::H1_RUNS; k += 128) {
        const int rr = k / G::H1_RUNS, s = k % G::H1_RUNS;
        const int r = e_next + rr;
        const int qc0 = s * G::H1_RUN;
        const int n = min(G::H1_RUN, QW - qc0);
        if (n > 0)
          hrun<R, G::H1_RUN>(S.e[eslot + rr] + rem, qc0 + R, n, S.t1[r & (G::RS - 1)] + qc0, x0 - R + qc0, W, w);
      }
      __syncthreads();
      // 2. vertical pass of blur #1 and the ratio on rows [q_next, q_hi), column tid
      {
        const int x = x0 - R + tid, n = q_hi - q_next;
        if (n > 0 && (unsigned)x < (unsigned)W) {
          float win[BH + 2 * R];
          if (n == BH && q_next - R >= 0 && q_next + BH + R <= H) {  // no mirrored rows
            const int r0 = q_next - R;
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j) win[j] = S.t1[(r0 + j) & (G::RS - 1)][tid];
          } else {
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j)
              win[j] = j < n + 2 * R ? S.t1[mirror_row(q_next - R + j, H) & (G::RS - 1)][tid] : 0.0f;
          }
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            if (j < n) {
              float b = 0.0f;
#pragma unroll
              for (int t = 0; t < T; ++t) b += win[j + t] * w[t];
              S.q[(q_next + j) & (BH - 1)][tid] = gq[j] / rmax(b, FLOOR);
            }
          }
        }
      }
      __syncthreads();
      if (edge) {
        // Ratio entries outside the image within R of it take their mirror's value.
        const int x = x0 - R + tid;
        if ((unsigned)x >= (unsigned)W && x >= -R && x < W + R) {
          const int src = mirror_half(x, W) - (x0 - R);
          for (int y = q_next; y < q_hi; ++y) S.q[y & (BH - 1)][tid] = S.q[y & (BH - 1)][src];
        }
        __syncthreads();
      }
      // 3. horizontal pass of blur #2 on rows [q_next, q_hi), output columns
      for (int k = tid; k < (q_hi - q_next) * G::H2_RUNS; k += 128) {
        const int r = q_next + k / G::H2_RUNS, s = k % G::H2_RUNS;
        const int c0 = s * G::H2_RUN;
        const int n = min(min(G::H2_RUN, SW - c0), W - (x0 + c0));
        if (n > 0) hrun<R, G::H2_RUN>(S.q[r & (BH - 1)], c0 + R, n, S.t2[r & (G::RS - 1)] + c0, x0 + c0, W, w);
      }
      __syncthreads();
      // 4. vertical pass of blur #2 and the bounded update on rows [o_next, o_hi)
      {
        const int x = x0 + tid, n = o_hi - o_next;
        if (tid < SW && x < W && n > 0) {
          float win[BH + 2 * R];
          if (n == BH && o_next - R >= 0 && o_next + BH + R <= H) {  // no mirrored rows
            const int r0 = o_next - R;
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j) win[j] = S.t2[(r0 + j) & (G::RS - 1)][tid];
          } else {
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j)
              win[j] = j < n + 2 * R ? S.t2[mirror_row(o_next - R + j, H) & (G::RS - 1)][tid] : 0.0f;
          }
          const long long o0 = (long long)o_next * W + x;
          const int es = (o_next - ebase) % G::RIN;
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            if (j < n) {
              float b = 0.0f;
#pragma unroll
              for (int t = 0; t < T; ++t) b += win[j + t] * w[t];
              const long long o = o0 + (long long)j * W;
              const float g = go[j];
              const int slot = es + j < G::RIN ? es + j : es + j - G::RIN;
              float e = S.e[slot][tid + 2 * R + rem] * b;
              const float lo = g * 0.5f, hi = g * 2.0f;
              if (e < lo) e = lo;
              if (e > hi) e = hi;
              est_out[o] = e;
            }
          }
        }
      }
      e_next = e_hi;
      q_next = q_hi;
      o_next = o_hi;
      __syncthreads();
    }
    // Drain the (empty) trailing copy group before the rings are reused.
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
  }
  if (use_tma) cw.drain(S.bar, 3);
}

template <int R>
Status launch_rl_iter(Context& ctx, const float* est, const float* guide, float* out, int W, int H, const Taps& taps,
                      const CUtensorMap* est_map, int segs) {
  using G = StreamGeom<R>;
  const size_t smem = sizeof(StreamSmem<R>);
  RD_CUDA_TRY(cudaFuncSetAttribute(rl_stream_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  RD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_stream_kernel<R>, 128, smem));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int slots = std::max(1, occ) * sms;
  const int strips = (W + G::SW - 1) / G::SW;
  const int seg_h = (H + segs - 1) / segs;
  const int nseg = (H + seg_h - 1) / seg_h;
  const int items = strips * nseg;
  const int grid = std::min(items, slots);
  CUtensorMap none{};
  RD_LAUNCH(ctx, K_RL_ITER, rl_stream_kernel<R><<<grid, 128, smem, ctx.stream>>>(
                                est, guide, out, W, H, strips, seg_h, items, taps, est_map ? *est_map : none,
                                est_map ? 1 : 0, ctx.d_error, ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES,
                                ctx.wait_withhold == RD_WAIT_RL_COPY ? 1 : 0));
  return Status{};
}

// ---- RL iteration, constant-lag streaming ------------------------------------
// The same iteration as rl_stream_kernel for images of at least 256 x 64, with
// less bookkeeping per row. Each step loads one 8-row estimate block E..E+7 and
// always advances every stage by 8 rows at fixed lags: blur #1 and the ratio
// produce rows E-R..E-R+7, blur #2 and the update rows E-2R..E-2R+7. The 2R
// rows each vertical pass needs from earlier steps (and the estimate values of
// the update rows) are carried in registers, so every shared-memory access in
// a step is a per-step base plus a compile-time offset. Rows a segment does not
// own are computed and dropped instead of being skipped.
//  * Rows outside the image are mirrored on load (half-sample symmetric, as
//    the reference samples). The first blur is row-wise, so its mirrored rows
//    equal the rows they mirror bit for bit; the ratio is not (its vertical
//    sum would run in reverse order), so the second blur's mirrored rows are
//    copied from the rows they mirror inside the register window: at the
//    image top in step R/2 of the first segment, at the bottom in the last
//    step of the last segment, whose start is aligned so that this step ends
//    exactly at the last image row. Columns outside the image are handled as
//    in rl_stream_kernel (mirrored estimate columns, copied ratio columns).
//  * With tensor maps (rows of a multiple of 16 bytes) the guide rows of a
//    step (E-2R .. E-R+7) arrive as one tensor copy beside the estimate block,
//    two steps ahead, and are read from shared memory; rows and columns
//    outside the image read the fill value 0 and only feed dropped outputs or
//    ratio columns that are overwritten by their mirrors.
//  * Horizontal passes run 9-column windows from registers over rows padded
//    so that every run of a step takes the same path (15 runs cover the 128
//    blur #1 columns, 14 the strip's output columns; the extra outputs land
//    in the padding and are never read).
//  * A sum starts from its first product instead of from zero: every value of
//    the iteration is positive (estimate >= guide / 2 > 0, ratio >= 0, taps >
//    0), and 0 + p = p for every such p, so the sums are unchanged.
// Work item idx -> (strip, segment) for the dynamically scheduled strip
// kernels: the items of the two edge strips (per-thread copies with mirrored
// columns, the slowest) are handed out first, then the interior strips', so
// that the longest items start early and the shorter ones fill in behind them.
__device__ __forceinline__ void strip_item(int idx, int strips, int segs, int& strip, int& seg) {
  const int ne = strips >= 2 ? 2 : 1;
  if (idx < ne * segs) {
    strip = (idx % ne) ? strips - 1 : 0;
    seg = idx / ne;
    return;
  }
  const int j = idx - ne * segs, ni = strips - ne;
  strip = 1 + j % ni;
  seg = j / ni;
}

// Next work item of the CTA from the context's counter, broadcast through
// shared memory; the barrier in front also ends every read of the previous
// item's shared buffers. Every CTA stops at its first fetch past the last item,
// so the launch makes exactly items + gridDim.x fetches; the one that returns
// the largest value is the launch's last and puts the counter back to 0 for
// the next launch.
__device__ __forceinline__ int next_item(unsigned* work, int items, int& s_item) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned v = atomicAdd(work, 1u);
    if (v == (unsigned)items + gridDim.x - 1u) atomicExch(work, 0u);
    s_item = (int)v;
  }
  __syncthreads();
  return s_item;
}

template <int R>
struct StepGeom {
  static constexpr int QW = 128;         // blur #1 / ratio columns [x0 - R, x0 - R + 128)
  static constexpr int SW = QW - 2 * R;  // output columns of a strip
  static constexpr int EW = QW + 2 * R;  // estimate columns [x0 - 2R, x0 - 2R + EW)
  static constexpr int BH = 8;
  static constexpr int GH = BH + R;      // guide rows of a step: E-2R .. E-R+7
  static constexpr int RUN = 9, H1_RUNS = 15, H2_RUNS = 14;
  static constexpr int PW = 144;                    // row stride of the blur and ratio rows
  static constexpr int EWP = R <= 3 ? 144 : 176;    // estimate / guide row stride = tensor-copy box width
  static constexpr int GSLOT = (GH * EWP + 31) & ~31;  // guide slot, a multiple of 128 bytes
  static_assert(RUN * H1_RUNS >= QW && RUN * H2_RUNS >= SW, "runs cover the rows");
  static_assert(3 + RUN * H1_RUNS - 1 + 2 * R < EWP, "blur #1 windows stay inside an estimate row");
  static_assert(RUN * H2_RUNS - 1 + 2 * R < PW && RUN * H1_RUNS <= PW, "blur #2 windows stay inside a ratio row");
  static_assert(EW + 3 <= EWP && (EWP * 4) % 16 == 0 && (BH * EWP * 4) % 128 == 0, "estimate ring layout");
  static_assert(H1_RUNS * BH <= 128 && H2_RUNS * BH <= 128, "one run per thread");
};

template <int R, bool TMA>
struct __align__(128) StepSmem {
  using G = StepGeom<R>;
  float e[3 * G::BH][G::EWP];       // three 8-row estimate blocks (tensor-copy targets)
  float g[TMA ? 3 : 1][G::GSLOT];   // three guide slots (tensor-copy targets)
  float t[G::BH][G::PW];            // blur #1 rows E..E+7, then blur #2 rows E-R..E-R+7
  float q[G::BH][G::PW];            // ratio rows E-R..E-R+7
  unsigned long long bar[3];
};

template <int R, int RUN>
__device__ __forceinline__ void hrun_full(const float* __restrict__ src, float* __restrict__ dst,
                                          const float (&w)[2 * R + 1], const float2 (&w2)[2 * R + 1], float2 z) {
  constexpr int T = 2 * R + 1, HALF = RUN / 2;
  float win[RUN + 2 * R];
#pragma unroll
  for (int k = 0; k < RUN + 2 * R; ++k) win[k] = src[k];
  // Outputs j and j + HALF in the two lanes of a packed sum.
#pragma unroll
  for (int j = 0; j < HALF; ++j) {
    float2 v = pmul(make_float2(win[j], win[j + HALF]), w2[0], z);
#pragma unroll
    for (int t = 1; t < T; ++t) v = padd(v, pmul(make_float2(win[j + t], win[j + HALF + t]), w2[t], z));
    dst[j] = v.x;
    dst[j + HALF] = v.y;
  }
#pragma unroll
  for (int j = 2 * HALF; j < RUN; ++j) {
    float v = win[j] * w[0];
#pragma unroll
    for (int t = 1; t < T; ++t) v += win[j + t] * w[t];
    dst[j] = v;
  }
}

// The vertical tap sums of BH consecutive rows from a window of BH + 2R rows:
// out[j] = sum_t win[j + t] w[t], rows j and j + BH/2 in the two lanes.
template <int R, int BH>
__device__ __forceinline__ void vsum_packed(const float (&win)[BH + 2 * R], const float2 (&w2)[2 * R + 1], float2 z,
                                            float (&out)[BH]) {
  constexpr int T = 2 * R + 1, HALF = BH / 2;
  static_assert(BH % 2 == 0, "rows pair up");
#pragma unroll
  for (int j = 0; j < HALF; ++j) {
    float2 v = pmul(make_float2(win[j], win[j + HALF]), w2[0], z);
#pragma unroll
    for (int t = 1; t < T; ++t) v = padd(v, pmul(make_float2(win[j + t], win[j + HALF + t]), w2[t], z));
    out[j] = v.x;
    out[j + HALF] = v.y;
  }
}

// Row segments: 8-row units spread evenly; every boundary lies at
// H + 4R (mod 8) so that the last segment's final step ends at row H - 1.
// Segment s covers [seg_row(s), seg_row(s + 1)).
struct StepSegments {
  int q, rem, r8, segs;
};
__host__ __device__ __forceinline__ int seg_row(const StepSegments& sg, int s, int H) {
  if (s <= 0) return 0;
  if (s >= sg.segs) return H;
  return sg.r8 + 8 * (s * sg.q + min(s, sg.rem));
}
StepSegments step_segments(int H, int R, int want) {
  const int m = (4 * R) % 8;
  const int n8 = (H - m) / 8;
  const int segs = std::max(2, std::min(want, n8));
  return {n8 / segs, n8 % segs, (H - m) % 8, segs};
}

// One image of an iteration launch: its estimate (in and out) and guide
// planes, its size, strips, row segments and work items, and the tensor maps
// of its estimate and guide planes (null without tensor copies).
struct StepImage {
  const float* est_in;
  const float* guide;
  float* est_out;
  int W, H, strips, items;
  StepSegments sg;
  const CUtensorMap* est_map;
  const CUtensorMap* guide_map;
};

// A thread's part of an iteration launch: the taps (scalar and packed), the
// -0.0 addend of the packed products, and the run it computes in each
// horizontal pass (row, first column).
template <int R>
struct StepThread {
  using G = StepGeom<R>;
  float w[2 * R + 1];
  float2 w2[2 * R + 1];
  float2 z2;
  bool h1_on, h2_on;
  int h1_row, h1_col, h2_row, h2_col;
  __device__ __forceinline__ explicit StepThread(const Taps& taps) {
#pragma unroll
    for (int k = 0; k < 2 * R + 1; ++k) {
      w[k] = taps.w[k];
      w2[k] = make_float2(taps.w[k], taps.w[k]);
    }
    z2 = make_float2(taps.neg_zero, taps.neg_zero);
    const int tid = threadIdx.x;
    h1_on = tid < G::H1_RUNS * G::BH;
    h2_on = tid < G::H2_RUNS * G::BH;
    h1_row = tid / G::H1_RUNS;
    h1_col = (tid % G::H1_RUNS) * G::RUN;
    h2_row = tid / G::H2_RUNS;
    h2_col = (tid % G::H2_RUNS) * G::RUN;
  }
};

// One work item (a strip and a row segment) of one image's iteration. Every
// thread of the CTA calls it.
template <int R, bool TMA>
__device__ __forceinline__ void step_item(StepSmem<R, TMA>& S, const StepImage& im, int item, const StepThread<R>& th,
                                          CopyWaits& cw) {
  using G = StepGeom<R>;
  constexpr int SW = G::SW, BH = G::BH, N2 = 2 * R;
  const int tid = threadIdx.x;
  const float(&w)[2 * R + 1] = th.w;
  const float2(&w2)[2 * R + 1] = th.w2;
  const float2 z2 = th.z2;
  const bool h1_on = th.h1_on, h2_on = th.h2_on;
  const int h1_row = th.h1_row, h1_col = th.h1_col, h2_row = th.h2_row, h2_col = th.h2_col;
  const float* __restrict__ est_in = im.est_in;
  const float* __restrict__ guide = im.guide;
  float* __restrict__ est_out = im.est_out;
  const int W = im.W, H = im.H, strips = im.strips;
  const StepSegments sg = im.sg;
  int strip, seg;
  strip_item(item, strips, sg.segs, strip, seg);
  const int x0 = strip * SW;
  const int y0 = seg_row(sg, seg, H), y1 = seg_row(sg, seg + 1, H);
  const int E0 = y0 - N2;
  const int nsteps = (y1 - y0 + 2 * N2 - BH + 7) / BH + 1;
  const bool inside = x0 - N2 >= 0 && x0 - N2 + G::EW <= W;
  const bool tma_strip = TMA && inside;
  const bool edge_q = x0 < R || x0 + SW + R > W;
  const int xal = (x0 - N2) & ~3;  // rounds down, also below 0
  const int rem = TMA ? (x0 - N2) - xal : 0;
  // Guide boxes stay inside the image columns (a box crossing the image edge
  // takes the tensor unit much longer); reads shift by xal - gx. Columns the
  // shifted box misses lie outside the image and only feed ratio columns
  // that are overwritten by their mirrors and outputs that are not stored.
  const int gx = TMA ? min(max(xal, 0), W - G::EWP) : 0;
  const int xa = x0 - N2 + tid, xb = xa + 128;
  const int sxa = (unsigned)xa < (unsigned)W ? xa : mirror_half(xa, W);
  const bool has_b = tid + 128 < G::EW;
  const int sxb = has_b ? ((unsigned)xb < (unsigned)W ? xb : mirror_half(xb, W)) : 0;
  // Step k's estimate block (rows [E0 + 8k, +8)) goes to ring block k % 3, by
  // one tensor copy when the rows and the window lie inside the image, else
  // by per-thread copies with rows and columns mirrored into the image; its
  // guide rows go to guide slot k % 3 by one tensor copy.
  auto e_by_tma = [&](int k) {
    const int r0 = E0 + BH * k;
    return tma_strip && r0 >= 0 && r0 + BH <= H;
  };
  auto issue = [&](int k) {
    if (k >= nsteps) return;
    const int r0 = E0 + BH * k, b = k % 3;
    const bool et = e_by_tma(k);
    if (TMA && cw.issue_block(b) && tid == 0) {
      fence_proxy_async();
      mbar_expect_tx(&S.bar[b], (et ? BH * G::EWP * sizeof(float) : 0) + G::GH * G::EWP * sizeof(float));
      if (et) tma_load_2d(S.e[b * BH], im.est_map, xal, r0, &S.bar[b]);
      tma_load_2d(S.g[b], im.guide_map, gx, r0 - N2, &S.bar[b]);
    }
    if (et) return;
#pragma unroll
    for (int j = 0; j < BH; ++j) {
      const float* src = est_in + (long long)mirror_row(r0 + j, H) * W;
      float* dst = S.e[b * BH + j] + rem;
      cp_async4(dst + tid, src + sxa);
      if (has_b) cp_async4(dst + tid + 128, src + sxb);
    }
  };
  issue(0);
  cp_async_commit();
  issue(1);
  cp_async_commit();
  // Carried rows: blur #1 rows [E-2R, E), blur #2 rows [E-3R, E-R), estimate
  // rows [E-2R, E) of this thread's output column.
  float c1[N2], c2[N2], ed[N2];
#pragma unroll
  for (int i = 0; i < N2; ++i) c1[i] = c2[i] = ed[i] = 1.0f;
  const int xq = x0 - R + tid, xo = x0 + tid;
  const bool okq = (unsigned)xq < (unsigned)W;
  const bool oko = tid < SW && xo < W;
  for (int k = 0; k < nsteps; ++k) {
    const int E = E0 + BH * k;
    // Without tensor maps: guide values of the ratio rows and of the update rows.
    float gq[BH], go[BH];
    if (!TMA) {
#pragma unroll
      for (int j = 0; j < BH; ++j) {
        const int rq = E - R + j, ro = E - N2 + j;
        gq[j] = okq && (unsigned)rq < (unsigned)H ? __ldg(guide + (long long)rq * W + xq) : 0.0f;
        go[j] = oko && ro >= y0 && ro < y1 ? __ldg(guide + (long long)ro * W + xo) : 0.0f;
      }
    }
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    if (TMA) cw.wait(&S.bar[k % 3], k % 3);
    __syncthreads();
    // Block k + 2 reuses the slots of block k - 1, whose estimate rows were
    // last read before the second barrier of step k - 1 and whose guide rows
    // before the barrier above.
    issue(k + 2);
    cp_async_commit();
    const float* eb = S.e[(k % 3) * BH] + rem;
    const float* gb = S.g[TMA ? k % 3 : 0] + rem + (xal - gx);
    // 1. blur #1, horizontal: rows E..E+7, columns x0-R .. x0-R+134
    if (h1_on) hrun_full<R, G::RUN>(eb + h1_row * G::EWP + h1_col, S.t[h1_row] + h1_col, w, w2, z2);
    float ec[BH];
#pragma unroll
    for (int j = 0; j < BH; ++j) ec[j] = eb[j * G::EWP + tid + N2];
    __syncthreads();
    // 2. blur #1, vertical, and the ratio: rows E-R .. E-R+7, column x0-R+tid
    {
      float win[BH + N2];
#pragma unroll
      for (int i = 0; i < N2; ++i) win[i] = c1[i];
#pragma unroll
      for (int j = 0; j < BH; ++j) win[N2 + j] = S.t[j][tid];
      float bs[BH];
      vsum_packed<R, BH>(win, w2, z2, bs);
#pragma unroll
      for (int j = 0; j < BH; ++j) {
        const float b = bs[j];
        const float g = TMA ? gb[(R + j) * G::EWP + R + tid] : gq[j];
        // fmaxf(b, FLOOR) equals rmax(b, FLOOR): the floor is not NaN, and
        // a NaN b gives the floor either way.
        S.q[j][tid] = g / fmaxf(b, FLOOR);
      }
#pragma unroll
      for (int i = 0; i < N2; ++i) c1[i] = win[BH + i];
    }
    __syncthreads();
    if (edge_q) {
      // Ratio columns outside the image within R of it take their mirror's value.
      if ((unsigned)xq >= (unsigned)W && xq >= -R && xq < W + R) {
        const int src = mirror_half(xq, W) - (x0 - R);
#pragma unroll
        for (int j = 0; j < BH; ++j) S.q[j][tid] = S.q[j][src];
      }
      __syncthreads();
    }
    // 3. blur #2, horizontal: rows E-R .. E-R+7, output columns (over blur #1,
    //    whose rows every thread has read before the barrier above)
    if (h2_on) hrun_full<R, G::RUN>(S.q[h2_row] + h2_col, S.t[h2_row] + h2_col, w, w2, z2);
    __syncthreads();
    // 4. blur #2, vertical, and the bounded update: rows E-2R .. E-2R+7
    {
      float win[BH + N2];
#pragma unroll
      for (int i = 0; i < N2; ++i) win[i] = c2[i];
#pragma unroll
      for (int j = 0; j < BH; ++j) win[N2 + j] = S.t[j][tid];
#pragma unroll
      for (int i = 0; i < N2; ++i) c2[i] = win[BH + i];
      if (y0 == 0 && k == R / 2) {
        // Window position p holds row E - 3R + p; rows -1 .. -R take rows 0 .. R-1.
        constexpr int P0 = 5 * R - 8 * (R / 2);
#pragma unroll
        for (int i = 1; i <= R; ++i) win[P0 - i] = win[P0 + i - 1];
      }
      if (y1 == H && k == nsteps - 1) {
        // This step ends at row H - 1: rows H .. H+R-1 take rows H-1 .. H-R.
#pragma unroll
        for (int i = 0; i < R; ++i) win[BH + R + i] = win[BH + R - 1 - i];
      }
      if (oko && E - N2 + BH > y0) {
        float* po = est_out + (long long)(E - N2) * W + xo;
        float eo[BH];
        float bs[BH];
        vsum_packed<R, BH>(win, w2, z2, bs);
#pragma unroll
        for (int j = 0; j < BH; ++j) {
          const float b = bs[j];
          const float e = (j < N2 ? ed[j] : ec[j - N2]) * b;
          const float g = TMA ? gb[j * G::EWP + N2 + tid] : go[j];
          // The develop rejects non-finite capture input, so e is never NaN
          // here, and min / max give the reference's compare-and-replace.
          eo[j] = fminf(fmaxf(e, g * 0.5f), g * 2.0f);
        }
        if (E - N2 >= y0 && E - N2 + BH <= y1) {
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            *po = eo[j];
            po += W;
          }
        } else {
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            const int o = E - N2 + j;
            if (o >= y0 && o < y1) *po = eo[j];
            po += W;
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < N2; ++i) ed[i] = ec[BH - N2 + i];
  }
}

template <int R, bool TMA>
__global__ void __launch_bounds__(128, 5) rl_step_kernel(const float* __restrict__ est_in,
                                                          const float* __restrict__ guide,
                                                          float* __restrict__ est_out, int W, int H, int strips,
                                                          const StepSegments sg, int items, const Taps taps,
                                                          const __grid_constant__ CUtensorMap est_map,
                                                          const __grid_constant__ CUtensorMap guide_map,
                                                          unsigned* work, unsigned* error, unsigned wait_tries,
                                                          int withhold) {
  extern __shared__ __align__(128) float4 rl_step_raw[];
  StepSmem<R, TMA>& S = *reinterpret_cast<StepSmem<R, TMA>*>(rl_step_raw);
  const StepThread<R> th(taps);
  if (TMA && threadIdx.x == 0) {
    for (int b = 0; b < 3; ++b) mbar_init(&S.bar[b]);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  CopyWaits cw(wait_tries, TMA && withhold != 0, error);
  const StepImage im{est_in, guide, est_out, W, H, strips, items, sg, &est_map, &guide_map};
  __shared__ int s_item;
  for (int item = next_item(work, items, s_item); item < items; item = next_item(work, items, s_item))
    step_item<R, TMA>(S, im, item, th, cw);
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  if (TMA) cw.drain(S.bar, 3);
}

// One iteration of several images in one launch (the batched develop's flat
// pass): work items of every image from one counter, image by image in the
// table's order; first_item[i] is image i's first item (first_item[n] = items).
// The images share the taps; each brings its own planes, size and tensor maps
// (kept in global memory).
template <int R, bool TMA>
__global__ void __launch_bounds__(128, 5) rl_step_images_kernel(const StepImage* __restrict__ images,
                                                                 const int* __restrict__ first_item, int nimages,
                                                                 int items, const Taps taps, unsigned* work,
                                                                 unsigned* error, unsigned wait_tries, int withhold) {
  extern __shared__ __align__(128) float4 rl_step_raw[];
  StepSmem<R, TMA>& S = *reinterpret_cast<StepSmem<R, TMA>*>(rl_step_raw);
  const StepThread<R> th(taps);
  if (TMA && threadIdx.x == 0) {
    for (int b = 0; b < 3; ++b) mbar_init(&S.bar[b]);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  CopyWaits cw(wait_tries, TMA && withhold != 0, error);
  __shared__ int s_item, s_local;
  __shared__ StepImage s_im;
  for (;;) {
    // The barrier in front ends every read of the previous item's buffers.
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned v = atomicAdd(work, 1u);
      if (v == (unsigned)items + gridDim.x - 1u) atomicExch(work, 0u);
      s_item = (int)v;
      if ((int)v < items) {
        int lo = 0, hi = nimages;
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (first_item[mid] <= (int)v) lo = mid;
          else hi = mid;
        }
        s_im = images[lo];
        s_local = (int)v - first_item[lo];
      }
    }
    __syncthreads();
    if (s_item >= items) break;
    const StepImage im = s_im;
    step_item<R, TMA>(S, im, s_local, th, cw);
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  if (TMA) cw.drain(S.bar, 3);
}

// The constant-lag kernel serves images of at least 256 x 64; smaller ones
// keep the per-step bookkeeping of rl_stream_kernel.
bool rl_uses_step_kernel(int W, int H, int R) { return W >= 256 && H >= 64 && R >= 1 && R <= 4; }

template <int R, bool TMA>
int step_occupancy() {
  int occ = 0;
  const size_t smem = sizeof(StepSmem<R, TMA>);
  cudaFuncSetAttribute(rl_step_kernel<R, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_step_kernel<R, TMA>, 128, smem);
  cudaGetLastError();
  return std::max(1, occ);
}

template <int R, bool TMA>
Status launch_rl_step_t(Context& ctx, const float* est, const float* guide, float* out, int W, int H,
                        const Taps& taps, const CUtensorMap* est_map, const CUtensorMap* guide_map, int segs) {
  using G = StepGeom<R>;
  const size_t smem = sizeof(StepSmem<R, TMA>);
  RD_CUDA_TRY(cudaFuncSetAttribute(rl_step_kernel<R, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  RD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_step_kernel<R, TMA>, 128, smem));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int slots = std::max(1, occ) * sms;
  const int strips = (W + G::SW - 1) / G::SW;
  const StepSegments sg = step_segments(H, R, segs);
  const int items = strips * sg.segs;
  const int grid = std::min(items, slots);
  CUtensorMap none{};
  RD_LAUNCH(ctx, K_RL_ITER, rl_step_kernel<R, TMA><<<grid, 128, smem, ctx.stream>>>(
                                est, guide, out, W, H, strips, sg, items, taps, est_map ? *est_map : none,
                                guide_map ? *guide_map : none, ctx.d_work, ctx.d_error,
                                ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES,
                                ctx.wait_withhold == RD_WAIT_RL_COPY ? 1 : 0));
  return Status{};
}

template <int R>
Status launch_rl_step(Context& ctx, const float* est, const float* guide, float* out, int W, int H, const Taps& taps,
                      const CUtensorMap* est_map, const CUtensorMap* guide_map, int segs) {
  if (est_map && guide_map)
    return launch_rl_step_t<R, true>(ctx, est, guide, out, W, H, taps, est_map, guide_map, segs);
  return launch_rl_step_t<R, false>(ctx, est, guide, out, W, H, taps, nullptr, nullptr, segs);
}

// ---- guide and mask, streamed down column strips ---------------------------
// sharpening.rs:180-230 before the iterations: guide = max(sum max(c,0)/3,
// 1e-6) and mask = 1 - smoothstep(0.85, 0.98, max c/ceil_c) for every pixel,
// then mask = min(mask, blur(mask)^4) * smoothstep(thr, 3 thr, |g - blur(g)|)
// * smoothstep(0.001, 0.01, g). One CTA walks a strip of SW = 128 - 2R output
// columns down a row segment: each arriving row is turned into guide and mask
// values for the strip plus R mirrored columns on each side, blurred
// horizontally, and R rows later blurred vertically and combined. The guide
// doubles as the first estimate of the iterations.
template <int R>
struct PrepSmem {
  static constexpr int QW = 128, SW = QW - 2 * R, RS = 16;
  float g[RS][QW];   // guide
  float m[RS][QW];   // initial mask
  float tg[RS][QW];  // horizontal blur of the guide (first SW columns)
  float tm[RS][QW];  // horizontal blur of the mask
};

template <int R>
__global__ void __launch_bounds__(128) rl_prep_kernel(const float* __restrict__ rgb, long long plane, float c0,
                                                      float c1, float c2, float noise, float* __restrict__ guide,
                                                      float* __restrict__ mask, int W, int H, int strips, int seg_h,
                                                      int items, unsigned* error, const Taps taps) {
  using S_ = PrepSmem<R>;
  constexpr int T = 2 * R + 1, SW = S_::SW, RS = S_::RS, BH = 8;
  extern __shared__ float4 rl_smem_raw[];
  S_& S = *reinterpret_cast<S_*>(rl_smem_raw);
  float w[T];
#pragma unroll
  for (int k = 0; k < T; ++k) w[k] = taps.w[k];
  const int tid = threadIdx.x;
  bool bad = false;
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int x0 = (item % strips) * SW, y0 = (item / strips) * seg_h;
    const int y1 = min(y0 + seg_h, H);
    const int e_end = min(y1 + R, H);
    int e_next = max(y0 - R, 0), o_next = y0;
    const int xq = x0 - R + tid;  // this thread's column of the guide / mask rows
    const int sx = (unsigned)xq < (unsigned)W ? xq : mirror_half(xq, W);
    while (o_next < y1) {
      const int e_hi = min(e_next + BH, e_end);
      const int o_avail = e_hi >= H ? y1 : e_hi - R;
      const int o_hi = max(o_next, min(min(o_next + BH, y1), o_avail));
      // 1. guide and initial mask of rows [e_next, e_hi) (rl_init, sharpening.rs:187-203)
      for (int y = e_next; y < e_hi; ++y) {
        const long long i = (long long)y * W + sx;
        const float r = rgb[i], g = rgb[plane + i], b = rgb[2 * plane + i];
        if (!isfinite(r) || !isfinite(g) || !isfinite(b)) bad = true;
        float s = -0.0f;
        s += rmax(r, 0.0f) / 3.0f;
        s += rmax(g, 0.0f) / 3.0f;
        s += rmax(b, 0.0f) / 3.0f;
        float peak = 0.0f;
        peak = rmax(peak, r / c0);
        peak = rmax(peak, g / c1);
        peak = rmax(peak, b / c2);
        S.g[y & (RS - 1)][tid] = rmax(s, FLOOR);
        S.m[y & (RS - 1)][tid] = 1.0f - smoothstep(0.85f, 0.98f, peak);
      }
      __syncthreads();
      // 2. horizontal blurs of rows [e_next, e_hi), output columns, runs of 8
      {
        constexpr int RUN = 8, RUNS = (SW + RUN - 1) / RUN;
        for (int k = tid; k < (e_hi - e_next) * RUNS * 2; k += 128) {
          const int field = k & 1, rest = k >> 1;
          const int y = e_next + rest / RUNS, c0 = (rest % RUNS) * RUN;
          const int n = min(min(RUN, SW - c0), W - (x0 + c0));
          if (n <= 0) continue;
          const float* src = field ? S.m[y & (RS - 1)] : S.g[y & (RS - 1)];
          float* dst = field ? S.tm[y & (RS - 1)] : S.tg[y & (RS - 1)];
          hrun<R, RUN>(src, c0 + R, n, dst + c0, x0 + c0, W, w);
        }
      }
      __syncthreads();
      // 3. vertical blurs and the mask refinement of rows [o_next, o_hi) (sharpening.rs:205-230)
      {
        const int x = x0 + tid, n = o_hi - o_next;
        if (tid < SW && x < W && n > 0) {
          float wg[BH + 2 * R], wm[BH + 2 * R];
          if (n == BH && o_next - R >= 0 && o_next + BH + R <= H) {  // no mirrored rows
            const int r0 = o_next - R;
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j) {
              wg[j] = S.tg[(r0 + j) & (RS - 1)][tid];
              wm[j] = S.tm[(r0 + j) & (RS - 1)][tid];
            }
          } else {
#pragma unroll
            for (int j = 0; j < BH + 2 * R; ++j) {
              const int row = j < n + 2 * R ? mirror_row(o_next - R + j, H) & (RS - 1) : 0;
              wg[j] = S.tg[row][tid];
              wm[j] = S.tm[row][tid];
            }
          }
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            if (j < n) {
              float bm = 0.0f, bg = 0.0f;
#pragma unroll
              for (int t = 0; t < T; ++t) {
                bm += wm[j + t] * w[t];
                bg += wg[j + t] * w[t];
              }
              const int y = o_next + j;
              const float m0 = S.m[y & (RS - 1)][tid + R];
              const float g = S.g[y & (RS - 1)][tid + R];
              const float b2 = bm * bm;
              float m = rmin(m0, b2 * b2);
              const float threshold = 0.0005f + noise * 0.008f + bg * noise * 0.02f;
              const float detail = fabsf(g - bg);
              m *= smoothstep(threshold, threshold * 3.0f, detail) * smoothstep(0.001f, 0.01f, g);
              const long long o = (long long)y * W + x;
              mask[o] = m;
              guide[o] = g;
            }
          }
        }
      }
      e_next = e_hi;
      o_next = o_hi;
      __syncthreads();
    }
  }
  if (bad) atomicOr(error, 2u);
}

// Constant-lag form of rl_prep_kernel for images of at least 256 x 64. Step k
// turns RGB rows E..E+7 (E = E0 + 8k) into guide and initial-mask rows, blurs
// them horizontally and emits the refined rows E-R..E-R+7. Every thread owns
// one column of the 128-column window [x0 - R, x0 - R + 128) in every phase,
// so the guide and mask values the refinement needs R rows later, and the 2R
// blurred rows the vertical pass needs from the previous step, stay in its
// registers. Rows and columns outside the image are loaded from their mirror
// positions; the guide and mask are pointwise and the horizontal blur is
// row-wise, so every mirrored value equals the one it mirrors bit for bit and
// no segment needs special treatment. RGB blocks arrive by tensor copy (one
// per plane, two steps ahead) when the window lies inside the image, else by
// per-thread copies. Sums start from their first product: guide > 0 and
// mask >= 0 (never -0.0), so 0 + p = p.
template <int R>
struct PrepGeom {
  static constexpr int T = 2 * R + 1, QW = 128, SW = QW - 2 * R, BH = 8;
  static constexpr int RUN = 9, H_RUNS = 14;  // 14 runs of 9 cover the output columns
  static constexpr int PW = 144;              // guide / mask row stride
  static constexpr int CWP = 132;             // RGB row stride = tensor-copy box width
  static_assert(RUN * H_RUNS >= SW && RUN * H_RUNS - 1 + 2 * R < PW && R + RUN * H_RUNS <= PW, "runs fit the rows");
  static_assert(QW + 3 <= CWP && (CWP * 4) % 16 == 0 && (BH * CWP * 4) % 128 == 0, "RGB block layout");
};

template <int R>
struct __align__(128) PrepStepSmem {
  using G = PrepGeom<R>;
  float rgb[2][3 * G::BH][G::CWP];  // two slots of three 8-row plane blocks
  float g[G::BH][G::PW], m[G::BH][G::PW];
  float tg[G::BH][G::PW], tm[G::BH][G::PW];
  unsigned long long bar[2];
};

template <int R, bool TMA>
__global__ void __launch_bounds__(128, 4) rl_prep_step_kernel(const float* __restrict__ rgb, long long plane, float c0,
                                                               float c1, float c2, float noise,
                                                               float* __restrict__ guide, float* __restrict__ mask,
                                                               int W, int H, int strips, int segs, int items,
                                                               const Taps taps, const __grid_constant__ CUtensorMap rgb_map,
                                                               unsigned* work, unsigned* error, unsigned wait_tries,
                                                               int withhold) {
  using G = PrepGeom<R>;
  constexpr int T = G::T, SW = G::SW, BH = G::BH, N2 = 2 * R;
  extern __shared__ __align__(128) float4 rl_prep_raw[];
  PrepStepSmem<R>& S = *reinterpret_cast<PrepStepSmem<R>*>(rl_prep_raw);
  float w[T];
  float2 w2[T];
#pragma unroll
  for (int k = 0; k < T; ++k) {
    w[k] = taps.w[k];
    w2[k] = make_float2(taps.w[k], taps.w[k]);
  }
  const float2 z2 = make_float2(taps.neg_zero, taps.neg_zero);
  const int tid = threadIdx.x;
  if (TMA && tid == 0) {
    for (int b = 0; b < 2; ++b) mbar_init(&S.bar[b]);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  CopyWaits cw(wait_tries, TMA && withhold != 0, error);
  bool bad = false;
  const bool h_on = tid < G::H_RUNS * BH;
  const int h_row = tid / G::H_RUNS, h_col = (tid % G::H_RUNS) * G::RUN;
  __shared__ int s_item;
  for (int item = next_item(work, items, s_item); item < items; item = next_item(work, items, s_item)) {
    int strip, seg;
    strip_item(item, strips, segs, strip, seg);
    const int x0 = strip * SW;
    const int y0 = (int)((long long)seg * H / segs), y1 = (int)((long long)(seg + 1) * H / segs);
    const int E0 = y0 - R;
    const int nsteps = (y1 - y0 + N2 - BH + 7) / BH + 1;
    const bool inside = x0 - R >= 0 && x0 - R + G::QW <= W;
    const bool tma_strip = TMA && inside;
    const int xal = (x0 - R) & ~3;
    const int rem = tma_strip ? (x0 - R) - xal : 0;
    const int xc = x0 - R + tid;
    const int sxc = (unsigned)xc < (unsigned)W ? xc : mirror_half(xc, W);
    auto by_tma = [&](int k) {
      const int r0 = E0 + BH * k;
      return tma_strip && r0 >= 0 && r0 + BH <= H;
    };
    // Block k: RGB rows [E0 + 8k, +8) of the window into slot k & 1.
    auto issue = [&](int k) {
      if (k >= nsteps) return;
      const int r0 = E0 + BH * k, b = k & 1;
      if (by_tma(k)) {
        if (cw.issue_block(b) && tid == 0) {
          fence_proxy_async();
          mbar_expect_tx(&S.bar[b], 3 * BH * G::CWP * sizeof(float));
#pragma unroll
          for (int c = 0; c < 3; ++c) tma_load_2d(S.rgb[b][c * BH], &rgb_map, xal, c * H + r0, &S.bar[b]);
        }
        return;
      }
#pragma unroll
      for (int j = 0; j < BH; ++j) {
        const float* src = rgb + (long long)mirror_row(r0 + j, H) * W + sxc;
#pragma unroll
        for (int c = 0; c < 3; ++c) cp_async4(&S.rgb[b][c * BH + j][rem + tid], src + c * plane);
      }
    };
    auto arrive = [&](int k) {  // this thread's view of block k is complete
      if (by_tma(k)) cw.wait(&S.bar[k & 1], k & 1);
    };
    issue(0);
    cp_async_commit();
    issue(1);
    cp_async_commit();
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    arrive(0);
    __syncthreads();
    // Carried rows: blurred guide / mask rows [E-2R, E); guide and initial
    // mask rows [E-R, E) of this thread's column.
    float ctg[N2], ctm[N2], cg[R], cm[R];
#pragma unroll
    for (int i = 0; i < N2; ++i) ctg[i] = ctm[i] = 1.0f;
#pragma unroll
    for (int i = 0; i < R; ++i) cg[i] = cm[i] = 1.0f;
    const int xo = xc;  // output column of this thread, when it is one
    const bool store_col = tid >= R && tid < R + SW && xo < W;
    for (int k = 0; k < nsteps; ++k) {
      const int E = E0 + BH * k;
      // 1. guide and initial mask of rows E..E+7 (sharpening.rs:187-203)
      float gcur[BH], mcur[BH];
      {
        const float* pr = &S.rgb[k & 1][0][rem + tid];
#pragma unroll
        for (int j = 0; j < BH; ++j) {
          const float r = pr[j * G::CWP], g = pr[(BH + j) * G::CWP], b = pr[(2 * BH + j) * G::CWP];
          if (!isfinite(r) || !isfinite(g) || !isfinite(b)) bad = true;
          // fmaxf returns the non-NaN operand, as rmax does; the two can only
          // differ in the sign of a zero, which neither the guide (floored
          // at 1e-6) nor the smoothstep of the peak can see.
          float s = -0.0f;
          s += fmaxf(r, 0.0f) / 3.0f;
          s += fmaxf(g, 0.0f) / 3.0f;
          s += fmaxf(b, 0.0f) / 3.0f;
          float peak = 0.0f;
          peak = fmaxf(peak, r / c0);
          peak = fmaxf(peak, g / c1);
          peak = fmaxf(peak, b / c2);
          gcur[j] = fmaxf(s, FLOOR);
          mcur[j] = 1.0f - smoothstep(0.85f, 0.98f, peak);
          S.g[j][tid] = gcur[j];
          S.m[j][tid] = mcur[j];
        }
      }
      __syncthreads();
      // Slot k & 1 has been read: refill it with block k + 2.
      issue(k + 2);
      cp_async_commit();
      // 2. horizontal blurs of rows E..E+7, output columns of the window
      if (h_on) {
        hrun_full<R, G::RUN>(S.g[h_row] + h_col, S.tg[h_row] + R + h_col, w, w2, z2);
        hrun_full<R, G::RUN>(S.m[h_row] + h_col, S.tm[h_row] + R + h_col, w, w2, z2);
      }
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      if (k + 1 < nsteps) arrive(k + 1);
      __syncthreads();
      // 3. vertical blurs and the mask refinement of rows E-R..E-R+7 (sharpening.rs:205-230)
      {
        float wg[BH + N2], wm[BH + N2];
#pragma unroll
        for (int i = 0; i < N2; ++i) {
          wg[i] = ctg[i];
          wm[i] = ctm[i];
        }
#pragma unroll
        for (int j = 0; j < BH; ++j) {
          wg[N2 + j] = S.tg[j][tid];
          wm[N2 + j] = S.tm[j][tid];
        }
        if (store_col && E - R + BH > y0) {
          float* pm = mask + (long long)(E - R) * W + xo;
          float* pg = guide + (long long)(E - R) * W + xo;
#pragma unroll
          for (int j = 0; j < BH; ++j) {
            const int y = E - R + j;
            float bm = wm[j] * w[0], bg = wg[j] * w[0];
#pragma unroll
            for (int t = 1; t < T; ++t) {
              bm += wm[j + t] * w[t];
              bg += wg[j + t] * w[t];
            }
            const float m0 = j < R ? cm[j] : mcur[j - R];
            const float g = j < R ? cg[j] : gcur[j - R];
            const float b2 = bm * bm;
            float m = fminf(m0, b2 * b2);  // m0 >= +0, never NaN: as rmin
            const float threshold = 0.0005f + noise * 0.008f + bg * noise * 0.02f;
            const float detail = fabsf(g - bg);
            m *= smoothstep(threshold, threshold * 3.0f, detail) * smoothstep(0.001f, 0.01f, g);
            if (y >= y0 && y < y1) {
              pm[(long long)j * W] = m;
              pg[(long long)j * W] = g;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < N2; ++i) {
          ctg[i] = wg[BH + i];
          ctm[i] = wm[BH + i];
        }
#pragma unroll
        for (int i = 0; i < R; ++i) {
          cg[i] = gcur[BH - R + i];
          cm[i] = mcur[BH - R + i];
        }
      }
    }
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  if (TMA) cw.drain(S.bar, 2);
  if (bad) atomicOr(error, 2u);
}

bool rl_prep_uses_step_kernel(int W, int H, int R) { return W >= 256 && H >= 64 && R >= 1 && R <= 4; }

template <int R, bool TMA>
Status launch_rl_prep_step(Context& ctx, const Taps& taps, const float* rgb, long long plane, const float ceil[3],
                           float noise, float* guide, float* mask, int W, int H, const CUtensorMap* rgb_map) {
  using G = PrepGeom<R>;
  const size_t smem = sizeof(PrepStepSmem<R>);
  RD_CUDA_TRY(cudaFuncSetAttribute(rl_prep_step_kernel<R, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  RD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_prep_step_kernel<R, TMA>, 128, smem));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int slots = std::max(1, occ) * sms;
  const int strips = (W + G::SW - 1) / G::SW;
  // Row segments per strip: tuned across calls per image shape (the
  // segmentation changes only the schedule), from about three work items per
  // resident CTA, each at least 32 rows.
  const int per_round = std::max(1, slots / strips);
  const int fallback = std::max(1, std::min(3 * per_round, H / 32));
  std::vector<int> cands;
  for (int m : {2, 3, 4, 5, 6})
    if (H / (m * per_round) >= 32) cands.push_back(m * per_round);
  const ShapeKey key{TUNE_RL_PREP, W, H, R};
  const ShapePick pick = shape_begin(ctx, key, fallback, cands);
  const int segs = pick.value;
  const int items = strips * segs;
  const int grid = std::min(items, slots);
  CUtensorMap none{};
  RD_LAUNCH(ctx, K_RL_MASK, rl_prep_step_kernel<R, TMA><<<grid, 128, smem, ctx.stream>>>(
                                rgb, plane, ceil[0], ceil[1], ceil[2], noise, guide, mask, W, H, strips, segs, items,
                                taps, rgb_map ? *rgb_map : none, ctx.d_work, ctx.d_error,
                                ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES,
                                ctx.wait_withhold == RD_WAIT_RL_COPY ? 1 : 0));
  shape_end(ctx, key, pick);
  return Status{};
}

template <int R>
Status launch_rl_prep(Context& ctx, const Taps& taps, const float* rgb, long long plane, const float ceil[3], float noise, float* guide,
                      float* mask, int W, int H) {
  using S_ = PrepSmem<R>;
  const size_t smem = sizeof(S_);
  RD_CUDA_TRY(cudaFuncSetAttribute(rl_prep_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  RD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_prep_kernel<R>, 128, smem));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int slots = std::max(1, occ) * sms;
  const int strips = (W + S_::SW - 1) / S_::SW;
  const int per_round = std::max(1, slots / strips);
  int segs = std::min(per_round, std::max(1, H / 32));
  while ((H + segs - 1) / segs > 512) segs += per_round;
  const int seg_h = (H + segs - 1) / segs;
  const int nseg = (H + seg_h - 1) / seg_h;
  const int items = strips * nseg;
  const int grid = std::min(items, slots);
  RD_LAUNCH(ctx, K_RL_MASK, rl_prep_kernel<R><<<grid, 128, smem, ctx.stream>>>(
                                rgb, plane, ceil[0], ceil[1], ceil[2], noise, guide, mask, W, H, strips, seg_h, items,
                                ctx.d_error, taps));
  return Status{};
}

Status rl_prep(Context& ctx, int r, const Taps& taps, const float* rgb, long long plane, const float ceil[3], float noise, float* guide,
               float* mask, int W, int H, const CUtensorMap* rgb_map) {
  if (rl_prep_uses_step_kernel(W, H, r)) {
    switch (r) {
#define RD_PREP_CASE(RR)                                                                                   \
  case RR:                                                                                                 \
    return rgb_map ? launch_rl_prep_step<RR, true>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H, rgb_map) \
                   : launch_rl_prep_step<RR, false>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H, nullptr);
      RD_PREP_CASE(1)
      RD_PREP_CASE(2)
      RD_PREP_CASE(3)
      RD_PREP_CASE(4)
#undef RD_PREP_CASE
      default: break;
    }
  }
  switch (r) {
    case 1: return launch_rl_prep<1>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H);
    case 2: return launch_rl_prep<2>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H);
    case 3: return launch_rl_prep<3>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H);
    case 4: return launch_rl_prep<4>(ctx, taps, rgb, plane, ceil, noise, guide, mask, W, H);
    default: return Status{RD_INVALID_INPUT, "capture radius outside 1..4"};
  }
}

// ---- launch-shape tuning of the RL iteration -----------------------------------
// How many row segments each strip is cut into is a pure scheduling choice:
// every output of an iteration is computed the same way whatever the
// segmentation. The first develop of an image shape (width, height, radius)
// therefore runs iterations 1..K-1 under the candidate segment counts in turn
// (iteration 0, which may pay for loading the kernel, under the heuristic's
// count and untimed), each timed with events; after the develop's
// synchronisation the candidate with the fastest iteration is kept for that
// shape in a process-wide table, and later develops of the shape use it.
struct RlShape {
  int W, H, R;
  bool operator<(const RlShape& o) const {
    return W != o.W ? W < o.W : (H != o.H ? H < o.H : R < o.R);
  }
};
struct RlChoice {
  int segs = 0, default_segs = 0;
  float best_ms = 0.0f, default_ms = 0.0f;
};
std::mutex g_rl_tune_mutex;
std::map<RlShape, RlChoice> g_rl_tuned;

// The occupancy heuristic: one round of (strip, segment) items over all
// resident CTAs, each segment at least 32 rows (vertical halos) and at most
// 512 (more rounds).
int rl_default_segments(int W, int H, int R, int sms) {
  int occ = 0;
  size_t smem = 0;
  if (rl_uses_step_kernel(W, H, R)) R += 4;  // cases 5..8: the constant-lag kernel (tensor-copy form)
  switch (R) {
    case 5: occ = step_occupancy<1, true>(); break;
    case 6: occ = step_occupancy<2, true>(); break;
    case 7: occ = step_occupancy<3, true>(); break;
    case 8: occ = step_occupancy<4, true>(); break;
    case 1: smem = sizeof(StreamSmem<1>); cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_stream_kernel<1>, 128, smem); break;
    case 2: smem = sizeof(StreamSmem<2>); cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_stream_kernel<2>, 128, smem); break;
    case 3: smem = sizeof(StreamSmem<3>); cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_stream_kernel<3>, 128, smem); break;
    default: smem = sizeof(StreamSmem<4>); cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_stream_kernel<4>, 128, smem); break;
  }
  cudaGetLastError();
  if (R > 4) R -= 4;
  const int slots = std::max(1, occ) * std::max(1, sms);
  const int strips = (W + (128 - 2 * R) - 1) / (128 - 2 * R);
  const int per_round = std::max(1, slots / strips);
  int segs = std::min(per_round, std::max(1, H / 32));
  while ((H + segs - 1) / segs > 512) segs += per_round;
  return segs;
}

// Candidate segment counts around the heuristic's (each segment >= 32 rows):
// fewer, equal and several times more work items than resident CTAs.
std::vector<int> rl_candidates(int H, int d) {
  std::vector<int> c{d};
  for (int v : {2 * d, 3 * d, 4 * d, 6 * d, std::max(1, d / 2)})
    if (H / v >= 32 && std::find(c.begin(), c.end(), v) == c.end()) c.push_back(v);
  return c;
}

}  // namespace

void resolve_rl_tuning(Context& ctx) {
  std::map<int, float> best;  // candidate -> fastest timed iteration
  for (auto& r : ctx.tune_runs) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, r.second.first, r.second.second) == cudaSuccess) {
      auto it = best.find(r.first);
      if (it == best.end() || ms < it->second) best[r.first] = ms;
    }
    ctx.event_pool.push_back(r.second.first);
    ctx.event_pool.push_back(r.second.second);
  }
  ctx.tune_runs.clear();
  cudaGetLastError();
  const RlShape key{ctx.tune_shape[0], ctx.tune_shape[1], ctx.tune_shape[2]};
  const int d = rl_default_segments(key.W, key.H, key.R, ctx.sm_count > 0 ? ctx.sm_count : 152);
  RlChoice c;
  c.default_segs = d;
  for (auto& kv : best) {
    if (kv.first == d) c.default_ms = kv.second;
    if (c.segs == 0 || kv.second < c.best_ms) {
      c.segs = kv.first;
      c.best_ms = kv.second;
    }
  }
  if (c.segs == 0) return;
  std::lock_guard<std::mutex> lk(g_rl_tune_mutex);
  g_rl_tuned[key] = c;
}

namespace {

// Estimate-ring box width (floats) of the kernel that runs an iteration.
int rl_box_width(int W, int H, int R) {
  if (!rl_uses_step_kernel(W, H, R)) return StreamGeom<1>::EWP;
  return R <= 3 ? StepGeom<1>::EWP : StepGeom<4>::EWP;
}

// Tensor map of one f32 plane for the estimate ring's box_w x 8 boxes; false
// when TMA cannot address it (row stride not a multiple of 16 bytes, or no
// encoder).
bool make_plane_map(CUtensorMap* map, const float* plane, int W, int H, int box_w, int box_h = 8) {
  return make_tensor_map_2d(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, plane, W, H, (uint64_t)W * sizeof(float), box_w,
                            box_h);
}

Status rl_iteration(Context& ctx, int r, const Taps& taps, const float* est, const float* guide, float* out, int W,
                    int H, const CUtensorMap* est_map, const CUtensorMap* guide_map, int segs) {
  if (rl_uses_step_kernel(W, H, r)) {
    switch (r) {
      case 1: return launch_rl_step<1>(ctx, est, guide, out, W, H, taps, est_map, guide_map, segs);
      case 2: return launch_rl_step<2>(ctx, est, guide, out, W, H, taps, est_map, guide_map, segs);
      case 3: return launch_rl_step<3>(ctx, est, guide, out, W, H, taps, est_map, guide_map, segs);
      case 4: return launch_rl_step<4>(ctx, est, guide, out, W, H, taps, est_map, guide_map, segs);
      default: break;
    }
  }
  switch (r) {
    case 1: return launch_rl_iter<1>(ctx, est, guide, out, W, H, taps, est_map, segs);
    case 2: return launch_rl_iter<2>(ctx, est, guide, out, W, H, taps, est_map, segs);
    case 3: return launch_rl_iter<3>(ctx, est, guide, out, W, H, taps, est_map, segs);
    case 4: return launch_rl_iter<4>(ctx, est, guide, out, W, H, taps, est_map, segs);
    default: return Status{RD_INVALID_INPUT, "capture radius outside 1..4"};
  }
}


// Vignetting radius scan (correction.rs:239-262): r2 advances along each row
// by the row-independent increment d[k] = 2 ns x_k + ns^2 with f32 rounding at
// every step, so the value at a column depends on the whole row prefix. One
// thread per row walks the row and records r2 at every SEG-th column; the
// apply kernel resumes each SEG-column segment from its checkpoint exactly.
constexpr int SEG = 32;
constexpr int VIGNETTE_MAX_WIDTH = 24576;  // the staged increments fit in shared memory

// One thread per row. The increments are the same for every row, so a block
// stages them in shared memory and every read is a broadcast; what remains on
// a row is its chain of dependent additions. Checkpoints are stored segment
// major (checkpoints[s * H + y]) so that a warp's stores are contiguous.
__global__ void __launch_bounds__(64) vignette_scan_kernel(const float* __restrict__ incr,
                                                           const float* __restrict__ r2_start, int W, int H,
                                                           float* __restrict__ checkpoints, int segs) {
  extern __shared__ __align__(16) float s_incr[];
  // Staged 16 bytes at a time, four loads in flight per thread (incr is the
  // start of a device allocation, so 16-byte aligned).
  const int n4 = W >> 2;
#pragma unroll 4
  for (int i = threadIdx.x; i < n4; i += blockDim.x)
    reinterpret_cast<float4*>(s_incr)[i] = __ldg(reinterpret_cast<const float4*>(incr) + i);
  for (int i = 4 * n4 + threadIdx.x; i < W; i += blockDim.x) s_incr[i] = incr[i];
  __syncthreads();
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= H) return;
  float r2 = r2_start[y];
  const int full = W / SEG;
  for (int s = 0; s < full; ++s) {
    checkpoints[(long long)s * H + y] = r2;
    const float4* v = reinterpret_cast<const float4*>(s_incr + s * SEG);
#pragma unroll
    for (int q = 0; q < SEG / 4; ++q) {
      const float4 t = v[q];
      r2 += t.x;
      r2 += t.y;
      r2 += t.z;
      r2 += t.w;
    }
  }
  // A last partial segment needs only its start.
  if (full < segs) checkpoints[(long long)full * H + y] = r2;
}

struct ApplyParams {
  float* rgb;
  long long plane;
  int W, H;
  float amount;
  const float* mask;
  const float* est;
  const float* guide;
};

// sharpening.rs:110-118: the bounded common gain 1 + amount * mask * (est /
// guide - 1) on all three channels, skipped when it is 1 or would make a
// channel non-finite. One thread per pixel, coalesced planes.
__global__ void __launch_bounds__(256) rl_apply_kernel(const ApplyParams p) {
  const long long o = (long long)blockIdx.x * 256 + threadIdx.x;
  if (o >= p.plane) return;
  float v0 = p.rgb[o], v1 = p.rgb[p.plane + o], v2 = p.rgb[2 * p.plane + o];
  const float gain = 1.0f + p.amount * p.mask[o] * (p.est[o] / p.guide[o] - 1.0f);
  if (gain != 1.0f && isfinite(v0 * gain) && isfinite(v1 * gain) && isfinite(v2 * gain)) {
    p.rgb[o] = v0 * gain;
    p.rgb[p.plane + o] = v1 * gain;
    p.rgb[2 * p.plane + o] = v2 * gain;
  }
}

}  // namespace

// Host contract: Gaussian kernel weights (crates/detail/src/gaussian.rs:9-17).
int gaussian_kernel(float sigma, float* weights, int max_taps) {
  const int radius = (int)std::ceil(3.0f * sigma);
  const int taps = 2 * radius + 1;
  if (taps > max_taps) return -1;
  float sum = -0.0f;
  for (int i = 0; i < taps; ++i) {
    const float t = (float)(i - radius) / sigma;
    weights[i] = std::exp(-0.5f * (t * t));
    sum += weights[i];
  }
  for (int i = 0; i < taps; ++i) weights[i] /= sum;
  return taps;
}

namespace {
struct VignetteTables {
  float* incr = nullptr;
  float* r2_start = nullptr;
  float* checkpoints = nullptr;
  int segs = 0;
  size_t bytes = 0;
};

// Host side of the vignetting scan: the column increments and the row starts
// follow correction.rs:226-243 operation by operation in f32.
Status prepare_vignetting(Context& ctx, const rd_optics_desc& o, int W, int H, VignetteTables& t) {
  if (W > VIGNETTE_MAX_WIDTH) return Status{RD_INVALID_DIMENSIONS, "vignetting supports widths up to 24576"};
  const float ns = (float)o.norm_scale;
  const float step = 2.0f * ns, step_sq = ns * ns;
  const float start_x = (float)(-o.center_x), start_y = (float)(-o.center_y);
  std::vector<float> incr(W), r2s(H);
  float x = start_x;
  for (int k = 0; k < W; ++k) {
    incr[k] = step * x + step_sq;
    x += ns;
  }
  for (int row = 0; row < H; ++row) {
    const float y = start_y + ns * (float)row;
    r2s[row] = start_x * start_x + y * y;
  }
  t.segs = (W + SEG - 1) / SEG;
  t.bytes = sizeof(float) * ((size_t)W + H + (size_t)H * t.segs);
  void* p = nullptr;
  RD_TRY(device_alloc(ctx, t.bytes, &p));
  t.incr = static_cast<float*>(p);
  t.r2_start = t.incr + W;
  t.checkpoints = t.r2_start + H;
  RD_TRY(upload(ctx, t.incr, incr.data(), sizeof(float) * W));
  RD_TRY(upload(ctx, t.r2_start, r2s.data(), sizeof(float) * H));
  const int smem = (int)(sizeof(float) * W);
  // The limit is set to the largest size the kernel takes, never to this
  // launch's: contexts on other threads launch it with other widths.
  RD_CUDA_TRY(cudaFuncSetAttribute(vignette_scan_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(float) * VIGNETTE_MAX_WIDTH)));
  RD_LAUNCH(ctx, K_VIGNETTE, vignette_scan_kernel<<<(H + 63) / 64, 64, smem, ctx.stream>>>(t.incr, t.r2_start, W, H,
                                                                                         t.checkpoints, t.segs));
  RD_CUDA_TRY(cudaGetLastError());
  return Status{};
}
}  // namespace

// Vignetting multiplier plane: mult[y][x] = 1 / (1 + k1 r2 + k2 r2^2 + k3 r2^3)
// with r2 from the exact incremental scan. The optics gather and the area
// reduction multiply each source sample by it on load, so the resident source
// itself is never modified. One warp per row: in a pass, lane l resumes the
// scan of segment 32g + l from its checkpoint and computes the segment's 32
// multipliers from increments staged in shared memory with one pad word per
// 32 (lane stride 33 words, no bank conflicts); the warp then writes the
// pass's 1024 values with coalesced stores through a transposition buffer.
constexpr int VP_WARPS = 16;
size_t vignette_plane_smem(int W) { return sizeof(float) * ((size_t)W + W / 32 + 1 + VP_WARPS * 32 * 33); }

__global__ void __launch_bounds__(VP_WARPS * 32) vignette_plane_kernel(const float* __restrict__ incr,
                                                                      const float* __restrict__ checkpoints, int W,
                                                                      int H, int segs, float k1, float k2, float k3,
                                                                      float* __restrict__ mult, unsigned* error) {
  extern __shared__ float vsm[];
  float* s_incr = vsm;
  float* tbuf = vsm + W + W / 32 + 1;
  const int n4 = W >> 2;  // four consecutive increments never straddle a pad word
#pragma unroll 4
  for (int i = threadIdx.x; i < n4; i += blockDim.x) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(incr) + i);
    float* d = s_incr + 4 * i + (i >> 3);
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
    d[3] = v.w;
  }
  for (int i = 4 * n4 + threadIdx.x; i < W; i += blockDim.x) s_incr[i + (i >> 5)] = incr[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int y = blockIdx.x * VP_WARPS + warp;
  if (y >= H) return;
  float* t = tbuf + warp * 32 * 33;
  bool bad = false;
  for (int g = 0; g * 32 < segs; ++g) {
    const int s = g * 32 + lane;
    if (s < segs) {
      float r2 = checkpoints[(long long)s * H + y];
      const int xs = s * SEG;
      const float* inc = s_incr + s * (SEG + 1);
#pragma unroll 8
      for (int j = 0; j < SEG; ++j) {
        float m = 1.0f;
        if (xs + j < W) {
          const float r4 = r2 * r2, r6 = r4 * r2;
          const float gain = 1.0f + k1 * r2 + k2 * r4 + k3 * r6;
          if (!isfinite(gain) || gain == 0.0f) bad = true;
          m = 1.0f / gain;
          r2 += inc[j];
        }
        t[lane * 33 + j] = m;
      }
    }
    __syncwarp();
    for (int j = 0; j < 32; ++j) {
      const int sj = g * 32 + j;
      const int x = sj * SEG + lane;
      if (sj < segs && x < W) mult[(long long)y * W + x] = t[j * 33 + lane];
    }
    __syncwarp();
  }
  if (bad) atomicOr(error, 4u);
}

Status run_vignette_plane(Context& ctx, const rd_optics_desc& optics, float* mult) {
  const int W = (int)optics.width, H = (int)optics.height;
  VignetteTables vt;
  RD_TRY(prepare_vignetting(ctx, optics, W, H, vt));
  const size_t smem = vignette_plane_smem(W);
  // The largest size the kernel takes (contexts on other threads launch it
  // with other widths), not this launch's.
  cudaError_t launch = cudaFuncSetAttribute(vignette_plane_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)vignette_plane_smem(VIGNETTE_MAX_WIDTH));
  if (launch == cudaSuccess) {
    RD_LAUNCH(ctx, K_VIGNETTE, vignette_plane_kernel<<<(H + VP_WARPS - 1) / VP_WARPS, VP_WARPS * 32, smem, ctx.stream>>>(
                                   vt.incr, vt.checkpoints, W, H, vt.segs, optics.vignetting_k[0],
                                   optics.vignetting_k[1], optics.vignetting_k[2], mult, ctx.d_error));
    launch = cudaGetLastError();
  }
  device_free(ctx, vt.incr, vt.bytes);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

// Capture sharpening (and, when given, vignetting) on planar RGB in place.
Status run_capture(Context& ctx, float* rgb, int W, int H, const rd_detail_desc& detail) {
  const bool capture = detail.enabled && detail.amount > 0.0f;
  if (!capture) return Status{};
  const long long plane = (long long)W * H;
  float* planes = nullptr;
  size_t plane_bytes = 0;
  int r = 0;
  Taps taps{};
  if (capture) {
    if (!(detail.radius >= 0.3f && detail.radius <= 1.2f) || !(detail.amount <= 1.0f) ||
        !(detail.noise_protection >= 0.0f && detail.noise_protection <= 1.0f))
      return Status{RD_INVALID_INPUT, "capture sharpening settings are outside their ranges"};
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(detail.ceilings[c]) || !(detail.ceilings[c] > 0.0f))
        return Status{RD_INVALID_INPUT, "capture ceilings must be finite and positive"};
    const int ntaps = gaussian_kernel(detail.radius, taps.w, MAX_TAPS);
    taps.neg_zero = -0.0f;
    if (ntaps < 0) return Status{RD_INVALID_INPUT, "capture radius too large"};
    r = ntaps / 2;
    plane_bytes = sizeof(float) * (size_t)plane * 4;
    void* p = nullptr;
    RD_TRY(device_alloc(ctx, plane_bytes, &p));
    planes = static_cast<float*>(p);
  }
  float* guide = planes;
  float* mask = planes ? planes + plane : nullptr;
  float* est_buf[2] = {planes ? planes + 2 * plane : nullptr, planes ? planes + 3 * plane : nullptr};
  // The estimate starts as the guide (sharpening.rs:203), so the first
  // iteration reads the guide plane itself.
  const float* est = guide;
  Status st;
  if (capture) {
    // The RGB planes as one (W, 3H) tensor for the prep kernel's tensor copies.
    CUtensorMap rgb_map;
    const bool rgb_tma =
        rl_prep_uses_step_kernel(W, H, r) && make_plane_map(&rgb_map, rgb, W, 3 * H, PrepGeom<1>::CWP, 8);
    st = rl_prep(ctx, r, taps, rgb, plane, detail.ceilings, detail.noise_protection, guide, mask, W, H,
                 rgb_tma ? &rgb_map : nullptr);
    // Tensor maps of the three planes an iteration can read (guide, then the
    // ping-pong estimates), for the TMA-fed estimate ring.
    CUtensorMap maps[3];
    const int box_w = rl_box_width(W, H, r);
    const bool tma = make_plane_map(&maps[0], guide, W, H, box_w) && make_plane_map(&maps[1], est_buf[0], W, H, box_w) &&
                     make_plane_map(&maps[2], est_buf[1], W, H, box_w);
    const CUtensorMap* in_map = tma ? &maps[0] : nullptr;
    // The constant-lag kernel also reads each step's guide rows (8 + R) by tensor copy.
    CUtensorMap guide_map;
    const bool guide_tma = tma && rl_uses_step_kernel(W, H, r) && make_plane_map(&guide_map, guide, W, H, box_w, 8 + r);
    // Launch shape: the tuned segment count of this image shape, or a tuning
    // run over the candidates (not while the stream is being captured).
    const RlShape shape{W, H, r};
    int segs = 0;
    {
      std::lock_guard<std::mutex> lk(g_rl_tune_mutex);
      auto it = g_rl_tuned.find(shape);
      if (it != g_rl_tuned.end()) segs = it->second.segs;
    }
    std::vector<int> cands;
    if (segs == 0) {
      segs = rl_default_segments(W, H, r, ctx.sm_count > 0 ? ctx.sm_count : 152);
      if (!ctx.capturing && ctx.tune_runs.empty() && detail.iterations >= 2) cands = rl_candidates(H, segs);
    }
    if (!cands.empty()) {
      ctx.tune_shape[0] = W;
      ctx.tune_shape[1] = H;
      ctx.tune_shape[2] = r;
    }
    for (int it = 0; it < detail.iterations && st.ok(); ++it) {
      const bool timed = !cands.empty() && it > 0;
      const int s_it = timed ? cands[(it - 1) % cands.size()] : segs;
      cudaEvent_t a = nullptr, b = nullptr;
      if (timed) {
        for (cudaEvent_t* e : {&a, &b}) {
          if (!ctx.event_pool.empty()) {
            *e = ctx.event_pool.back();
            ctx.event_pool.pop_back();
          } else {
            cudaEventCreate(e);
          }
        }
        cudaEventRecord(a, ctx.stream);
      }
      st = rl_iteration(ctx, r, taps, est, guide, est_buf[it & 1], W, H, in_map, guide_tma ? &guide_map : nullptr,
                        s_it);
      if (timed) {
        cudaEventRecord(b, ctx.stream);
        ctx.tune_runs.push_back({s_it, {a, b}});
      }
      est = est_buf[it & 1];
      in_map = tma ? &maps[1 + (it & 1)] : nullptr;
    }
    if (st.ok() && cudaGetLastError() != cudaSuccess) st = Status{RD_SYNCHRONIZATION, "capture kernels failed to launch"};
  }
  if (st.ok()) {
    ApplyParams ap{};
    ap.rgb = rgb;
    ap.plane = plane;
    ap.W = W;
    ap.H = H;
    ap.amount = detail.amount;
    ap.mask = mask;
    ap.est = est;
    ap.guide = guide;
    RD_LAUNCH(ctx, K_RL_APPLY, rl_apply_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, ctx.stream>>>(ap));
    if (cudaGetLastError() != cudaSuccess) st = Status{RD_SYNCHRONIZATION, "capture apply failed to launch"};
  }
  if (planes) device_free(ctx, planes, plane_bytes);
  return st;
}


// ---- capture sharpening of several images at once ---------------------------
namespace {

template <int R, bool TMA>
Status launch_rl_step_images(Context& ctx, const StepImage* d_images, const int* d_first, int nimages, int items,
                             const Taps& taps) {
  const size_t smem = sizeof(StepSmem<R, TMA>);
  RD_CUDA_TRY(
      cudaFuncSetAttribute(rl_step_images_kernel<R, TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  RD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rl_step_images_kernel<R, TMA>, 128, smem));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const int grid = std::min(items, std::max(1, occ) * sms);
  RD_LAUNCH(ctx, K_RL_ITER,
            rl_step_images_kernel<R, TMA><<<grid, 128, smem, ctx.stream>>>(
                d_images, d_first, nimages, items, taps, ctx.d_work, ctx.d_error,
                ctx.wait_limit ? ctx.wait_limit : RL_DEFAULT_WAIT_TRIES, ctx.wait_withhold == RD_WAIT_RL_COPY ? 1 : 0));
  return Status{};
}

Status rl_step_images(Context& ctx, int r, bool tma, const StepImage* d_images, const int* d_first, int nimages,
                      int items, const Taps& taps) {
  switch (r) {
#define RD_STEP_IMAGES_CASE(RR)                                                                       \
  case RR:                                                                                            \
    return tma ? launch_rl_step_images<RR, true>(ctx, d_images, d_first, nimages, items, taps)        \
               : launch_rl_step_images<RR, false>(ctx, d_images, d_first, nimages, items, taps);
    RD_STEP_IMAGES_CASE(1)
    RD_STEP_IMAGES_CASE(2)
    RD_STEP_IMAGES_CASE(3)
    RD_STEP_IMAGES_CASE(4)
#undef RD_STEP_IMAGES_CASE
    default:
      return Status{RD_INVALID_INPUT, "capture radius outside 1..4"};
  }
}

// Per image of run_capture_images: its RL planes, taps and step geometry, and
// the device copies of its four tensor maps (guide, the two estimates, and
// the guide for the step kernel's 8 + R row boxes).
struct CapturePlanes {
  int job = -1, r = 0, iterations = 0;
  Taps taps{};
  float* planes = nullptr;
  size_t bytes = 0;
  bool tma = false;
  CUtensorMap maps[4];
  StepSegments sg{};
  int strips = 0, items = 0;
};

}  // namespace

Status run_capture_images(Context& ctx, CaptureJob* jobs, int n) {
  std::vector<CapturePlanes> prepared;
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  // 1. Settings, planes and the guide / mask pass, image by image; images the
  //    step kernel does not serve take the per-image path whole.
  for (int j = 0; j < n; ++j) {
    CaptureJob& job = jobs[j];
    const rd_detail_desc& d = job.detail;
    if (!job.st.ok() || !(d.enabled && d.amount > 0.0f)) continue;
    const int W = job.W, H = job.H;
    CapturePlanes cp;
    cp.job = j;
    const int ntaps = gaussian_kernel(d.radius, cp.taps.w, MAX_TAPS);
    cp.taps.neg_zero = -0.0f;
    cp.r = ntaps / 2;
    if (ntaps < 0 || !rl_uses_step_kernel(W, H, cp.r) || d.iterations < 1) {
      job.st = run_capture(ctx, job.rgb, W, H, d);
      continue;
    }
    if (!(d.radius >= 0.3f && d.radius <= 1.2f) || !(d.amount <= 1.0f) ||
        !(d.noise_protection >= 0.0f && d.noise_protection <= 1.0f)) {
      job.st = Status{RD_INVALID_INPUT, "capture sharpening settings are outside their ranges"};
      continue;
    }
    bool ceilings_ok = true;
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(d.ceilings[c]) || !(d.ceilings[c] > 0.0f)) ceilings_ok = false;
    if (!ceilings_ok) {
      job.st = Status{RD_INVALID_INPUT, "capture ceilings must be finite and positive"};
      continue;
    }
    const long long plane = (long long)W * H;
    cp.bytes = sizeof(float) * (size_t)plane * 4;
    void* p = nullptr;
    job.st = device_alloc(ctx, cp.bytes, &p);
    if (!job.st.ok()) continue;
    cp.planes = static_cast<float*>(p);
    float* guide = cp.planes;
    float* mask = cp.planes + plane;
    CUtensorMap rgb_map;
    const bool rgb_tma =
        rl_prep_uses_step_kernel(W, H, cp.r) && make_plane_map(&rgb_map, job.rgb, W, 3 * H, PrepGeom<1>::CWP, 8);
    job.st = rl_prep(ctx, cp.r, cp.taps, job.rgb, plane, d.ceilings, d.noise_protection, guide, mask, W, H,
                     rgb_tma ? &rgb_map : nullptr);
    if (!job.st.ok()) {
      device_free(ctx, cp.planes, cp.bytes);
      continue;
    }
    const int box_w = rl_box_width(W, H, cp.r);
    cp.tma = make_plane_map(&cp.maps[0], guide, W, H, box_w) &&
             make_plane_map(&cp.maps[1], cp.planes + 2 * plane, W, H, box_w) &&
             make_plane_map(&cp.maps[2], cp.planes + 3 * plane, W, H, box_w) &&
             make_plane_map(&cp.maps[3], guide, W, H, box_w, 8 + cp.r);
    int segs = 0;
    {
      std::lock_guard<std::mutex> lk(g_rl_tune_mutex);
      auto it = g_rl_tuned.find(RlShape{W, H, cp.r});
      if (it != g_rl_tuned.end()) segs = it->second.segs;
    }
    if (segs == 0) segs = rl_default_segments(W, H, cp.r, sms);
    cp.sg = step_segments(H, cp.r, segs);
    cp.iterations = d.iterations;
    prepared.push_back(cp);
  }
  // 2. The iterations: images with the same taps and tensor-copy ability
  //    share one launch per iteration; an image leaves after its last one.
  Status st;
  std::vector<bool> done(prepared.size(), false);
  for (size_t g = 0; g < prepared.size() && st.ok(); ++g) {
    if (done[g]) continue;
    std::vector<size_t> group;
    for (size_t k = g; k < prepared.size(); ++k)
      if (!done[k] && prepared[k].r == prepared[g].r && prepared[k].tma == prepared[g].tma &&
          std::memcmp(prepared[k].taps.w, prepared[g].taps.w, sizeof(float) * (2 * prepared[g].r + 1)) == 0) {
        group.push_back(k);
        done[k] = true;
      }
    const int r = prepared[g].r;
    const bool tma = prepared[g].tma;
    int max_k = 0;
    for (size_t k : group) max_k = std::max(max_k, prepared[k].iterations);
    // Device tables: the group's tensor maps, then per iteration the image
    // table and its first-item offsets.
    const size_t map_bytes = sizeof(CUtensorMap) * 4 * group.size();
    const size_t img_bytes = (sizeof(StepImage) * group.size() + 63) & ~(size_t)63;
    const size_t first_bytes = (sizeof(int) * (group.size() + 1) + 63) & ~(size_t)63;
    const size_t table_bytes = map_bytes + (size_t)max_k * (img_bytes + first_bytes);
    void* t = nullptr;
    st = device_alloc(ctx, table_bytes + 64, &t);
    if (!st.ok()) break;
    unsigned char* tb =
        reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(t) + 63) & ~static_cast<uintptr_t>(63));
    std::vector<unsigned char> host(table_bytes, 0);
    const CUtensorMap* d_maps = reinterpret_cast<const CUtensorMap*>(tb);
    for (size_t i = 0; i < group.size(); ++i)
      std::memcpy(host.data() + sizeof(CUtensorMap) * 4 * i, prepared[group[i]].maps, sizeof(CUtensorMap) * 4);
    std::vector<int> counts((size_t)max_k, 0), totals((size_t)max_k, 0);
    for (int it = 0; it < max_k; ++it) {
      StepImage* images = reinterpret_cast<StepImage*>(host.data() + map_bytes + (size_t)it * (img_bytes + first_bytes));
      int* first = reinterpret_cast<int*>(host.data() + map_bytes + (size_t)it * (img_bytes + first_bytes) + img_bytes);
      int m = 0, items = 0;
      for (size_t i = 0; i < group.size(); ++i) {
        const CapturePlanes& cp = prepared[group[i]];
        if (cp.iterations <= it) continue;
        const CaptureJob& job = jobs[cp.job];
        const long long plane = (long long)job.W * job.H;
        float* est[2] = {cp.planes + 2 * plane, cp.planes + 3 * plane};
        StepImage& im = images[m];
        im.est_in = it == 0 ? cp.planes : est[(it - 1) & 1];
        im.guide = cp.planes;
        im.est_out = est[it & 1];
        im.W = job.W;
        im.H = job.H;
        im.strips = (job.W + StepGeom<1>::QW - 2 * r - 1) / (StepGeom<1>::QW - 2 * r);
        im.sg = cp.sg;
        im.items = im.strips * cp.sg.segs;
        // The first iteration reads the guide, later ones the estimate the one before wrote.
        im.est_map = tma ? d_maps + 4 * i + (it == 0 ? 0 : 1 + ((it - 1) & 1)) : nullptr;
        im.guide_map = tma ? d_maps + 4 * i + 3 : nullptr;
        first[m] = items;
        items += im.items;
        ++m;
      }
      first[m] = items;
      counts[(size_t)it] = m;
      totals[(size_t)it] = items;
    }
    st = upload(ctx, tb, host.data(), table_bytes);
    for (int it = 0; it < max_k && st.ok(); ++it) {
      const unsigned char* base = tb + map_bytes + (size_t)it * (img_bytes + first_bytes);
      st = rl_step_images(ctx, r, tma, reinterpret_cast<const StepImage*>(base),
                          reinterpret_cast<const int*>(base + img_bytes), counts[(size_t)it], totals[(size_t)it],
                          prepared[g].taps);
    }
    if (st.ok() && cudaGetLastError() != cudaSuccess) st = Status{RD_SYNCHRONIZATION, "capture kernels failed to launch"};
    device_free(ctx, t, table_bytes + 64);
  }
  // 3. The gain, image by image (sharpening.rs:110-118), then the planes go.
  for (CapturePlanes& cp : prepared) {
    CaptureJob& job = jobs[cp.job];
    const long long plane = (long long)job.W * job.H;
    if (st.ok()) {
      ApplyParams ap{};
      ap.rgb = job.rgb;
      ap.plane = plane;
      ap.W = job.W;
      ap.H = job.H;
      ap.amount = job.detail.amount;
      ap.mask = cp.planes + plane;
      ap.est = cp.planes + (2 + ((cp.iterations - 1) & 1)) * plane;
      ap.guide = cp.planes;
      RD_LAUNCH(ctx, K_RL_APPLY, rl_apply_kernel<<<(unsigned)((plane + 255) / 256), 256, 0, ctx.stream>>>(ap));
      if (cudaGetLastError() != cudaSuccess) st = Status{RD_SYNCHRONIZATION, "capture apply failed to launch"};
    }
    if (!st.ok()) job.st = st;
    device_free(ctx, cp.planes, cp.bytes);
  }
  return st;
}

}  // namespace rd

extern "C" rd_status rd_rl_launch_shape(uint32_t width, uint32_t height, float radius, int32_t* segments,
                                        int32_t* default_segments, float* best_ms, float* default_ms) {
  float w[rd::MAX_TAPS];
  const int taps = rd::gaussian_kernel(radius, w, rd::MAX_TAPS);
  if (taps < 0 || !segments) return RD_INVALID_INPUT;
  const rd::RlShape key{(int)width, (int)height, taps / 2};
  std::lock_guard<std::mutex> lk(rd::g_rl_tune_mutex);
  auto it = rd::g_rl_tuned.find(key);
  if (it == rd::g_rl_tuned.end()) return RD_UNSUPPORTED;
  *segments = it->second.segs;
  if (default_segments) *default_segments = it->second.default_segs;
  if (best_ms) *best_ms = it->second.best_ms;
  if (default_ms) *default_ms = it->second.default_ms;
  return RD_OK;
}

extern "C" rd_status rd_launch_shape(int32_t stage, uint32_t width, uint32_t height, float radius, int32_t* value,
                                     int32_t* default_value, float* best_ms, float* default_ms) {
  if (!value || (stage != RD_SHAPE_RL_MASK && stage != RD_SHAPE_COLOR && stage != RD_SHAPE_OPTICS))
    return RD_INVALID_INPUT;
  int c = 0;
  if (stage == RD_SHAPE_RL_MASK) {
    float w[rd::MAX_TAPS];
    const int taps = rd::gaussian_kernel(radius, w, rd::MAX_TAPS);
    if (taps < 0) return RD_INVALID_INPUT;
    c = taps / 2;
  }
  const int kernel = stage == RD_SHAPE_RL_MASK ? rd::TUNE_RL_PREP : stage == RD_SHAPE_COLOR ? rd::TUNE_COLOR : rd::TUNE_OPTICS;
  const rd::ShapeKey key{kernel, (int)width, (int)height, c};
  int v = 0, d = 0;
  float b = 0.0f, dm = 0.0f;
  if (!rd::shape_record(key, &v, &d, &b, &dm)) return RD_UNSUPPORTED;
  *value = v;
  if (default_value) *default_value = d;
  if (best_ms) *best_ms = b;
  if (default_ms) *default_ms = dm;
  return RD_OK;
}
