// Opposed highlight reconstruction on sm_103a (crates/highlight/src/
// {opposed,cells,regions,support,region_correction}.rs).
//
// Pipeline (all on the device, no host round trip between kernels):
//   1. suspected-site count (early exit as opposed.rs:75-81 when zero: every
//      later kernel reads the count and returns), in the same pass as
//   2. cell summaries (cells.rs:41-113): per 2x2 cell, channel means of the
//      clean positive samples and usable / suspected flags. The pass reads the
//      raw u16 samples and normalizes them itself (writing the f32 mosaic the
//      estimate and the demosaic read), so no separate normalize pass runs;
//   3. dilated mask (regions.rs:127-182): a cell is inside when any cell of
//      its 3x3 neighbourhood holds a suspected sample (DILATION_CELLS = 1);
//      the inside cells are also appended to a list, and every labelling
//      kernel after this one runs over that list only (a few percent of the
//      cells in a typical frame) instead of over the whole cell grid;
//   4. 8-connected labelling (regions.rs:188-281) as a lock-free union-find
//      whose root is always the smallest cell index of the component; the
//      roots are marked in a bitmap of the cell grid, and the prefix count of
//      that bitmap in raster order gives exactly the reference's compact
//      labels (numbered by first appearance in raster order);
//   5. per-region clipped channels and wanted (channel, support) slots
//      (region_correction.rs:134-178);
//   6. two-pass trimmed means over each region's clean border ring plus the
//      image-wide pool, f64 accumulators (region_correction.rs:196-256);
//   7. per-site estimate (opposed.rs:86-330): local median over clean cells
//      1..3 cells away, region/pool correction, chromaticity guard, 4x level
//      bound, raise or neutralise.
// The f64 accumulation order of step 6 differs from the reference's raster
// scan; the trimmed means agree to f64 rounding, which is far below f32.
// Every retry loop carries an iteration limit and reports through the error
// word instead of spinning.
#include <algorithm>

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr float DARK_SUPPORT_FRACTION = 0.2f;
constexpr float CROSS_CHANNEL_TOLERANCE_EV = 0.75f;
constexpr int SLOTS = 9, PATTERNS = 3;
constexpr unsigned MIN_BORDER_CELLS = 3;
constexpr double TRIM_DEVIATIONS = 2.0;
constexpr float TRIM_FLOOR = 1e-5f;
constexpr float BORDER_MIN_FRACTION = 0.5f;
constexpr int LAST_RADIUS = 3, MAX_CANDIDATES = 48, MIN_CANDIDATES = 3;
constexpr float MAX_ESTIMATE_MULT = 4.0f;
constexpr int UNION_LIMIT = 1 << 20;
constexpr unsigned OPPOSED_ERROR = 16u;

// The estimate runs on tiles of ETX x ETY target cells; a tile stages the
// cells within LAST_RADIUS of its own (ESW x ESH) in shared memory.
constexpr int ETX = 16, ETY = 8, ETHREADS = 128;
constexpr int ESW = ETX + 2 * LAST_RADIUS, ESH = ETY + 2 * LAST_RADIUS, ESN = ESW * ESH;

struct Cell {
  float m[3];
  unsigned flags;
};

struct OpposedParams {
  MosaicSource src;          // normalized samples (raw u16, or the f32 mosaic itself)
  float* mosaic;             // reconstructed crop-sized mosaic
  int write_mosaic;          // 1: the cell pass stores every normalized sample to `mosaic`
  int W, H, cw, ch, cfa;
  float levels[3];
  int has_ceiling;
  float ceiling[3];
  float4* cells;             // xyz = means, w = flags (as bits)
  unsigned char* dilated;
  unsigned char* suspected;  // per cell: suspected-channel bits
  unsigned* tile_flags;      // per estimate tile: 1 once a cell of it holds a suspected sample
  unsigned* tile_list;       // the flagged estimate tiles, counters[2] of them
  unsigned* cell_list;       // the dilated cells, counters[3] of them
  unsigned* parent;          // union-find links (dilated cells only)
  unsigned* labels;          // per dilated cell: its root, then its compact label
  unsigned* root_bits;       // one bit per cell: the component roots
  unsigned* word_prefix;     // per root_bits word: roots in the earlier words of its block
  unsigned* block_sums;      // per RANK_BLOCK words: roots, then their exclusive prefix
  unsigned* region_clipped;  // per label
  unsigned* wanted;          // per label; wanted[0] = union over regions
  double* acc;               // per (label, slot): count, kept, accum, second (4 doubles)
  float* trim;               // per (label, slot): mean, tolerance
  unsigned max_labels;
  unsigned long long* stats; // 9 counters (reconstructed etc. at [1..5])
  unsigned* counters;        // [0] suspected count, [1] region count, [2] estimate tiles, [3] dilated cells,
                             // [4] estimate tiles handed out
  int tiles_x;               // estimate tiles per row
  unsigned* error;
};

__device__ __forceinline__ Cell load_cell(const OpposedParams& p, int x, int y) {
  const float4 v = p.cells[(long long)y * p.cw + x];
  Cell c;
  c.m[0] = v.x;
  c.m[1] = v.y;
  c.m[2] = v.z;
  c.flags = __float_as_uint(v.w);
  return c;
}
__device__ __forceinline__ bool usable(const Cell& c, int ch) { return c.flags & (1u << ch); }
__device__ __forceinline__ bool clean(const Cell& c, int ch) { return !(c.flags & (1u << (ch + 3))); }
__device__ __forceinline__ bool bright_clean(const Cell& c, int ch, const float* lv) {
  return usable(c, ch) && clean(c, ch) && c.m[ch] > DARK_SUPPORT_FRACTION * lv[ch];
}
__device__ __forceinline__ unsigned support_mask(const Cell& c, int target, const float* lv) {
  unsigned m = 0;
  for (int ch = 0; ch < 3; ++ch)
    if (ch != target && bright_clean(c, ch, lv)) m |= 1u << ch;
  return m;
}
// support.rs:56-77
__device__ bool reference_value(const Cell& c, unsigned support, float& out) {
  if (__popc(support) == 1) {
    const float v = c.m[__ffs(support) - 1];
    if (isfinite(v) && v > 0.0f) {
      out = v;
      return true;
    }
    return false;
  }
  float sum = 0.0f;
  int count = 0;
  for (int ch = 0; ch < 3; ++ch) {
    if (!(support & (1u << ch))) continue;
    const float v = c.m[ch];
    if (!isfinite(v) || v <= 0.0f) return false;
    sum += cbrtf(v);
    count += 1;
  }
  if (count == 0) return false;
  const float root = sum / (float)count;
  out = root * root * root;
  return true;
}
__device__ bool correction(const Cell& c, int target, unsigned support, const float* lv, float& out) {
  if (!bright_clean(c, target, lv)) return false;
  for (int ch = 0; ch < 3; ++ch)
    if ((support & (1u << ch)) && !bright_clean(c, ch, lv)) return false;
  float ref;
  if (!reference_value(c, support, ref)) return false;
  const float v = c.m[target] - ref;
  if (!isfinite(v)) return false;
  out = v;
  return true;
}
__device__ bool log_ratio(const Cell& c, unsigned support, float& out) {
  if (__popc(support) != 2) return false;
  const int first = __ffs(support) - 1;
  const int second = __ffs(support & ~(1u << first)) - 1;
  const float ratio = c.m[first] / c.m[second];
  if (!(isfinite(ratio) && ratio > 0.0f)) return false;
  out = log2f(ratio);
  return true;
}
__device__ __forceinline__ bool chroma_agrees(unsigned support, bool ht, float t, bool he, float e) {
  if (__popc(support) < 2) return true;
  if (ht && he) return fabsf(t - e) <= CROSS_CHANNEL_TOLERANCE_EV;
  return false;
}
__device__ __forceinline__ void support_patterns(int ch, unsigned out[3]) {
  const int o0 = ch == 0 ? 1 : 0;
  const int o1 = ch == 2 ? 1 : 2;
  out[0] = 1u << o0;
  out[1] = 1u << o1;
  out[2] = (1u << o0) | (1u << o1);
}
__device__ __forceinline__ int pattern_position(int ch, unsigned support) {
  unsigned p[3];
  support_patterns(ch, p);
  for (int k = 0; k < 3; ++k)
    if (p[k] == support) return k;
  return -1;
}

// 1 + 2. suspected sites and cell summaries (cells.rs:41-113) in one pass over
// the mosaic: per 2x2 cell the channel means of the clean positive samples
// (summed in raster order), the usable / suspected flags, a byte of suspected
// bits for the dilation, the estimate tiles holding suspected samples, and the
// suspected-site counts per channel, reduced per block before they reach the
// global counters.
__global__ void __launch_bounds__(128) cells_kernel(const OpposedParams p) {
  __shared__ unsigned block_counts[4];
  if (threadIdx.x < 4) block_counts[threadIdx.x] = 0;
  __syncthreads();
  const int cx = blockIdx.x * blockDim.x + threadIdx.x, cy = blockIdx.y;
  unsigned n_ch[3] = {0, 0, 0};
  unsigned smask = 0;  // suspected positions of the cell, bit 2 dy + dx
  if (cx < p.cw) {
    float sums[3] = {0.0f, 0.0f, 0.0f};
    unsigned counts[3] = {0, 0, 0};
    unsigned flags = 0;
    float v[2][2];
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const int y = 2 * cy + dy, x = 2 * cx + dx;
        v[dy][dx] = (y < p.H && x < p.W) ? source_normalized(p.src, x, y) : 0.0f;
      }
    if (p.write_mosaic) {
#pragma unroll
      for (int dy = 0; dy < 2; ++dy) {
        const int y = 2 * cy + dy, x = 2 * cx;
        if (y >= p.H) continue;
        float* row = p.mosaic + (long long)y * p.W;
        if (x + 1 < p.W && ((((long long)y * p.W + x) & 1) == 0)) {
          *reinterpret_cast<float2*>(row + x) = make_float2(v[dy][0], v[dy][1]);
        } else {
          row[x] = v[dy][0];
          if (x + 1 < p.W) row[x + 1] = v[dy][1];
        }
      }
    }
#pragma unroll
    for (int dy = 0; dy < 2; ++dy)
#pragma unroll
      for (int dx = 0; dx < 2; ++dx) {
        const int y = 2 * cy + dy, x = 2 * cx + dx;
        if (y >= p.H || x >= p.W) continue;
        const int ch = color_at(p.cfa, x, y);
        const float s = v[dy][dx];
        const bool susp = s >= p.levels[ch], clean = !susp && s > 0.0f;
        if (susp) {
          flags |= 1u << (ch + 3);
          smask |= 1u << (2 * dy + dx);
        }
        // Channel selects keep the per-channel values in registers.
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (c == ch && susp) n_ch[c] += 1;
          if (c == ch && clean) {
            sums[c] += s;
            counts[c] += 1;
          }
        }
      }
    float m[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
      if (counts[ch] != 0) {
        m[ch] = sums[ch] / (float)counts[ch];
        flags |= 1u << ch;
      }
    const long long i = (long long)cy * p.cw + cx;
    p.cells[i] = make_float4(m[0], m[1], m[2], __uint_as_float(flags));
    p.suspected[i] = (unsigned char)(flags >> 3);
  }
  // Flag the cell's estimate tile; its first flagging appends it to the tile list.
  if (smask) {
    const unsigned tile = (unsigned)((cy / ETY) * p.tiles_x + cx / ETX);
    if (atomicExch(&p.tile_flags[tile], 1u) == 0u) p.tile_list[atomicAdd(&p.counters[2], 1u)] = tile;
  }
  // A cell holds at most four sites, so the per-channel counts of a warp fit
  // 8-bit fields of one word.
  const unsigned packed = n_ch[0] | n_ch[1] << 8 | n_ch[2] << 16;
  const unsigned sum = __reduce_add_sync(0xffffffffu, packed);
  if ((threadIdx.x & 31) == 0 && sum)
    for (int c = 0; c < 3; ++c) atomicAdd(&block_counts[c], (sum >> (8 * c)) & 255u);
  __syncthreads();
  if (threadIdx.x < 3 && block_counts[threadIdx.x]) {
    atomicAdd(&p.counters[0], block_counts[threadIdx.x]);
    atomicAdd(&p.stats[6 + threadIdx.x], (unsigned long long)block_counts[threadIdx.x]);
  }
}

// 3. dilation + union-find initialisation, DILATE_CELLS cells of a row per
// thread (their 3x3 neighbourhoods share columns, and the loads of a thread
// are independent); the inside cells are appended to the cell list, one
// atomic per warp.
constexpr int DILATE_CELLS = 4;
__global__ void __launch_bounds__(128) dilate_kernel(const OpposedParams p) {
  if (p.counters[0] == 0) return;
  const int cx0 = (blockIdx.x * blockDim.x + threadIdx.x) * DILATE_CELLS, cy = blockIdx.y;
  unsigned inside = 0;  // bit j: cell cx0 + j is inside
  if (cx0 < p.cw) {
    const int y0 = max(cy - 1, 0), y1 = min(cy + 1, p.ch - 1);
    unsigned cols = 0;  // bit k: column cx0 - 1 + k holds a suspected cell in rows y0..y1
#pragma unroll
    for (int k = 0; k < DILATE_CELLS + 2; ++k) {
      const int x = cx0 - 1 + k;
      if (x < 0 || x >= p.cw) continue;
      unsigned v = 0;
      for (int y = y0; y <= y1; ++y) v |= p.suspected[(long long)y * p.cw + x];
      if (v) cols |= 1u << k;
    }
#pragma unroll
    for (int j = 0; j < DILATE_CELLS; ++j) {
      const int x = cx0 + j;
      if (x >= p.cw) break;
      const bool in = ((cols >> j) & 7u) != 0;  // columns x - 1, x, x + 1
      const long long i = (long long)cy * p.cw + x;
      p.dilated[i] = in;
      if (in) {
        p.parent[i] = (unsigned)i;
        inside |= 1u << j;
      }
    }
  }
  const unsigned FULL = 0xffffffffu, lane = threadIdx.x & 31;
  const unsigned n = __popc(inside);
  unsigned incl = n;
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned v = __shfl_up_sync(FULL, incl, off);
    if (lane >= (unsigned)off) incl += v;
  }
  const unsigned total = __shfl_sync(FULL, incl, 31);
  unsigned base = 0;
  if (lane == 31 && total) base = atomicAdd(&p.counters[3], total);
  base = __shfl_sync(FULL, base, 31) + incl - n;
  for (int j = 0; j < DILATE_CELLS; ++j)
    if (inside & (1u << j)) p.cell_list[base++] = (unsigned)((long long)cy * p.cw + cx0 + j);
}

// Root of i. Links only ever point to smaller indices, so shortening a path
// with atomicMin (never raising a link) keeps every component intact.
__device__ unsigned find_root(unsigned* parent, unsigned i, unsigned* error) {
  for (int k = 0; k < UNION_LIMIT; ++k) {
    const unsigned q = parent[i];
    if (q == i) return i;
    const unsigned g = parent[q];
    if (g < q) atomicMin(&parent[i], g);
    i = q;
  }
  atomicOr(error, OPPOSED_ERROR);
  return i;
}

// Link the roots of a and b, the larger root pointing at the smaller.
__device__ void unite(unsigned* parent, unsigned a, unsigned b, unsigned* error) {
  for (int k = 0; k < UNION_LIMIT; ++k) {
    a = find_root(parent, a, error);
    b = find_root(parent, b, error);
    if (a == b) return;
    if (a > b) {
      const unsigned t = a;
      a = b;
      b = t;
    }
    const unsigned old = atomicMin(&parent[b], a);
    if (old == b) return;
    b = old;
  }
  atomicOr(error, OPPOSED_ERROR);
}

// Grid-stride loops over the dilated cells of the list.
#define FOR_LISTED_CELLS(k) \
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x, k##_n = p.counters[3]; k < k##_n; \
       k += gridDim.x * blockDim.x)

__global__ void __launch_bounds__(256) union_kernel(const OpposedParams p) {
  FOR_LISTED_CELLS(k) {
    const unsigned i = p.cell_list[k];
    const unsigned cy = i / (unsigned)p.cw, cx = i - cy * (unsigned)p.cw;
    if (cx > 0 && p.dilated[i - 1]) unite(p.parent, i, i - 1, p.error);
    if (cy > 0) {
      const unsigned up = i - p.cw;
      if (cx > 0 && p.dilated[up - 1]) unite(p.parent, i, up - 1, p.error);
      if (p.dilated[up]) unite(p.parent, i, up, p.error);
      if (cx + 1 < (unsigned)p.cw && p.dilated[up + 1]) unite(p.parent, i, up + 1, p.error);
    }
  }
}

// Root of every dilated cell (provisional label: the component's smallest
// cell index), and the roots marked in the bitmap.
__global__ void __launch_bounds__(256) flatten_kernel(const OpposedParams p) {
  FOR_LISTED_CELLS(k) {
    const unsigned i = p.cell_list[k];
    const unsigned r = find_root(p.parent, i, p.error);
    p.labels[i] = r;
    if (r == i) atomicOr(&p.root_bits[i >> 5], 1u << (i & 31));
  }
}

// Roots before each bitmap word within its block of RANK_BLOCK words, and
// each block's roots.
constexpr int RANK_BLOCK = 1024;
__global__ void __launch_bounds__(RANK_BLOCK) rank_words_kernel(const OpposedParams p, unsigned words) {
  if (p.counters[0] == 0) return;
  __shared__ unsigned warp_sums[RANK_BLOCK / 32];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned w = blockIdx.x * RANK_BLOCK + threadIdx.x;
  const unsigned c = w < words ? __popc(p.root_bits[w]) : 0u;
  unsigned x = c;
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned y = __shfl_up_sync(FULL, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned v = warp_sums[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned y = __shfl_up_sync(FULL, v, off);
      if (lane >= off) v += y;
    }
    warp_sums[lane] = v;
  }
  __syncthreads();
  const unsigned before = (warp ? warp_sums[warp - 1] : 0u) + x - c;
  if (w < words) p.word_prefix[w] = before;
  if (threadIdx.x == RANK_BLOCK - 1) p.block_sums[blockIdx.x] = before + c;
}

// Exclusive scan of the per-block root counts (one block); the total is the
// region count.
__global__ void scan_blocks_kernel(const OpposedParams p, int blocks) {
  if (p.counters[0] == 0) return;
  __shared__ unsigned carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < blocks; base += blockDim.x) {
    const int k = base + threadIdx.x;
    const unsigned v = k < blocks ? p.block_sums[k] : 0;
    // Inclusive warp scan, then across warps through shared memory.
    unsigned x = v;
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, off);
      if ((threadIdx.x & 31) >= off) x += y;
    }
    __shared__ unsigned wsum[32];
    if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      unsigned w = threadIdx.x < blockDim.x / 32 ? wsum[threadIdx.x] : 0;
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, w, off);
        if (threadIdx.x >= off) w += y;
      }
      wsum[threadIdx.x] = w;
    }
    __syncthreads();
    const unsigned before = (threadIdx.x >= 32 ? wsum[(threadIdx.x >> 5) - 1] : 0) + x - v;
    if (k < blocks) p.block_sums[k] = carry + before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += before + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) p.counters[1] = carry;
}

// Zero the per-label tables of the labels in use (label 0 is the pool).
__global__ void clear_tables_kernel(const OpposedParams p) {
  if (p.counters[0] == 0) return;
  const unsigned labels = min(p.counters[1] + 1u, p.max_labels);
  const unsigned stride = gridDim.x * blockDim.x, t = blockIdx.x * blockDim.x + threadIdx.x;
  for (unsigned k = t; k < labels; k += stride) {
    p.region_clipped[k] = 0;
    p.wanted[k] = 0;
  }
  const unsigned long long doubles = (unsigned long long)labels * SLOTS * 4;
  for (unsigned long long k = t; k < doubles; k += stride) p.acc[k] = 0.0;
}

// OR `bits` into word[key] once per distinct key of the warp (neighbouring
// cells nearly always share their region).
__device__ __forceinline__ void warp_or(unsigned* word, unsigned key, unsigned bits) {
  namespace cg = cooperative_groups;
  const cg::coalesced_group active = cg::coalesced_threads();
  const cg::coalesced_group peers = cg::labeled_partition(active, key);
  const unsigned v = cg::reduce(peers, bits, cg::bit_or<unsigned>());
  if (peers.thread_rank() == 0 && v) atomicOr(&word[key], v);
}

// Final compact label of each dilated cell (1 + the roots before its root in
// raster order), the per-region clipped channels, and 5. the wanted
// (channel, support) slots per region (region_correction.rs:134-178), in one
// pass: both need only the cell's own label.
__global__ void __launch_bounds__(256) relabel_kernel(const OpposedParams p) {
  FOR_LISTED_CELLS(k) {
    const unsigned i = p.cell_list[k];
    const unsigned r = p.labels[i], w = r >> 5;
    unsigned label =
        p.block_sums[w / RANK_BLOCK] + p.word_prefix[w] + __popc(p.root_bits[w] & ((1u << (r & 31)) - 1u)) + 1u;
    if (label >= p.max_labels) {  // cannot happen for 8-connected regions of a 3x3 dilation
      atomicOr(p.error, OPPOSED_ERROR);
      label = 0;
    }
    p.labels[i] = label;
    if (label == 0) continue;
    const unsigned cy = i / (unsigned)p.cw, cx = i - cy * (unsigned)p.cw;
    const Cell c = load_cell(p, (int)cx, (int)cy);
    const unsigned clipped = c.flags >> 3;
    if (clipped == 0) continue;
    warp_or(p.region_clipped, label, clipped);
    unsigned bits = 0;
    for (int ch = 0; ch < 3; ++ch) {
      if (!(clipped & (1u << ch))) continue;
      bool has_clean = false;
      for (int o = 0; o < 3; ++o)
        if (o != ch && usable(c, o) && clean(c, o)) has_clean = true;
      if (!has_clean) continue;
      const int pos = pattern_position(ch, support_mask(c, ch, p.levels));
      if (pos >= 0) bits |= 1u << (ch * PATTERNS + pos);
    }
    if (bits) {
      warp_or(p.wanted, label, bits);
      warp_or(p.wanted, 0u, bits);
    }
  }
}

// 6. region border statistics over the dilated cells; pass 0 = moments, pass
// 1 = trimmed sums.
__global__ void __launch_bounds__(256) border_kernel(const OpposedParams p, int pass) {
  if (p.counters[0] == 0) return;
  __shared__ double pool[SLOTS][3];
  __shared__ unsigned pool_n[SLOTS];
  if (threadIdx.x < SLOTS) {
    pool[threadIdx.x][0] = pool[threadIdx.x][1] = pool[threadIdx.x][2] = 0.0;
    pool_n[threadIdx.x] = 0;
  }
  __syncthreads();
  FOR_LISTED_CELLS(k) {
    const unsigned i = p.cell_list[k];
    const unsigned label = p.labels[i];
    if (label == 0) continue;
    const unsigned cy = i / (unsigned)p.cw, cx = i - cy * (unsigned)p.cw;
    const Cell c = load_cell(p, (int)cx, (int)cy);
    if ((c.flags >> 3) == 0) {
      const unsigned rclip = p.region_clipped[label];
      const unsigned want_r = p.wanted[label], want_any = p.wanted[0];
      for (int ch = 0; ch < 3; ++ch) {
        if (!(rclip & (1u << ch))) continue;
        if (c.m[ch] < BORDER_MIN_FRACTION * p.levels[ch]) continue;
        unsigned pats[3];
        support_patterns(ch, pats);
        for (int k = 0; k < 3; ++k) {
          const int off = ch * PATTERNS + k;
          const bool for_region = want_r & (1u << off);
          const bool for_pool = want_any & (1u << off);
          if (!for_region && !for_pool) continue;
          float value;
          if (!correction(c, ch, pats[k], p.levels, value)) continue;
          float ratio = 0.0f;
          const bool has_ratio = log_ratio(c, pats[k], ratio);
          const double wide = (double)value;
          auto add = [&](long long slot, bool shared_pool) {
            double* a = p.acc + slot * 4;
            if (pass == 0) {
              if (shared_pool) {
                atomicAdd(&pool_n[off], 1u);
                atomicAdd(&pool[off][0], wide);
                atomicAdd(&pool[off][1], wide * wide);
              } else {
                atomicAdd(&a[0], 1.0);
                atomicAdd(&a[2], wide);
                atomicAdd(&a[3], wide * wide);
              }
            } else {
              const float* t = p.trim + slot * 2;
              if (fabsf(value - t[0]) <= t[1]) {
                const double r = (double)(has_ratio ? ratio : 0.0f);
                if (shared_pool) {
                  atomicAdd(&pool_n[off], 1u);
                  atomicAdd(&pool[off][0], wide);
                  atomicAdd(&pool[off][2], r);
                } else {
                  atomicAdd(&a[1], 1.0);
                  atomicAdd(&a[2], wide);
                  atomicAdd(&a[3], r);
                }
              }
            }
          };
          if (for_region) add((long long)label * SLOTS + off, false);
          if (for_pool) add(off, true);
        }
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < SLOTS && pool_n[threadIdx.x]) {
    double* a = p.acc + threadIdx.x * 4;
    if (pass == 0) {
      atomicAdd(&a[0], (double)pool_n[threadIdx.x]);
      atomicAdd(&a[2], pool[threadIdx.x][0]);
      atomicAdd(&a[3], pool[threadIdx.x][1]);
    } else {
      atomicAdd(&a[1], (double)pool_n[threadIdx.x]);
      atomicAdd(&a[2], pool[threadIdx.x][0]);
      atomicAdd(&a[3], pool[threadIdx.x][2]);
    }
  }
}

// Slot::finish_moments (region_correction.rs:73-86): trimming window, then
// the accumulators restart for the trimmed pass.
__global__ void finish_moments_kernel(const OpposedParams p) {
  if (p.counters[0] == 0) return;
  const unsigned slots = (p.counters[1] + 1) * SLOTS;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < slots; s += gridDim.x * blockDim.x) {
    double* a = p.acc + (long long)s * 4;
    const double count = a[0];
    if (count != 0.0) {
      const double mean = a[2] / count;
      double variance = a[3] / count - mean * mean;
      if (variance < 0.0) variance = 0.0;
      p.trim[(long long)s * 2] = (float)mean;
      p.trim[(long long)s * 2 + 1] = (float)(TRIM_DEVIATIONS * sqrt(variance)) + TRIM_FLOOR;
    }
    a[2] = 0.0;
    a[3] = 0.0;
  }
}

// Slot::value (region_correction.rs:90-103)
__device__ bool slot_value(const OpposedParams& p, long long slot, bool has_ratio, float& offset, bool& hr,
                           float& ratio) {
  const double* a = p.acc + slot * 4;
  if (a[0] < (double)MIN_BORDER_CELLS || a[1] == 0.0) return false;
  offset = (float)(a[2] / a[1]);
  hr = has_ratio;
  if (has_ratio) ratio = (float)(a[3] / a[1]);
  return true;
}

__device__ __forceinline__ bool total_less(float a, float b) {
  if (a == b) return signbit(a) && !signbit(b);
  return a < b;
}

// Cell offsets (dx, dy) of the rings at Chebyshev distance 1, 2 and 3 (8, 16
// and 24 cells), ring after ring, each in raster order.
__constant__ char2 c_ring[48] = {
    {-1, -1}, {0, -1}, {1, -1}, {-1, 0}, {1, 0}, {-1, 1}, {0, 1}, {1, 1},
    {-2, -2}, {-1, -2}, {0, -2}, {1, -2}, {2, -2}, {-2, -1}, {2, -1}, {-2, 0},
    {2, 0}, {-2, 1}, {2, 1}, {-2, 2}, {-1, 2}, {0, 2}, {1, 2}, {2, 2},
    {-3, -3}, {-2, -3}, {-1, -3}, {0, -3}, {1, -3}, {2, -3}, {3, -3}, {-3, -2},
    {3, -2}, {-3, -1}, {3, -1}, {-3, 0}, {3, 0}, {-3, 1}, {3, 1}, {-3, 2},
    {3, 2}, {-3, 3}, {-2, 3}, {-1, 3}, {0, 3}, {1, 3}, {2, 3}, {3, 3},
};

// 7. per-site estimate (opposed.rs:86-180, 236-330) on tiles of target cells.
// A candidate cell's correction for (channel, support) and its log ratio for
// a channel pair depend only on the cell, so a tile computes them once for
// every cell it stages (9 corrections, 3 pair ratios; NaN = the candidate is
// skipped) and its sites read them from shared memory. The values are the
// ones correction() and log_ratio() return, so the candidates, their median
// and every estimate are unchanged.
struct EstimateSmem {
  float4 cell[ESN];
  float root[ESN][3];   // cube root of each bright-clean channel's mean (else 0)
  float corr[ESN][9];   // [channel * PATTERNS + pattern]
  float ratio[ESN][3];  // [channel]: log ratio of the other two channels when both are bright-clean
};

__device__ void stage_candidate(const OpposedParams& p, EstimateSmem& S, int k, int gx, int gy) {
  const float qnan = __int_as_float(0x7fc00000);
  if ((unsigned)gx >= (unsigned)p.cw || (unsigned)gy >= (unsigned)p.ch) {
    S.cell[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int j = 0; j < 3; ++j) S.root[k][j] = 0.0f;
    for (int j = 0; j < 9; ++j) S.corr[k][j] = qnan;
    for (int j = 0; j < 3; ++j) S.ratio[k][j] = qnan;
    return;
  }
  const Cell c = load_cell(p, gx, gy);
  S.cell[k] = make_float4(c.m[0], c.m[1], c.m[2], __uint_as_float(c.flags));
  // correction(), reference_value() and log_ratio() restated from the
  // bright-clean channels. A bright-clean mean is finite and positive (it
  // exceeds a positive level), so reference_value() succeeds for any
  // non-empty support of them, and its pair reference sums the two cube roots
  // in channel order from 0 (0 + r = r): each root is taken once per cell.
  bool bright[3];
  float root[3];
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    bright[ch] = bright_clean(c, ch, p.levels);
    root[ch] = bright[ch] ? cbrtf(c.m[ch]) : 0.0f;
    S.root[k][ch] = root[ch];
  }
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) {
    const int o0 = ch == 0 ? 1 : 0, o1 = ch == 2 ? 1 : 2;  // support_patterns: {o0}, {o1}, {o0, o1}
    const bool pair = bright[o0] && bright[o1];
    const float mean_root = (root[o0] + root[o1]) / 2.0f;
    const float ref[3] = {c.m[o0], c.m[o1], mean_root * mean_root * mean_root};
    const bool ok[3] = {bright[ch] && bright[o0], bright[ch] && bright[o1], bright[ch] && pair};
#pragma unroll
    for (int q = 0; q < PATTERNS; ++q) {
      const float v = c.m[ch] - ref[q];
      S.corr[k][ch * PATTERNS + q] = ok[q] && isfinite(v) ? v : qnan;
    }
    float r = qnan;
    if (pair) {
      const float ratio = c.m[o0] / c.m[o1];
      if (isfinite(ratio) && ratio > 0.0f) r = log2f(ratio);
    }
    S.ratio[k][ch] = r;
  }
}

// The estimate of one suspected site (x, y) of target cell (lx, ly) of the
// tile (staged coordinates); counts[5]: reconstructed, changed, fallback,
// unsupported, neutralised.
__device__ void estimate_site(const OpposedParams& p, const EstimateSmem& S, int x, int y, int lx, int ly,
                              unsigned (&counts)[5]) {
  float& s = p.mosaic[(long long)y * p.W + x];
  const int ch = color_at(p.cfa, x, y);
  const float level = p.levels[ch];
  const int sx = lx + LAST_RADIUS, sy = ly + LAST_RADIUS;
  const float4 tv = S.cell[sy * ESW + sx];
  Cell target;
  target.m[0] = tv.x;
  target.m[1] = tv.y;
  target.m[2] = tv.z;
  target.flags = __float_as_uint(tv.w);
  int support_count = 0;
  for (int o = 0; o < 3; ++o)
    if (o != ch && usable(target, o) && clean(target, o)) support_count++;
  bool ok = false;
  float estimate = 0.0f;
  if (support_count != 0) {
    const unsigned support = support_mask(target, ch, p.levels);
    // reference_value(target, support) and log_ratio(target, support) from the
    // staged roots and ratio (the support channels are bright-clean).
    if (support != 0) {
      const int t = sy * ESW + sx;
      const bool pair = __popc(support) == 2;
      float ref;
      if (pair) {
        const int o0 = ch == 0 ? 1 : 0, o1 = ch == 2 ? 1 : 2;
        const float mean_root = (S.root[t][o0] + S.root[t][o1]) / 2.0f;
        ref = mean_root * mean_root * mean_root;
      } else {
        ref = target.m[__ffs(support) - 1];
      }
      const float tratio = pair ? S.ratio[t][ch] : 0.0f;
      const bool has_tratio = pair && tratio == tratio;
      const int col = ch * PATTERNS + pattern_position(ch, support);  // support != 0 here
      float corr[MAX_CANDIDATES];
      int count = 0;
      bool has_local = false;
      float local = 0.0f;
      int local_radius = 0;
      for (int radius = 1; radius <= LAST_RADIUS && !has_local; ++radius) {
        // The ring's cells from the offset table (no pass over the square's
        // interior); the candidates are sorted below, so the visiting order
        // does not matter, and the three rings hold 48 = MAX_CANDIDATES cells.
        const int ring0 = 4 * radius * (radius - 1), ring_n = 8 * radius;
        for (int q = 0; q < ring_n; ++q) {
          const int k = (sy + c_ring[ring0 + q].y) * ESW + sx + c_ring[ring0 + q].x;
          const float value = S.corr[k][col];
          if (value != value) continue;  // not a usable candidate (or outside the image)
          if (pair) {  // chroma_agrees with both ratios required
            const float cratio = S.ratio[k][ch];
            if (!has_tratio || cratio != cratio || !(fabsf(tratio - cratio) <= CROSS_CHANNEL_TOLERANCE_EV)) continue;
          }
          corr[count++] = value;
        }
        if (count >= MIN_CANDIDATES) {
          for (int a = 1; a < count; ++a) {  // insertion sort, total order
            const float v = corr[a];
            int b = a - 1;
            while (b >= 0 && total_less(v, corr[b])) {
              corr[b + 1] = corr[b];
              --b;
            }
            corr[b + 1] = v;
          }
          const int mid = count / 2;
          local = count % 2 == 0 ? (corr[mid - 1] + corr[mid]) * 0.5f : corr[mid];
          local_radius = radius;
          has_local = true;
        }
      }
      const unsigned label = p.labels[(long long)(y / 2) * p.cw + x / 2];
      bool has_region = false;
      float region = 0.0f;
      const int pos = pattern_position(ch, support);
      if (pos >= 0) {
        const int off = ch * PATTERNS + pos;
        float bratio = 0.0f;
        bool has_bratio = false;
        if (slot_value(p, (long long)label * SLOTS + off, pair, region, has_bratio, bratio) ||
            slot_value(p, off, pair, region, has_bratio, bratio))
          has_region = chroma_agrees(support, has_tratio, tratio, has_bratio, bratio);
      }
      float correction_value = 0.0f;
      bool have = true;
      if (has_local && has_region) {
        const float weight = (float)(LAST_RADIUS + 1 - local_radius) / (float)LAST_RADIUS;
        correction_value = weight * local + (1.0f - weight) * region;
      } else if (has_local) {
        correction_value = local;
      } else if (has_region) {
        correction_value = region;
      } else {
        have = false;
      }
      if (have) {
        estimate = ref + correction_value;
        ok = isfinite(estimate) && estimate > 0.0f;
      }
    }
  }
  bool neutralise = false;
  if (!ok) {
    counts[2]++;
    if (support_count == 0) counts[3]++;
    neutralise = true;
  } else {
    counts[0]++;
    float bounded = MAX_ESTIMATE_MULT * level;
    if (estimate < bounded) bounded = estimate;  // f32::min of finite values
    if (bounded > s) {
      s = bounded;
      counts[1]++;
    } else {
      neutralise = true;
    }
  }
  if (neutralise && p.has_ceiling && s > p.ceiling[ch]) {
    s = p.ceiling[ch];
    counts[4]++;
  }
}

// 7. the estimate over the flagged tiles, a grid-stride loop: stage the tile's
// cells and their candidate values, queue the suspected samples of the tile's
// target cells (the cell pass's test, s >= level), then estimate them (each
// site reads and writes only its own sample).
__global__ void __launch_bounds__(ETHREADS) estimate_kernel(const OpposedParams p) {
  __shared__ EstimateSmem S;
  __shared__ unsigned short queue[ETX * ETY * 4];  // the tile's suspected samples
  __shared__ int queued;
  __shared__ unsigned s_tile;
  unsigned counts[5] = {0, 0, 0, 0, 0};
  const unsigned FULL = 0xffffffffu, lane = threadIdx.x & 31;
  const unsigned tiles = p.counters[2];
  for (;;) {
    __syncthreads();  // the previous tile's sites are done with S and the queue
    // Tiles from a counter: a CTA takes the next one as soon as it is free, so
    // tiles with many sites do not pile up on some CTAs.
    if (threadIdx.x == 0) {
      s_tile = atomicAdd(&p.counters[4], 1u);
      queued = 0;
    }
    __syncthreads();
    const unsigned t = s_tile;
    if (t >= tiles) break;
    const unsigned tile = p.tile_list[t];
    const int tx0 = (int)(tile % (unsigned)p.tiles_x) * ETX, ty0 = (int)(tile / (unsigned)p.tiles_x) * ETY;
    for (int k = threadIdx.x; k < ESN; k += blockDim.x)
      stage_candidate(p, S, k, tx0 - LAST_RADIUS + k % ESW, ty0 - LAST_RADIUS + k / ESW);
    // Queue the suspected samples, so that full warps take the sites.
    for (int q = threadIdx.x; q < ETX * ETY * 4; q += blockDim.x) {
      const int lc = q >> 2;
      const int x = 2 * (tx0 + lc % ETX) + (q & 1), y = 2 * (ty0 + lc / ETX) + ((q >> 1) & 1);
      bool suspected = false;
      if (x < p.W && y < p.H) suspected = p.mosaic[(long long)y * p.W + x] >= p.levels[color_at(p.cfa, x, y)];
      const unsigned ballot = __ballot_sync(FULL, suspected);
      if (ballot) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&queued, __popc(ballot));
        base = __shfl_sync(FULL, base, 0);
        if (suspected) queue[base + __popc(ballot & ((1u << lane) - 1u))] = (unsigned short)q;
      }
    }
    __syncthreads();
    const int n = queued;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int q = queue[i], lc = q >> 2, lx = lc % ETX, ly = lc / ETX;
      estimate_site(p, S, 2 * (tx0 + lx) + (q & 1), 2 * (ty0 + ly) + ((q >> 1) & 1), lx, ly, counts);
    }
  }
  for (int k = 0; k < 5; ++k) {
    const unsigned sum = __reduce_add_sync(FULL, counts[k]);
    if (lane == 0 && sum) atomicAdd(&p.stats[1 + k], (unsigned long long)sum);
  }
  if (threadIdx.x == 0 && blockIdx.x == 0) p.stats[0] = p.counters[0];
}

// The compact label of every dilated cell into a zeroed cell grid.
__global__ void __launch_bounds__(256) labels_out_kernel(const OpposedParams p, uint32_t* out) {
  FOR_LISTED_CELLS(k) {
    const unsigned i = p.cell_list[k];
    out[i] = p.labels[i];
  }
}

}  // namespace

// reconstruct_opposed_cancellable on the crop-sized normalized mosaic of
// `src`, written to `mosaic` (in place when src.f32 == mosaic). d_stats (9
// counters) follows OpposedStats; labels_out (optional, device,
// ceil(w/2)*ceil(h/2)) receives the compact region labels.
Status run_opposed_labels(Context& ctx, const MosaicSource& src, float* mosaic, const float levels[3],
                          const float* ceiling, unsigned long long* d_stats, uint32_t* labels_out,
                          uint32_t* region_count_out) {
  const int W = src.width, H = src.height;
  const int cw = W / 2 + W % 2, chh = H / 2 + H % 2;
  const long long cells = (long long)cw * chh;
  // max_regions (regions.rs:117-124): raw-mask cells of separate regions are >= 4 cells apart.
  const unsigned max_labels = (unsigned)(((cw + 3) / 4) * ((chh + 3) / 4) + 1);
  const unsigned words = (unsigned)((cells + 31) / 32);
  const int rank_blocks = (int)((words + RANK_BLOCK - 1) / RANK_BLOCK);
  size_t bytes = 0;
  auto take = [&](size_t n) {
    const size_t at = bytes;
    bytes += (n + 255) & ~(size_t)255;
    return at;
  };
  const size_t o_cells = take(sizeof(float4) * cells);
  const size_t o_dil = take(cells);
  const size_t o_susp = take(cells);
  const size_t o_parent = take(sizeof(unsigned) * cells);
  const size_t o_labels = take(sizeof(unsigned) * cells);
  const size_t o_list = take(sizeof(unsigned) * cells);
  const int tiles_x = (cw + ETX - 1) / ETX;
  const size_t tiles = (size_t)tiles_x * ((chh + ETY - 1) / ETY);
  const size_t o_tiles = take(sizeof(unsigned) * tiles);
  const size_t o_prefix = take(sizeof(unsigned) * words);
  const size_t o_bsum = take(sizeof(unsigned) * rank_blocks);
  const size_t o_rclip = take(sizeof(unsigned) * max_labels);
  const size_t o_wanted = take(sizeof(unsigned) * max_labels);
  const size_t o_acc = take(sizeof(double) * 4 * SLOTS * (size_t)max_labels);
  const size_t o_trim = take(sizeof(float) * 2 * SLOTS * (size_t)max_labels);
  // The root bitmap, the tile flags and the counters, the only memory zeroed
  // before the kernels.
  const size_t o_bits = take(sizeof(unsigned) * words);
  const size_t o_flags = take(sizeof(unsigned) * tiles);
  const size_t o_cnt = take(sizeof(unsigned) * 8);
  void* base = nullptr;
  RD_TRY(device_alloc(ctx, bytes, &base));
  char* b = static_cast<char*>(base);
  OpposedParams p{};
  p.src = src;
  p.src.clip = 0;
  p.mosaic = mosaic;
  p.write_mosaic = src.f32 == mosaic ? 0 : 1;
  p.W = W;
  p.H = H;
  p.cw = cw;
  p.ch = chh;
  p.cfa = src.cfa;
  for (int c = 0; c < 3; ++c) {
    p.levels[c] = levels[c];
    p.ceiling[c] = ceiling ? ceiling[c] : 0.0f;
  }
  p.has_ceiling = ceiling ? 1 : 0;
  p.cells = reinterpret_cast<float4*>(b + o_cells);
  p.dilated = reinterpret_cast<unsigned char*>(b + o_dil);
  p.suspected = reinterpret_cast<unsigned char*>(b + o_susp);
  p.tile_list = reinterpret_cast<unsigned*>(b + o_tiles);
  p.tile_flags = reinterpret_cast<unsigned*>(b + o_flags);
  p.tiles_x = tiles_x;
  p.cell_list = reinterpret_cast<unsigned*>(b + o_list);
  p.parent = reinterpret_cast<unsigned*>(b + o_parent);
  p.labels = reinterpret_cast<unsigned*>(b + o_labels);
  p.root_bits = reinterpret_cast<unsigned*>(b + o_bits);
  p.word_prefix = reinterpret_cast<unsigned*>(b + o_prefix);
  p.block_sums = reinterpret_cast<unsigned*>(b + o_bsum);
  p.region_clipped = reinterpret_cast<unsigned*>(b + o_rclip);
  p.wanted = reinterpret_cast<unsigned*>(b + o_wanted);
  p.acc = reinterpret_cast<double*>(b + o_acc);
  p.trim = reinterpret_cast<float*>(b + o_trim);
  p.max_labels = max_labels;
  p.stats = d_stats;
  p.counters = reinterpret_cast<unsigned*>(b + o_cnt);
  p.error = ctx.d_error;
  RD_CUDA_TRY(cudaMemsetAsync(b + o_bits, 0, bytes - o_bits, ctx.stream));
  const int sms = ctx.sm_count > 0 ? ctx.sm_count : 152;
  const dim3 cgrid((cw + 127) / 128, chh);
  const dim3 dgrid((cw + 128 * DILATE_CELLS - 1) / (128 * DILATE_CELLS), chh);
  const int lgrid = sms * 8;  // list kernels: 256-thread blocks, grid-stride
  RD_LAUNCH(ctx, K_OPPOSED, cells_kernel<<<cgrid, 128, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, dilate_kernel<<<dgrid, 128, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, union_kernel<<<lgrid, 256, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, flatten_kernel<<<lgrid, 256, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, rank_words_kernel<<<rank_blocks, RANK_BLOCK, 0, ctx.stream>>>(p, words));
  RD_LAUNCH(ctx, K_OPPOSED, scan_blocks_kernel<<<1, 1024, 0, ctx.stream>>>(p, rank_blocks));
  RD_LAUNCH(ctx, K_OPPOSED, clear_tables_kernel<<<sms * 2, 256, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, relabel_kernel<<<lgrid, 256, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, border_kernel<<<lgrid, 256, 0, ctx.stream>>>(p, 0));
  RD_LAUNCH(ctx, K_OPPOSED, finish_moments_kernel<<<256, 256, 0, ctx.stream>>>(p));
  RD_LAUNCH(ctx, K_OPPOSED, border_kernel<<<lgrid, 256, 0, ctx.stream>>>(p, 1));
  int est_occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&est_occ, estimate_kernel, ETHREADS, 0) != cudaSuccess) est_occ = 0;
  RD_LAUNCH(ctx, K_OPPOSED, estimate_kernel<<<sms * std::max(est_occ, 1), ETHREADS, 0, ctx.stream>>>(p));
  cudaError_t launch = cudaGetLastError();
  if (launch == cudaSuccess && labels_out) {
    // Cells outside every region keep label 0 (with no suspected site, all of them).
    launch = cudaMemsetAsync(labels_out, 0, sizeof(uint32_t) * cells, ctx.stream);
    if (launch == cudaSuccess) {
      RD_LAUNCH(ctx, K_OPPOSED, labels_out_kernel<<<lgrid, 256, 0, ctx.stream>>>(p, labels_out));
      launch = cudaGetLastError();
    }
  }
  if (launch == cudaSuccess && region_count_out) {
    unsigned counters[2] = {0, 0};
    launch = cudaMemcpyAsync(counters, p.counters, sizeof(counters), cudaMemcpyDeviceToHost, ctx.stream);
    if (launch == cudaSuccess) launch = cudaStreamSynchronize(ctx.stream);
    *region_count_out = counters[0] ? counters[1] : 0;
  }
  device_free(ctx, base, bytes);
  if (launch != cudaSuccess) return Status{RD_SYNCHRONIZATION, cudaGetErrorString(launch)};
  return Status{};
}

Status run_opposed(Context& ctx, const MosaicSource& src, float* mosaic, const float levels[3], const float* ceiling,
                   unsigned long long* d_stats, uint32_t* region_count) {
  return run_opposed_labels(ctx, src, mosaic, levels, ceiling, d_stats, nullptr, region_count);
}

}  // namespace rd
