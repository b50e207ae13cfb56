// PNG encoding of the export's interleaved RGB rows, on the device.
//
// Replaces the PNG arms of export::encode (crates/core/src/export.rs:176-211):
// the reference hands tightly packed 8-bit or 16-bit RGB rows, the ICC
// profile of the output colour space and optional EXIF to the `image`
// crate's PngEncoder (image 0.25, Cargo.toml:39; not vendored). The file here
// decodes to exactly those samples and carries the same metadata chunks; the
// compressed bytes are this encoder's own (any PNG encoder's are).
//
// Six launches on the context's stream:
//  1. png_filter_kernel   one CTA per scanline: PNG filter selection by the
//                         minimum sum of absolute filtered values (the
//                         heuristic the PNG specification recommends, ties to
//                         the lower filter type), then the filtered scanline
//                         with its filter byte into the stream buffer;
//  2. png_histogram_kernel  one CTA per 32 KiB segment of the stream: the
//                         segment's token (literal / run) symbol counts and
//                         Adler-32 partial sums;
//  3. png_code_kernel     one warp per segment: Huffman code and block header;
//  4. png_pack_kernel     one CTA per segment: the byte-aligned deflate block
//                         (deflate.cuh) into the segment's slot;
//  5. png_layout_kernel   one CTA: prefix sum of the IDAT chunk sizes, the
//                         stream's Adler-32, the IEND chunk;
//  6. png_chunk_kernel    one CTA per segment: the IDAT chunk (length, type,
//                         zlib header on the first, Adler-32 on the last) with
//                         its CRC-32, stored at its offset in the file.
// The signature, IHDR, iCCP and eXIf chunks are built on the host and copied
// in front. The stream is HBM-resident byte work: every kernel reads its bytes
// once with coalesced accesses and stages them in shared memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "deflate.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

using namespace png;

constexpr unsigned FULL_MASK = 0xFFFFFFFFu;

// ---- 1. scanline filters ----------------------------------------------------
constexpr int FILTER_THREADS = 256;
constexpr int FILTER_TILE = 4096;
constexpr int FILTER_HALO = 8;  // >= bytes per pixel

// The five PNG filters on four bytes at once (x: the bytes, a: the bytes
// one pixel to the left, b: above, c: above-left), with CUDA's per-byte SIMD
// arithmetic; every result is the filtered byte modulo 256.
__device__ __forceinline__ uint32_t paeth4(uint32_t a, uint32_t b, uint32_t c) {
  // Paeth predictor: the neighbour closest to p = a + b - c, ties to a, then b;
  // |p - a| = |b - c|, |p - b| = |a - c|, |p - c| = |a + b - 2c| (up to 510),
  // so the bytes are spread over 16-bit lanes, two at a time.
  uint32_t r = 0;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    const int sh = 8 * half;
    const uint32_t A = (a >> sh) & 0x00FF00FFu, B = (b >> sh) & 0x00FF00FFu, C = (c >> sh) & 0x00FF00FFu;
    const uint32_t pa = __vabsdiffu2(B, C);
    const uint32_t pb = __vabsdiffu2(A, C);
    const uint32_t pc = __vabsdiffu2(__vadd2(A, B), __vadd2(C, C));
    const uint32_t use_a = __vcmpleu2(pa, pb) & __vcmpleu2(pa, pc);
    const uint32_t use_b = __vcmpleu2(pb, pc);
    const uint32_t p = (A & use_a) | (~use_a & ((B & use_b) | (C & ~use_b)));
    r |= p << sh;
  }
  return r;
}

__device__ __forceinline__ uint32_t filtered4(int type, uint32_t x, uint32_t a, uint32_t b, uint32_t c) {
  switch (type) {
    case 0: return x;
    case 1: return __vsub4(x, a);
    case 2: return __vsub4(x, b);
    case 3: return __vsub4(x, __vhaddu4(a, b));  // floor((a + b) / 2) per byte
    default: return __vsub4(x, paeth4(a, b, c));
  }
}

// Sum over the bytes selected by `keep` of |filtered byte read as signed|.
__device__ __forceinline__ uint32_t magnitude4(uint32_t f, uint32_t keep) {
  return __vsadu4(__vminu4(f, __vneg4(f)) & keep, 0u);
}

// Bytes t0 - BPP .. t0 + count - 1 of PNG scanline r into
// tile[FILTER_HALO - BPP ...]: 8-bit samples as they are, 16-bit samples most
// significant byte first (the row's memory byte m is line byte m ^ 1); bytes
// before the start of the line are zero. The aligned middle of the span
// arrives in 16-byte loads, so a warp keeps 512 bytes in flight per load;
// the unaligned ends go byte by byte.
template <bool WIDE>
__device__ __forceinline__ void load_scanline_tile(const void* __restrict__ rgb, int W, int r, int64_t t0, int count,
                                                   uint8_t* tile) {
  constexpr int BPP = WIDE ? 6 : 3;
  constexpr int SWAP = WIDE ? 1 : 0;
  const int64_t rb = (int64_t)W * BPP;
  const uint8_t* row = static_cast<const uint8_t*>(rgb) + (int64_t)r * rb;
  const int64_t lo = t0 - BPP, hi = t0 + count;
  uint8_t* dst = tile + FILTER_HALO - BPP;  // dst[p - lo] = line byte p
  const int tid = threadIdx.x;
  if (lo < 0 && tid < -lo) dst[tid] = 0;
  const int64_t start = lo < 0 ? 0 : lo;  // even when WIDE: t0 and BPP are
  const int64_t head = min((int64_t)((16u - ((uintptr_t)(row + start) & 15u)) & 15u), hi - start);
  const int64_t nvec = (hi - start - head) / 16;
  const int64_t body = start + head, tail = body + 16 * nvec;
  for (int64_t m = start + tid; m < body; m += FILTER_THREADS) dst[(m ^ SWAP) - lo] = __ldg(row + m);
  for (int64_t m = tail + tid; m < hi; m += FILTER_THREADS) dst[(m ^ SWAP) - lo] = __ldg(row + m);
  const uint4* vec = reinterpret_cast<const uint4*>(row + body);
  for (int64_t v = tid; v < nvec; v += FILTER_THREADS) {
    const uint4 q = __ldg(vec + v);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
    const int64_t m0 = body + 16 * v;
#pragma unroll
    for (int i = 0; i < 16; ++i) dst[((m0 + i) ^ SWAP) - lo] = (uint8_t)(w[i >> 2] >> (8 * (i & 3)));
  }
}

// Word k of a tile: bytes 4k..4k+3 of it (x), the bytes BPP before (a), and
// the same from the line above (b, c). Tiles start FILTER_HALO bytes into
// their shared arrays, so x is an aligned word and a a funnel shift of two.
template <int BPP>
__device__ __forceinline__ void tile_words(const uint32_t* cur, const uint32_t* up, int k, uint32_t& x,
                                           uint32_t& a, uint32_t& b, uint32_t& c) {
  constexpr int W0 = FILTER_HALO / 4;
  constexpr int AW = (FILTER_HALO - BPP) / 4;        // word holding byte 4k - BPP
  constexpr int AS = 8 * ((FILTER_HALO - BPP) % 4);  // its bit offset there
  x = cur[W0 + k];
  b = up[W0 + k];
  a = __funnelshift_r(cur[AW + k], cur[AW + k + 1], AS);
  c = __funnelshift_r(up[AW + k], up[AW + k + 1], AS);
}

template <bool WIDE>
__global__ void __launch_bounds__(FILTER_THREADS, 5) png_filter_kernel(const void* __restrict__ rgb, int W,
                                                                    uint8_t* __restrict__ stream) {
  constexpr int BPP = WIDE ? 6 : 3;
  __shared__ __align__(16) uint8_t cur[FILTER_HALO + FILTER_TILE];
  __shared__ __align__(16) uint8_t up[FILTER_HALO + FILTER_TILE];
  __shared__ unsigned long long part[FILTER_THREADS / 32][5];
  __shared__ int s_type;
  const int r = blockIdx.x;
  const int64_t rb = (int64_t)W * BPP;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t* cur32 = reinterpret_cast<const uint32_t*>(cur);
  const uint32_t* up32 = reinterpret_cast<const uint32_t*>(up);

  unsigned long long sums[5] = {0, 0, 0, 0, 0};
  for (int64_t t0 = 0; t0 < rb; t0 += FILTER_TILE) {
    const int count = (int)min((int64_t)FILTER_TILE, rb - t0);
    load_scanline_tile<WIDE>(rgb, W, r, t0, count, cur);
    if (r > 0) {
      load_scanline_tile<WIDE>(rgb, W, r - 1, t0, count, up);
    } else {
      for (int j = tid; j < count + BPP; j += FILTER_THREADS) up[FILTER_HALO - BPP + j] = 0;
    }
    __syncthreads();
    uint32_t s[5] = {0, 0, 0, 0, 0};
    for (int k = tid; 4 * k < count; k += FILTER_THREADS) {
      uint32_t x, a, b, c;
      tile_words<BPP>(cur32, up32, k, x, a, b, c);
      const int valid = count - 4 * k;
      const uint32_t keep = valid >= 4 ? 0xFFFFFFFFu : (1u << (8 * valid)) - 1u;  // bytes past the line
      s[0] += magnitude4(x, keep);
      s[1] += magnitude4(__vsub4(x, a), keep);
      s[2] += magnitude4(__vsub4(x, b), keep);
      s[3] += magnitude4(__vsub4(x, __vhaddu4(a, b)), keep);
      s[4] += magnitude4(__vsub4(x, paeth4(a, b, c)), keep);
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) sums[k] += s[k];
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    unsigned long long v = sums[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL_MASK, v, o);
    if (lane == 0) part[warp][k] = v;
  }
  __syncthreads();
  if (tid == 0) {
    int best = 0;
    unsigned long long best_sum = 0;
    for (int k = 0; k < 5; ++k) {
      unsigned long long v = 0;
      for (int w = 0; w < FILTER_THREADS / 32; ++w) v += part[w][k];
      if (k == 0 || v < best_sum) {
        best = k;
        best_sum = v;
      }
    }
    s_type = best;
  }
  __syncthreads();
  const int type = s_type;
  uint8_t* line = stream + (uint64_t)r * (uint64_t)(1 + rb);
  if (tid == 0) line[0] = (uint8_t)type;
  for (int64_t t0 = 0; t0 < rb; t0 += FILTER_TILE) {
    const int count = (int)min((int64_t)FILTER_TILE, rb - t0);
    // A single tile is still resident from the selection pass.
    if (rb > FILTER_TILE) {
      __syncthreads();
      load_scanline_tile<WIDE>(rgb, W, r, t0, count, cur);
      if (r > 0) load_scanline_tile<WIDE>(rgb, W, r - 1, t0, count, up);
      __syncthreads();
    }
    uint8_t* dst = line + 1 + t0;
    for (int k = tid; 4 * k < count; k += FILTER_THREADS) {
      uint32_t x, a, b, c;
      tile_words<BPP>(cur32, up32, k, x, a, b, c);
      const uint32_t f = filtered4(type, x, a, b, c);
      const int valid = min(4, count - 4 * k);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < valid) dst[4 * k + q] = (uint8_t)(f >> (8 * q));
    }
  }
}

// ---- 2. deflate segments -----------------------------------------------------
// Three launches: png_histogram_kernel counts each segment's symbols,
// png_code_kernel builds each segment's Huffman code and block header (one
// warp per segment, so every segment's serial tree construction runs at once),
// png_pack_kernel writes the block. A thread of the per-segment kernels holds
// its 64 bytes in registers; runs of repeated bytes are found with a 64-bit
// mask of the positions where a run cannot continue.
constexpr int DEFLATE_THREADS = SEG / CHUNK;  // 1024
constexpr int DEFLATE_WARPS = DEFLATE_THREADS / 32;
constexpr int HIST_STRIDE = 288;               // literal/length symbols per segment row, padded
constexpr int CODE_WARPS = 4;                  // segments per png_code_kernel CTA

// Code of one segment: its block header (BFINAL, BTYPE and the dynamic
// Huffman header) and the literal/length code.
struct __align__(16) SegCode {
  uint32_t header_bits;
  uint32_t header[HEADER_WORDS];
  uint16_t code[HIST_STRIDE];
  uint8_t len[HIST_STRIDE];
};

struct Chunk {
  uint32_t w[CHUNK_WORDS];
  int c0, count;
  uint64_t breaks;
};

// Bytes [c0, c0 + 64) of the segment that starts at `seg`, n bytes long. The
// stream buffer is padded to 16 bytes and segments start at multiples of SEG,
// so whole 16-byte loads stay inside it; bytes past n are masked by count.
__device__ __forceinline__ void load_chunk(const uint8_t* __restrict__ seg, int n, Chunk& ch) {
  ch.c0 = min((int)threadIdx.x * CHUNK, n);
  ch.count = min(CHUNK, n - ch.c0);
  const uint4* src = reinterpret_cast<const uint4*>(seg + ch.c0);
#pragma unroll
  for (int v = 0; v < CHUNK / 16; ++v) {
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    if (v * 16 < ch.count) q = __ldg(src + v);
    ch.w[4 * v] = q.x;
    ch.w[4 * v + 1] = q.y;
    ch.w[4 * v + 2] = q.z;
    ch.w[4 * v + 3] = q.w;
  }
  const uint32_t prev = ch.c0 > 0 ? seg[ch.c0 - 1] : 0u;
  ch.breaks = chunk_breaks(ch.w, ch.count, prev, ch.c0 == 0);
}

// The last break before this thread's chunk and the first at or after its end
// (n when none), from every thread's chunk breaks. Block-wide: all threads call.
__device__ __forceinline__ void run_bounds(const Chunk& ch, int n, int* s_last, int* s_first, int* before,
                                           int* after) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int pre = ch.breaks ? ch.c0 + 63 - clz64(ch.breaks) : -1;
  int suf = ch.breaks ? ch.c0 + ctz64(ch.breaks) : n;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL_MASK, pre, o);
    if (lane >= o) pre = max(pre, t);
    const int u = __shfl_down_sync(FULL_MASK, suf, o);
    if (lane + o < 32) suf = min(suf, u);
  }
  if (lane == 31) s_last[warp] = pre;
  if (lane == 0) s_first[warp] = suf;
  __syncthreads();
  int b = __shfl_up_sync(FULL_MASK, pre, 1);
  if (lane == 0) b = -1;
  for (int w = 0; w < warp; ++w) b = max(b, s_last[w]);
  int a = __shfl_down_sync(FULL_MASK, suf, 1);
  if (lane == 31) a = n;
  for (int w = warp + 1; w < DEFLATE_WARPS; ++w) a = min(a, s_first[w]);
  *before = b;
  *after = a;
}

__global__ void __launch_bounds__(DEFLATE_THREADS)
    png_histogram_kernel(const uint8_t* __restrict__ stream, uint64_t total, uint32_t nseg,
                         uint32_t* __restrict__ seg_freq, uint2* __restrict__ seg_sums) {
  __shared__ uint32_t hist[DEFLATE_WARPS][HIST_STRIDE];
  __shared__ int s_last[DEFLATE_WARPS], s_first[DEFLATE_WARPS];
  __shared__ unsigned long long s_sums[DEFLATE_WARPS][2];
  const uint32_t seg = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t base = (uint64_t)seg * SEG;
  const int n = (int)min((uint64_t)SEG, total - base);
  for (int i = tid; i < DEFLATE_WARPS * HIST_STRIDE; i += DEFLATE_THREADS) (&hist[0][0])[i] = 0u;
  Chunk ch;
  load_chunk(stream + base, n, ch);
  // Adler-32 partial sums: S1 = sum d_j, S2 = sum (n - j) d_j over the segment.
  unsigned long long s1 = 0, s2 = 0;
#pragma unroll
  for (int j = 0; j < CHUNK; ++j) {
    if (j < ch.count) {
      const uint32_t x = chunk_byte(ch.w, j);
      s1 += x;
      s2 += (unsigned long long)(n - ch.c0 - j) * x;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(FULL_MASK, s1, o);
    s2 += __shfl_down_sync(FULL_MASK, s2, o);
  }
  if (lane == 0) {
    s_sums[warp][0] = s1;
    s_sums[warp][1] = s2;
  }
  int before, after;
  run_bounds(ch, n, s_last, s_first, &before, &after);  // includes a block barrier
  uint32_t* mine = hist[warp];
  chunk_tokens(ch.w, ch.breaks, ch.c0, ch.count, before, after, [&](uint32_t lit, int len) {
    int eb, ev;
    atomicAdd(mine + (len ? length_symbol(len, &eb, &ev) : (int)lit), 1u);
  });
  __syncthreads();
  uint32_t* out = seg_freq + (uint64_t)seg * HIST_STRIDE;
  for (int s = tid; s < HIST_STRIDE; s += DEFLATE_THREADS) {
    uint32_t f = s == END_OF_BLOCK ? 1u : 0u;
    for (int w = 0; w < DEFLATE_WARPS; ++w) f += hist[w][s];
    out[s] = f;
  }
  if (tid == 0) {
    uint32_t a = 0, b = 0;
    for (int w = 0; w < DEFLATE_WARPS; ++w) {
      a = (uint32_t)((a + s_sums[w][0]) % ADLER_MOD);
      b = (uint32_t)((b + s_sums[w][1]) % ADLER_MOD);
    }
    seg_sums[seg] = make_uint2(a, b);
  }
}

struct CodeScratch {
  uint32_t freq[LIT_SYMBOLS];
  uint32_t leaf[LIT_SYMBOLS];
  uint32_t weight[2 * LIT_SYMBOLS];
  uint16_t parent[2 * LIT_SYMBOLS];
  uint16_t order[LIT_SYMBOLS];
  uint16_t code[LIT_SYMBOLS];
  uint8_t len[HIST_STRIDE];
  uint32_t count[MAX_BITS + 1];
  uint32_t next[MAX_BITS + 1];
  HeaderScratch header;
  uint32_t header_words[HEADER_WORDS];
};

// Ascending bitonic sort of 512 keys held 16 per lane (key i = lane * 16 + j):
// compare-exchanges within a lane's registers for partners under 16 apart,
// lane shuffles for the rest.
__device__ __forceinline__ void warp_sort512(uint32_t (&e)[16], int lane) {
#pragma unroll
  for (int k = 2; k <= 512; k <<= 1) {
#pragma unroll
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      if (jj >= 16) {
        const int lm = jj >> 4;
        const bool lower = (lane & lm) == 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const bool asc = ((lane * 16 + j) & k) == 0;
          const uint32_t other = __shfl_xor_sync(FULL_MASK, e[j], lm);
          e[j] = (lower == asc) ? min(e[j], other) : max(e[j], other);
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int p = j ^ jj;
          if (p > j) {
            const bool asc = ((lane * 16 + j) & k) == 0;
            const uint32_t a = e[j], b = e[p];
            e[j] = asc ? min(a, b) : max(a, b);
            e[p] = asc ? max(a, b) : min(a, b);
          }
        }
      }
    }
  }
}

// One warp per segment; no block-wide barrier, so a warp past the last
// segment simply returns.
__global__ void __launch_bounds__(32 * CODE_WARPS)
    png_code_kernel(const uint32_t* __restrict__ seg_freq, uint32_t nseg, SegCode* __restrict__ codes) {
  __shared__ CodeScratch scratch[CODE_WARPS];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t seg = blockIdx.x * CODE_WARPS + warp;
  if (seg >= nseg) return;
  CodeScratch& C = scratch[warp];
  const uint32_t* f = seg_freq + (uint64_t)seg * HIST_STRIDE;
  for (int s = lane; s < HIST_STRIDE; s += 32) {
    if (s < LIT_SYMBOLS) C.freq[s] = f[s];
    C.len[s] = 0;
  }
  for (int i = lane; i < HEADER_WORDS; i += 32) C.header_words[i] = 0u;
  if (lane <= MAX_BITS) C.count[lane] = 0u;
  __syncwarp();
  // Used symbols by ascending (frequency, symbol): keys frequency << 9 | symbol
  // (frequencies are at most SEG + 1 < 2^16), unused symbols last.
  uint32_t keys[16];
  int used = 0;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int sym = lane * 16 + j;
    const uint32_t fs = sym < LIT_SYMBOLS ? C.freq[sym] : 0u;
    keys[j] = fs ? (fs << 9) | (uint32_t)sym : 0xFFFFFFFFu;
    used += fs != 0u;
  }
  for (int o = 16; o > 0; o >>= 1) used += __shfl_xor_sync(FULL_MASK, used, o);
  warp_sort512(keys, lane);
#pragma unroll
  for (int j = 0; j < 16; ++j)
    if (lane * 16 + j < used) C.order[lane * 16 + j] = (uint16_t)(keys[j] & 511u);
  __syncwarp();
  // used >= 2: the end-of-block symbol and the segment's first byte.
  for (int i = lane; i < used; i += 32) C.leaf[i] = C.freq[C.order[i]];
  const int root = 2 * used - 2;
  for (;;) {
    __syncwarp();
    if (lane == 0) huffman_tree(C.leaf, used, C.weight, C.parent);
    __syncwarp();
    int deepest = 0;
    for (int i = lane; i < used; i += 32) {
      int d = 0;
      for (int j = i; j != root; j = C.parent[j]) ++d;
      C.len[C.order[i]] = (uint8_t)d;
      deepest = max(deepest, d);
    }
    for (int o = 16; o > 0; o >>= 1) deepest = max(deepest, __shfl_xor_sync(FULL_MASK, deepest, o));
    if (deepest <= MAX_BITS) break;
    // Too deep: halve the frequencies (rounding up keeps them non-zero and in order) and rebuild.
    for (int i = lane; i < used; i += 32) C.leaf[i] = (C.leaf[i] + 1) >> 1;
  }
  __syncwarp();
  // Canonical codes (RFC 1951 3.2.2): the next code of each length, then each
  // symbol's rank among the symbols of its length.
  for (int s = lane; s < LIT_SYMBOLS; s += 32)
    if (C.len[s]) atomicAdd(&C.count[C.len[s]], 1u);
  __syncwarp();
  if (lane == 0) {
    uint32_t c = 0;
    C.next[0] = 0;
    for (int bits = 1; bits <= MAX_BITS; ++bits) {
      c = (c + (bits > 1 ? C.count[bits - 1] : 0u)) << 1;
      C.next[bits] = c;
    }
  }
  __syncwarp();
  // Symbols in groups of 32, in order: a symbol's rank within its group among
  // those of its length, plus the codes of that length handed out before.
  if (lane <= MAX_BITS) C.count[lane] = 0u;
  __syncwarp();
  for (int g = 0; g < HIST_STRIDE; g += 32) {
    const int sym = g + lane;
    const int l = sym < LIT_SYMBOLS ? C.len[sym] : 0;
    const unsigned same = __match_any_sync(FULL_MASK, l);
    const uint32_t ahead = (uint32_t)__popc(same & ((1u << lane) - 1u));
    if (sym < LIT_SYMBOLS) C.code[sym] = l ? (uint16_t)reverse_bits(C.next[l] + C.count[l] + ahead, l) : (uint16_t)0;
    __syncwarp();
    if (l && ahead == 0) C.count[l] += (uint32_t)__popc(same);
    __syncwarp();
  }
  uint32_t header_bits = 0;
  if (lane == 0) {
    BitWriter w{C.header_words, 0};
    header_bits = write_dynamic_header(w, seg + 1 == nseg, C.len, C.header);
  }
  header_bits = __shfl_sync(FULL_MASK, header_bits, 0);
  __syncwarp();
  SegCode& out = codes[seg];
  if (lane == 0) out.header_bits = header_bits;
  for (int i = lane; i < HEADER_WORDS; i += 32) out.header[i] = C.header_words[i];
  for (int s = lane; s < HIST_STRIDE; s += 32) {
    out.code[s] = s < LIT_SYMBOLS ? C.code[s] : (uint16_t)0;
    out.len[s] = C.len[s];
  }
}

__global__ void __launch_bounds__(DEFLATE_THREADS)
    png_pack_kernel(const uint8_t* __restrict__ stream, uint64_t total, uint32_t nseg,
                    const SegCode* __restrict__ codes, uint8_t* __restrict__ slots, uint32_t* __restrict__ seg_bytes) {
  __shared__ __align__(16) uint32_t out[SEG_CAP / 4];
  __shared__ uint32_t s_sym[HIST_STRIDE];  // code | length << 16
  __shared__ int s_last[DEFLATE_WARPS], s_first[DEFLATE_WARPS];
  __shared__ uint32_t s_bits[DEFLATE_WARPS];
  const uint32_t seg = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t base = (uint64_t)seg * SEG;
  const int n = (int)min((uint64_t)SEG, total - base);
  const bool last = seg + 1 == nseg;
  const SegCode& sc = codes[seg];
  const uint32_t header_bits = sc.header_bits;
  for (int i = tid; i < SEG_CAP / 4; i += DEFLATE_THREADS) out[i] = i < HEADER_WORDS ? sc.header[i] : 0u;
  for (int s = tid; s < HIST_STRIDE; s += DEFLATE_THREADS) s_sym[s] = sc.code[s] | ((uint32_t)sc.len[s] << 16);
  Chunk ch;
  load_chunk(stream + base, n, ch);
  int before, after;
  run_bounds(ch, n, s_last, s_first, &before, &after);  // includes a block barrier

  // Bit offsets of each thread's tokens.
  uint32_t bits = 0;
  chunk_tokens(ch.w, ch.breaks, ch.c0, ch.count, before, after, [&](uint32_t lit, int len) {
    if (len) {
      int eb, ev;
      bits += (s_sym[length_symbol(len, &eb, &ev)] >> 16) + eb + 1;  // distance symbol 0: one bit
    } else {
      bits += s_sym[lit] >> 16;
    }
  });
  uint32_t incl = bits;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL_MASK, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) s_bits[warp] = incl;
  __syncthreads();
  uint32_t offset = header_bits + incl - bits;
  uint32_t token_bits = 0;
  for (int w = 0; w < DEFLATE_WARPS; ++w) {
    if (w < warp) offset += s_bits[w];
    token_bits += s_bits[w];
  }
  const uint32_t eob_at = header_bits + token_bits;
  const uint32_t end = eob_at + (s_sym[END_OF_BLOCK] >> 16);
  // After the last block the stream pads to a byte; after any other, an empty
  // stored block (3 zero bits, padding, LEN 0, NLEN 0xFFFF) realigns it.
  const uint32_t dyn_bytes = last ? (end + 7) / 8 : (end + 3 + 7) / 8 + 4;
  const uint32_t stored_bytes = (uint32_t)n + STORED_OVERHEAD;
  const bool stored = dyn_bytes >= stored_bytes;  // the same in every thread

  if (!stored) {
    // The thread's bits gather in a 64-bit accumulator that starts at its
    // offset's position within a word; each full word is ORed out (the first
    // and last words of a thread's range are shared with its neighbours').
    uint32_t word = offset >> 5;
    unsigned long long acc = 0;
    int held = (int)(offset & 31u);
    auto emit = [&](uint32_t value, int n) {  // n <= 21, so held stays below 64
      acc |= (unsigned long long)value << held;
      held += n;
      if (held >= 32) {
        if ((uint32_t)acc) atomicOr(out + word, (uint32_t)acc);
        ++word;
        acc >>= 32;
        held -= 32;
      }
    };
    chunk_tokens(ch.w, ch.breaks, ch.c0, ch.count, before, after, [&](uint32_t lit, int len) {
      if (len) {
        int eb, ev;
        const uint32_t e = s_sym[length_symbol(len, &eb, &ev)];
        const int l = (int)(e >> 16);
        // length code, extra bits, then distance symbol 0's one-bit code 0
        emit((e & 0xFFFFu) | ((uint32_t)ev << l), l + eb + 1);
      } else {
        const uint32_t e = s_sym[lit];
        emit(e & 0xFFFFu, (int)(e >> 16));
      }
    });
    if (held > 0 && (uint32_t)acc) atomicOr(out + word, (uint32_t)acc);
    __syncthreads();
    if (tid == 0) {
      BitWriter w{out, eob_at};
      w.put(s_sym[END_OF_BLOCK] & 0xFFFFu, (int)(s_sym[END_OF_BLOCK] >> 16));
      if (!last) {
        uint8_t* bytes = reinterpret_cast<uint8_t*>(out);
        const uint32_t at = (end + 3 + 7) / 8;
        bytes[at + 2] = 0xFF;
        bytes[at + 3] = 0xFF;
      }
    }
  } else {
    // Every thread has read the header words; the block is rewritten as a stored one.
    for (int i = tid; i < HEADER_WORDS; i += DEFLATE_THREADS) out[i] = 0u;
    __syncthreads();
    uint8_t* bytes = reinterpret_cast<uint8_t*>(out);
    if (tid == 0) {
      bytes[0] = last ? 1 : 0;  // BFINAL, BTYPE 00
      bytes[1] = (uint8_t)n;
      bytes[2] = (uint8_t)(n >> 8);
      bytes[3] = (uint8_t)~n;
      bytes[4] = (uint8_t)(~n >> 8);
    }
#pragma unroll
    for (int j = 0; j < CHUNK; ++j)
      if (j < ch.count) bytes[STORED_OVERHEAD + ch.c0 + j] = (uint8_t)chunk_byte(ch.w, j);
  }
  __syncthreads();
  const uint32_t nbytes = stored ? stored_bytes : dyn_bytes;
  uint4* slot = reinterpret_cast<uint4*>(slots + (uint64_t)seg * SEG_CAP);
  const uint4* src = reinterpret_cast<const uint4*>(out);
  for (uint32_t i = tid; i < (nbytes + 15) / 16; i += DEFLATE_THREADS) slot[i] = src[i];
  if (tid == 0) seg_bytes[seg] = nbytes;
}

// ---- 3. file layout ---------------------------------------------------------
constexpr int LAYOUT_THREADS = 1024;

__device__ __forceinline__ uint64_t idat_chunk_bytes(const uint32_t* seg_bytes, uint32_t s, uint32_t nseg) {
  return 12ull + seg_bytes[s] + (s == 0 ? 2u : 0u) + (s + 1 == nseg ? 4u : 0u);
}

__global__ void __launch_bounds__(LAYOUT_THREADS)
    png_layout_kernel(const uint32_t* __restrict__ seg_bytes, const uint2* __restrict__ seg_sums, uint32_t nseg,
                      uint64_t total, uint64_t header_bytes, uint32_t iend_crc, uint64_t* __restrict__ chunk_at,
                      uint32_t* __restrict__ adler_out, uint64_t* __restrict__ png_bytes, uint8_t* __restrict__ png) {
  __shared__ unsigned long long warp_sum[LAYOUT_THREADS / 32][3];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = (nseg + LAYOUT_THREADS - 1) / LAYOUT_THREADS;
  const uint32_t s0 = min((uint32_t)tid * per, nseg), s1 = min(s0 + per, nseg);
  unsigned long long mine = 0, a = 0, b = 0;
  for (uint32_t s = s0; s < s1; ++s) {
    mine += idat_chunk_bytes(seg_bytes, s, nseg);
    const uint64_t o = (uint64_t)s * SEG;
    const uint64_t n = min((uint64_t)SEG, total - o);
    const uint2 q = seg_sums[s];
    a += q.x;
    b = (b + adler_combine_term(total, o, n, q.x, q.y)) % ADLER_MOD;
  }
  unsigned long long incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(FULL_MASK, incl, o);
    if (lane >= o) incl += t;
  }
  unsigned long long ra = a, rbv = b;
  for (int o = 16; o > 0; o >>= 1) {
    ra += __shfl_down_sync(FULL_MASK, ra, o);
    rbv += __shfl_down_sync(FULL_MASK, rbv, o);
  }
  if (lane == 31) warp_sum[warp][0] = incl;
  if (lane == 0) {
    warp_sum[warp][1] = ra;
    warp_sum[warp][2] = rbv;
  }
  __syncthreads();
  unsigned long long at = header_bytes + incl - mine, all = 0;
  for (int w = 0; w < LAYOUT_THREADS / 32; ++w) {
    if (w < warp) at += warp_sum[w][0];
    all += warp_sum[w][0];
  }
  for (uint32_t s = s0; s < s1; ++s) {
    chunk_at[s] = at;
    at += idat_chunk_bytes(seg_bytes, s, nseg);
  }
  if (tid == 0) {
    unsigned long long asum = 0, bsum = 0;
    for (int w = 0; w < LAYOUT_THREADS / 32; ++w) {
      asum += warp_sum[w][1];
      bsum += warp_sum[w][2];
    }
    const uint32_t A = (uint32_t)((1ull + asum) % ADLER_MOD);
    const uint32_t B = (uint32_t)((total % ADLER_MOD + bsum) % ADLER_MOD);
    *adler_out = (B << 16) | A;
    const uint64_t size = header_bytes + all + 12;
    *png_bytes = size;
    uint8_t* iend = png + size - 12;
    const uint8_t fixed[8] = {0, 0, 0, 0, 'I', 'E', 'N', 'D'};
    for (int k = 0; k < 8; ++k) iend[k] = fixed[k];
    for (int k = 0; k < 4; ++k) iend[8 + k] = (uint8_t)(iend_crc >> (24 - 8 * k));
  }
}

// ---- 4. IDAT chunks ----------------------------------------------------------
constexpr int CHUNK_THREADS = 256;

struct ChunkParams {
  const uint8_t* slots;
  const uint32_t* seg_bytes;
  const uint64_t* chunk_at;
  const uint32_t* adler;
  uint8_t* png;
  uint32_t nseg;
  CrcShifts shifts;
};

__global__ void __launch_bounds__(CHUNK_THREADS) png_chunk_kernel(const __grid_constant__ ChunkParams P) {
  __shared__ __align__(16) uint8_t buf[SEG_CAP + 32];
  __shared__ uint32_t table[256];
  __shared__ uint32_t warp_crc[CHUNK_THREADS / 32];
  const uint32_t s = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool first = s == 0, last = s + 1 == P.nseg;
  const uint32_t nb = P.seg_bytes[s];
  const uint32_t dl = nb + (first ? 2u : 0u) + (last ? 4u : 0u);  // chunk data bytes
  const uint32_t size = dl + 12;
  table[tid] = crc_byte_entry((uint32_t)tid);
  if (tid == 0) {
    for (int k = 0; k < 4; ++k) buf[k] = (uint8_t)(dl >> (24 - 8 * k));
    buf[4] = 'I';
    buf[5] = 'D';
    buf[6] = 'A';
    buf[7] = 'T';
    if (first) {
      buf[8] = 0x78;  // deflate, 32 KiB window
      buf[9] = 0x9C;  // default level, no dictionary; 0x789C is a multiple of 31
    }
    if (last) {
      const uint32_t adler = *P.adler;
      for (int k = 0; k < 4; ++k) buf[8 + dl - 4 + k] = (uint8_t)(adler >> (24 - 8 * k));
    }
  }
  const uint32_t d0 = first ? 10u : 8u;
  const uint4* src = reinterpret_cast<const uint4*>(P.slots + (uint64_t)s * SEG_CAP);
  for (uint32_t v = tid; v < (nb + 15) / 16; v += CHUNK_THREADS) {
    const uint4 q = __ldg(src + v);
    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const uint32_t i = v * 16 + k;
      if (i < nb) buf[d0 + i] = (uint8_t)(w[k >> 2] >> (8 * (k & 3)));
    }
  }
  __syncthreads();
  // CRC-32 over the chunk type and data, each thread over its own bytes.
  const uint32_t crc_len = 4 + dl;
  const uint32_t per = (crc_len + CHUNK_THREADS - 1) / CHUNK_THREADS;
  const uint32_t b0 = min((uint32_t)tid * per, crc_len), b1 = min(b0 + per, crc_len);
  uint32_t part = 0;
  if (b1 > b0) part = crc_shift(P.shifts, crc_update(table, 0u, buf + 4 + b0, b1 - b0), crc_len - b1);
  if (tid == 0) part ^= crc_shift(P.shifts, 0xFFFFFFFFu, crc_len);
  for (int o = 16; o > 0; o >>= 1) part ^= __shfl_down_sync(FULL_MASK, part, o);
  if (lane == 0) warp_crc[warp] = part;
  __syncthreads();
  if (tid == 0) {
    uint32_t reg = 0;
    for (int w = 0; w < CHUNK_THREADS / 32; ++w) reg ^= warp_crc[w];
    const uint32_t crc = reg ^ 0xFFFFFFFFu;
    for (int k = 0; k < 4; ++k) buf[8 + dl + k] = (uint8_t)(crc >> (24 - 8 * k));
  }
  __syncthreads();
  // Whole 32-bit words inside the chunk are stored as words; the bytes at
  // either end share a word with the neighbouring chunk and go one by one.
  const uint64_t at = P.chunk_at[s];
  uint8_t* out = P.png + at;
  const uint32_t head = min((uint32_t)((4u - (uint32_t)(at & 3u)) & 3u), size);
  const uint32_t words = (size - head) / 4;
  for (uint32_t i = tid; i < head; i += CHUNK_THREADS) out[i] = buf[i];
  uint32_t* ow = reinterpret_cast<uint32_t*>(out + head);
  for (uint32_t w = tid; w < words; w += CHUNK_THREADS) {
    const uint32_t k = head + 4 * w;
    ow[w] = (uint32_t)buf[k] | ((uint32_t)buf[k + 1] << 8) | ((uint32_t)buf[k + 2] << 16) |
            ((uint32_t)buf[k + 3] << 24);
  }
  for (uint32_t i = head + 4 * words + tid; i < size; i += CHUNK_THREADS) out[i] = buf[i];
}

// ---- host: chunks built on the CPU ----------------------------------------
struct HostCrc {
  uint32_t table[256];
  HostCrc() {
    for (uint32_t i = 0; i < 256; ++i) table[i] = crc_byte_entry(i);
  }
  uint32_t operator()(const uint8_t* p, size_t n) const { return crc_update(table, 0xFFFFFFFFu, p, n) ^ 0xFFFFFFFFu; }
};

const HostCrc& host_crc() {
  static const HostCrc crc;
  return crc;
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
  for (int k = 0; k < 4; ++k) v.push_back((uint8_t)(x >> (24 - 8 * k)));
}

void add_chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put_be32(out, (uint32_t)data.size());
  const size_t at = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put_be32(out, host_crc()(out.data() + at, 4 + data.size()));
}

// A zlib stream of stored deflate blocks (RFC 1950/1951): the profile is a
// few kilobytes and rides uncompressed inside its wrapper.
std::vector<uint8_t> zlib_stored(const uint8_t* p, size_t n) {
  std::vector<uint8_t> z = {0x78, 0x01};
  size_t at = 0;
  do {
    const size_t len = std::min<size_t>(65535, n - at);
    const bool final_block = at + len == n;
    z.push_back(final_block ? 1 : 0);
    z.push_back((uint8_t)len);
    z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)~len);
    z.push_back((uint8_t)(~len >> 8));
    z.insert(z.end(), p + at, p + at + len);
    at += len;
  } while (at < n);
  uint32_t a = 1, b = 0;
  for (size_t i = 0; i < n; ++i) {
    a = (a + p[i]) % ADLER_MOD;
    b = (b + a) % ADLER_MOD;
  }
  put_be32(z, (b << 16) | a);
  return z;
}

const char* ICC_PROFILE_NAME = "ICC profile";

}  // namespace

uint64_t png_stream_bytes(int W, int H, int depth) { return (uint64_t)H * (1ull + (uint64_t)W * (depth / 8) * 3); }

uint64_t png_segments(uint64_t stream_bytes) { return (stream_bytes + SEG - 1) / SEG; }

// Largest metadata a PNG chunk carries: the chunk length is a 31-bit count
// and the profile's chunk adds its name and zlib framing.
constexpr uint64_t PNG_METADATA_LIMIT = 0x7FF00000ull;

bool png_metadata_ok(uint64_t icc_len, uint64_t exif_len) {
  return icc_len <= PNG_METADATA_LIMIT && exif_len <= PNG_METADATA_LIMIT;
}

uint64_t png_header_bytes(uint64_t icc_len, uint64_t exif_len) {
  uint64_t n = 8 + 25;  // signature, IHDR
  if (icc_len) {
    const uint64_t blocks = (icc_len + 65534) / 65535;
    n += 12 + std::strlen(ICC_PROFILE_NAME) + 2 + 2 + 5 * blocks + icc_len + 4;
  }
  if (exif_len) n += 12 + exif_len;
  return n;
}

Status png_header(int W, int H, int depth, const uint8_t* icc, size_t icc_len, const uint8_t* exif, size_t exif_len,
                  std::vector<uint8_t>* out) {
  if (!png_metadata_ok(icc_len, exif_len)) return Status{RD_INVALID_INPUT, "metadata too large for a PNG chunk"};
  std::vector<uint8_t>& h = *out;
  h = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  std::vector<uint8_t> ihdr;
  put_be32(ihdr, (uint32_t)W);
  put_be32(ihdr, (uint32_t)H);
  ihdr.push_back((uint8_t)depth);
  ihdr.push_back(2);  // truecolour RGB
  ihdr.push_back(0);  // deflate
  ihdr.push_back(0);  // adaptive filtering with the five basic filters
  ihdr.push_back(0);  // no interlace
  add_chunk(h, "IHDR", ihdr);
  if (icc && icc_len) {
    std::vector<uint8_t> iccp(ICC_PROFILE_NAME, ICC_PROFILE_NAME + std::strlen(ICC_PROFILE_NAME));
    iccp.push_back(0);  // name terminator
    iccp.push_back(0);  // compression method: zlib
    const std::vector<uint8_t> z = zlib_stored(icc, icc_len);
    iccp.insert(iccp.end(), z.begin(), z.end());
    if (iccp.size() > 0x7FFFFFFFu) return Status{RD_INVALID_INPUT, "ICC profile does not fit in a PNG chunk"};
    add_chunk(h, "iCCP", iccp);
  }
  if (exif && exif_len) {
    if (exif_len > 0x7FFFFFFFu) return Status{RD_INVALID_INPUT, "EXIF block does not fit in a PNG chunk"};
    add_chunk(h, "eXIf", std::vector<uint8_t>(exif, exif + exif_len));
  }
  return Status{};
}

uint64_t png_bound(int W, int H, int depth, uint64_t header_bytes) {
  const uint64_t L = png_stream_bytes(W, H, depth);
  const uint64_t nseg = png_segments(L);
  // Each segment is at most a stored block; zlib header and Adler-32; IEND.
  return header_bytes + L + nseg * (12 + STORED_OVERHEAD) + 6 + 12;
}

Status run_png_encode(Context& ctx, const void* d_rgb, int W, int H, int depth, const std::vector<uint8_t>& header,
                      uint8_t* d_png, uint64_t* d_png_bytes) {
  const uint64_t L = png_stream_bytes(W, H, depth);
  const uint64_t nseg = png_segments(L);
  if (nseg > 0x7FFFFFFFull) return Status{RD_INVALID_DIMENSIONS, "image too large for one PNG stream"};
  auto round16 = [](uint64_t v) { return (v + 15) & ~15ull; };
  const uint64_t stream_bytes = round16(L);
  const uint64_t slot_bytes = nseg * SEG_CAP;
  const uint64_t count_bytes = round16(nseg * 4);
  const uint64_t sum_bytes = round16(nseg * 8);
  const uint64_t at_bytes = round16(nseg * 8);
  const uint64_t freq_bytes = round16(nseg * HIST_STRIDE * 4);
  const uint64_t code_bytes = nseg * sizeof(SegCode);
  const uint64_t total = stream_bytes + slot_bytes + count_bytes + sum_bytes + at_bytes + 16 + freq_bytes + code_bytes;
  void* scratch = nullptr;
  RD_TRY(device_alloc(ctx, total, &scratch));
  uint8_t* p = static_cast<uint8_t*>(scratch);
  uint8_t* stream = p;
  uint8_t* slots = stream + stream_bytes;
  uint32_t* seg_bytes = reinterpret_cast<uint32_t*>(slots + slot_bytes);
  uint2* seg_sums = reinterpret_cast<uint2*>(reinterpret_cast<uint8_t*>(seg_bytes) + count_bytes);
  uint64_t* chunk_at = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(seg_sums) + sum_bytes);
  uint32_t* adler = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(chunk_at) + at_bytes);
  uint32_t* seg_freq = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(adler) + 16);
  SegCode* codes = reinterpret_cast<SegCode*>(reinterpret_cast<uint8_t*>(seg_freq) + freq_bytes);

  Status st = upload(ctx, d_png, header.data(), header.size());
  if (st.ok()) {
    if (depth == 16) {
      RD_LAUNCH(ctx, K_ENCODE, png_filter_kernel<true><<<H, FILTER_THREADS, 0, ctx.stream>>>(d_rgb, W, stream));
    } else {
      RD_LAUNCH(ctx, K_ENCODE, png_filter_kernel<false><<<H, FILTER_THREADS, 0, ctx.stream>>>(d_rgb, W, stream));
    }
    RD_LAUNCH(ctx, K_ENCODE,
              png_histogram_kernel<<<(unsigned)nseg, DEFLATE_THREADS, 0, ctx.stream>>>(stream, L, (uint32_t)nseg,
                                                                                     seg_freq, seg_sums));
    RD_LAUNCH(ctx, K_ENCODE,
              png_code_kernel<<<(unsigned)((nseg + CODE_WARPS - 1) / CODE_WARPS), 32 * CODE_WARPS, 0, ctx.stream>>>(
                  seg_freq, (uint32_t)nseg, codes));
    RD_LAUNCH(ctx, K_ENCODE,
              png_pack_kernel<<<(unsigned)nseg, DEFLATE_THREADS, 0, ctx.stream>>>(stream, L, (uint32_t)nseg, codes,
                                                                                slots, seg_bytes));
    const uint32_t iend_crc = host_crc()(reinterpret_cast<const uint8_t*>("IEND"), 4);
    RD_LAUNCH(ctx, K_ENCODE,
              png_layout_kernel<<<1, LAYOUT_THREADS, 0, ctx.stream>>>(seg_bytes, seg_sums, (uint32_t)nseg, L,
                                                                      header.size(), iend_crc, chunk_at, adler,
                                                                      d_png_bytes, d_png));
    ChunkParams cp{};
    cp.slots = slots;
    cp.seg_bytes = seg_bytes;
    cp.chunk_at = chunk_at;
    cp.adler = adler;
    cp.png = d_png;
    cp.nseg = (uint32_t)nseg;
    crc_shift_table(cp.shifts);
    RD_LAUNCH(ctx, K_ENCODE, png_chunk_kernel<<<(unsigned)nseg, CHUNK_THREADS, 0, ctx.stream>>>(cp));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = Status{RD_SYNCHRONIZATION, std::string("PNG encode launch: ") + cudaGetErrorString(e)};
  }
  device_free(ctx, scratch, total);
  return st;
}

}  // namespace rd
