// PNG encoding of the export's interleaved RGB rows, on the device.
//
// Replaces the PNG arms of export::encode (crates/core/src/export.rs:176-211):
// the reference hands tightly packed 8-bit or 16-bit RGB rows, the ICC
// profile of the output colour space and optional EXIF to the `image`
// crate's PngEncoder (image 0.25, Cargo.toml:39; not vendored). The file here
// decodes to exactly those samples and carries the same metadata chunks; the
// compressed bytes are this encoder's own (any PNG encoder's are).
//
// Four launches on the context's stream:
//  1. png_filter_kernel   one CTA per scanline: PNG filter selection by the
//                         minimum sum of absolute filtered values (the
//                         heuristic the PNG specification recommends, ties to
//                         the lower filter type), then the filtered scanline
//                         with its filter byte into the stream buffer;
//  2. png_deflate_kernel  one CTA per 32 KiB segment of the stream: one
//                         byte-aligned deflate block each (deflate.cuh), and
//                         the segment's Adler-32 partial sums;
//  3. png_layout_kernel   one CTA: prefix sum of the IDAT chunk sizes, the
//                         stream's Adler-32, the IEND chunk;
//  4. png_chunk_kernel    one CTA per segment: the IDAT chunk (length, type,
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

__device__ __forceinline__ uint32_t magnitude(int v) {
  const uint32_t b = (uint32_t)v & 0xFFu;  // the filtered byte, read as a signed value
  return b < 128u ? b : 256u - b;
}

// PNG Paeth predictor: the neighbour closest to a + b - c, ties to a, then b.
__device__ __forceinline__ int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

__device__ __forceinline__ int filtered(int type, int x, int a, int b, int c) {
  switch (type) {
    case 0: return x;
    case 1: return x - a;
    case 2: return x - b;
    case 3: return x - ((a + b) >> 1);
    default: return x - paeth(a, b, c);
  }
}

// Bytes t0 - BPP .. t0 + count - 1 of PNG scanline r into tile[FILTER_HALO - BPP ...]:
// 8-bit samples as they are, 16-bit samples most significant byte first.
// Bytes before the start of the line are zero.
template <bool WIDE>
__device__ __forceinline__ void load_scanline_tile(const void* __restrict__ rgb, int W, int r, int64_t t0, int count,
                                                   uint8_t* tile) {
  constexpr int BPP = WIDE ? 6 : 3;
  if (WIDE) {
    const uint16_t* row = static_cast<const uint16_t*>(rgb) + (int64_t)r * 3 * W;
    const int64_t s0 = (t0 - BPP) / 2;  // t0 and BPP are even
    const int samples = (count + BPP) / 2;
    for (int j = threadIdx.x; j < samples; j += FILTER_THREADS) {
      const int64_t s = s0 + j;
      const uint32_t v = s >= 0 ? __ldg(row + s) : 0u;
      tile[FILTER_HALO - BPP + 2 * j] = (uint8_t)(v >> 8);
      tile[FILTER_HALO - BPP + 2 * j + 1] = (uint8_t)v;
    }
  } else {
    const uint8_t* row = static_cast<const uint8_t*>(rgb) + (int64_t)r * 3 * W;
    for (int j = threadIdx.x; j < count + BPP; j += FILTER_THREADS) {
      const int64_t q = t0 - BPP + j;
      tile[FILTER_HALO - BPP + j] = q >= 0 ? __ldg(row + q) : (uint8_t)0;
    }
  }
}

template <bool WIDE>
__global__ void __launch_bounds__(FILTER_THREADS) png_filter_kernel(const void* __restrict__ rgb, int W,
                                                                    uint8_t* __restrict__ stream) {
  constexpr int BPP = WIDE ? 6 : 3;
  __shared__ uint8_t cur[FILTER_HALO + FILTER_TILE];
  __shared__ uint8_t up[FILTER_HALO + FILTER_TILE];
  __shared__ unsigned long long part[FILTER_THREADS / 32][5];
  __shared__ int s_type;
  const int r = blockIdx.x;
  const int64_t rb = (int64_t)W * BPP;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

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
    for (int i = tid; i < count; i += FILTER_THREADS) {
      const int x = cur[FILTER_HALO + i], a = cur[FILTER_HALO + i - BPP];
      const int b = up[FILTER_HALO + i], c = up[FILTER_HALO + i - BPP];
      s[0] += magnitude(x);
      s[1] += magnitude(x - a);
      s[2] += magnitude(x - b);
      s[3] += magnitude(x - ((a + b) >> 1));
      s[4] += magnitude(x - paeth(a, b, c));
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
    for (int i = tid; i < count; i += FILTER_THREADS) {
      const int x = cur[FILTER_HALO + i], a = cur[FILTER_HALO + i - BPP];
      const int b = up[FILTER_HALO + i], c = up[FILTER_HALO + i - BPP];
      line[1 + t0 + i] = (uint8_t)filtered(type, x, a, b, c);
    }
  }
}

// ---- 2. deflate segments ----------------------------------------------------
constexpr int DEFLATE_THREADS = 512;
constexpr int DEFLATE_PER = SEG / DEFLATE_THREADS;  // stream bytes per thread
constexpr int DEFLATE_WARPS = DEFLATE_THREADS / 32;

struct __align__(16) DeflateSmem {
  uint8_t in[SEG];
  uint32_t out[SEG_CAP / 4];
  uint32_t freq[LIT_SYMBOLS];
  uint32_t leaf[LIT_SYMBOLS];
  uint32_t weight[2 * LIT_SYMBOLS];
  uint16_t parent[2 * LIT_SYMBOLS];
  uint16_t order[LIT_SYMBOLS];
  uint16_t code[LIT_SYMBOLS];
  uint8_t depth[2 * LIT_SYMBOLS];
  uint8_t len[LIT_SYMBOLS];
  HeaderScratch header;
  int last_break[DEFLATE_WARPS];
  int first_break[DEFLATE_WARPS];
  uint32_t warp_bits[DEFLATE_WARPS];
  unsigned long long warp_sums[DEFLATE_WARPS][2];
  uint32_t header_bits;
};

// Bits are ORed into shared words that neighbouring threads' tokens share.
__device__ __forceinline__ void put_bits_shared(uint32_t* words, uint32_t pos, uint32_t value, int bits) {
  if (bits == 0 || value == 0) return;
  const unsigned long long v = (unsigned long long)value << (pos & 31u);
  atomicOr(words + (pos >> 5), (uint32_t)v);
  if ((uint32_t)(v >> 32)) atomicOr(words + (pos >> 5) + 1, (uint32_t)(v >> 32));
}

__global__ void __launch_bounds__(DEFLATE_THREADS, 2)
    png_deflate_kernel(const uint8_t* __restrict__ stream, uint64_t total, uint32_t nseg, uint8_t* __restrict__ slots,
                       uint32_t* __restrict__ seg_bytes, uint2* __restrict__ seg_sums) {
  extern __shared__ __align__(16) unsigned char deflate_smem[];
  DeflateSmem& S = *reinterpret_cast<DeflateSmem*>(deflate_smem);
  const uint32_t seg = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t base = (uint64_t)seg * SEG;
  const int n = (int)min((uint64_t)SEG, total - base);
  const bool last = seg + 1 == nseg;

  {
    // The stream buffer is padded to 16 bytes, and segments start at multiples of SEG.
    const uint4* src = reinterpret_cast<const uint4*>(stream + base);
    uint4* dst = reinterpret_cast<uint4*>(S.in);
    const int vecs = (n + 15) >> 4;
    for (int i = tid; i < vecs; i += DEFLATE_THREADS) dst[i] = __ldg(src + i);
  }
  for (int i = tid; i < SEG_CAP / 4; i += DEFLATE_THREADS) S.out[i] = 0;
  for (int i = tid; i < LIT_SYMBOLS; i += DEFLATE_THREADS) S.freq[i] = i == END_OF_BLOCK ? 1u : 0u;
  __syncthreads();

  // Run boundaries around this thread's bytes, and the Adler-32 partial sums.
  const int c0 = min(tid * DEFLATE_PER, n);
  const int c1 = min(c0 + DEFLATE_PER, n);
  int first_break = n, last_break = -1;
  unsigned long long s1 = 0, s2 = 0;
  for (int p = c0; p < c1; ++p) {
    const uint32_t x = S.in[p];
    if (p == 0 || x != S.in[p - 1]) {
      if (first_break == n) first_break = p;
      last_break = p;
    }
    s1 += x;
    s2 += (unsigned long long)(n - p) * x;
  }
  int pre = last_break, suf = first_break;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL_MASK, pre, o);
    if (lane >= o) pre = max(pre, t);
    const int u = __shfl_down_sync(FULL_MASK, suf, o);
    if (lane + o < 32) suf = min(suf, u);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_down_sync(FULL_MASK, s1, o);
    s2 += __shfl_down_sync(FULL_MASK, s2, o);
  }
  if (lane == 31) S.last_break[warp] = pre;
  if (lane == 0) {
    S.first_break[warp] = suf;
    S.warp_sums[warp][0] = s1;
    S.warp_sums[warp][1] = s2;
  }
  __syncthreads();
  int before = __shfl_up_sync(FULL_MASK, pre, 1);
  if (lane == 0) before = -1;
  for (int w = 0; w < warp; ++w) before = max(before, S.last_break[w]);
  int after = __shfl_down_sync(FULL_MASK, suf, 1);
  if (lane == 31) after = n;
  for (int w = warp + 1; w < DEFLATE_WARPS; ++w) after = min(after, S.first_break[w]);

  // Symbol frequencies.
  for_each_token(S.in, c0, c1, before, after, [&](uint32_t lit, int len) {
    if (len) {
      int eb, ev;
      atomicAdd(&S.freq[length_symbol(len, &eb, &ev)], 1u);
    } else {
      atomicAdd(&S.freq[lit], 1u);
    }
  });
  __syncthreads();

  // Used symbols by ascending (frequency, symbol), then the code and the block header.
  if (tid < LIT_SYMBOLS) {
    const uint32_t f = S.freq[tid];
    if (f) {
      int rank = 0;
      for (int s = 0; s < LIT_SYMBOLS; ++s) {
        const uint32_t g = S.freq[s];
        rank += (g != 0u) & ((g < f) | ((g == f) & (s < tid)));
      }
      S.order[rank] = (uint16_t)tid;
    }
    S.len[tid] = 0;
  }
  __syncthreads();
  if (tid == 0) {
    int used = 0;
    for (int s = 0; s < LIT_SYMBOLS; ++s) used += S.freq[s] != 0u;
    // used >= 2: the end-of-block symbol and the segment's first byte.
    huffman_lengths(S.freq, S.order, used, MAX_BITS, S.leaf, S.weight, S.parent, S.depth, S.len);
    canonical_codes(S.len, LIT_SYMBOLS, MAX_BITS, S.code);
    BitWriter w{S.out, 0};
    S.header_bits = write_dynamic_header(w, last, S.len, S.header);
    uint32_t s1_total = 0, s2_total = 0;
    for (int v = 0; v < DEFLATE_WARPS; ++v) {
      s1_total = (uint32_t)((s1_total + S.warp_sums[v][0]) % ADLER_MOD);
      s2_total = (uint32_t)((s2_total + S.warp_sums[v][1]) % ADLER_MOD);
    }
    seg_sums[seg] = make_uint2(s1_total, s2_total);
  }
  __syncthreads();

  // Bit offsets of each thread's tokens.
  uint32_t bits = 0;
  for_each_token(S.in, c0, c1, before, after, [&](uint32_t lit, int len) {
    if (len) {
      int eb, ev;
      bits += S.len[length_symbol(len, &eb, &ev)] + eb + 1;  // distance symbol 0: one bit
    } else {
      bits += S.len[lit];
    }
  });
  uint32_t incl = bits;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL_MASK, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) S.warp_bits[warp] = incl;
  __syncthreads();
  uint32_t offset = S.header_bits + incl - bits;
  uint32_t token_bits = 0;
  for (int w = 0; w < DEFLATE_WARPS; ++w) {
    if (w < warp) offset += S.warp_bits[w];
    token_bits += S.warp_bits[w];
  }
  const uint32_t eob_at = S.header_bits + token_bits;
  const uint32_t end = eob_at + S.len[END_OF_BLOCK];
  // After the last block the stream pads to a byte; after any other, an empty
  // stored block (3 zero bits, padding, LEN 0, NLEN 0xFFFF) realigns it.
  const uint32_t dyn_bytes = last ? (end + 7) / 8 : (end + 3 + 7) / 8 + 4;
  const uint32_t stored_bytes = (uint32_t)n + STORED_OVERHEAD;
  const bool stored = dyn_bytes >= stored_bytes;

  if (!stored) {
    for_each_token(S.in, c0, c1, before, after, [&](uint32_t lit, int len) {
      if (len) {
        int eb, ev;
        const int sym = length_symbol(len, &eb, &ev);
        put_bits_shared(S.out, offset, S.code[sym], S.len[sym]);
        offset += S.len[sym];
        put_bits_shared(S.out, offset, (uint32_t)ev, eb);
        offset += eb + 1;  // distance symbol 0 has the one-bit code 0
      } else {
        put_bits_shared(S.out, offset, S.code[lit], S.len[lit]);
        offset += S.len[lit];
      }
    });
    __syncthreads();
    if (tid == 0) {
      BitWriter w{S.out, eob_at};
      w.put(S.code[END_OF_BLOCK], S.len[END_OF_BLOCK]);
      if (!last) {
        uint8_t* bytes = reinterpret_cast<uint8_t*>(S.out);
        const uint32_t at = (end + 3 + 7) / 8;
        bytes[at + 2] = 0xFF;
        bytes[at + 3] = 0xFF;
      }
    }
  } else {
    uint8_t* bytes = reinterpret_cast<uint8_t*>(S.out);
    if (tid == 0) {
      bytes[0] = last ? 1 : 0;  // BFINAL, BTYPE 00
      bytes[1] = (uint8_t)n;
      bytes[2] = (uint8_t)(n >> 8);
      bytes[3] = (uint8_t)~n;
      bytes[4] = (uint8_t)(~n >> 8);
    }
    for (int i = tid; i < n; i += DEFLATE_THREADS) bytes[STORED_OVERHEAD + i] = S.in[i];
  }
  __syncthreads();
  const uint32_t nbytes = stored ? stored_bytes : dyn_bytes;
  uint4* slot = reinterpret_cast<uint4*>(slots + (uint64_t)seg * SEG_CAP);
  const uint4* src = reinterpret_cast<const uint4*>(S.out);
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

Status png_header(int W, int H, int depth, const uint8_t* icc, size_t icc_len, const uint8_t* exif, size_t exif_len,
                  std::vector<uint8_t>* out) {
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
  const uint64_t total = stream_bytes + slot_bytes + count_bytes + sum_bytes + at_bytes + 16;
  void* scratch = nullptr;
  RD_TRY(device_alloc(ctx, total, &scratch));
  uint8_t* p = static_cast<uint8_t*>(scratch);
  uint8_t* stream = p;
  uint8_t* slots = stream + stream_bytes;
  uint32_t* seg_bytes = reinterpret_cast<uint32_t*>(slots + slot_bytes);
  uint2* seg_sums = reinterpret_cast<uint2*>(reinterpret_cast<uint8_t*>(seg_bytes) + count_bytes);
  uint64_t* chunk_at = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(seg_sums) + sum_bytes);
  uint32_t* adler = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(chunk_at) + at_bytes);

  Status st = upload(ctx, d_png, header.data(), header.size());
  if (st.ok()) {
    if (depth == 16) {
      RD_LAUNCH(ctx, K_ENCODE, png_filter_kernel<true><<<H, FILTER_THREADS, 0, ctx.stream>>>(d_rgb, W, stream));
    } else {
      RD_LAUNCH(ctx, K_ENCODE, png_filter_kernel<false><<<H, FILTER_THREADS, 0, ctx.stream>>>(d_rgb, W, stream));
    }
    cudaFuncSetAttribute(png_deflate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(DeflateSmem));
    RD_LAUNCH(ctx, K_ENCODE,
              png_deflate_kernel<<<(unsigned)nseg, DEFLATE_THREADS, sizeof(DeflateSmem), ctx.stream>>>(
                  stream, L, (uint32_t)nseg, slots, seg_bytes, seg_sums));
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
