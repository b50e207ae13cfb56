// JPEG encoding of the export's 8-bit RGB rows, on the device.
//
// Replaces the JPEG arm of export::encode (crates/core/src/export.rs:166-175):
// the reference hands tightly packed 8-bit RGB rows, a quality of 1..100, the
// output colour space's ICC profile and optional EXIF to the `image` crate's
// JpegEncoder (image 0.25, Cargo.toml:39; not vendored). Its DCT and table
// choices are not visible, so this encoder's coefficients are its own (in the
// integer arithmetic of jpeg.cuh) and the file is a standard baseline JPEG of
// them (ITU-T T.81): JFIF, 4:4:4, quantisation tables scaled from Annex K by
// the quality, Huffman tables built for the image, restart markers every 32
// MCUs.
//
// Launches on the context's stream:
//  1. jpeg_coef_kernel    8 rows x 256 pixels per CTA: colour conversion, DCT
//                         (row pass, then column pass through shared memory),
//                         quantisation, coefficients in zigzag order;
//  2. jpeg_hist_kernel    one thread per block and component: the Huffman
//                         symbols' counts of the four tables;
//  (host: the counts come back, the tables and the file header are built and
//  the codes go up)
//  3. jpeg_pack_kernel    one CTA per restart interval: bit offsets by a scan,
//                         the blocks' bits packed most significant first,
//                         1-padding, 0xFF byte stuffing, the RST marker;
//  4. jpeg_layout_kernel  one CTA: offsets of the intervals in the file, EOI;
//  5. jpeg_copy_kernel    one CTA per interval: its bytes into the file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "deflate.cuh"
#include "jpeg.cuh"
#include "rd_internal.cuh"

namespace rd {
namespace {

using namespace jpeg;

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr int COEF_THREADS = 256;  // 8 pixel rows x 32 blocks
constexpr int COEF_BLOCKS = 32;
constexpr int COEF_STRIDE = 194;  // int16 per block in shared memory: 3 x 64, padded to an odd word count
constexpr int BLOCK_STRIDE = 66;  // int16 per block-component in shared memory: 64, padded to 33 words
constexpr int HIST_THREADS = 256;
constexpr int PACK_THREADS = INTERVAL_BLOCKS;  // one per block of the interval
constexpr int LAYOUT_THREADS = 1024;
constexpr int COPY_THREADS = 256;
constexpr int TABLES = 4;  // DC luminance, AC luminance, DC chrominance, AC chrominance

struct CoefParams {
  const uint8_t* rgb;
  int W, H, bw, bh;
  int16_t* coef;  // [block][component][64], zigzag order, blocks in raster order
  uint8_t quant[2][64];
  uint32_t recip[2][64];  // quant_reciprocal of each step
  uint8_t zigzag_of[64];  // natural index -> zigzag position
};

__global__ void __launch_bounds__(COEF_THREADS) jpeg_coef_kernel(const __grid_constant__ CoefParams P) {
  // t[c][y][u][block]: the row pass result, the block index innermost so that
  // the lanes of a warp (consecutive blocks) hit consecutive banks.
  __shared__ int t[3][8][8][COEF_BLOCKS];
  __shared__ __align__(16) int16_t q[COEF_BLOCKS * COEF_STRIDE];
  const int lane = threadIdx.x & 31, rowu = threadIdx.x >> 5;
  const int bx = blockIdx.x * COEF_BLOCKS + lane, by = blockIdx.y;
  {
    // Row pass: pixel row `rowu` of block `lane`, edges replicated.
    const int y = min(by * 8 + rowu, P.H - 1);
    const uint8_t* row = P.rgb + (int64_t)y * 3 * P.W;
    int s[3][8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int x = min(bx * 8 + i, P.W - 1);
      int yy, cb, cr;
      rgb_to_ycc(row[3 * x], row[3 * x + 1], row[3 * x + 2], &yy, &cb, &cr);
      s[0][i] = yy - 128;
      s[1][i] = cb - 128;
      s[2][i] = cr - 128;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      int out[8];
      dct8(s[c], out, 11);
#pragma unroll
      for (int u = 0; u < 8; ++u) t[c][rowu][u][lane] = out[u];
    }
  }
  __syncthreads();
  // Column pass: column u = rowu of block `lane`; the quantised coefficients
  // gather in q[block][component][zigzag], a block's 192 values padded to 97
  // words so that the 32 lanes (blocks) of a warp store to 32 banks.
  const int u = rowu;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    int col[8], f[8];
#pragma unroll
    for (int y = 0; y < 8; ++y) col[y] = t[c][y][u][lane];
    dct8(col, f, 15);
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const int nat = v * 8 + u;
      const int tq = c == 0 ? 0 : 1;
      q[lane * COEF_STRIDE + c * 64 + P.zigzag_of[nat]] = (int16_t)quantize(f[v], P.quant[tq][nat], P.recip[tq][nat]);
    }
  }
  __syncthreads();
  // The CTA's blocks are consecutive in raster order: one contiguous run of
  // 384-byte blocks, stored as 32-bit words.
  const int nb = min(COEF_BLOCKS, P.bw - (int)blockIdx.x * COEF_BLOCKS);
  uint32_t* dst = reinterpret_cast<uint32_t*>(P.coef + ((int64_t)by * P.bw + blockIdx.x * COEF_BLOCKS) * 3 * 64);
  const uint32_t* src = reinterpret_cast<const uint32_t*>(q);
  for (int w = threadIdx.x; w < nb * 96; w += COEF_THREADS) dst[w] = src[(w / 96) * (COEF_STRIDE / 2) + w % 96];
}

// Symbols of one block: the DC difference's category, then (run, category)
// pairs, 0xF0 for sixteen zeros, 0x00 at the end of the block's non-zeros.
template <class Visit>
__device__ __forceinline__ void block_symbols(const int16_t* z, int pred, Visit&& visit) {
  const int diff = z[0] - pred;
  const int dc = category(diff);
  visit(true, dc, extra_bits(diff, dc), dc);
  int run = 0;
  for (int k = 1; k < 64; ++k) {
    const int v = z[k];
    if (v == 0) {
      ++run;
      continue;
    }
    while (run > 15) {
      visit(false, 0xF0, 0u, 0);
      run -= 16;
    }
    const int cat = category(v);
    visit(false, (run << 4) | cat, extra_bits(v, cat), cat);
    run = 0;
  }
  if (run > 0) visit(false, 0x00, 0u, 0);
}

// Block-components [g0, g0 + n) (64 coefficients each, contiguous in
// global memory) into dst with BLOCK_STRIDE per block-component, as 32-bit
// words: coalesced loads, and lanes reading their own blocks later hit 32
// different banks.
template <int THREADS>
__device__ __forceinline__ void stage_blocks(const int16_t* __restrict__ coef, int64_t g0, int n, int16_t* dst) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(coef + g0 * 64);
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  for (int w = threadIdx.x; w < n * 32; w += THREADS) d[(w >> 5) * (BLOCK_STRIDE / 2) + (w & 31)] = src[w];
}

__global__ void __launch_bounds__(HIST_THREADS)
    jpeg_hist_kernel(const int16_t* __restrict__ coef, int64_t blocks, uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[TABLES][256];
  __shared__ __align__(16) int16_t z[HIST_THREADS * BLOCK_STRIDE];
  for (int i = threadIdx.x; i < TABLES * 256; i += HIST_THREADS) (&h[0][0])[i] = 0u;
  const int64_t g0 = (int64_t)blockIdx.x * HIST_THREADS;
  const int n = (int)min((int64_t)HIST_THREADS, blocks * 3 - g0);
  stage_blocks<HIST_THREADS>(coef, g0, n, z);
  __syncthreads();
  const int local = threadIdx.x;
  if (local < n) {
    const int64_t g = g0 + local;
    const int64_t blk = g / 3;
    const int c = (int)(g % 3);
    const int table = c == 0 ? 0 : 2;
    // DC prediction: the previous block of the component, 0 at the first MCU of an interval.
    const int pred = blk % RESTART_MCUS == 0 ? 0 : (local >= 3 ? z[(local - 3) * BLOCK_STRIDE] : coef[(g - 3) * 64]);
    block_symbols(z + local * BLOCK_STRIDE, pred, [&](bool dc, int sym, uint32_t, int) {
      atomicAdd(&h[table + (dc ? 0 : 1)][sym], 1u);
    });
  }
  __syncthreads();
  for (int i = threadIdx.x; i < TABLES * 256; i += HIST_THREADS) {
    const uint32_t v = (&h[0][0])[i];
    if (v) atomicAdd(hist + i, v);
  }
}

// Bits go out most significant first; each byte is ORed into the shared
// buffer, since the first and last bytes of a thread's range are shared with
// its neighbours'.
struct MsbWriter {
  uint32_t* words;
  uint32_t byte;
  unsigned long long acc;
  int held;
  __device__ __forceinline__ void or_byte(uint32_t i, uint32_t v) {
    if (v) atomicOr(words + (i >> 2), v << (8 * (i & 3u)));
  }
  __device__ __forceinline__ void put(uint32_t value, int n) {  // n <= 16
    acc = (acc << n) | value;
    held += n;
    while (held >= 8) {
      held -= 8;
      or_byte(byte++, (uint32_t)(acc >> held) & 0xFFu);
    }
    acc &= (1ull << held) - 1ull;
  }
  __device__ __forceinline__ void finish() {
    if (held > 0) or_byte(byte, (uint32_t)(acc << (8 - held)) & 0xFFu);
  }
};

__global__ void __launch_bounds__(PACK_THREADS)
    jpeg_pack_kernel(const int16_t* __restrict__ coef, int64_t blocks, const uint32_t* __restrict__ codes,
                     uint8_t* __restrict__ slots, uint32_t* __restrict__ interval_bytes, int64_t intervals) {
  __shared__ uint32_t s_codes[TABLES][256];  // code | length << 16
  __shared__ __align__(16) uint32_t words[(INTERVAL_BYTES + 3) / 4 + 1];
  __shared__ uint32_t warp_sum[PACK_THREADS / 32];
  __shared__ __align__(16) int16_t s_coef[INTERVAL_BLOCKS * BLOCK_STRIDE];
  const int64_t interval = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < TABLES * 256; i += PACK_THREADS) (&s_codes[0][0])[i] = codes[i];
  for (int i = tid; i < (INTERVAL_BYTES + 3) / 4 + 1; i += PACK_THREADS) words[i] = 0u;
  const int64_t g0 = interval * INTERVAL_BLOCKS;
  const int n = (int)min((int64_t)INTERVAL_BLOCKS, blocks * 3 - g0);
  stage_blocks<PACK_THREADS>(coef, g0, n, s_coef);
  __syncthreads();
  // Thread tid codes block-component tid of the interval: MCU tid / 3,
  // component tid % 3; the interval starts a new DC prediction.
  const bool active = tid < n;
  const int c = tid % 3;
  const int table = c == 0 ? 0 : 2;
  const int16_t* z = s_coef + tid * BLOCK_STRIDE;
  const int pred = (active && tid >= 3) ? s_coef[(tid - 3) * BLOCK_STRIDE] : 0;

  uint32_t bits = 0;
  if (active)
    block_symbols(z, pred, [&](bool dc, int sym, uint32_t, int extra) {
      bits += (s_codes[table + (dc ? 0 : 1)][sym] >> 16) + extra;
    });
  uint32_t incl = bits;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  uint32_t offset = incl - bits, total = 0;
  for (int w = 0; w < PACK_THREADS / 32; ++w) {
    if (w < warp) offset += warp_sum[w];
    total += warp_sum[w];
  }
  if (active) {
    MsbWriter wr{words, offset >> 3, 0ull, (int)(offset & 7u)};
    block_symbols(z, pred, [&](bool dc, int sym, uint32_t value, int extra) {
      const uint32_t e = s_codes[table + (dc ? 0 : 1)][sym];
      wr.put(e & 0xFFFFu, (int)(e >> 16));
      if (extra) wr.put(value, extra);
    });
    wr.finish();
  }
  __syncthreads();
  uint8_t* bytes = reinterpret_cast<uint8_t*>(words);
  if (tid == 0 && (total & 7u)) bytes[total >> 3] |= (uint8_t)((1u << (8 - (total & 7u))) - 1u);  // 1-padding
  __syncthreads();
  // Byte stuffing: a 0x00 after every 0xFF, each thread over its own bytes.
  const uint32_t nbytes = (total + 7) / 8;
  const uint32_t per = (nbytes + PACK_THREADS - 1) / PACK_THREADS;
  const uint32_t b0 = min((uint32_t)tid * per, nbytes), b1 = min(b0 + per, nbytes);
  uint32_t ff = 0;
  for (uint32_t i = b0; i < b1; ++i) ff += bytes[i] == 0xFFu;
  uint32_t ffi = ff;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(FULL, ffi, o);
    if (lane >= o) ffi += v;
  }
  __syncthreads();
  if (lane == 31) warp_sum[warp] = ffi;
  __syncthreads();
  uint32_t at = b0 + ffi - ff, all_ff = 0;
  for (int w = 0; w < PACK_THREADS / 32; ++w) {
    if (w < warp) at += warp_sum[w];
    all_ff += warp_sum[w];
  }
  uint8_t* slot = slots + interval * INTERVAL_SLOT;
  for (uint32_t i = b0; i < b1; ++i) {
    const uint8_t v = bytes[i];
    slot[at++] = v;
    if (v == 0xFFu) slot[at++] = 0x00;
  }
  if (tid == 0) {
    uint32_t size = nbytes + all_ff;
    if (interval + 1 < intervals) {
      slot[size] = 0xFF;
      slot[size + 1] = (uint8_t)(0xD0 | (interval & 7));
      size += 2;
    }
    interval_bytes[interval] = size;
  }
}

__global__ void __launch_bounds__(LAYOUT_THREADS)
    jpeg_layout_kernel(const uint32_t* __restrict__ interval_bytes, int64_t intervals, uint64_t header_bytes,
                       uint64_t* __restrict__ interval_at, uint64_t* __restrict__ file_bytes, uint8_t* __restrict__ file) {
  __shared__ unsigned long long warp_sum[LAYOUT_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t per = (intervals + LAYOUT_THREADS - 1) / LAYOUT_THREADS;
  const int64_t i0 = min((int64_t)tid * per, intervals), i1 = min(i0 + per, intervals);
  unsigned long long mine = 0;
  for (int64_t i = i0; i < i1; ++i) mine += interval_bytes[i];
  unsigned long long incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  unsigned long long at = header_bytes + incl - mine, all = 0;
  for (int w = 0; w < LAYOUT_THREADS / 32; ++w) {
    if (w < warp) at += warp_sum[w];
    all += warp_sum[w];
  }
  for (int64_t i = i0; i < i1; ++i) {
    interval_at[i] = at;
    at += interval_bytes[i];
  }
  if (tid == 0) {
    const uint64_t end = header_bytes + all;
    file[end] = 0xFF;  // EOI
    file[end + 1] = 0xD9;
    *file_bytes = end + 2;
  }
}

__global__ void __launch_bounds__(COPY_THREADS)
    jpeg_copy_kernel(const uint8_t* __restrict__ slots, const uint32_t* __restrict__ interval_bytes,
                     const uint64_t* __restrict__ interval_at, uint8_t* __restrict__ file) {
  const int64_t i = blockIdx.x;
  const uint8_t* src = slots + i * INTERVAL_SLOT;
  uint8_t* dst = file + interval_at[i];
  const uint32_t n = interval_bytes[i];
  for (uint32_t k = threadIdx.x; k < n; k += COPY_THREADS) dst[k] = src[k];
}

// ---- host: Huffman tables and the header ----------------------------------
// Code lengths of one table from its symbol counts (T.81 K.2 in effect): the
// reserved symbol 256 takes count 1 and sorts first among the least frequent,
// so it is merged first and holds the longest length; listed last among its
// length it takes the all-ones code, which T.81 forbids for real symbols, and
// is then dropped. Trees deeper than 16 are rebuilt from halved counts.
struct HuffTable {
  uint8_t counts[MAX_CODE_BITS + 1] = {};  // counts[l]: real symbols of length l
  std::vector<uint8_t> values;              // symbols by length, then by value
  uint32_t code[256] = {};                  // code | length << 16
};

HuffTable build_table(const uint32_t* hist) {
  uint32_t freq[TABLE_SYMBOLS];
  for (int s = 0; s < 256; ++s) freq[s] = hist[s];
  freq[256] = 1;
  std::vector<uint16_t> order;
  for (int s = 0; s < TABLE_SYMBOLS; ++s)
    if (freq[s]) order.push_back((uint16_t)s);
  // Ascending count; among equal counts the larger symbol first.
  std::stable_sort(order.begin(), order.end(), [&](uint16_t a, uint16_t b) {
    return freq[a] != freq[b] ? freq[a] < freq[b] : a > b;
  });
  const int n = (int)order.size();
  HuffTable t;
  uint8_t len[TABLE_SYMBOLS] = {};
  uint32_t leaf[TABLE_SYMBOLS], weight[2 * TABLE_SYMBOLS];
  uint16_t parent[2 * TABLE_SYMBOLS];
  uint8_t depth[2 * TABLE_SYMBOLS];
  png::huffman_lengths(freq, order.data(), n, MAX_CODE_BITS, leaf, weight, parent, depth, len);
  // Canonical codes (T.81 C.2) over symbols by length, then value, the reserved one last.
  uint32_t code = 0;
  for (int l = 1; l <= MAX_CODE_BITS; ++l) {
    for (int s = 0; s < 256; ++s) {
      if (len[s] != l) continue;
      t.counts[l]++;
      t.values.push_back((uint8_t)s);
      t.code[s] = code | ((uint32_t)l << 16);
      ++code;
    }
    if (len[256] == l) ++code;  // the all-ones code of the longest length, unused
    code <<= 1;
  }
  return t;
}

void put16(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void marker(std::vector<uint8_t>& v, uint8_t m, const std::vector<uint8_t>& body) {
  v.push_back(0xFF);
  v.push_back(m);
  put16(v, (uint32_t)body.size() + 2);
  v.insert(v.end(), body.begin(), body.end());
}

}  // namespace

bool jpeg_metadata_ok(uint64_t icc_len, uint64_t exif_len) {
  // APP1 holds "Exif\0\0" and the block in one segment; APP2 segments carry
  // up to 65519 profile bytes each, numbered 1..255.
  return exif_len <= 65527 && icc_len <= 255ull * 65519;
}

Status jpeg_check(int W, int H, int quality) {
  if (quality < 1 || quality > 100) return Status{RD_INVALID_INPUT, "JPEG quality must be 1..100"};
  if (W > 65535 || H > 65535) return Status{RD_INVALID_DIMENSIONS, "JPEG dimensions are limited to 65535"};
  return Status{};
}

uint64_t jpeg_bound(int W, int H, uint64_t icc_len, uint64_t exif_len) {
  const uint64_t blocks = (uint64_t)((W + 7) / 8) * ((H + 7) / 8);
  const uint64_t intervals = (blocks + RESTART_MCUS - 1) / RESTART_MCUS;
  const uint64_t icc_chunks = (icc_len + 65518) / 65519;
  const uint64_t header = 2 + 18 + (exif_len ? 4 + 6 + exif_len : 0) + icc_chunks * 18 + icc_len + 134 + 19 +
                          4 * (5 + 16 + 256) + 6 + 14;
  return header + intervals * (uint64_t)INTERVAL_SLOT + 2;
}

Status run_jpeg_encode(Context& ctx, const uint8_t* d_rgb, int W, int H, int quality, const uint8_t* icc,
                       size_t icc_len, const uint8_t* exif, size_t exif_len, uint8_t* d_file, uint64_t* d_file_bytes) {
  RD_TRY(jpeg_check(W, H, quality));
  if (!jpeg_metadata_ok(icc_len, exif_len)) return Status{RD_INVALID_INPUT, "metadata too large for JPEG segments"};
  if (ctx.capturing) return Status{RD_INVALID_INPUT, "the JPEG encoder reads its symbol counts back mid-way"};
  const int bw = (W + 7) / 8, bh = (H + 7) / 8;
  const int64_t blocks = (int64_t)bw * bh;
  const int64_t intervals = (blocks + RESTART_MCUS - 1) / RESTART_MCUS;
  auto round256 = [](uint64_t v) { return (v + 255) & ~255ull; };
  const uint64_t coef_bytes = round256((uint64_t)blocks * 3 * 64 * 2);
  const uint64_t hist_bytes = round256(TABLES * 256 * 4);
  const uint64_t slot_bytes = (uint64_t)intervals * INTERVAL_SLOT;
  const uint64_t count_bytes = round256((uint64_t)intervals * 4);
  const uint64_t at_bytes = round256((uint64_t)intervals * 8);
  const uint64_t total = coef_bytes + 2 * hist_bytes + slot_bytes + count_bytes + at_bytes;
  void* scratch = nullptr;
  RD_TRY(device_alloc(ctx, total, &scratch));
  uint8_t* p = static_cast<uint8_t*>(scratch);
  int16_t* coef = reinterpret_cast<int16_t*>(p);
  uint32_t* hist = reinterpret_cast<uint32_t*>(p + coef_bytes);
  uint32_t* codes = reinterpret_cast<uint32_t*>(p + coef_bytes + hist_bytes);
  uint8_t* slots = p + coef_bytes + 2 * hist_bytes;
  uint32_t* interval_bytes = reinterpret_cast<uint32_t*>(slots + slot_bytes);
  uint64_t* interval_at = reinterpret_cast<uint64_t*>(reinterpret_cast<uint8_t*>(interval_bytes) + count_bytes);

  CoefParams cp{};
  cp.rgb = d_rgb;
  cp.W = W;
  cp.H = H;
  cp.bw = bw;
  cp.bh = bh;
  cp.coef = coef;
  quant_table(0, quality, cp.quant[0]);
  quant_table(1, quality, cp.quant[1]);
  for (int t = 0; t < 2; ++t)
    for (int i = 0; i < 64; ++i) cp.recip[t][i] = quant_reciprocal(cp.quant[t][i]);
  uint8_t zz[64];
  zigzag_order(zz);
  for (int k = 0; k < 64; ++k) cp.zigzag_of[zz[k]] = (uint8_t)k;

  Status st;
  uint32_t h_hist[TABLES * 256];
  if (cudaMemsetAsync(hist, 0, TABLES * 256 * 4, ctx.stream) != cudaSuccess)
    st = Status{RD_SYNCHRONIZATION, "histogram clear failed"};
  if (st.ok()) {
    RD_LAUNCH(ctx, K_ENCODE,
              jpeg_coef_kernel<<<dim3((unsigned)((bw + COEF_BLOCKS - 1) / COEF_BLOCKS), (unsigned)bh), COEF_THREADS, 0,
                                 ctx.stream>>>(cp));
    RD_LAUNCH(ctx, K_ENCODE,
              jpeg_hist_kernel<<<(unsigned)((blocks * 3 + HIST_THREADS - 1) / HIST_THREADS), HIST_THREADS, 0,
                                 ctx.stream>>>(coef, blocks, hist));
    if (cudaMemcpyAsync(h_hist, hist, sizeof(h_hist), cudaMemcpyDeviceToHost, ctx.stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx.stream) != cudaSuccess)
      st = Status{RD_SYNCHRONIZATION, "JPEG symbol counts readback failed"};
  }
  std::vector<uint8_t> header;
  uint32_t h_codes[TABLES * 256];
  if (st.ok()) {
    HuffTable tables[TABLES];
    for (int t = 0; t < TABLES; ++t) {
      tables[t] = build_table(h_hist + 256 * t);
      std::memcpy(h_codes + 256 * t, tables[t].code, sizeof(tables[t].code));
    }
    header = {0xFF, 0xD8};  // SOI
    marker(header, 0xE0, {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0});  // JFIF 1.01, no units, 1:1
    if (exif && exif_len) {
      std::vector<uint8_t> b = {'E', 'x', 'i', 'f', 0, 0};
      b.insert(b.end(), exif, exif + exif_len);
      marker(header, 0xE1, b);
    }
    const size_t chunk = 65519;
    const size_t nchunks = (icc_len + chunk - 1) / chunk;
    for (size_t k = 0; icc && k < nchunks; ++k) {
      std::vector<uint8_t> b = {'I', 'C', 'C', '_', 'P', 'R', 'O', 'F', 'I', 'L', 'E', 0, (uint8_t)(k + 1),
                                (uint8_t)nchunks};
      const size_t a = k * chunk, e = std::min(icc_len, a + chunk);
      b.insert(b.end(), icc + a, icc + e);
      marker(header, 0xE2, b);
    }
    std::vector<uint8_t> dqt;
    for (int q = 0; q < 2; ++q) {
      dqt.push_back((uint8_t)q);
      for (int k = 0; k < 64; ++k) dqt.push_back(cp.quant[q][zz[k]]);
    }
    marker(header, 0xDB, dqt);
    std::vector<uint8_t> sof = {8};
    put16(sof, (uint32_t)H);
    put16(sof, (uint32_t)W);
    sof.insert(sof.end(), {3, 1, 0x11, 0, 2, 0x11, 1, 3, 0x11, 1});
    marker(header, 0xC0, sof);
    std::vector<uint8_t> dht;
    const uint8_t ids[TABLES] = {0x00, 0x10, 0x01, 0x11};
    for (int t = 0; t < TABLES; ++t) {
      dht.push_back(ids[t]);
      for (int l = 1; l <= MAX_CODE_BITS; ++l) dht.push_back(tables[t].counts[l]);
      dht.insert(dht.end(), tables[t].values.begin(), tables[t].values.end());
    }
    marker(header, 0xC4, dht);
    std::vector<uint8_t> dri;
    put16(dri, RESTART_MCUS);
    marker(header, 0xDD, dri);
    marker(header, 0xDA, {3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0});
  }
  if (st.ok()) st = upload(ctx, codes, h_codes, sizeof(h_codes));
  if (st.ok()) st = upload(ctx, d_file, header.data(), header.size());
  if (st.ok()) {
    RD_LAUNCH(ctx, K_ENCODE,
              jpeg_pack_kernel<<<(unsigned)intervals, PACK_THREADS, 0, ctx.stream>>>(coef, blocks, codes, slots,
                                                                                  interval_bytes, intervals));
    RD_LAUNCH(ctx, K_ENCODE,
              jpeg_layout_kernel<<<1, LAYOUT_THREADS, 0, ctx.stream>>>(interval_bytes, intervals, header.size(),
                                                                       interval_at, d_file_bytes, d_file));
    RD_LAUNCH(ctx, K_ENCODE,
              jpeg_copy_kernel<<<(unsigned)intervals, COPY_THREADS, 0, ctx.stream>>>(slots, interval_bytes,
                                                                                   interval_at, d_file));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) st = Status{RD_SYNCHRONIZATION, std::string("JPEG encode launch: ") + cudaGetErrorString(e)};
  }
  device_free(ctx, scratch, total);
  return st;
}

}  // namespace rd
