// Baseline JPEG arithmetic of the JPEG encoder (k_jpeg.cu): colour
// conversion, the 8x8 forward DCT, quantisation and the symbols of the
// entropy coder, all in integers so that any implementation of the same steps
// gets the same coefficients. Plain functions of their arguments, compiled for
// the device and the host.
//
// Format: ITU-T T.81 baseline sequential DCT, 8-bit samples, three components
// (Y, Cb, Cr as in JFIF) with 1x1 sampling (one 8x8 block of each per MCU),
// Huffman tables built for each image, restart markers every RESTART_MCUS
// MCUs so that each restart interval is entropy-coded on its own.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define RD_JHD __host__ __device__ __forceinline__
#else
#define RD_JHD inline
#endif

namespace rd {
namespace jpeg {

constexpr int RESTART_MCUS = 32;              // MCUs per restart interval
constexpr int BLOCKS_PER_MCU = 3;             // Y, Cb, Cr
constexpr int INTERVAL_BLOCKS = RESTART_MCUS * BLOCKS_PER_MCU;
// Largest entropy-coded block: a DC code (<= 16 bits) with 11 extra bits,
// then 63 AC codes (<= 16 bits) with 10 extra bits each.
constexpr int MAX_BLOCK_BITS = 16 + 11 + 63 * (16 + 10);
constexpr int INTERVAL_BYTES = (INTERVAL_BLOCKS * MAX_BLOCK_BITS + 7) / 8;
// An interval's slot: every byte may be stuffed with a 0x00, then a 2-byte RST marker.
constexpr int INTERVAL_SLOT = ((2 * INTERVAL_BYTES + 2 + 15) / 16) * 16;
constexpr int AC_SYMBOLS = 256;
constexpr int DC_SYMBOLS = 12;
constexpr int TABLE_SYMBOLS = 257;            // a table's symbols plus the reserved one (256)
constexpr int MAX_CODE_BITS = 16;

// Quantisation table at `quality` (1..100), row-major: the luminance (0) or
// chrominance (1) table of T.81 Annex K (K.1, K.2), scaled as the Independent
// JPEG Group's reference software does (5000 / q percent below quality 50,
// 200 - 2q above), rounded and limited to the 8-bit range of baseline tables.
inline void quant_table(int which, int quality, uint8_t* out) {
  static const uint8_t BASE[2][64] = {
      {16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57,
       69, 56, 14, 17, 22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64,
       81, 104, 113, 92, 49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99},
      {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99,
       99, 99, 47, 66, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
       99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99}};
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  for (int i = 0; i < 64; ++i) {
    const int v = ((int)BASE[which][i] * scale + 50) / 100;
    out[i] = (uint8_t)(v < 1 ? 1 : (v > 255 ? 255 : v));
  }
}

// zigzag[k] = natural (row-major) index of the k-th coefficient in zigzag
// order: anti-diagonals s = row + col in turn, even ones from bottom-left to
// top-right, odd ones from top-right to bottom-left.
inline void zigzag_order(uint8_t* zigzag) {
  int k = 0;
  for (int s = 0; s < 15; ++s) {
    const int lo = s < 8 ? 0 : s - 7, hi = s < 8 ? s : 7;
    for (int t = 0; t <= hi - lo; ++t) {
      const int row = (s & 1) ? lo + t : hi - t;
      zigzag[k++] = (uint8_t)(row * 8 + (s - row));
    }
  }
}

// JFIF colour conversion (ITU-R BT.601 full range) in 16-bit fixed point.
RD_JHD void rgb_to_ycc(int r, int g, int b, int* y, int* cb, int* cr) {
  *y = (19595 * r + 38470 * g + 7471 * b + 32768) >> 16;
  const int u = (-11059 * r - 21709 * g + 32768 * b + (128 << 16) + 32768) >> 16;
  const int v = (32768 * r - 27439 * g - 5329 * b + (128 << 16) + 32768) >> 16;
  *cb = u > 255 ? 255 : u;
  *cr = v > 255 ? 255 : v;
}

// One 8-point pass of the forward DCT: out[u] = (sum_x B[u][x] in[x] +
// 2^(shift-1)) >> shift with the 13-bit basis B[u][x] = round(8192 * c(u) / 2
// * cos((2x + 1) u pi / 16)), c(0) = 1/sqrt(2), c(u > 0) = 1 (no entry lies
// within 0.02 of a rounding boundary). The row pass on level-shifted samples
// uses shift 11 (two fraction bits kept), the column pass shift 15, which
// leaves the coefficient at the scale of T.81's FDCT (A.3.3).
RD_JHD void dct8(const int* in, int* out, int shift) {
  constexpr int16_t B[8][8] = {
      {2896, 2896, 2896, 2896, 2896, 2896, 2896, 2896},
      {4017, 3406, 2276, 799, -799, -2276, -3406, -4017},
      {3784, 1567, -1567, -3784, -3784, -1567, 1567, 3784},
      {3406, -799, -4017, -2276, 2276, 4017, 799, -3406},
      {2896, -2896, -2896, 2896, 2896, -2896, -2896, 2896},
      {2276, -4017, 799, 3406, -3406, -799, 4017, -2276},
      {1567, -3784, 3784, -1567, -1567, 3784, -3784, 1567},
      {799, -2276, 3406, -4017, 4017, -3406, 2276, -799}};
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int u = 0; u < 8; ++u) {
    int acc = 0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int x = 0; x < 8; ++x) acc += B[u][x] * in[x];
    out[u] = (acc + (1 << (shift - 1))) >> shift;
  }
}

// m = ceil(2^31 / q) for a step q of 1..255: with m = (2^31 + e) / q,
// 0 <= e < q, (n * m) >> 31 = floor(n / q + n e / (q 2^31)) = floor(n / q)
// whenever n e < 2^31, which holds for every n below 2^23.
RD_JHD uint32_t quant_reciprocal(int q) { return (uint32_t)(((1ull << 31) + (uint64_t)q - 1) / (uint64_t)q); }

// coef / q rounded to the nearest integer, halves away from zero, with m the
// step's reciprocal (|coef| stays far below 2^22 for 8-bit samples).
RD_JHD int quantize(int coef, int q, uint32_t m) {
  const uint32_t n = (uint32_t)(coef >= 0 ? coef : -coef) + (uint32_t)(q >> 1);
  const int r = (int)(((uint64_t)n * m) >> 31);
  return coef >= 0 ? r : -r;
}

// Magnitude category (T.81 F.1.2.1): bits of |v|, 0 for 0.
RD_JHD int category(int v) {
  const unsigned a = (unsigned)(v < 0 ? -v : v);
#if defined(__CUDA_ARCH__)
  return 32 - __clz((int)a);
#else
  return a ? 32 - __builtin_clz(a) : 0;
#endif
}

// The `cat` extra bits that follow a symbol: v itself when positive, v - 1 in
// two's complement (the ones' complement of |v|) when negative.
RD_JHD uint32_t extra_bits(int v, int cat) { return (uint32_t)(v >= 0 ? v : v + (1 << cat) - 1) & ((1u << cat) - 1u); }

}  // namespace jpeg
}  // namespace rd
