// JPEG coefficients and baseline JPEG decoding for the export encoder's tests
// (test infrastructure).
//
// The reference encodes JPEG files in export::encode (crates/core/src/export.rs:
// 166-175) through the `image` crate's JpegEncoder (`image = "0.25"`,
// Cargo.toml:39), which is not vendored: its DCT, quantisation and Huffman
// choices cannot be pinned here (parity against the reference's bytes is
// unpinned). What the reference's own tests hold of a JPEG export is that it
// decodes, and that a higher quality gives a larger file with different
// decoded pixels (crates/core/tests/export.rs:152-179).
//
// ro_jpeg_coefficients restates, independently, the integer arithmetic the
// GPU encoder documents (JFIF colour conversion in 16-bit fixed point, an
// 8x8 DCT whose 13-bit basis is derived here from cos(), T.81 Annex K tables
// scaled by quality as the Independent JPEG Group's software does, rounding
// halves away from zero), so the GPU's coefficients can be compared bit for
// bit. ro_jpeg_decode is a baseline decoder (ITU-T T.81 Annex F: Huffman
// decoding, DC prediction, restart intervals) that turns a file back into
// its quantised coefficients, so the test suite can check that the GPU's file
// carries exactly those coefficients.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "rd_oracle.h"

namespace {

// Natural (row-major) index of each zigzag position: walk the anti-diagonals,
// moving up-right on even ones and down-left on odd ones.
void zigzag(int* nat) {
  int r = 0, c = 0;
  for (int k = 0; k < 64; ++k) {
    nat[k] = r * 8 + c;
    if ((r + c) % 2 == 0) {  // moving up-right
      if (c == 7) {
        ++r;
      } else if (r == 0) {
        ++c;
      } else {
        --r;
        ++c;
      }
    } else {  // moving down-left
      if (r == 7) {
        ++c;
      } else if (c == 0) {
        ++r;
      } else {
        ++r;
        --c;
      }
    }
  }
}

const int ANNEX_K[2][64] = {
    {16, 11, 10, 16, 24, 40, 51, 61, 12, 12, 14, 19, 26, 58, 60, 55, 14, 13, 16, 24, 40, 57, 69, 56,
     14, 17, 22, 29, 51, 87, 80, 62, 18, 22, 37, 56, 68, 109, 103, 77, 24, 35, 55, 64, 81, 104, 113, 92,
     49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99},
    {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99, 24, 26, 56, 99, 99, 99, 99, 99,
     47, 66, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
     99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99}};

int scaled_quant(int which, int quality, int i) {
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  int v = (ANNEX_K[which][i] * scale + 50) / 100;
  if (v < 1) v = 1;
  if (v > 255) v = 255;
  return v;
}

struct BitReader {
  const uint8_t* p;
  size_t n, pos;
  uint32_t bits = 0;
  int count = 0;
  bool marker = false;  // a marker was reached: only zero bits follow
  int bit() {
    if (count == 0) {
      uint8_t b = 0;
      if (!marker && pos < n) {
        b = p[pos];
        if (b == 0xFF) {
          const uint8_t next = pos + 1 < n ? p[pos + 1] : 0;
          if (next == 0x00) {
            pos += 2;
          } else {
            marker = true;
            b = 0;
          }
        } else {
          ++pos;
        }
      }
      bits = b;
      count = 8;
    }
    --count;
    return (int)((bits >> count) & 1u);
  }
  int receive(int s) {
    int v = 0;
    for (int i = 0; i < s; ++i) v = (v << 1) | bit();
    return v;
  }
  void align() { count = 0; }
};

struct Huffman {
  int maxcode[18], mincode[17], valptr[17];
  std::vector<uint8_t> values;
  bool present = false;
  void build(const uint8_t* counts, const uint8_t* vals, int total) {
    values.assign(vals, vals + total);
    int code = 0, k = 0;
    for (int l = 1; l <= 16; ++l) {
      valptr[l] = k;
      mincode[l] = code;
      code += counts[l - 1];
      k += counts[l - 1];
      maxcode[l] = counts[l - 1] ? code - 1 : -1;
      code <<= 1;
    }
    maxcode[17] = 0x7FFFFFFF;
    present = true;
  }
  int decode(BitReader& br) const {
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
      code = (code << 1) | br.bit();
      if (maxcode[l] >= 0 && code <= maxcode[l]) return values[valptr[l] + code - mincode[l]];
    }
    return -1;
  }
};

int extend(int v, int s) { return s == 0 ? 0 : (v < (1 << (s - 1)) ? v - (1 << s) + 1 : v); }

uint32_t be16(const uint8_t* p) { return ((uint32_t)p[0] << 8) | p[1]; }

}  // namespace

extern "C" void ro_jpeg_coefficients(const uint8_t* rgb, int w, int h, int quality, int16_t* coef) {
  int basis[8][8];
  for (int u = 0; u < 8; ++u)
    for (int x = 0; x < 8; ++x) {
      const double cu = u == 0 ? 1.0 / std::sqrt(2.0) : 1.0;
      basis[u][x] = (int)std::lround(8192.0 * cu / 2.0 * std::cos((2 * x + 1) * u * M_PI / 16.0));
    }
  int nat[64];
  zigzag(nat);
  int q[2][64];
  for (int t = 0; t < 2; ++t)
    for (int i = 0; i < 64; ++i) q[t][i] = scaled_quant(t, quality, i);
  const int bw = (w + 7) / 8, bh = (h + 7) / 8;
  for (int by = 0; by < bh; ++by)
    for (int bx = 0; bx < bw; ++bx)
      for (int c = 0; c < 3; ++c) {
        int s[8][8];
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) {
            const int py = std::min(by * 8 + y, h - 1), px = std::min(bx * 8 + x, w - 1);
            const uint8_t* p = rgb + ((int64_t)py * w + px) * 3;
            const int r = p[0], g = p[1], b = p[2];
            int v;
            if (c == 0) {
              v = (19595 * r + 38470 * g + 7471 * b + 32768) >> 16;
            } else if (c == 1) {
              v = std::min(255, (-11059 * r - 21709 * g + 32768 * b + (128 << 16) + 32768) >> 16);
            } else {
              v = std::min(255, (32768 * r - 27439 * g - 5329 * b + (128 << 16) + 32768) >> 16);
            }
            s[y][x] = v - 128;
          }
        int t[8][8];  // t[y][u]
        for (int y = 0; y < 8; ++y)
          for (int u = 0; u < 8; ++u) {
            int acc = 0;
            for (int x = 0; x < 8; ++x) acc += basis[u][x] * s[y][x];
            t[y][u] = (acc + 1024) >> 11;
          }
        int16_t* out = coef + (((int64_t)by * bw + bx) * 3 + c) * 64;
        for (int k = 0; k < 64; ++k) {
          const int v = nat[k] / 8, u = nat[k] % 8;
          int acc = 0;
          for (int y = 0; y < 8; ++y) acc += basis[v][y] * t[y][u];
          const int f = (acc + 16384) >> 15;
          const int qq = q[c == 0 ? 0 : 1][nat[k]];
          out[k] = (int16_t)(f >= 0 ? (f + qq / 2) / qq : -((-f + qq / 2) / qq));
        }
      }
}

extern "C" int ro_jpeg_decode(const uint8_t* data, size_t n, int* width, int* height, int* restart,
                              uint8_t* quant /* 3 x 64: each component's table, natural order */, int16_t* coef, size_t coef_capacity) {
  if (n < 4 || data[0] != 0xFF || data[1] != 0xD8) return -1;
  size_t pos = 2;
  Huffman dc[4], ac[4];
  int qtab[4][64] = {};
  int comps = 0, comp_id[3] = {}, comp_q[3] = {}, comp_dc[3] = {}, comp_ac[3] = {};
  int W = 0, H = 0, ri = 0;
  int nat[64];
  zigzag(nat);
  while (pos + 4 <= n) {
    if (data[pos] != 0xFF) return -2;
    const uint8_t m = data[pos + 1];
    pos += 2;
    if (m == 0xD9) return -3;  // EOI before any scan
    const uint32_t len = be16(data + pos);
    if (len < 2 || pos + len > n) return -4;
    const uint8_t* s = data + pos + 2;
    const uint32_t body = len - 2;
    if (m == 0xDB) {
      for (uint32_t i = 0; i + 65 <= body; i += 65) {
        if (s[i] >> 4) return -5;  // 16-bit tables are not baseline
        for (int k = 0; k < 64; ++k) qtab[s[i] & 3][nat[k]] = s[i + 1 + k];
      }
    } else if (m == 0xC0) {
      if (s[0] != 8) return -6;
      H = (int)be16(s + 1);
      W = (int)be16(s + 3);
      comps = s[5];
      if (comps != 3) return -7;
      for (int c = 0; c < 3; ++c) {
        comp_id[c] = s[6 + 3 * c];
        if (s[7 + 3 * c] != 0x11) return -8;  // 1x1 sampling only
        comp_q[c] = s[8 + 3 * c] & 3;
      }
    } else if (m == 0xC4) {
      uint32_t i = 0;
      while (i + 17 <= body) {
        const int tc = s[i] >> 4, th = s[i] & 3;
        int total = 0;
        for (int l = 0; l < 16; ++l) total += s[i + 1 + l];
        if (i + 17 + total > body) return -9;
        (tc == 0 ? dc[th] : ac[th]).build(s + i + 1, s + i + 17, total);
        i += 17 + total;
      }
    } else if (m == 0xDD) {
      ri = (int)be16(s);
    } else if (m == 0xDA) {
      if (s[0] != 3) return -10;
      for (int k = 0; k < 3; ++k) {
        const int id = s[1 + 2 * k];
        int c = 0;
        while (c < 3 && comp_id[c] != id) ++c;
        if (c == 3) return -11;
        comp_dc[c] = s[2 + 2 * k] >> 4;
        comp_ac[c] = s[2 + 2 * k] & 3;
      }
      pos += len;
      break;
    }
    pos += len;
  }
  if (!W || !H || !comps) return -12;
  const int bw = (W + 7) / 8, bh = (H + 7) / 8;
  const int64_t mcus = (int64_t)bw * bh;
  if ((size_t)mcus * 3 * 64 > coef_capacity) return -13;
  BitReader br{data, n, pos};
  int pred[3] = {0, 0, 0};
  int next_rst = 0;
  for (int64_t m = 0; m < mcus; ++m) {
    if (ri && m > 0 && m % ri == 0) {
      // Restart: byte alignment, the RSTn marker in sequence, predictors reset.
      br.align();
      br.marker = false;
      if (br.pos + 2 > n || data[br.pos] != 0xFF || data[br.pos + 1] != (uint8_t)(0xD0 + next_rst)) return -14;
      br.pos += 2;
      next_rst = (next_rst + 1) & 7;
      pred[0] = pred[1] = pred[2] = 0;
    }
    for (int c = 0; c < 3; ++c) {
      int16_t* z = coef + (m * 3 + c) * 64;
      std::memset(z, 0, 64 * sizeof(int16_t));
      const Huffman& hd = dc[comp_dc[c]];
      const Huffman& ha = ac[comp_ac[c]];
      if (!hd.present || !ha.present) return -15;
      const int t = hd.decode(br);
      if (t < 0 || t > 11) return -16;
      pred[c] += extend(br.receive(t), t);
      z[0] = (int16_t)pred[c];
      for (int k = 1; k < 64;) {
        const int rs = ha.decode(br);
        if (rs < 0) return -17;
        const int r = rs >> 4, sz = rs & 15;
        if (sz == 0) {
          if (r != 15) break;  // end of block
          k += 16;
          continue;
        }
        k += r;
        if (k > 63) return -18;
        z[k++] = (int16_t)extend(br.receive(sz), sz);
      }
    }
  }
  // The scan ends on a byte boundary with EOI.
  br.align();
  if (br.pos + 2 > n || data[br.pos] != 0xFF || data[br.pos + 1] != 0xD9) return -19;
  *width = W;
  *height = H;
  *restart = ri;
  for (int t = 0; t < 3; ++t)
    for (int k = 0; k < 64; ++k) quant[t * 64 + k] = (uint8_t)qtab[comp_q[t]][k];
  return 0;
}
