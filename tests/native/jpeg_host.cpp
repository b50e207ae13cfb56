// Host harness of the JPEG encoder's arithmetic (test infrastructure).
//
// Compiles rohditor_gb300/csrc/jpeg.cuh for the CPU and computes quantised
// coefficients the way jpeg_coef_kernel does: colour conversion of each
// pixel (edges replicated), the row pass of the DCT, the column pass,
// quantisation with the quality's tables, zigzag order. The tests compare
// the result with the oracle's independent restatement.
//
//   jpeg_host IN OUT W H QUALITY   IN: W*H*3 bytes of RGB; OUT: int16
//                                  coefficients [block][Y, Cb, Cr][64]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../rohditor_gb300/csrc/jpeg.cuh"

using namespace rd::jpeg;

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: jpeg_host IN OUT W H QUALITY\n");
    return 1;
  }
  const int W = std::atoi(argv[3]), H = std::atoi(argv[4]), quality = std::atoi(argv[5]);
  std::vector<uint8_t> rgb((size_t)W * H * 3);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(rgb.data(), 1, rgb.size(), f) != rgb.size()) return 1;
  std::fclose(f);
  uint8_t quant[2][64], zz[64], zigzag_of[64];
  quant_table(0, quality, quant[0]);
  quant_table(1, quality, quant[1]);
  zigzag_order(zz);
  for (int k = 0; k < 64; ++k) zigzag_of[zz[k]] = (uint8_t)k;
  const int bw = (W + 7) / 8, bh = (H + 7) / 8;
  std::vector<int16_t> coef((size_t)bw * bh * 3 * 64);
  for (int by = 0; by < bh; ++by)
    for (int bx = 0; bx < bw; ++bx) {
      int t[3][8][8];  // t[c][y][u]
      for (int y = 0; y < 8; ++y) {
        const int py = by * 8 + y < H ? by * 8 + y : H - 1;
        int s[3][8];
        for (int i = 0; i < 8; ++i) {
          const int px = bx * 8 + i < W ? bx * 8 + i : W - 1;
          const uint8_t* p = &rgb[((size_t)py * W + px) * 3];
          int yy, cb, cr;
          rgb_to_ycc(p[0], p[1], p[2], &yy, &cb, &cr);
          s[0][i] = yy - 128;
          s[1][i] = cb - 128;
          s[2][i] = cr - 128;
        }
        for (int c = 0; c < 3; ++c) dct8(s[c], t[c][y], 11);
      }
      for (int c = 0; c < 3; ++c)
        for (int u = 0; u < 8; ++u) {
          int col[8], fv[8];
          for (int y = 0; y < 8; ++y) col[y] = t[c][y][u];
          dct8(col, fv, 15);
          for (int v = 0; v < 8; ++v) {
            const int nat = v * 8 + u;
            const int q = quant[c == 0 ? 0 : 1][nat];
            coef[(((size_t)by * bw + bx) * 3 + c) * 64 + zigzag_of[nat]] =
                (int16_t)quantize(fv[v], q, quant_reciprocal(q));
          }
        }
    }
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 1;
  std::fwrite(coef.data(), sizeof(int16_t), coef.size(), o);
  std::fclose(o);
  return 0;
}
