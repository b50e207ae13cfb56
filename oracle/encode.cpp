// PNG scanline filtering of the export encoder (test infrastructure).
//
// The reference encodes PNG files in export::encode (crates/core/src/export.rs:
// 176-211) through the `image` crate's PngEncoder (`image = "0.25"`,
// Cargo.toml:39, png and jpeg features), which is not vendored. Its file bytes
// cannot be pinned here; what the reference's own tests hold of it is that the
// file decodes to exactly the samples it was given, including 16-bit samples
// that are not multiples of 257 (crates/core/tests/export.rs:115-148), with the
// ICC profile and EXIF embedded (:19-64). These functions restate the published
// PNG algorithms (PNG specification, filter type 0 with the five basic filters
// and the minimum-sum-of-absolute-differences filter selection the
// specification recommends, ties to the lower filter type) so that the test
// suite can check the GPU's filtered stream byte for byte and decode any file.
#include <cstdint>
#include <cstdlib>

#include "rd_oracle.h"

namespace {

int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  if (pb <= pc) return b;
  return c;
}

int predict(int type, int a, int b, int c) {
  switch (type) {
    case 0: return 0;
    case 1: return a;
    case 2: return b;
    case 3: return (a + b) / 2;
    default: return paeth(a, b, c);
  }
}

// Byte i of scanline r as the file stores it: 8-bit samples as they are,
// 16-bit samples most significant byte first.
uint8_t line_byte(const uint8_t* image, int w, int depth, int64_t r, int64_t i) {
  if (depth == 8) return image[r * 3 * w + i];
  const uint16_t* s = reinterpret_cast<const uint16_t*>(image);
  const uint16_t v = s[r * 3 * w + i / 2];
  return (i & 1) ? (uint8_t)(v & 0xFF) : (uint8_t)(v >> 8);
}

}  // namespace

extern "C" void ro_png_filter(const uint8_t* image, int w, int h, int depth, uint8_t* stream) {
  const int bpp = depth == 8 ? 3 : 6;
  const int64_t rb = (int64_t)w * bpp;
  for (int64_t r = 0; r < h; ++r) {
    auto x = [&](int64_t i) { return i < 0 ? 0 : (int)line_byte(image, w, depth, r, i); };
    auto up = [&](int64_t i) { return (r == 0 || i < 0) ? 0 : (int)line_byte(image, w, depth, r - 1, i); };
    uint64_t best_sum = 0;
    int best = 0;
    for (int type = 0; type < 5; ++type) {
      uint64_t sum = 0;
      for (int64_t i = 0; i < rb; ++i) {
        const int v = (x(i) - predict(type, x(i - bpp), up(i), up(i - bpp))) & 0xFF;
        sum += v < 128 ? v : 256 - v;
      }
      if (type == 0 || sum < best_sum) {
        best_sum = sum;
        best = type;
      }
    }
    uint8_t* line = stream + r * (1 + rb);
    line[0] = (uint8_t)best;
    for (int64_t i = 0; i < rb; ++i)
      line[1 + i] = (uint8_t)((x(i) - predict(best, x(i - bpp), up(i), up(i - bpp))) & 0xFF);
  }
}

extern "C" int ro_png_unfilter(const uint8_t* stream, int w, int h, int depth, uint8_t* out) {
  const int bpp = depth == 8 ? 3 : 6;
  const int64_t rb = (int64_t)w * bpp;
  for (int64_t r = 0; r < h; ++r) {
    const uint8_t* line = stream + r * (1 + rb);
    const int type = line[0];
    if (type > 4) return -1;
    uint8_t* row = out + r * rb;
    const uint8_t* prev = r > 0 ? out + (r - 1) * rb : nullptr;
    for (int64_t i = 0; i < rb; ++i) {
      const int a = i >= bpp ? row[i - bpp] : 0;
      const int b = prev ? prev[i] : 0;
      const int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
      row[i] = (uint8_t)((line[1 + i] + predict(type, a, b, c)) & 0xFF);
    }
  }
  return 0;
}
