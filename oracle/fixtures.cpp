// Test fixtures restated from the reference's own tests (test infrastructure).
//
// * ro_fixture_amaze_golden: the integer-LCG mosaic of
//   crates/demosaic/tests/amaze_golden.rs:20-42 (513x389), whose AMaZE output
//   hashes are pinned there (:75-84).
// * ro_fixture_amaze_probe: the signed 53x47 mosaic of
//   crates/demosaic/src/amaze/mod.rs:276-296 used by the stage snapshot.
// * ro_fnv1a_f32: FNV-1a over f32 bit patterns (amaze_golden.rs:45-50).
#include <cstring>

#include "rd_oracle_fixtures.h"

extern "C" void ro_fixture_amaze_golden(int width, int height, float* out) {
  uint32_t state = 12345u;
  for (int index = 0; index < width * height; ++index) {
    state = state * 1664525u + 1013904223u;
    const float noise = (float)(state >> 8) / 16777216.0f;
    const int x = index % width, y = index / width;
    const float stripes = (float)((x * 3 + y * 5) % 7) / 7.0f;
    const float gradient = (float)(x + 2 * y) / (3.0f * (float)width);
    const float value = 0.1f + 0.5f * stripes + 0.3f * gradient + 0.2f * (noise - 0.5f);
    float v;
    if ((y / 40 + x / 60) % 5 == 0) {
      v = 1.1f;
    } else if ((x / 90 + y / 70) % 4 == 1) {
      v = 0.35f + 0.1f * noise;
    } else {
      v = value > -0.05f ? value : -0.05f;
    }
    out[index] = v;
  }
}

extern "C" void ro_fixture_amaze_probe(float* out) {
  const int width = 53, height = 47;
  for (int i = 0; i < width * height; ++i) {
    const int x = i % width, y = i / width;
    float v;
    switch ((x + 3 * y) % 11) {
      case 0: v = -0.0f; break;
      case 1: v = 1.0e-6f; break;
      case 2: v = -1.0e-6f; break;
      case 3: v = 1.5f; break;
      case 4: v = -0.2f; break;
      case 5: v = 2.0f; break;
      default: v = (float)((x * 37 + y * 19 + x * y) % 101) / 63.0f - 0.4f;
    }
    out[i] = v;
  }
}

extern "C" uint64_t ro_fnv1a_f32(const float* values, size_t count) {
  uint64_t hash = 0xcbf29ce484222325ull;
  for (size_t i = 0; i < count; ++i) {
    uint32_t bits;
    std::memcpy(&bits, &values[i], 4);
    hash = (hash ^ (uint64_t)bits) * 0x100000001b3ull;
  }
  return hash;
}
