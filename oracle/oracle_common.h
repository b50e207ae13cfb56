// Shared helpers of the CPU oracle.
//
// The oracle is TEST INFRASTRUCTURE: a plain C++17 restatement of the
// reference's deterministic CPU sensor-development pipeline (Rohditor, Rust).
// It is only ever linked by the test-suite, by the smoke check and by the
// bench's CPU-baseline leg, as the checker. The product library never links it.
//
// Arithmetic rules that keep it bit-compatible with the Rust reference:
//  * every value is binary32 and every literal carries an `f` suffix, because
//    Rust infers f32 for literals mixed with f32 operands;
//  * expressions keep Rust's left-to-right association and the file is built
//    with -ffp-contract=off, because rustc never fuses a*b+c into an FMA unless
//    the source calls mul_add (which the oracle then writes as std::fmaf);
//  * Rust's `f32::min/max` return the non-NaN operand; the AMaZE helpers
//    `fmin/fmax` are plain compare-selects (crates/demosaic/src/amaze/math.rs:94-104).
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>

namespace oracle {

// Bayer layouts in the reference's order (crates/image/src/lib.rs:52-57) and
// the C ABI's CFA codes: 0 RGGB, 1 BGGR, 2 GRBG, 3 GBRG.
enum Pattern : int { RGGB = 0, BGGR = 1, GRBG = 2, GBRG = 3 };

// BayerPattern::color_at (crates/image/src/lib.rs:88-116): channel 0/1/2.
inline int color_at(int pattern, std::size_t x, std::size_t y) {
  static const int table[4][4] = {{0, 1, 1, 2}, {2, 1, 1, 0}, {1, 0, 2, 1}, {1, 2, 0, 1}};
  return table[pattern][((y & 1) << 1) | (x & 1)];
}

// BayerPattern::shifted (crates/image/src/lib.rs:119-133).
inline int shifted(int pattern, std::size_t x, std::size_t y) {
  const int px = static_cast<int>(x & 1), py = static_cast<int>(y & 1);
  if (px == 0 && py == 0) return pattern;
  switch (pattern) {
    case RGGB: return px && py ? BGGR : (px ? GRBG : GBRG);
    case BGGR: return px && py ? RGGB : (px ? GBRG : GRBG);
    case GRBG: return px && py ? GBRG : (px ? RGGB : BGGR);
    default:   return px && py ? GRBG : (px ? BGGR : RGGB);  // GBRG
  }
}

// Rust f32::max / f32::min: the non-NaN operand wins.
inline float rmax(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a > b ? a : (b > a ? b : (std::signbit(a) ? b : a));
}
inline float rmin(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a < b ? a : (b < a ? b : (std::signbit(a) ? a : b));
}
// Rust f32::clamp(lo, hi): NaN stays NaN.
inline float rclamp(float v, float lo, float hi) {
  if (v < lo) v = lo;
  if (v > hi) v = hi;
  return v;
}

// mirror_coordinate (crates/demosaic/src/amaze_geometry.rs:80-88): whole-sample
// reflection that keeps coordinate parity.
inline std::size_t mirror_coordinate(long long index, std::size_t length) {
  if (length <= 1) return 0;
  const long long period = 2LL * static_cast<long long>(length - 1);
  long long wrapped = index % period;
  if (wrapped < 0) wrapped += period;
  const long long other = period - wrapped;
  return static_cast<std::size_t>(wrapped < other ? wrapped : other);
}

}  // namespace oracle
