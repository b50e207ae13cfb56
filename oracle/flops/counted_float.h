// Operation-counting binary32 for the oracle's FLOP census (test and
// measurement infrastructure). A CountedFloat holds one float and performs
// every operation in binary32 exactly as the plain type does, incrementing a
// per-thread counter per operation class, so an instrumented build of an
// oracle stage returns bit-identical results together with its operation mix.
#pragma once

#include <cmath>
#include <cstdint>

namespace oracle_flops {

enum Op { ADD, MUL, DIV, CMP, ABS, MINMAX, N_OPS };
extern thread_local uint64_t g_ops[N_OPS];

struct CountedFloat {
  float v;
  constexpr CountedFloat() : v(0.0f) {}
  constexpr CountedFloat(float x) : v(x) {}  // NOLINT: implicit, as a float literal converts
  constexpr CountedFloat(double x) : v((float)x) {}
  constexpr CountedFloat(int x) : v((float)x) {}
  explicit operator float() const { return v; }
  explicit operator int() const { return (int)v; }
  explicit operator bool() const { return v != 0.0f; }
};
using CF = CountedFloat;

// Constant expressions (the stage constants) are evaluated without counting.
constexpr void count(Op op) {
  if (!__builtin_is_constant_evaluated()) ++g_ops[op];
}
constexpr CF operator+(CF a, CF b) { count(ADD); return CF(a.v + b.v); }
constexpr CF operator-(CF a, CF b) { count(ADD); return CF(a.v - b.v); }
constexpr CF operator*(CF a, CF b) { count(MUL); return CF(a.v * b.v); }
constexpr CF operator/(CF a, CF b) { count(DIV); return CF(a.v / b.v); }
constexpr CF operator-(CF a) { return CF(-a.v); }
inline CF& operator+=(CF& a, CF b) { return a = a + b; }
inline CF& operator-=(CF& a, CF b) { return a = a - b; }
inline CF& operator*=(CF& a, CF b) { return a = a * b; }
inline CF& operator/=(CF& a, CF b) { return a = a / b; }
inline bool operator<(CF a, CF b) { ++g_ops[CMP]; return a.v < b.v; }
inline bool operator>(CF a, CF b) { ++g_ops[CMP]; return a.v > b.v; }
inline bool operator<=(CF a, CF b) { ++g_ops[CMP]; return a.v <= b.v; }
inline bool operator>=(CF a, CF b) { ++g_ops[CMP]; return a.v >= b.v; }
inline bool operator==(CF a, CF b) { ++g_ops[CMP]; return a.v == b.v; }
inline bool operator!=(CF a, CF b) { ++g_ops[CMP]; return a.v != b.v; }

}  // namespace oracle_flops

namespace std {
inline oracle_flops::CF fabs(oracle_flops::CF a) {
  ++oracle_flops::g_ops[oracle_flops::ABS];
  return oracle_flops::CF(std::fabs(a.v));
}
inline oracle_flops::CF abs(oracle_flops::CF a) { return std::fabs(a); }
inline const oracle_flops::CF& min(const oracle_flops::CF& a, const oracle_flops::CF& b) {
  ++oracle_flops::g_ops[oracle_flops::MINMAX];
  return b.v < a.v ? b : a;
}
inline const oracle_flops::CF& max(const oracle_flops::CF& a, const oracle_flops::CF& b) {
  ++oracle_flops::g_ops[oracle_flops::MINMAX];
  return a.v < b.v ? b : a;
}
inline bool isfinite(oracle_flops::CF a) { return std::isfinite(a.v); }
inline bool isnan(oracle_flops::CF a) { return std::isnan(a.v); }
inline bool signbit(oracle_flops::CF a) { return std::signbit(a.v); }
inline oracle_flops::CF floor(oracle_flops::CF a) { return oracle_flops::CF(std::floor(a.v)); }
}  // namespace std
