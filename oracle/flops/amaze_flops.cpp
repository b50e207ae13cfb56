// FLOP census of the oracle's AMaZE (measurement infrastructure): amaze.cpp
// compiled with every float replaced by CountedFloat, so its per-pixel
// operation mix can be read next to the reconstruction it produces. Built
// without OpenMP into its own library (librd_oracle_flops.so).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "counted_float.h"

namespace oracle_flops {
thread_local uint64_t g_ops[N_OPS];
}

#define float oracle_flops::CountedFloat
#include "../amaze.cpp"

// Small images fall back to bilinear in the reference; the census only runs
// images larger than one tile, so the fallback is never taken here.
extern "C" void ro_bilinear_reconstruct(const float*, int, int, int, int, const float*, float*, int) {}
#undef float

extern "C" void ro_flops_reset() {
  for (int k = 0; k < oracle_flops::N_OPS; ++k) oracle_flops::g_ops[k] = 0;
}
// ops: add/sub, mul, div, compare, abs, min/max
extern "C" void ro_flops_read(uint64_t ops[6]) {
  for (int k = 0; k < oracle_flops::N_OPS; ++k) ops[k] = oracle_flops::g_ops[k];
}
