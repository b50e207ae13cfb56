// Opaque handles of the C ABI (include/rd_gpu.h), shared by the entry points
// and the served loop.
#pragma once

#include "rd_internal.cuh"

struct rd_ctx {
  rd::Context c;
};
struct rd_source {
  rd_ctx* ctx;
  float* rgb;  // planar camera-native RGB
  int W, H;
  size_t bytes;
};
struct rd_base {
  rd_ctx* ctx;
  float* rgb;  // planar linear Rec.2020 RGB
  int W, H;
  size_t bytes;
  uint8_t* d_srgb;             // device output of rd_render_device
  unsigned long long* d_hist;  // 1024 bins
  size_t out_bytes;
};
