// Launch-shape tuning across calls, for kernels launched once per call whose
// launch shape changes only the schedule of their work, never a value (the RL
// guide / mask kernel's row segments, the colour kernel's grid size).
//
// A process-wide table maps (kernel, width, height, radius) to the state of
// its tuning: the candidate shapes, the best time seen for each, and, once
// every candidate has been timed twice, the chosen one. Until then each call
// launches the next candidate still to be timed, bracketed by events on its
// context's stream; the call's synchronisation (check_kernel_error) folds the
// times into the table. Under stream capture a call launches the chosen
// shape, or the default while the shape is still being tuned, untimed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "rd_internal.cuh"

namespace rd {
namespace {

constexpr int TIMINGS_PER_CANDIDATE = 2;

struct ShapeState {
  std::vector<int> cands;
  std::vector<float> best;   // fastest time per candidate (ms), < 0 until timed
  std::vector<int> timings;  // timed launches per candidate
  std::vector<int> issued;   // launches handed out per candidate (timed or pending)
  int default_value = 0;
  int chosen = 0;            // 0 until every candidate is timed
};

std::mutex g_mutex;
std::map<ShapeKey, ShapeState> g_table;

cudaEvent_t take_event(Context& ctx) {
  cudaEvent_t e = nullptr;
  if (!ctx.event_pool.empty()) {
    e = ctx.event_pool.back();
    ctx.event_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    e = nullptr;
  }
  return e;
}

}  // namespace

ShapePick shape_begin(Context& ctx, const ShapeKey& key, int default_value, const std::vector<int>& candidates) {
  ShapePick pick;
  pick.value = default_value;
  std::lock_guard<std::mutex> lk(g_mutex);
  auto it = g_table.find(key);
  if (it == g_table.end()) {
    ShapeState st;
    st.cands = candidates;
    if (std::find(st.cands.begin(), st.cands.end(), default_value) == st.cands.end())
      st.cands.insert(st.cands.begin(), default_value);
    st.best.assign(st.cands.size(), -1.0f);
    st.timings.assign(st.cands.size(), 0);
    st.issued.assign(st.cands.size(), 0);
    st.default_value = default_value;
    it = g_table.emplace(key, std::move(st)).first;
  }
  ShapeState& st = it->second;
  if (st.chosen) {
    pick.value = st.chosen;
    return pick;
  }
  if (ctx.capturing) return pick;
  // The candidate with the fewest launches handed out so far.
  size_t next = 0;
  for (size_t k = 1; k < st.cands.size(); ++k)
    if (st.issued[k] < st.issued[next]) next = k;
  if (st.issued[next] >= TIMINGS_PER_CANDIDATE) return pick;  // the rest are in flight
  pick.start = take_event(ctx);
  if (!pick.start) return pick;
  ++st.issued[next];
  pick.value = st.cands[next];
  cudaEventRecord(pick.start, ctx.stream);
  return pick;
}

void shape_end(Context& ctx, const ShapeKey& key, const ShapePick& pick) {
  if (!pick.start) return;
  cudaEvent_t b = take_event(ctx);
  if (!b) {
    ctx.event_pool.push_back(pick.start);
    return;
  }
  cudaEventRecord(b, ctx.stream);
  ctx.shape_runs.push_back({key, pick.value, pick.start, b});
}

void resolve_shape_tuning(Context& ctx) {
  std::lock_guard<std::mutex> lk(g_mutex);
  for (const Context::ShapeRun& r : ctx.shape_runs) {
    float ms = 0.0f;
    const bool ok = cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess;
    ctx.event_pool.push_back(r.a);
    ctx.event_pool.push_back(r.b);
    auto it = g_table.find(r.key);
    if (it == g_table.end()) continue;
    ShapeState& st = it->second;
    const auto pos = std::find(st.cands.begin(), st.cands.end(), r.value);
    if (pos == st.cands.end()) continue;
    const size_t k = (size_t)(pos - st.cands.begin());
    if (!ok) {
      --st.issued[k];  // hand it out again
      continue;
    }
    ++st.timings[k];
    if (st.best[k] < 0.0f || ms < st.best[k]) st.best[k] = ms;
    bool done = !st.chosen;
    for (int n : st.timings) done = done && n >= TIMINGS_PER_CANDIDATE;
    if (done) {
      size_t best = 0;
      for (size_t j = 1; j < st.cands.size(); ++j)
        if (st.best[j] < st.best[best]) best = j;
      st.chosen = st.cands[best];
    }
  }
  ctx.shape_runs.clear();
  cudaGetLastError();
}

bool shape_record(const ShapeKey& key, int* value, int* default_value, float* best_ms, float* default_ms) {
  std::lock_guard<std::mutex> lk(g_mutex);
  auto it = g_table.find(key);
  if (it == g_table.end() || !it->second.chosen) return false;
  const ShapeState& st = it->second;
  if (value) *value = st.chosen;
  if (default_value) *default_value = st.default_value;
  for (size_t k = 0; k < st.cands.size(); ++k) {
    if (st.cands[k] == st.chosen && best_ms) *best_ms = st.best[k];
    if (st.cands[k] == st.default_value && default_ms) *default_ms = st.best[k];
  }
  return true;
}

}  // namespace rd
