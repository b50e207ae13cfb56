// CPU oracle: normalization contract, Clip and Opposed highlight
// reconstruction. Test infrastructure only (see oracle_common.h).
//
//  normalize  crates/core/src/pipeline/sensor.rs:221-277, 598-610
//  clip       crates/highlight/src/clip.rs:23-72, detect.rs:6-16
//  opposed    crates/highlight/src/{opposed,cells,regions,support,region_correction}.rs
#include <algorithm>
#include <cstring>
#include <vector>

#include "oracle_common.h"
#include "rd_oracle.h"

using namespace oracle;

extern "C" int ro_normalize(const uint16_t* mosaic, const ro_sensor* s, float* out) {
  const int crop_pattern = shifted(s->pattern, s->crop_x, s->crop_y);
#pragma omp parallel for schedule(static)
  for (int oy = 0; oy < s->crop_h; ++oy) {
    const int sy = s->crop_y + oy;
    for (int ox = 0; ox < s->crop_w; ++ox) {
      const int sx = s->crop_x + ox;
      const uint16_t sample = mosaic[(std::size_t)sy * s->row_stride + sx];
      const int bi = (sy % s->black_h) * s->black_w + (sx % s->black_w);
      const float black = s->black[bi];
      float white;
      if (s->white_count == 1) white = s->white[0];
      else if (s->white_count == 3) white = s->white[color_at(s->pattern, sx, sy)];
      else white = s->white[bi];
      out[(std::size_t)oy * s->crop_w + ox] = ((float)sample - black) / (white - black);
    }
  }
  return crop_pattern;
}

extern "C" int ro_clip(float* m, int w, int h, int pattern, const float levels[3], uint64_t stats[6]) {
  uint64_t affected = 0, changed = 0, over = 0, ar = 0, ag = 0, ab = 0;
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : affected, changed, over, ar, ag, ab) reduction(| : bad)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float& s = m[(std::size_t)y * w + x];
      if (!std::isfinite(s)) { bad |= 1; continue; }
      const int c = color_at(pattern, x, y);
      const float limit = levels[c];
      if (s >= limit) {
        affected++;
        (c == 0 ? ar : c == 1 ? ag : ab)++;
      }
      if (s > 1.0f) over++;
      if (s > limit) { changed++; s = limit; }
    }
  stats[0] = affected; stats[1] = changed; stats[2] = over; stats[3] = ar; stats[4] = ag; stats[5] = ab;
  return bad ? -1 : 0;
}

// ------------------------------------------------------------------ Opposed
namespace {

constexpr int FIRST_RADIUS = 1, LAST_RADIUS = 3, MAX_CANDIDATES = 48, MIN_CANDIDATES = 3;
constexpr float MAXIMUM_ESTIMATE_MULTIPLIER = 4.0f;
constexpr float DARK_SUPPORT_FRACTION = 0.2f;          // support.rs:13
constexpr float CROSS_CHANNEL_TOLERANCE_EV = 0.75f;    // support.rs:18
constexpr int DILATION = 1;                            // regions.rs:18
constexpr int PATTERNS = 3, SLOTS = 9;                 // region_correction.rs:21-23
constexpr unsigned MIN_BORDER_CELLS = 3;
constexpr double TRIM_DEVIATIONS = 2.0;
constexpr float TRIM_FLOOR = 1e-5f;
constexpr float BORDER_MIN_FRACTION = 0.5f;

struct Cell {
  float means[3];
  uint8_t flags;
  bool usable(int c) const { return flags & (1 << c); }
  bool suspected(int c) const { return flags & (1 << (c + 3)); }
  bool clean(int c) const { return !suspected(c); }
};

int popcount(unsigned m) { return __builtin_popcount(m); }

bool bright_clean(const Cell& cell, int c, const float* levels) {
  return cell.usable(c) && cell.clean(c) && cell.means[c] > DARK_SUPPORT_FRACTION * levels[c];
}
unsigned support_mask(const Cell& cell, int target, const float* levels) {
  unsigned m = 0;
  for (int c = 0; c < 3; ++c)
    if (c != target && bright_clean(cell, c, levels)) m |= 1u << c;
  return m;
}
// support.rs:56-77
bool reference(const Cell& cell, unsigned support, float* out) {
  if (popcount(support) == 1) {
    const float v = cell.means[__builtin_ctz(support)];
    if (std::isfinite(v) && v > 0.0f) { *out = v; return true; }
    return false;
  }
  float sum = 0.0f;
  int count = 0;
  for (int c = 0; c < 3; ++c) {
    if (!(support & (1u << c))) continue;
    const float v = cell.means[c];
    if (!std::isfinite(v) || v <= 0.0f) return false;
    sum += std::cbrt(v);
    count += 1;
  }
  if (count == 0) return false;
  const float root = sum / (float)count;
  *out = root * root * root;
  return true;
}
// support.rs:83-99
bool correction(const Cell& cell, int target, unsigned support, const float* levels, float* out) {
  if (!bright_clean(cell, target, levels)) return false;
  for (int c = 0; c < 3; ++c)
    if ((support & (1u << c)) && !bright_clean(cell, c, levels)) return false;
  float ref;
  if (!reference(cell, support, &ref)) return false;
  const float v = cell.means[target] - ref;
  if (!std::isfinite(v)) return false;
  *out = v;
  return true;
}
// support.rs:104-113
bool log_ratio(const Cell& cell, unsigned support, float* out) {
  if (popcount(support) != 2) return false;
  int first = -1, second = -1;
  for (int c = 0; c < 3; ++c)
    if (support & (1u << c)) (first < 0 ? first : second) = c;
  const float ratio = cell.means[first] / cell.means[second];
  if (!(std::isfinite(ratio) && ratio > 0.0f)) return false;
  *out = std::log2(ratio);
  return true;
}
// support.rs:119-131
bool chroma_agrees(unsigned support, bool has_t, float t, bool has_e, float e) {
  if (popcount(support) < 2) return true;
  if (has_t && has_e) return std::fabs(t - e) <= CROSS_CHANNEL_TOLERANCE_EV;
  return false;
}
void support_patterns(int channel, unsigned out[3]) {
  int o[2], k = 0;
  for (int c = 0; c < 3; ++c)
    if (c != channel) o[k++] = c;
  out[0] = 1u << o[0];
  out[1] = 1u << o[1];
  out[2] = (1u << o[0]) | (1u << o[1]);
}
int pattern_position(int channel, unsigned support) {
  unsigned p[3];
  support_patterns(channel, p);
  for (int k = 0; k < 3; ++k)
    if (p[k] == support) return k;
  return -1;
}

struct Slot {
  uint32_t count = 0, kept = 0;
  double accum = 0.0, second = 0.0;
  float mean = 0.0f, tolerance = 0.0f;
  void add(int pass, float value, bool has_ratio, float ratio) {
    const double wide = (double)value;
    if (pass == 0) {
      count += 1;
      accum += wide;
      second += wide * wide;
    } else if (std::fabs(value - mean) <= tolerance) {
      kept += 1;
      accum += wide;
      second += (double)(has_ratio ? ratio : 0.0f);
    }
  }
  void finish_moments() {
    if (count != 0) {
      const double n = (double)count;
      const double m = accum / n;
      const double var = std::max(second / n - m * m, 0.0);
      mean = (float)m;
      tolerance = (float)(TRIM_DEVIATIONS * std::sqrt(var)) + TRIM_FLOOR;
    }
    accum = 0.0;
    second = 0.0;
  }
  bool value(bool has_ratio, float* offset, bool* out_has_ratio, float* ratio) const {
    if (count < MIN_BORDER_CELLS || kept == 0) return false;
    const double k = (double)kept;
    *offset = (float)(accum / k);
    *out_has_ratio = has_ratio;
    if (has_ratio) *ratio = (float)(second / k);
    return true;
  }
};

uint32_t find_root(std::vector<uint32_t>& parent, uint32_t label) {
  while (parent[label] != label) {
    const uint32_t gp = parent[parent[label]];
    parent[label] = gp;
    label = gp;
  }
  return label;
}

}  // namespace

// regions.rs:188-281
extern "C" uint32_t ro_label_components(uint32_t* labels, int width, int height) {
  std::vector<uint32_t> parent;
  parent.push_back(0);
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      const std::size_t index = (std::size_t)y * width + x;
      if (labels[index] == 0) continue;
      uint32_t nb[4] = {0, 0, 0, 0};
      if (x > 0) nb[0] = labels[index - 1];
      if (y > 0) {
        if (x > 0) nb[1] = labels[index - width - 1];
        nb[2] = labels[index - width];
        if (x + 1 < width) nb[3] = labels[index - width + 1];
      }
      uint32_t smallest = 0;
      for (uint32_t l : nb)
        if (l != 0) {
          const uint32_t r = find_root(parent, l);
          if (smallest == 0 || r < smallest) smallest = r;
        }
      if (smallest == 0) {
        const uint32_t fresh = (uint32_t)parent.size();
        parent.push_back(fresh);
        labels[index] = fresh;
      } else {
        for (uint32_t l : nb)
          if (l != 0) parent[find_root(parent, l)] = smallest;
        labels[index] = smallest;
      }
    }
  uint32_t count = 0;
  for (std::size_t p = 1; p < parent.size(); ++p) {
    if (parent[p] == p) parent[p] = ++count;
    else parent[p] = parent[parent[p]];
  }
  for (std::size_t i = 0; i < (std::size_t)width * height; ++i)
    if (labels[i] != 0) labels[i] = parent[labels[i]];
  return count;
}

extern "C" int ro_opposed(float* m, int w, int h, int pattern, const float levels[3], const float* ceiling,
                          uint64_t stats[9], uint32_t* labels_out, uint32_t* region_count) {
  for (int k = 0; k < 9; ++k) stats[k] = 0;
  if (region_count) *region_count = 0;
  // ChannelDetectionLevels / ChannelClipLevels::validate (crates/highlight/src/lib.rs:63-118):
  // every level finite and positive, checked before any sample is read.
  for (int c = 0; c < 3; ++c) {
    if (!std::isfinite(levels[c]) || !(levels[c] > 0.0f)) return -2;
    if (ceiling && (!std::isfinite(ceiling[c]) || !(ceiling[c] > 0.0f))) return -2;
  }
  // validate_visible_samples, opposed.rs:182-219
  uint64_t suspected = 0, sc[3] = {0, 0, 0};
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const float s = m[(std::size_t)y * w + x];
      if (!std::isfinite(s)) return -1;
      const int c = color_at(pattern, x, y);
      if (s >= levels[c]) { suspected++; sc[c]++; }
    }
  stats[0] = suspected; stats[6] = sc[0]; stats[7] = sc[1]; stats[8] = sc[2];
  const int cw = w / 2 + w % 2, ch = h / 2 + h % 2;
  if (suspected == 0) {
    if (labels_out) std::memset(labels_out, 0, sizeof(uint32_t) * (std::size_t)cw * ch);
    return 0;
  }
  // CellSummaries::build, cells.rs:41-113
  std::vector<Cell> cells((std::size_t)cw * ch);
#pragma omp parallel for schedule(static)
  for (int cy = 0; cy < ch; ++cy)
    for (int cx = 0; cx < cw; ++cx) {
      float sums[3] = {0.0f, 0.0f, 0.0f};
      uint32_t counts[3] = {0, 0, 0};
      uint8_t flags = 0;
      for (int y = 2 * cy; y < std::min(2 * cy + 2, h); ++y)
        for (int x = 2 * cx; x < std::min(2 * cx + 2, w); ++x) {
          const int c = color_at(pattern, x, y);
          const float s = m[(std::size_t)y * w + x];
          if (s >= levels[c]) flags |= 1 << (c + 3);
          else if (s > 0.0f) { sums[c] += s; counts[c] += 1; }
        }
      Cell& cell = cells[(std::size_t)cy * cw + cx];
      for (int c = 0; c < 3; ++c) {
        cell.means[c] = 0.0f;
        if (counts[c] != 0) {
          cell.means[c] = sums[c] / (float)counts[c];
          flags |= 1 << c;
        }
      }
      cell.flags = flags;
    }
  auto clipped_at = [&](int x, int y) { return (uint8_t)(cells[(std::size_t)y * cw + x].flags >> 3); };
  auto usable_clean = [&](int x, int y, int c) {
    const uint8_t f = cells[(std::size_t)y * cw + x].flags;
    return (f & (1 << c)) && !(f & (1 << (c + 3)));
  };
  // dilated_mask, regions.rs:127-182
  std::vector<uint8_t> horiz((std::size_t)cw * ch, 0);
  for (int y = 0; y < ch; ++y) {
    long last = -1;
    for (int x = 0; x < cw; ++x) {
      if (clipped_at(x, y)) last = x;
      horiz[(std::size_t)y * cw + x] = last >= 0 && x - last <= DILATION;
    }
    long next = -1;
    for (int x = cw - 1; x >= 0; --x) {
      if (clipped_at(x, y)) next = x;
      horiz[(std::size_t)y * cw + x] |= next >= 0 && next - x <= DILATION;
    }
  }
  std::vector<uint32_t> labels((std::size_t)cw * ch, 0);
  for (int y = 0; y < ch; ++y) {
    const int first = std::max(y - DILATION, 0), last = std::min(y + DILATION, ch - 1);
    for (int sy = first; sy <= last; ++sy)
      for (int x = 0; x < cw; ++x) labels[(std::size_t)y * cw + x] |= horiz[(std::size_t)sy * cw + x];
  }
  const uint32_t count = ro_label_components(labels.data(), cw, ch);
  if (region_count) *region_count = count;
  if (labels_out) std::memcpy(labels_out, labels.data(), sizeof(uint32_t) * labels.size());
  std::vector<uint8_t> region_clipped(count + 1, 0);
  for (int y = 0; y < ch; ++y)
    for (int x = 0; x < cw; ++x) {
      const uint32_t l = labels[(std::size_t)y * cw + x];
      if (l) region_clipped[l] |= clipped_at(x, y);
    }
  // WantedSlots::scan, region_correction.rs:134-178
  std::vector<uint16_t> wanted(count + 1, 0);
  uint16_t any = 0;
  for (int y = 0; y < ch; ++y)
    for (int x = 0; x < cw; ++x) {
      const uint32_t label = labels[(std::size_t)y * cw + x];
      const uint8_t clipped = clipped_at(x, y);
      if (label == 0 || clipped == 0) continue;
      auto has_clean = [&](int c) {
        for (int o = 0; o < 3; ++o)
          if (o != c && usable_clean(x, y, o)) return true;
        return false;
      };
      auto candidate = [&](int c) { return (clipped & (1 << c)) && has_clean(c); };
      const Cell& cell = cells[(std::size_t)y * cw + x];
      for (int c = 0; c < 3; ++c) {
        if (!candidate(c)) continue;
        const int p = pattern_position(c, support_mask(cell, c, levels));
        if (p >= 0) {
          const uint16_t bit = (uint16_t)(1u << (c * PATTERNS + p));
          wanted[label] |= bit;
          any |= bit;
        }
      }
    }
  // RegionCorrections::build, region_correction.rs:196-256
  std::vector<Slot> slots((std::size_t)(count + 1) * SLOTS);
  for (int pass = 0; pass < 2; ++pass) {
    for (int y = 0; y < ch; ++y)
      for (int x = 0; x < cw; ++x) {
        const uint32_t label = labels[(std::size_t)y * cw + x];
        if (label == 0 || clipped_at(x, y) != 0) continue;
        const Cell& cell = cells[(std::size_t)y * cw + x];
        for (int c = 0; c < 3; ++c) {
          if (!(region_clipped[label] & (1 << c))) continue;
          if (cell.means[c] < BORDER_MIN_FRACTION * levels[c]) continue;
          unsigned pats[3];
          support_patterns(c, pats);
          for (int p = 0; p < 3; ++p) {
            const int offset = c * PATTERNS + p;
            const bool for_region = wanted[label] & (1 << offset);
            const bool for_pool = any & (1 << offset);
            if (!for_region && !for_pool) continue;
            float value;
            if (!correction(cell, c, pats[p], levels, &value)) continue;
            float ratio = 0.0f;
            const bool has_ratio = log_ratio(cell, pats[p], &ratio);
            if (for_region) slots[(std::size_t)label * SLOTS + offset].add(pass, value, has_ratio, ratio);
            if (for_pool) slots[offset].add(pass, value, has_ratio, ratio);
          }
        }
      }
    if (pass == 0)
      for (auto& s : slots) s.finish_moments();
  }
  auto lookup = [&](uint32_t label, int channel, unsigned support, float* offset, bool* has_ratio, float* ratio) {
    const int p = pattern_position(channel, support);
    if (p < 0) return false;
    const int off = channel * PATTERNS + p;
    const bool hr = popcount(support) == 2;
    if (slots[(std::size_t)label * SLOTS + off].value(hr, offset, has_ratio, ratio)) return true;
    return slots[off].value(hr, offset, has_ratio, ratio);
  };
  // estimate_site / local_correction, opposed.rs:236-330
  auto estimate_site = [&](const Cell& target, int channel, int tx, int ty, float* out) {
    const unsigned support = support_mask(target, channel, levels);
    float ref;
    if (!reference(target, support, &ref)) return false;
    float tratio = 0.0f;
    const bool has_tratio = log_ratio(target, support, &tratio);
    // local_correction
    float corr[MAX_CANDIDATES];
    int n = 0;
    bool has_local = false;
    float local = 0.0f;
    int local_radius = 0;
    for (int radius = FIRST_RADIUS; radius <= LAST_RADIUS && !has_local; ++radius) {
      for (int cy = std::max(ty - radius, 0); cy <= std::min(ty + radius, ch - 1); ++cy)
        for (int cx = std::max(tx - radius, 0); cx <= std::min(tx + radius, cw - 1); ++cx) {
          if (std::max(std::abs(tx - cx), std::abs(ty - cy)) != radius) continue;
          if (!usable_clean(cx, cy, channel)) continue;
          const Cell& cand = cells[(std::size_t)cy * cw + cx];
          float value;
          if (!correction(cand, channel, support, levels, &value)) continue;
          float cratio = 0.0f;
          const bool has_cratio = log_ratio(cand, support, &cratio);
          if (!chroma_agrees(support, has_tratio, tratio, has_cratio, cratio)) continue;
          if (n < MAX_CANDIDATES) corr[n++] = value;
        }
      if (n >= MIN_CANDIDATES) {
        // total_cmp sort; values are finite so a plain sort with -0 < +0 suffices.
        std::sort(corr, corr + n, [](float a, float b) {
          if (a == b) return std::signbit(a) && !std::signbit(b);
          return a < b;
        });
        const int mid = n / 2;
        local = n % 2 == 0 ? (corr[mid - 1] + corr[mid]) * 0.5f : corr[mid];
        local_radius = radius;
        has_local = true;
      }
    }
    const uint32_t label = labels[(std::size_t)ty * cw + tx];
    float region = 0.0f, bratio = 0.0f;
    bool has_bratio = false;
    bool has_region = lookup(label, channel, support, &region, &has_bratio, &bratio);
    if (has_region && !chroma_agrees(support, has_tratio, tratio, has_bratio, bratio)) has_region = false;
    float corr_value;
    if (has_local && has_region) {
      const float weight = (float)(LAST_RADIUS + 1 - local_radius) / (float)LAST_RADIUS;
      corr_value = weight * local + (1.0f - weight) * region;
    } else if (has_local) {
      corr_value = local;
    } else if (has_region) {
      corr_value = region;
    } else {
      return false;
    }
    const float estimate = ref + corr_value;
    if (!(std::isfinite(estimate) && estimate > 0.0f)) return false;
    *out = estimate;
    return true;
  };
  uint64_t reconstructed = 0, changed = 0, fallback = 0, unsupported = 0, neutralised = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : reconstructed, changed, fallback, unsupported, neutralised)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float& s = m[(std::size_t)y * w + x];
      const int c = color_at(pattern, x, y);
      const float level = levels[c];
      if (!(s >= level)) continue;
      const int tx = x / 2, ty = y / 2;
      const Cell& target = cells[(std::size_t)ty * cw + tx];
      int support_count = 0;
      for (int o = 0; o < 3; ++o)
        if (o != c && target.usable(o) && target.clean(o)) support_count++;
      float estimate = 0.0f;
      const bool ok = support_count != 0 && estimate_site(target, c, tx, ty, &estimate);
      auto neutralise = [&]() {
        if (!ceiling) return;
        if (s > ceiling[c]) { s = ceiling[c]; neutralised++; }
      };
      if (!ok) {
        fallback++;
        if (support_count == 0) unsupported++;
        neutralise();
        continue;
      }
      reconstructed++;
      const float bounded = rmin(estimate, MAXIMUM_ESTIMATE_MULTIPLIER * level);
      if (bounded > s) {
        s = bounded;
        changed++;
      } else {
        neutralise();
      }
    }
  stats[1] = reconstructed; stats[2] = changed; stats[3] = fallback; stats[4] = unsupported; stats[5] = neutralised;
  return 0;
}
