// Host harness of the PNG encoder's deflate arithmetic (test infrastructure).
//
// Compiles rohditor_gb300/csrc/deflate.cuh for the CPU and runs the segment
// encoder the way png_histogram_kernel and png_pack_kernel do, with their
// 1024 threads played one after another: the same per-thread byte ranges, run
// boundaries, token walk,
// Huffman construction, header, bit offsets and stored-block decision. The
// tests feed its zlib stream to Python's zlib, so the block format is checked
// without a GPU.
//
//   deflate_host IN OUT   reads IN, writes the zlib stream to OUT and prints
//                         "<crc32> <adler32> <segments> <stored segments>"
//                         where the checksums come from the combine rules
//                         (CRC over 256 slices, Adler-32 over segments).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <vector>

#include "../../rohditor_gb300/csrc/deflate.cuh"

using namespace rd::png;

namespace {

constexpr int THREADS = SEG / CHUNK;

struct Segment {
  std::vector<uint8_t> bytes;
  uint32_t s1 = 0, s2 = 0;
  bool stored = false;
};

struct ThreadChunk {
  uint32_t w[CHUNK_WORDS] = {};
  int c0 = 0, count = 0, before = -1, after = 0;
  uint64_t breaks = 0;
};

Segment encode_segment(const uint8_t* in, int n, bool last) {
  Segment out;
  std::vector<ThreadChunk> ch(THREADS);
  unsigned long long s1 = 0, s2 = 0;
  for (int t = 0; t < THREADS; ++t) {
    ThreadChunk& c = ch[t];
    c.c0 = std::min(t * CHUNK, n);
    c.count = std::min(CHUNK, n - c.c0);
    std::memcpy(c.w, in + c.c0, (size_t)c.count);  // little-endian host: byte j is chunk_byte(w, j)
    c.breaks = chunk_breaks(c.w, c.count, c.c0 > 0 ? in[c.c0 - 1] : 0u, c.c0 == 0);
    for (int j = 0; j < c.count; ++j) {
      s1 += in[c.c0 + j];
      s2 += (unsigned long long)(n - c.c0 - j) * in[c.c0 + j];
    }
  }
  int run = -1;
  for (int t = 0; t < THREADS; ++t) {
    ch[t].before = run;
    if (ch[t].breaks) run = std::max(run, ch[t].c0 + 63 - clz64(ch[t].breaks));
  }
  run = n;
  for (int t = THREADS - 1; t >= 0; --t) {
    ch[t].after = run;
    if (ch[t].breaks) run = std::min(run, ch[t].c0 + ctz64(ch[t].breaks));
  }
  out.s1 = (uint32_t)(s1 % ADLER_MOD);
  out.s2 = (uint32_t)(s2 % ADLER_MOD);
  auto tokens = [&](int t, auto&& visit) {
    const ThreadChunk& c = ch[t];
    chunk_tokens(c.w, c.breaks, c.c0, c.count, c.before, c.after, visit);
  };

  uint32_t freq[LIT_SYMBOLS] = {};
  freq[END_OF_BLOCK] = 1;
  for (int t = 0; t < THREADS; ++t)
    tokens(t, [&](uint32_t lit, int len) {
      int eb, ev;
      freq[len ? length_symbol(len, &eb, &ev) : (int)lit]++;
    });
  uint16_t order[LIT_SYMBOLS];
  int used = 0;
  for (int s = 0; s < LIT_SYMBOLS; ++s) {
    if (!freq[s]) continue;
    int rank = 0;
    for (int u = 0; u < LIT_SYMBOLS; ++u)
      rank += freq[u] && (freq[u] < freq[s] || (freq[u] == freq[s] && u < s));
    order[rank] = (uint16_t)s;
    ++used;
  }
  uint32_t leaf[LIT_SYMBOLS], weight[2 * LIT_SYMBOLS];
  uint16_t parent[2 * LIT_SYMBOLS], code[LIT_SYMBOLS];
  uint8_t depth[2 * LIT_SYMBOLS], len[LIT_SYMBOLS] = {};
  huffman_lengths(freq, order, used, MAX_BITS, leaf, weight, parent, depth, len);
  canonical_codes(len, LIT_SYMBOLS, MAX_BITS, code);
  std::vector<uint32_t> words(SEG_CAP / 4, 0);
  BitWriter w{words.data(), 0};
  static HeaderScratch hs;
  const uint32_t header_bits = write_dynamic_header(w, last, len, hs);

  std::vector<uint32_t> bits(THREADS, 0), offset(THREADS);
  for (int t = 0; t < THREADS; ++t)
    tokens(t, [&](uint32_t lit, int l) {
      int eb, ev;
      bits[t] += l ? len[length_symbol(l, &eb, &ev)] + eb + 1 : len[lit];
    });
  uint32_t acc = header_bits;
  for (int t = 0; t < THREADS; ++t) {
    offset[t] = acc;
    acc += bits[t];
  }
  const uint32_t eob_at = acc;
  const uint32_t end = eob_at + len[END_OF_BLOCK];
  const uint32_t dyn_bytes = last ? (end + 7) / 8 : (end + 3 + 7) / 8 + 4;
  const uint32_t stored_bytes = (uint32_t)n + STORED_OVERHEAD;
  out.stored = dyn_bytes >= stored_bytes;
  if (!out.stored) {
    for (int t = 0; t < THREADS; ++t) {
      BitWriter tw{words.data(), offset[t]};
      tokens(t, [&](uint32_t lit, int l) {
        if (l) {
          int eb, ev;
          const int sym = length_symbol(l, &eb, &ev);
          tw.put(code[sym], len[sym]);
          tw.put((uint32_t)ev, eb);
          tw.put(0u, 1);
        } else {
          tw.put(code[lit], len[lit]);
        }
      });
      if (tw.pos != offset[t] + bits[t]) {
        std::fprintf(stderr, "bit count mismatch in thread %d\n", t);
        std::exit(2);
      }
    }
    BitWriter ew{words.data(), eob_at};
    ew.put(code[END_OF_BLOCK], len[END_OF_BLOCK]);
    uint8_t* bytes = reinterpret_cast<uint8_t*>(words.data());
    if (!last) {
      const uint32_t at = (end + 3 + 7) / 8;
      bytes[at + 2] = 0xFF;
      bytes[at + 3] = 0xFF;
    }
    out.bytes.assign(bytes, bytes + dyn_bytes);
  } else {
    out.bytes.push_back(last ? 1 : 0);
    out.bytes.push_back((uint8_t)n);
    out.bytes.push_back((uint8_t)(n >> 8));
    out.bytes.push_back((uint8_t)~n);
    out.bytes.push_back((uint8_t)(~n >> 8));
    out.bytes.insert(out.bytes.end(), in, in + n);
  }
  return out;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: deflate_host IN OUT\n");
    return 1;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 1;
  std::vector<uint8_t> data;
  uint8_t buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + got);
  std::fclose(f);
  const uint64_t L = data.size();
  if (L == 0) return 1;
  const uint64_t nseg = (L + SEG - 1) / SEG;
  std::vector<uint8_t> z = {0x78, 0x9C};
  uint64_t asum = 0, bsum = 0;
  int stored = 0;
  for (uint64_t s = 0; s < nseg; ++s) {
    const uint64_t o = s * SEG;
    const int n = (int)std::min<uint64_t>(SEG, L - o);
    const Segment seg = encode_segment(data.data() + o, n, s + 1 == nseg);
    z.insert(z.end(), seg.bytes.begin(), seg.bytes.end());
    asum += seg.s1;
    bsum = (bsum + adler_combine_term(L, o, (uint64_t)n, seg.s1, seg.s2)) % ADLER_MOD;
    stored += seg.stored;
  }
  const uint32_t A = (uint32_t)((1 + asum) % ADLER_MOD);
  const uint32_t B = (uint32_t)((L % ADLER_MOD + bsum) % ADLER_MOD);
  const uint32_t adler = (B << 16) | A;
  for (int k = 0; k < 4; ++k) z.push_back((uint8_t)(adler >> (24 - 8 * k)));
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 1;
  std::fwrite(z.data(), 1, z.size(), o);
  std::fclose(o);

  // CRC-32 of the input from 256 slices, combined as png_chunk_kernel does.
  uint32_t table[256];
  for (uint32_t i = 0; i < 256; ++i) table[i] = crc_byte_entry(i);
  CrcShifts shifts;
  crc_shift_table(shifts);
  const uint64_t per = (L + 255) / 256;
  uint32_t reg = crc_shift(shifts, 0xFFFFFFFFu, L);
  for (uint64_t t = 0; t < 256; ++t) {
    const uint64_t b0 = std::min(t * per, L), b1 = std::min(b0 + per, L);
    if (b1 > b0) reg ^= crc_shift(shifts, crc_update(table, 0u, data.data() + b0, b1 - b0), L - b1);
  }
  std::printf("%u %u %llu %d\n", reg ^ 0xFFFFFFFFu, adler, (unsigned long long)nseg, stored);
  return 0;
}
