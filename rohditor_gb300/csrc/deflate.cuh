// Deflate (RFC 1951), zlib (RFC 1950) and PNG CRC-32 arithmetic of the PNG
// encoder (k_encode.cu). Everything here is a plain function of its
// arguments, compiled for the device and, by the host test harness, for the
// CPU, so that the block format is checked against zlib without a GPU.
//
// Stream layout. The filtered PNG scanlines form one byte stream that is cut
// into segments of SEG bytes. Each segment becomes exactly one deflate block
// that starts on a byte boundary:
//  * a dynamic-Huffman block (BTYPE 10) whose matches all have distance 1
//    (runs of a repeated byte), followed, unless it is the last block, by an
//    empty stored block that pads the stream to the next byte boundary;
//  * or, when that would be larger, one stored block (BTYPE 00) of the bytes.
// Byte-aligned blocks concatenate without bit shifting, so segments are
// encoded independently and their bytes are laid out by a prefix sum.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define RD_HD __host__ __device__ __forceinline__
#else
#define RD_HD inline
#endif

namespace rd {
namespace png {

constexpr int SEG = 32768;                // filtered-stream bytes per deflate block
constexpr int STORED_OVERHEAD = 5;        // BFINAL/BTYPE byte, LEN, NLEN
constexpr int SEG_CAP = SEG + 64;         // bytes reserved per encoded segment (16-byte multiple)
constexpr int LIT_SYMBOLS = 286;          // literal/length alphabet, 0..285
constexpr int END_OF_BLOCK = 256;
constexpr int MAX_BITS = 15;              // literal/length and distance code length limit
constexpr int CLEN_SYMBOLS = 19;          // code-length alphabet
constexpr int CLEN_MAX_BITS = 7;
constexpr int MAX_RUN = 258;              // longest deflate match
constexpr int HEADER_ITEMS = LIT_SYMBOLS + 2;  // code lengths sent: HLIT + HDIST (HDIST = 2)
constexpr int HEADER_WORDS = 130;          // >= 3 + 14 + 19*3 + (286 + 2) * (7 + 7) header bits, in words
constexpr uint32_t ADLER_MOD = 65521u;
constexpr uint32_t CRC_POLY = 0xEDB88320u;  // CRC-32 of PNG / zlib, reflected

static_assert(SEG_CAP % 16 == 0, "segment slots hold 16-byte vectors");
static_assert(SEG + STORED_OVERHEAD <= SEG_CAP, "a stored segment fits its slot");
static_assert(SEG <= 65535, "one stored block holds a segment");
static_assert(32 * HEADER_WORDS >= 3 + 14 + 3 * CLEN_SYMBOLS + HEADER_ITEMS * (7 + 7), "header words");

RD_HD int floor_log2(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return 31 - __clz((int)v);
#else
  return 31 - __builtin_clz(v);
#endif
}

// Literal/length symbol of a match length 3..258 (RFC 1951 3.2.5): lengths
// 3..10 have symbols 257..264 and no extra bits; above that every group of
// four symbols doubles the span, so with v = len - 3 the number of extra bits
// is floor(log2 v) - 2 and the two bits below the leading one select the
// symbol within its group; 258 has its own symbol 285.
RD_HD int length_symbol(int len, int* extra_bits, int* extra_value) {
  if (len == MAX_RUN) {
    *extra_bits = 0;
    *extra_value = 0;
    return 285;
  }
  const int v = len - 3;
  if (v < 8) {
    *extra_bits = 0;
    *extra_value = 0;
    return 257 + v;
  }
  const int e = floor_log2((uint32_t)v) - 2;
  const int group = (v >> e) & 3;
  *extra_bits = e;
  *extra_value = v - ((4 + group) << e);
  return 257 + 4 * e + 4 + group;
}

// Token that starts at position p of a run [a, b): positions a..b-1 each
// repeat the byte before them (position a - 1 is a literal). Matches of
// distance 1 cover the run greedily, 258 bytes at a time, and a tail shorter
// than 3 bytes is sent as literals. Returns 0 when p lies inside a match,
// 1 when p is a literal, or the length (3..258) of the match starting at p.
RD_HD int run_token(int p, int a, int b) {
  const int k = p - a;
  const int q = k - k % MAX_RUN;
  const int rest = b - a - q;
  if (rest >= 3) return k == q ? (rest < MAX_RUN ? rest : MAX_RUN) : 0;
  return 1;
}

RD_HD int clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return __builtin_clzll(v);
#endif
}
RD_HD int ctz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __ffsll((long long)v) - 1;
#else
  return __builtin_ctzll(v);
#endif
}

// A thread's share of a segment: CHUNK bytes at segment position c0, held in
// 16 little-endian words (registers on the device when indexed by constants).
constexpr int CHUNK = 32;  // below 64, so (1ull << count) - 1 is the mask of a full chunk
constexpr int CHUNK_WORDS = CHUNK / 4;

RD_HD uint32_t chunk_byte(const uint32_t* w, int j) { return (w[j >> 2] >> (8 * (j & 3))) & 0xFFu; }

// Bit j set when byte j of the chunk differs from the byte before it (`prev`
// for j = 0), and always for the first byte of a segment; bits at and above
// `count` are clear. The set bits are where a run of repeated bytes cannot
// continue: every token of the segment starts at one, or inside a run.
RD_HD uint64_t chunk_breaks(const uint32_t* w, int count, uint32_t prev, bool segment_start) {
  uint64_t m = 0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int j = 0; j < CHUNK; ++j) {
    const uint32_t b = chunk_byte(w, j);
    if (b != prev) m |= 1ull << j;
    prev = b;
  }
  if (segment_start) m |= 1ull;
  if (count < CHUNK) m &= (1ull << count) - 1ull;
  return m;
}

// Calls visit(literal, 0) or visit(0, length) for each token that starts in
// the chunk's first `count` bytes. `before` is the segment position of the
// last break before the chunk (position 0 always is one) and `after` the
// first break at or after its end (or the segment length): together with the
// chunk's own breaks they bound the run each repeated byte belongs to.
template <class Visit>
RD_HD void chunk_tokens(const uint32_t* w, uint64_t breaks, int c0, int count, int before, int after,
                        Visit&& visit) {
  if (breaks == (1ull << count) - 1ull) {  // no byte repeats its predecessor: all literals
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int j = 0; j < CHUNK; ++j) {
      if (j >= count) break;
      visit(chunk_byte(w, j), 0);
    }
    return;
  }
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int j = 0; j < CHUNK; ++j) {
    if (j >= count) break;
    const uint32_t x = chunk_byte(w, j);
    if ((breaks >> j) & 1ull) {
      visit(x, 0);
      continue;
    }
    const uint64_t upto = j == CHUNK - 1 ? ~0ull : (2ull << j) - 1ull;
    const uint64_t below = breaks & upto;
    const uint64_t above = breaks & ~upto;
    const int a = (below ? c0 + 63 - clz64(below) : before) + 1;
    const int b = above ? c0 + ctz64(above) : after;
    const int t = run_token(c0 + j, a, b);
    if (t == 1)
      visit(x, 0);
    else if (t >= 3)
      visit(0u, t);
  }
}

// The low `len` (1..16) bits of code in reverse order.
RD_HD uint32_t reverse_bits(uint32_t code, int len) {
#if defined(__CUDA_ARCH__)
  return __brev(code) >> (32 - len);
#else
  uint32_t r = 0;
  for (int i = 0; i < len; ++i) {
    r = (r << 1) | (code & 1u);
    code >>= 1;
  }
  return r;
#endif
}

// Huffman tree over n >= 2 leaf weights in ascending order: leaves and merged
// nodes are taken from two queues (both stay sorted), which builds an optimal
// tree in O(n). Nodes n..2n-2 are the merged ones, 2n-2 the root; parent[i]
// is the node that absorbed node i. Scratch weight[2n].
RD_HD void huffman_tree(const uint32_t* leaf, int n, uint32_t* weight, uint16_t* parent) {
  for (int i = 0; i < n; ++i) weight[i] = leaf[i];
  int next_leaf = 0, next_node = n, created = n;
  for (int k = 0; k < n - 1; ++k) {
    int pick[2];
    for (int j = 0; j < 2; ++j) {
      if (next_leaf < n && (next_node >= created || weight[next_leaf] <= weight[next_node]))
        pick[j] = next_leaf++;
      else
        pick[j] = next_node++;
    }
    weight[created] = weight[pick[0]] + weight[pick[1]];
    parent[pick[0]] = (uint16_t)created;
    parent[pick[1]] = (uint16_t)created;
    ++created;
  }
}

// Huffman code lengths of the n symbols whose indices `order` lists by
// ascending (frequency, symbol). When the tree is deeper than `limit`, every
// frequency is halved (rounding up, so none reaches zero and the order is
// kept) and the tree is rebuilt; a tree built this way is always complete,
// which inflaters require of the code. Scratch: leaf[n], weight[2n],
// parent[2n], depth[2n]. Writes len[order[i]].
RD_HD void huffman_lengths(const uint32_t* freq, const uint16_t* order, int n, int limit, uint32_t* leaf,
                           uint32_t* weight, uint16_t* parent, uint8_t* depth, uint8_t* len) {
  if (n < 2) {  // a lone symbol still needs a one-bit code
    if (n == 1) len[order[0]] = 1;
    return;
  }
  for (int i = 0; i < n; ++i) leaf[i] = freq[order[i]];
  for (;;) {
    huffman_tree(leaf, n, weight, parent);
    // Every node's parent was created after it, so depths resolve from the
    // root (the last node) downwards.
    const int root = 2 * n - 2;
    depth[root] = 0;
    int deepest = 0;
    for (int i = root - 1; i >= 0; --i) {
      depth[i] = (uint8_t)(depth[parent[i]] + 1);
      if (i < n && depth[i] > deepest) deepest = depth[i];
    }
    if (deepest <= limit) break;
    for (int i = 0; i < n; ++i) leaf[i] = (leaf[i] + 1) >> 1;
  }
  for (int i = 0; i < n; ++i) len[order[i]] = depth[i];
}

// Canonical codes of RFC 1951 3.2.2 from code lengths, bit-reversed so that
// they go out least significant bit first like every other deflate field.
RD_HD void canonical_codes(const uint8_t* len, int n, int max_bits, uint16_t* code) {
  uint32_t count[MAX_BITS + 1] = {};
  for (int s = 0; s < n; ++s) count[len[s]]++;
  count[0] = 0;
  uint32_t next[MAX_BITS + 2] = {};
  uint32_t c = 0;
  for (int bits = 1; bits <= max_bits; ++bits) {
    c = (c + count[bits - 1]) << 1;
    next[bits] = c;
  }
  for (int s = 0; s < n; ++s)
    code[s] = len[s] ? (uint16_t)reverse_bits(next[len[s]]++, len[s]) : (uint16_t)0;
}

// Order in which the code-length code's lengths are sent (RFC 1951 3.2.7).
RD_HD int clen_order(int i) {
  constexpr int ORDER[CLEN_SYMBOLS] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  return ORDER[i];
}

// Run-length form of a code-length sequence (RFC 1951 3.2.7): 16 repeats the
// previous length 3..6 times, 17 writes 3..10 zeros and 18 writes 11..138.
// Writes (symbol, extra value) pairs; returns their count (<= n).
RD_HD int clen_items(const uint8_t* lengths, int n, uint8_t* sym, uint8_t* extra) {
  int items = 0;
  int i = 0;
  while (i < n) {
    const uint8_t v = lengths[i];
    int run = 1;
    while (i + run < n && lengths[i + run] == v) ++run;
    i += run;
    if (v == 0) {
      while (run >= 11) {
        const int r = run < 138 ? run : 138;
        sym[items] = 18;
        extra[items++] = (uint8_t)(r - 11);
        run -= r;
      }
      if (run >= 3) {
        sym[items] = 17;
        extra[items++] = (uint8_t)(run - 3);
        run = 0;
      }
    } else {
      sym[items] = v;
      extra[items++] = 0;
      --run;
      while (run >= 3) {
        const int r = run < 6 ? run : 6;
        sym[items] = 16;
        extra[items++] = (uint8_t)(r - 3);
        run -= r;
      }
    }
    while (run > 0) {
      sym[items] = v;
      extra[items++] = 0;
      --run;
    }
  }
  return items;
}

RD_HD int clen_extra_bits(int sym) { return sym == 16 ? 2 : (sym == 17 ? 3 : (sym == 18 ? 7 : 0)); }

// Least-significant-bit-first writer over 32-bit words (the caller zeroes
// them). `bits` <= 32 per call.
struct BitWriter {
  uint32_t* words;
  uint32_t pos;
  RD_HD void put(uint32_t value, int bits) {
    if (bits == 0) return;
    const uint64_t v = (uint64_t)value << (pos & 31u);
    words[pos >> 5] |= (uint32_t)v;
    if ((pos & 31u) + (uint32_t)bits > 32u) words[(pos >> 5) + 1] |= (uint32_t)(v >> 32);
    pos += (uint32_t)bits;
  }
};

// The literal/length lengths of a segment and the scratch that turns them into
// a dynamic block header. Filled and used by one thread.
struct HeaderScratch {
  uint8_t seq[HEADER_ITEMS];  // code lengths sent: HLIT literal/length, then HDIST distance
  uint8_t sym[HEADER_ITEMS];
  uint8_t extra[HEADER_ITEMS];
  uint32_t freq[CLEN_SYMBOLS];
  uint16_t order[CLEN_SYMBOLS + 1];
  uint8_t len[CLEN_SYMBOLS + 1];
  uint16_t code[CLEN_SYMBOLS + 1];
  uint32_t leaf[CLEN_SYMBOLS + 1];
  uint32_t weight[2 * CLEN_SYMBOLS + 2];
  uint16_t parent[2 * CLEN_SYMBOLS + 2];
  uint8_t depth[2 * CLEN_SYMBOLS + 2];
};

// Writes the 3-bit block header and the dynamic-Huffman header of a block
// whose literal/length code has lengths `lit_len` (286 entries) and whose
// distance code is two one-bit codes (distance symbols 0 and 1; only symbol 0,
// distance 1, is used). Returns the bits written.
RD_HD uint32_t write_dynamic_header(BitWriter& w, bool final_block, const uint8_t* lit_len, HeaderScratch& h) {
  const uint32_t start = w.pos;
  int hlit = LIT_SYMBOLS;
  while (hlit > 257 && lit_len[hlit - 1] == 0) --hlit;
  const int hdist = 2;
  for (int s = 0; s < hlit; ++s) h.seq[s] = lit_len[s];
  h.seq[hlit] = 1;
  h.seq[hlit + 1] = 1;
  const int items = clen_items(h.seq, hlit + hdist, h.sym, h.extra);
  for (int s = 0; s < CLEN_SYMBOLS; ++s) h.freq[s] = 0;
  for (int i = 0; i < items; ++i) h.freq[h.sym[i]]++;
  // A code needs two symbols; a single used symbol gets a partner that is never sent.
  int used = 0;
  for (int s = 0; s < CLEN_SYMBOLS; ++s) used += h.freq[s] != 0;
  uint32_t freq[CLEN_SYMBOLS];
  for (int s = 0; s < CLEN_SYMBOLS; ++s) freq[s] = h.freq[s];
  if (used < 2) {
    for (int s = 0; s < CLEN_SYMBOLS; ++s)
      if (!freq[s]) {
        freq[s] = 1;
        break;
      }
  }
  // Ascending (frequency, symbol) by insertion; 19 symbols.
  int n = 0;
  for (int s = 0; s < CLEN_SYMBOLS; ++s) {
    if (!freq[s]) continue;
    int j = n++;
    while (j > 0 && freq[h.order[j - 1]] > freq[s]) {
      h.order[j] = h.order[j - 1];
      --j;
    }
    h.order[j] = (uint16_t)s;
  }
  for (int s = 0; s < CLEN_SYMBOLS; ++s) h.len[s] = 0;
  huffman_lengths(freq, h.order, n, CLEN_MAX_BITS, h.leaf, h.weight, h.parent, h.depth, h.len);
  canonical_codes(h.len, CLEN_SYMBOLS, CLEN_MAX_BITS, h.code);
  int hclen = CLEN_SYMBOLS;
  while (hclen > 4 && h.len[clen_order(hclen - 1)] == 0) --hclen;
  w.put(final_block ? 1u : 0u, 1);
  w.put(2u, 2);
  w.put((uint32_t)(hlit - 257), 5);
  w.put((uint32_t)(hdist - 1), 5);
  w.put((uint32_t)(hclen - 4), 4);
  for (int i = 0; i < hclen; ++i) w.put(h.len[clen_order(i)], 3);
  for (int i = 0; i < items; ++i) {
    const int s = h.sym[i];
    w.put(h.code[s], h.len[s]);
    w.put(h.extra[i], clen_extra_bits(s));
  }
  return w.pos - start;
}

// ---- CRC-32 ----------------------------------------------------------------
// CRC-32 as PNG chunks carry it (ISO 3309 polynomial, reflected, register
// preset to all ones and inverted at the end). In the reflected register, bit
// 31 holds the coefficient of x^0 and bit 0 that of x^31, so multiplying by x
// is a right shift that folds the polynomial back in when x^32 appears.
// Feeding a zero byte multiplies the register by x^8; with that, the CRC of a
// concatenation A||B is (register after A) * x^(8|B|) xor (register of B from
// zero), which lets each thread checksum its own bytes.
RD_HD uint32_t gf2_times_x(uint32_t v) { return (v & 1u) ? (v >> 1) ^ CRC_POLY : v >> 1; }

RD_HD uint32_t gf2_mul(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 0; i < 32; ++i) {
    if ((a >> (31 - i)) & 1u) p ^= b;
    b = gf2_times_x(b);
  }
  return p;
}

constexpr uint32_t GF2_ONE = 0x80000000u;  // x^0
constexpr uint32_t GF2_X8 = 0x00800000u;   // x^8

// xpow[k] = x^(8 * 2^k): the shift by 2^k zero bytes.
struct CrcShifts {
  uint32_t xpow[40];
};

RD_HD void crc_shift_table(CrcShifts& t) {
  t.xpow[0] = GF2_X8;
  for (int k = 1; k < 40; ++k) t.xpow[k] = gf2_mul(t.xpow[k - 1], t.xpow[k - 1]);
}

// Register v advanced over `bytes` zero bytes.
RD_HD uint32_t crc_shift(const CrcShifts& t, uint32_t v, uint64_t bytes) {
  uint32_t m = GF2_ONE;
  for (int k = 0; bytes; ++k, bytes >>= 1)
    if (bytes & 1u) m = gf2_mul(m, t.xpow[k]);
  return gf2_mul(v, m);
}

// Table of the register after one byte (the byte's value at zero register).
RD_HD uint32_t crc_byte_entry(uint32_t byte) {
  uint32_t c = byte;
  for (int k = 0; k < 8; ++k) c = (c & 1u) ? (c >> 1) ^ CRC_POLY : c >> 1;
  return c;
}

RD_HD uint32_t crc_update(const uint32_t* table, uint32_t reg, const uint8_t* p, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) reg = table[(reg ^ p[i]) & 0xFFu] ^ (reg >> 8);
  return reg;
}

// ---- Adler-32 ---------------------------------------------------------------
// zlib's checksum over L bytes d_0..d_{L-1}: A = 1 + sum d_i, B = sum over the
// prefixes of A = L + sum (L - i) d_i, both mod 65521. A segment of n bytes
// at offset o contributes (L - o - n) * S1 + S2 to B with S1 = sum d_j and
// S2 = sum (n - j) d_j over its own bytes.
RD_HD uint32_t adler_combine_term(uint64_t L, uint64_t o, uint64_t n, uint32_t s1, uint32_t s2) {
  const uint64_t w = (L - o - n) % ADLER_MOD;
  return (uint32_t)((w * s1 + s2) % ADLER_MOD);
}

}  // namespace png
}  // namespace rd
