// DEFLATE decoder (RFC 1951) for one BGZF block, usable on the device and on the host.
//
// A BGZF block (SAM/BAM specification §4.1) is a gzip member whose compressed payload is raw DEFLATE
// data of at most 64 KiB of output.  breseq reads its BAM through htslib, which inflates each block
// with zlib (a third-party library outside the reference tree); this is a restatement of the
// format's decoding procedure: stored, fixed-Huffman and dynamic-Huffman blocks, canonical Huffman
// codes decoded bit by bit from the code-length counts, and LZ77 length/distance copies.
//
// Every read of the input and every write or back-reference of the output is checked against its
// bounds; malformed data returns an error code instead of touching memory outside the buffers.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define BSQ_HD __host__ __device__ __forceinline__
#else
#define BSQ_HD inline
#endif

namespace bsq {
namespace inflate {

enum : int {
  kOk = 0,
  kErrInput = 1,       // ran past the end of the compressed data
  kErrBlockType = 2,   // block type 3
  kErrStored = 3,      // stored block length and its complement disagree
  kErrCode = 4,        // over-subscribed or unusable code lengths, or an undecodable symbol
  kErrOutput = 5,      // output larger than the capacity
  kErrDistance = 6,    // back-reference before the start of the output
  kErrSymbol = 7,      // length or distance symbol outside the alphabet
};

constexpr int kMaxBits = 15;

// Bit reader over a byte buffer, least significant bit first.
struct Bits {
  const uint8_t* in;
  uint32_t len, pos;   // bytes
  uint64_t buf;
  int cnt;             // bits in buf
  int err;
};

BSQ_HD void bits_init(Bits& b, const uint8_t* in, uint32_t len) {
  b.in = in; b.len = len; b.pos = 0; b.buf = 0; b.cnt = 0; b.err = 0;
}

// Ensures n <= 32 bits are buffered; past the end of the input sets kErrInput.
BSQ_HD bool bits_need(Bits& b, int n) {
  while (b.cnt < n) {
    if (b.pos >= b.len) { b.err = kErrInput; return false; }
    b.buf |= (uint64_t)b.in[b.pos++] << b.cnt;
    b.cnt += 8;
  }
  return true;
}

BSQ_HD uint32_t bits_get(Bits& b, int n) {   // n <= 24
  if (n == 0) return 0;
  if (!bits_need(b, n)) return 0;
  const uint32_t v = (uint32_t)(b.buf & ((1ull << n) - 1));
  b.buf >>= n;
  b.cnt -= n;
  return v;
}

// A canonical Huffman code: count[len] codes of each length, symbols in (length, value) order.
struct Code {
  uint16_t count[kMaxBits + 1];
  uint16_t symbol[288];
};

// Builds the code from the code lengths of n symbols.  Returns false when the lengths over-subscribe
// the code space.  A code may be incomplete (RFC 1951 allows a single distance code); an
// incomplete code's unused bit patterns fail when decoded.
BSQ_HD bool code_build(Code& c, const uint8_t* lengths, int n) {
  for (int l = 0; l <= kMaxBits; l++) c.count[l] = 0;
  for (int s = 0; s < n; s++) c.count[lengths[s]]++;
  int left = 1;
  for (int l = 1; l <= kMaxBits; l++) {
    left <<= 1;
    left -= c.count[l];
    if (left < 0) return false;
  }
  uint16_t offs[kMaxBits + 1];
  offs[1] = 0;
  for (int l = 1; l < kMaxBits; l++) offs[l + 1] = offs[l] + c.count[l];
  for (int s = 0; s < n; s++)
    if (lengths[s] != 0) c.symbol[offs[lengths[s]]++] = (uint16_t)s;
  return true;
}

// Decodes one symbol: the code's bits arrive most significant first, one stream bit at a time; codes
// of each length are consecutive integers starting at `first`.  Returns -1 on failure.
BSQ_HD int code_decode(Bits& b, const Code& c) {
  int code = 0, first = 0, index = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code |= (int)bits_get(b, 1);
    if (b.err) return -1;
    const int count = c.count[l];
    if (code - first < count) return c.symbol[index + (code - first)];
    index += count;
    first += count;
    first <<= 1;
    code <<= 1;
  }
  b.err = kErrCode;
  return -1;
}

// Length symbols 257..285 and distance symbols 0..29: base values and extra bits (RFC 1951 §3.2.5),
// from the tables' closed forms (a table in a function would be rebuilt at every call on the device).
BSQ_HD int length_extra(int i) { return (i < 8 || i == 28) ? 0 : (i - 4) >> 2; }
BSQ_HD uint32_t length_base(int i) {
  return i == 28 ? 258u : (i < 8 ? 3u + i : ((4u + (i & 3)) << length_extra(i)) + 3u);
}
BSQ_HD int dist_extra(int i) { return i < 4 ? 0 : (i - 2) >> 1; }
BSQ_HD uint32_t dist_base(int i) { return i < 4 ? 1u + i : ((2u + (i & 1)) << dist_extra(i)) + 1u; }

// Literal/length and distance symbols of one Huffman block until the end-of-block symbol.
BSQ_HD int decode_symbols(Bits& b, const Code& lit, const Code& dist, uint8_t* out, uint32_t cap, uint32_t& n) {
  for (;;) {
    const int sym = code_decode(b, lit);
    if (sym < 0) return b.err ? b.err : kErrCode;
    if (sym < 256) {
      if (n >= cap) return kErrOutput;
      out[n++] = (uint8_t)sym;
      continue;
    }
    if (sym == 256) return kOk;
    const int li = sym - 257;
    if (li >= 29) return kErrSymbol;
    const uint32_t len = length_base(li) + bits_get(b, length_extra(li));
    const int ds = code_decode(b, dist);
    if (ds < 0) return b.err ? b.err : kErrCode;
    if (ds >= 30) return kErrSymbol;
    const uint32_t d = dist_base(ds) + bits_get(b, dist_extra(ds));
    if (b.err) return b.err;
    if (d > n) return kErrDistance;
    if (len > cap - n) return kErrOutput;
    for (uint32_t k = 0; k < len; k++, n++) out[n] = out[n - d];   // overlapping copies repeat
  }
}

// Inflates raw DEFLATE data into out[0, cap).  *out_len gets the bytes produced.
BSQ_HD int inflate_raw(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  Bits b;
  bits_init(b, in, in_len);
  uint32_t n = 0;
  Code lit, dist;
  int last = 0;
  do {
    last = (int)bits_get(b, 1);
    const uint32_t type = bits_get(b, 2);
    if (b.err) return b.err;
    if (type == 0) {
      // stored: the rest of the current byte is skipped, then LEN, NLEN, LEN bytes
      b.buf = 0;
      b.cnt = 0;
      if (b.pos + 4 > b.len) return kErrInput;
      const uint32_t len = b.in[b.pos] | ((uint32_t)b.in[b.pos + 1] << 8);
      const uint32_t nlen = b.in[b.pos + 2] | ((uint32_t)b.in[b.pos + 3] << 8);
      b.pos += 4;
      if (len != (~nlen & 0xFFFFu)) return kErrStored;
      if (len > b.len - b.pos) return kErrInput;
      if (len > cap - n) return kErrOutput;
      for (uint32_t k = 0; k < len; k++) out[n++] = b.in[b.pos + k];
      b.pos += len;
    } else if (type == 1) {
      uint8_t lengths[288 + 30];
      for (int s = 0; s < 144; s++) lengths[s] = 8;
      for (int s = 144; s < 256; s++) lengths[s] = 9;
      for (int s = 256; s < 280; s++) lengths[s] = 7;
      for (int s = 280; s < 288; s++) lengths[s] = 8;
      for (int s = 0; s < 30; s++) lengths[288 + s] = 5;
      code_build(lit, lengths, 288);
      code_build(dist, lengths + 288, 30);
      const int e = decode_symbols(b, lit, dist, out, cap, n);
      if (e) return e;
    } else if (type == 2) {
      const int nlen = (int)bits_get(b, 5) + 257, ndist = (int)bits_get(b, 5) + 1, ncode = (int)bits_get(b, 4) + 4;
      if (b.err) return b.err;
      if (nlen > 286 || ndist > 30) return kErrCode;
      const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
      uint8_t lengths[288 + 32];
      for (int k = 0; k < 19; k++) lengths[k] = 0;
      for (int k = 0; k < ncode; k++) lengths[order[k]] = (uint8_t)bits_get(b, 3);
      if (b.err) return b.err;
      Code cl;
      if (!code_build(cl, lengths, 19)) return kErrCode;
      // literal/length then distance code lengths, with the repeat codes 16, 17, 18
      int k = 0;
      while (k < nlen + ndist) {
        const int sym = code_decode(b, cl);
        if (sym < 0) return b.err ? b.err : kErrCode;
        if (sym < 16) { lengths[k++] = (uint8_t)sym; continue; }
        uint8_t v = 0;
        int rep;
        if (sym == 16) {
          if (k == 0) return kErrCode;
          v = lengths[k - 1];
          rep = 3 + (int)bits_get(b, 2);
        } else if (sym == 17) {
          rep = 3 + (int)bits_get(b, 3);
        } else {
          rep = 11 + (int)bits_get(b, 7);
        }
        if (b.err) return b.err;
        if (k + rep > nlen + ndist) return kErrCode;
        while (rep--) lengths[k++] = v;
      }
      if (lengths[256] == 0) return kErrCode;   // no end-of-block code
      if (!code_build(lit, lengths, nlen) || !code_build(dist, lengths + nlen, ndist)) return kErrCode;
      const int e = decode_symbols(b, lit, dist, out, cap, n);
      if (e) return e;
    } else {
      return kErrBlockType;
    }
  } while (!last);
  *out_len = n;
  return kOk;
}

}  // namespace inflate
}  // namespace bsq

namespace bsq {
namespace inflate {

// ----------------------------------------------------------------------------- the device's decoder
// Two phases.  Phase 1, one thread per block: the Huffman decode alone, into one 32-bit token per
// symbol, (x << 16) | d: d = 0 for the literal byte x, else a copy of x + 3 bytes from distance d.
// It checks what phase 2 relies on: every distance within the bytes produced so far and the total
// equal to the block's size.  Each thread has its own small tables: 9-bit and 6-bit lookup tables for
// literal/length and distance codes, and for a longer code the canonical decode from the code's first
// code, first symbol index and count per length (RFC 1951 §3.2.2), all lengths at once from the next
// 15 bits reversed.  The decoder is a state machine of short steps (a block header with its tables,
// one symbol, or up to 8 stored bytes) so that 32 lanes, each in its own block, run one step per loop
// iteration side by side.  Input: a 64-bit bit buffer refilled four bytes at a time from aligned
// 32-bit loads.  Phase 2 (one warp per block, bsq_bam.cu) turns the tokens into bytes.

constexpr int kLaneLitBits = 9, kLaneDistBits = 6;
constexpr uint32_t kTokStage = 16;     // tokens staged per thread before a 64-byte store

// A canonical code (RFC 1951 §3.2.2) for the decode of codes longer than a table: the codes of length
// l are the consecutive values [first[l], limit[l]), and the code value v of length l is symbol
// symbol[v + base[l]] (base[l] = index of the length's first symbol - first[l], modulo 2^16); symbols in
// (length, value) order.  Scanning lengths upward, a value below limit[l] is a code: a smaller one
// would extend a shorter code, found before.
template <int kSyms>
struct LaneCode {
  uint16_t limit[kMaxBits + 1];
  uint16_t base[kMaxBits + 1];
  uint16_t symbol[kSyms];
};
// Per-thread tables (2244 bytes, an odd number of 32-bit words, so that the threads' copies in shared
// memory start on different banks).
struct LaneTables {
  uint16_t lit[1 << kLaneLitBits];     // (length << 9) | symbol, 0 = not in the table
  uint16_t dist[1 << kLaneDistBits];
  LaneCode<288> lc;                    // literal/length code
  LaneCode<32> dc;                     // distance code; during a header, the code-length code
  uint8_t lengths[288 + 32];
  uint16_t pad[2];
};

static_assert(sizeof(LaneTables) % 8 == 4, "an odd number of 32-bit words");

struct LaneIn {
  const uint8_t* in;
  uint32_t len, pos;                   // bytes of the block; bytes moved into buf
  uint64_t buf;
  int cnt;
};

// Four bytes at in[pos] from the two aligned words that hold them (in[] is readable up to 3 bytes on
// either side of the block, which the file's allocation guarantees); one byte at a time near the end.
BSQ_HD void lane_refill(LaneIn& b) {
  if (b.cnt > 32) return;
  if (b.pos + 4 <= b.len) {
    const uintptr_t a = (uintptr_t)(b.in + b.pos);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(a & ~(uintptr_t)3);
    const uint32_t sh = (uint32_t)(a & 3) * 8;
#ifdef __CUDA_ARCH__
    const uint32_t lo = __ldg(w), hi = sh ? __ldg(w + 1) : 0u;
#else
    const uint32_t lo = w[0], hi = sh ? w[1] : 0u;
#endif
    const uint32_t v = sh ? (lo >> sh) | (hi << (32 - sh)) : lo;
    b.buf |= (uint64_t)v << b.cnt;
    b.cnt += 32;
    b.pos += 4;
    return;
  }
  while (b.cnt <= 56 && b.pos < b.len) {
    b.buf |= (uint64_t)b.in[b.pos++] << b.cnt;
    b.cnt += 8;
  }
}

// k <= 16 bits; past the end of the block sets err.
BSQ_HD uint32_t lane_bits(LaneIn& b, int k, int& err) {
  if (k == 0) return 0;
  if (b.cnt < k) { lane_refill(b); if (b.cnt < k) { err = kErrInput; return 0; } }
  const uint32_t v = (uint32_t)(b.buf & ((1u << k) - 1));
  b.buf >>= k;
  b.cnt -= k;
  return v;
}

// Counts and first codes per length of n code lengths; false when they over-subscribe the code space.
BSQ_HD bool lane_counts(const uint8_t* lengths, int n, uint16_t* count, uint32_t* first) {
  for (int l = 0; l <= kMaxBits; l++) count[l] = 0;
  for (int s = 0; s < n; s++) count[lengths[s]]++;
  int left = 1;
  for (int l = 1; l <= kMaxBits; l++) {
    left = (left << 1) - count[l];
    if (left < 0) return false;
  }
  uint32_t code = 0;
  first[0] = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code = (code + (l > 1 ? count[l - 1] : 0u)) << 1;
    first[l] = code;
  }
  return true;
}

// The canonical code of n code lengths; false when they over-subscribe the code space.
template <int kSyms>
BSQ_HD bool lane_code(LaneCode<kSyms>& c, const uint8_t* lengths, int n) {
  uint16_t count[kMaxBits + 1];
  uint32_t first[kMaxBits + 1];
  if (!lane_counts(lengths, n, count, first)) return false;
  uint16_t offs[kMaxBits + 1];
  uint32_t idx = 0;
  for (int l = 0; l <= kMaxBits; l++) {
    idx += l > 1 ? count[l - 1] : 0u;
    offs[l] = (uint16_t)idx;
    c.limit[l] = (uint16_t)(first[l] + count[l]);
    c.base[l] = (uint16_t)(idx - first[l]);
  }
  for (int s = 0; s < n; s++)
    if (lengths[s] != 0 && offs[lengths[s]] < kSyms) c.symbol[offs[lengths[s]]++] = (uint16_t)s;
  return true;
}

// The k-bit lookup table of a code: each code of at most k bits, bit-reversed, fills its entries.
BSQ_HD void lane_table(uint16_t* table, int k, const uint8_t* lengths, int n) {
  for (int i = 0; i < (1 << k); i++) table[i] = 0;
  uint16_t count[kMaxBits + 1];
  uint32_t next[kMaxBits + 1];
  lane_counts(lengths, n, count, next);
  for (int s = 0; s < n; s++) {
    const int l = lengths[s];
    if (l == 0) continue;
    const uint32_t cd = next[l]++;
    if (l > k) continue;
    uint32_t rev = 0;
    for (int b = 0; b < l; b++) rev |= ((cd >> b) & 1u) << (l - 1 - b);
    for (uint32_t f = rev; f < (1u << k); f += 1u << l) table[f] = (uint16_t)((l << 9) | s);
  }
}

BSQ_HD uint32_t bitrev32(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __brev(x);
#else
  uint32_t r = 0;
  for (int i = 0; i < 32; i++) r |= ((x >> i) & 1u) << (31 - i);
  return r;
#endif
}

// One symbol through the table, or, for a code longer than it, the canonical decode: the next 15
// bits reversed hold every candidate code (the first bit most significant).  -1 on failure.
template <int kSyms>
BSQ_HD int lane_symbol(LaneIn& b, const uint16_t* table, int k, const LaneCode<kSyms>& c, int nsym, int& err) {
  if (b.cnt < kMaxBits) lane_refill(b);
  const uint16_t e = table[b.buf & ((1u << k) - 1)];
  if (e) {
    const int l = e >> 9;
    if (l > b.cnt) { err = kErrInput; return -1; }
    b.buf >>= l;
    b.cnt -= l;
    return e & 511;
  }
  const uint32_t c15 = bitrev32((uint32_t)b.buf) >> (32 - kMaxBits);
  for (int l = k + 1; l <= kMaxBits; l++) {
    const uint32_t code = c15 >> (kMaxBits - l);
    if (code < c.limit[l]) {
      if (l > b.cnt) { err = kErrInput; return -1; }
      const uint32_t i = (code + c.base[l]) & 0xFFFFu;
      if (i >= (uint32_t)nsym) { err = kErrCode; return -1; }
      b.buf >>= l;
      b.cnt -= l;
      return c.symbol[i];
    }
  }
  err = kErrCode;
  return -1;
}

enum : int { kLaneHeader = 0, kLaneStored = 1, kLaneSymbol = 2, kLaneDone = 4 };

// A block header: its type, and for Huffman blocks the code lengths and tables.  room: the bytes the
// block may still produce.  Returns the next mode (kLaneDone with err set on failure).
BSQ_HD int lane_header(LaneIn& b, LaneTables& T, int& last, int& err, uint32_t& left, uint32_t room) {
  last = (int)lane_bits(b, 1, err);
  const uint32_t type = lane_bits(b, 2, err);
  if (err) return kLaneDone;
  if (type == 0) {
    // stored: the rest of the current byte is skipped, then LEN, NLEN and the bytes
    const int drop = b.cnt & 7;
    b.buf >>= drop;
    b.cnt -= drop;
    const uint32_t len = lane_bits(b, 16, err), nlen = lane_bits(b, 16, err);
    if (err) return kLaneDone;
    if (len != (~nlen & 0xFFFFu)) { err = kErrStored; return kLaneDone; }
    if (len > room) { err = kErrOutput; return kLaneDone; }
    left = len;
    return kLaneStored;
  }
  if (type == 1) {
    for (int s = 0; s < 144; s++) T.lengths[s] = 8;
    for (int s = 144; s < 256; s++) T.lengths[s] = 9;
    for (int s = 256; s < 280; s++) T.lengths[s] = 7;
    for (int s = 280; s < 288; s++) T.lengths[s] = 8;
    for (int s = 0; s < 30; s++) T.lengths[288 + s] = 5;
    lane_code(T.lc, T.lengths, 288);
    lane_code(T.dc, T.lengths + 288, 30);
    lane_table(T.lit, kLaneLitBits, T.lengths, 288);
    lane_table(T.dist, kLaneDistBits, T.lengths + 288, 30);
    return kLaneSymbol;
  }
  if (type != 2) { err = kErrBlockType; return kLaneDone; }
  const int nlen = (int)lane_bits(b, 5, err) + 257, ndist = (int)lane_bits(b, 5, err) + 1;
  const int ncode = (int)lane_bits(b, 4, err) + 4;
  if (err) return kLaneDone;
  if (nlen > 286 || ndist > 30) { err = kErrCode; return kLaneDone; }
  const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  for (int k = 0; k < 19; k++) T.lengths[k] = 0;
  for (int k = 0; k < ncode; k++) T.lengths[order[k]] = (uint8_t)lane_bits(b, 3, err);
  if (err) return kLaneDone;
  // the code-length code, decoded through the distance table (codes of at most 7 bits)
  if (!lane_code(T.dc, T.lengths, 19)) { err = kErrCode; return kLaneDone; }
  lane_table(T.dist, kLaneDistBits, T.lengths, 19);
  int k = 0;
  while (k < nlen + ndist) {
    const int sym = lane_symbol(b, T.dist, kLaneDistBits, T.dc, 19, err);
    if (sym < 0) { if (!err) err = kErrCode; return kLaneDone; }
    if (sym < 16) { T.lengths[k++] = (uint8_t)sym; continue; }
    uint8_t v = 0;
    int rep;
    if (sym == 16) {
      if (k == 0) { err = kErrCode; return kLaneDone; }
      v = T.lengths[k - 1];
      rep = 3 + (int)lane_bits(b, 2, err);
    } else if (sym == 17) {
      rep = 3 + (int)lane_bits(b, 3, err);
    } else {
      rep = 11 + (int)lane_bits(b, 7, err);
    }
    if (err) return kLaneDone;
    if (k + rep > nlen + ndist) { err = kErrCode; return kLaneDone; }
    while (rep--) T.lengths[k++] = v;
  }
  if (T.lengths[256] == 0) { err = kErrCode; return kLaneDone; }
  if (!lane_code(T.lc, T.lengths, nlen) || !lane_code(T.dc, T.lengths + nlen, ndist)) {
    err = kErrCode;
    return kLaneDone;
  }
  lane_table(T.lit, kLaneLitBits, T.lengths, nlen);
  lane_table(T.dist, kLaneDistBits, T.lengths + nlen, ndist);
  return kLaneSymbol;
}

struct TokState {
  LaneIn b;
  uint32_t* tok;        // the block's token array, 16-byte aligned, room for cap tokens
  uint32_t* stage;      // kTokStage tokens, 16-byte aligned (the device keeps them in shared memory)
  uint32_t n, staged;   // tokens written to tok, tokens in the stage
  uint32_t bytes, cap;  // bytes the tokens make; the block's size
  int mode, last, err;
  uint32_t left;        // stored bytes left
};

BSQ_HD void tok_start(TokState& z, const uint8_t* in, uint32_t in_len, uint32_t* tok, uint32_t* stage, uint32_t cap) {
  z.b.in = in; z.b.len = in_len; z.b.pos = 0; z.b.buf = 0; z.b.cnt = 0;
  z.tok = tok; z.stage = stage; z.n = 0; z.staged = 0; z.bytes = 0; z.cap = cap;
  z.mode = kLaneHeader; z.last = 0; z.err = kOk; z.left = 0;
}

BSQ_HD void tok_flush(TokState& z) {
  if (z.staged == kTokStage) {
#ifdef __CUDA_ARCH__
    uint4* dst = reinterpret_cast<uint4*>(z.tok + z.n);
    const uint4* src = reinterpret_cast<const uint4*>(z.stage);
#pragma unroll
    for (int k = 0; k < 4; k++) dst[k] = src[k];
#else
    for (uint32_t k = 0; k < kTokStage; k++) z.tok[z.n + k] = z.stage[k];
#endif
  } else {
    for (uint32_t k = 0; k < z.staged; k++) z.tok[z.n + k] = z.stage[k];
  }
  z.n += z.staged;
  z.staged = 0;
}

BSQ_HD void tok_put(TokState& z, uint32_t t) {
  z.stage[z.staged++] = t;
  if (z.staged == kTokStage) tok_flush(z);
}

// One step: a block header with its tables, one symbol, or up to 8 stored bytes.
BSQ_HD void tok_step(TokState& z, LaneTables& T) {
  if (z.mode == kLaneDone) return;
  if (z.mode == kLaneHeader) {
    z.mode = lane_header(z.b, T, z.last, z.err, z.left, z.cap - z.bytes);
  } else if (z.mode == kLaneSymbol) {
    const int sym = lane_symbol(z.b, T.lit, kLaneLitBits, T.lc, 288, z.err);
    if (sym < 0) {
      if (!z.err) z.err = kErrCode;
    } else if (sym < 256) {
      if (z.bytes >= z.cap) z.err = kErrOutput;
      else { tok_put(z, (uint32_t)sym << 16); z.bytes++; }
    } else if (sym == 256) {
      z.mode = z.last ? kLaneDone : kLaneHeader;
    } else {
      const int li = sym - 257;
      if (li >= 29) { z.err = kErrSymbol; }
      else {
        const uint32_t len = length_base(li) + lane_bits(z.b, length_extra(li), z.err);
        const int ds = lane_symbol(z.b, T.dist, kLaneDistBits, T.dc, 32, z.err);
        if (ds < 0) { if (!z.err) z.err = kErrCode; }
        else if (ds >= 30) z.err = kErrSymbol;
        else {
          const uint32_t d = dist_base(ds) + lane_bits(z.b, dist_extra(ds), z.err);
          if (!z.err) {
            if (d > z.bytes) z.err = kErrDistance;
            else if (len > z.cap - z.bytes) z.err = kErrOutput;
            else { tok_put(z, ((len - 3) << 16) | d); z.bytes += len; }
          }
        }
      }
    }
  } else {
    // stored bytes, up to 8, as literals
    const uint32_t m = z.left < 8 ? z.left : 8;
    for (uint32_t j = 0; j < m && !z.err; j++) {
      const uint32_t v = lane_bits(z.b, 8, z.err);
      if (!z.err) { tok_put(z, v << 16); z.bytes++; }
    }
    z.left -= m;
    if (z.left == 0 && !z.err) z.mode = z.last ? kLaneDone : kLaneHeader;
  }
  if (z.err) z.mode = kLaneDone;
}

// The end of phase 1 for a block: the last staged tokens; kErrOutput when the bytes fall short.
BSQ_HD void tok_finish(TokState& z) {
  if (z.err) return;
  tok_flush(z);
  if (z.bytes != z.cap) z.err = kErrOutput;
}

// Phase 2 on one thread (the host form of the warp's work): the tokens' bytes into out.
BSQ_HD void tokens_to_bytes(const uint32_t* tok, uint32_t n, uint8_t* out) {
  uint32_t p = 0;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t d = tok[i] & 0xFFFFu, x = tok[i] >> 16;
    if (d == 0) { out[p++] = (uint8_t)x; continue; }
    for (uint32_t k = 0; k < x + 3; k++, p++) out[p] = out[p - d];
  }
}

// Both phases for one block on one thread; tok has room for cap tokens.
BSQ_HD int inflate_tokens(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len,
                          uint32_t* tok, uint32_t* n_tok, LaneTables& T) {
  alignas(16) uint32_t stage[kTokStage];
  TokState z;
  tok_start(z, in, in_len, tok, stage, cap);
  while (z.mode != kLaneDone) tok_step(z, T);
  tok_finish(z);
  *n_tok = z.n;
  *out_len = z.err ? 0 : z.bytes;
  if (z.err) return z.err;
  tokens_to_bytes(tok, z.n, out);
  return kOk;
}

// ----------------------------------------------------------------------------- CRC-32
// gzip's CRC-32 (reflected, polynomial 0xEDB88320).  Two CRCs combine as crc(AB) =
// crc(A) * x^(8 |B|) + crc(B) over GF(2) modulo the polynomial, the products taken in the
// reflected representation (bit 31 is x^0).
constexpr uint32_t kCrcPoly = 0xEDB88320u;

BSQ_HD uint32_t gf2_mulmod(uint32_t a, uint32_t b) {
  uint32_t p = 0;
  for (int i = 0; i < 32; i++) {
    if (a & (0x80000000u >> i)) p ^= b;
    b = (b & 1) ? (b >> 1) ^ kCrcPoly : b >> 1;
  }
  return p;
}

// x^(8 n) modulo the polynomial
BSQ_HD uint32_t gf2_x8n(uint64_t n) {
  uint32_t p = 0x80000000u;            // x^0
  uint32_t sq = 0x00800000u;           // x^8
  while (n) {
    if (n & 1) p = gf2_mulmod(sq, p);
    sq = gf2_mulmod(sq, sq);
    n >>= 1;
  }
  return p;
}

BSQ_HD uint32_t crc_combine(uint32_t crc_a, uint32_t crc_b, uint64_t len_b) {
  return gf2_mulmod(gf2_x8n(len_b), crc_a) ^ crc_b;
}

}  // namespace inflate
}  // namespace bsq
