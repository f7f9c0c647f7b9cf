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

// ----------------------------------------------------------------------------- resumable decoder
// The same format, decoded with lookup tables (10 bits for literal/length codes, 8 for distances; a
// code longer than the table falls back to the canonical bit-by-bit decode) and suspended whenever
// the staged output reaches a threshold or the staged input runs low, so a caller can move output
// out of a small ring buffer and move more input in.  Output: positions [n - kRing, n) are in
// ring[p & (kRing - 1)], everything before `flushed` is in out[] already, at most kRing bytes are
// unflushed.  Input: bytes [win_lo, win_hi) of the compressed data are in win[]; decoding pauses
// at a step boundary when fewer than kInMargin bytes remain staged, more than any one step (a
// dynamic block header, or a symbol with its extra bits) reads.

constexpr int kLitBits = 10, kDistBits = 8;
constexpr uint32_t kRing = 4096;
constexpr uint32_t kSuspend = kRing - 258 - 1;   // unflushed bytes at which decoding pauses
constexpr uint32_t kInMargin = 640;              // staged input bytes below which decoding pauses

// The lookup tables and code lengths of the current block (the device keeps them in shared memory)
struct Tables {
  uint16_t lit[1 << kLitBits];    // (length << 9) | symbol, 0 = not in the table
  uint16_t dist[1 << kDistBits];  // (length << 9) | symbol
  uint8_t lengths[288 + 32];
};
// The canonical codes, for building the tables and for codes longer than them (per thread)
struct Codes {
  Code lit_code, dist_code;
};

struct Inflater {
  const uint8_t* win;             // staged input: bytes [win_lo, win_hi) of the compressed data
  uint32_t win_lo, win_hi;
  uint32_t in_len, pos;
  uint64_t buf;
  int cnt;
  uint32_t n, flushed, cap;       // produced, moved to out, output capacity
  int state;                      // 0 block header, 1 stored bytes, 2 Huffman symbols, 3 done
  int last;
  uint32_t stored_left;
  int err;
};

BSQ_HD void inflater_init(Inflater& z, uint32_t in_len, uint32_t cap) {
  z.win = nullptr; z.win_lo = 0; z.win_hi = 0;
  z.in_len = in_len; z.pos = 0; z.buf = 0; z.cnt = 0;
  z.n = 0; z.flushed = 0; z.cap = cap; z.state = 0; z.last = 0; z.stored_left = 0; z.err = kOk;
}

BSQ_HD void z_refill(Inflater& z) {
  while (z.cnt <= 56 && z.pos < z.win_hi) {
    z.buf |= (uint64_t)z.win[z.pos - z.win_lo] << z.cnt;
    z.pos++;
    z.cnt += 8;
  }
}

// More input must be staged before the next step.
BSQ_HD bool z_input_low(const Inflater& z) { return z.win_hi < z.in_len && z.pos + kInMargin > z.win_hi; }

BSQ_HD uint32_t z_bits(Inflater& z, int k) {   // k <= 32
  if (k == 0) return 0;
  if (z.cnt < k) { z_refill(z); if (z.cnt < k) { z.err = kErrInput; return 0; } }
  const uint32_t v = (uint32_t)(z.buf & ((1ull << k) - 1));
  z.buf >>= k;
  z.cnt -= k;
  return v;
}

// Canonical codes of the lengths (RFC 1951 §3.2.2), bit-reversed into a k-bit lookup table.
BSQ_HD void table_build(uint16_t* table, int k, const uint8_t* lengths, int nsym, const Code& c) {
  for (int i = 0; i < (1 << k); i++) table[i] = 0;
  // first code of each length; unused symbols (length 0) take no codes
  uint32_t next[kMaxBits + 2];
  uint32_t code = 0;
  next[0] = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code = (code + (l > 1 ? c.count[l - 1] : 0u)) << 1;
    next[l] = code;
  }
  for (int s = 0; s < nsym; s++) {
    const int l = lengths[s];
    if (l == 0) continue;
    const uint32_t cd = next[l]++;
    if (l > k) continue;
    uint32_t rev = 0;
    for (int b = 0; b < l; b++) rev |= ((cd >> b) & 1u) << (l - 1 - b);
    for (uint32_t f = rev; f < (1u << k); f += 1u << l) table[f] = (uint16_t)((l << 9) | s);
  }
}

// One symbol: the table when the code is short enough, else the canonical decode.
BSQ_HD int z_symbol(Inflater& z, const uint16_t* table, int k, const Code& c) {
  if (z.cnt < kMaxBits) z_refill(z);
  const uint16_t e = table[z.buf & ((1u << k) - 1)];
  if (e) {
    const int l = e >> 9;
    if (l > z.cnt) { z.err = kErrInput; return -1; }
    z.buf >>= l;
    z.cnt -= l;
    return e & 511;
  }
  int code = 0, first = 0, index = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code |= (int)z_bits(z, 1);
    if (z.err) return -1;
    const int count = c.count[l];
    if (code - first < count) return c.symbol[index + (code - first)];
    index += count;
    first += count;
    first <<= 1;
    code <<= 1;
  }
  z.err = kErrCode;
  return -1;
}

// Reads one block header; builds the block's tables.
BSQ_HD void z_header(Inflater& z, Tables& T, Codes& K) {
  z.last = (int)z_bits(z, 1);
  const uint32_t type = z_bits(z, 2);
  if (z.err) return;
  if (type == 0) {
    // the rest of the current byte is skipped: whole bytes still buffered are given back
    const int drop = z.cnt & 7;
    z.buf >>= drop;
    z.cnt -= drop;
    const uint32_t len = z_bits(z, 16), nlen = z_bits(z, 16);
    if (z.err) return;
    if (len != (~nlen & 0xFFFFu)) { z.err = kErrStored; return; }
    z.stored_left = len;
    z.state = 1;
  } else if (type == 1) {
    for (int s = 0; s < 144; s++) T.lengths[s] = 8;
    for (int s = 144; s < 256; s++) T.lengths[s] = 9;
    for (int s = 256; s < 280; s++) T.lengths[s] = 7;
    for (int s = 280; s < 288; s++) T.lengths[s] = 8;
    for (int s = 0; s < 30; s++) T.lengths[288 + s] = 5;
    code_build(K.lit_code, T.lengths, 288);
    code_build(K.dist_code, T.lengths + 288, 30);
    table_build(T.lit, kLitBits, T.lengths, 288, K.lit_code);
    table_build(T.dist, kDistBits, T.lengths + 288, 30, K.dist_code);
    z.state = 2;
  } else if (type == 2) {
    const int nlen = (int)z_bits(z, 5) + 257, ndist = (int)z_bits(z, 5) + 1, ncode = (int)z_bits(z, 4) + 4;
    if (z.err) return;
    if (nlen > 286 || ndist > 30) { z.err = kErrCode; return; }
    const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    for (int k = 0; k < 19; k++) T.lengths[k] = 0;
    for (int k = 0; k < ncode; k++) T.lengths[order[k]] = (uint8_t)z_bits(z, 3);
    if (z.err) return;
    // the code-length code lives in dist_code while the lengths are read
    if (!code_build(K.dist_code, T.lengths, 19)) { z.err = kErrCode; return; }
    table_build(T.dist, kDistBits, T.lengths, 19, K.dist_code);
    int k = 0;
    while (k < nlen + ndist) {
      const int sym = z_symbol(z, T.dist, kDistBits, K.dist_code);
      if (sym < 0) { if (!z.err) z.err = kErrCode; return; }
      if (sym < 16) { T.lengths[k++] = (uint8_t)sym; continue; }
      uint8_t v = 0;
      int rep;
      if (sym == 16) {
        if (k == 0) { z.err = kErrCode; return; }
        v = T.lengths[k - 1];
        rep = 3 + (int)z_bits(z, 2);
      } else if (sym == 17) {
        rep = 3 + (int)z_bits(z, 3);
      } else {
        rep = 11 + (int)z_bits(z, 7);
      }
      if (z.err) return;
      if (k + rep > nlen + ndist) { z.err = kErrCode; return; }
      while (rep--) T.lengths[k++] = v;
    }
    if (T.lengths[256] == 0) { z.err = kErrCode; return; }
    if (!code_build(K.lit_code, T.lengths, nlen) || !code_build(K.dist_code, T.lengths + nlen, ndist)) {
      z.err = kErrCode;
      return;
    }
    table_build(T.lit, kLitBits, T.lengths, nlen, K.lit_code);
    table_build(T.dist, kDistBits, T.lengths + nlen, ndist, K.dist_code);
    z.state = 2;
  } else {
    z.err = kErrBlockType;
  }
}

// Decodes until kSuspend bytes are unflushed, the stream ends (state 3) or an error.  ring holds the
// recent output; out is read for back-references older than the ring.
BSQ_HD void z_run_body(Inflater& z, Tables& T, Codes& K, uint8_t* ring, const uint8_t* out) {
  while (z.err == kOk && z.state != 3 && z.n - z.flushed < kSuspend && !z_input_low(z)) {
    if (z.state == 0) {
      z_header(z, T, K);
    } else if (z.state == 1) {
      // stored bytes: whole buffered bytes first, then the input
      if (z.stored_left == 0) { z.state = z.last ? 3 : 0; continue; }
      if (z.n >= z.cap) { z.err = kErrOutput; return; }
      uint8_t byte;
      if (z.cnt >= 8) {
        byte = (uint8_t)(z.buf & 0xFF);
        z.buf >>= 8;
        z.cnt -= 8;
      } else {
        if (z.pos >= z.win_hi) { z.err = kErrInput; return; }
        byte = z.win[z.pos - z.win_lo];
        z.pos++;
      }
      ring[z.n & (kRing - 1)] = byte;
      z.n++;
      z.stored_left--;
    } else {
      // runs of literals whose codes are in the table, without the per-step checks above; the
      // run stops where a step must (output or input low, a longer code, anything but a literal)
      for (;;) {
        if (z.cnt < kMaxBits) z_refill(z);
        const uint16_t e = T.lit[z.buf & ((1u << kLitBits) - 1)];
        const int l = e >> 9;
        if (e == 0 || l > z.cnt || (e & 511) >= 256) break;
        if (z.n >= z.cap) { z.err = kErrOutput; return; }
        z.buf >>= l;
        z.cnt -= l;
        ring[z.n & (kRing - 1)] = (uint8_t)(e & 511);
        z.n++;
        if (z.n - z.flushed >= kSuspend || z_input_low(z)) break;
      }
      if (z.n - z.flushed >= kSuspend || z_input_low(z)) continue;
      const int sym = z_symbol(z, T.lit, kLitBits, K.lit_code);
      if (sym < 0) { if (!z.err) z.err = kErrCode; return; }
      if (sym < 256) {
        if (z.n >= z.cap) { z.err = kErrOutput; return; }
        ring[z.n & (kRing - 1)] = (uint8_t)sym;
        z.n++;
      } else if (sym == 256) {
        z.state = z.last ? 3 : 0;
      } else {
        const int li = sym - 257;
        if (li >= 29) { z.err = kErrSymbol; return; }
        const uint32_t len = length_base(li) + z_bits(z, length_extra(li));
        const int ds = z_symbol(z, T.dist, kDistBits, K.dist_code);
        if (ds < 0) { if (!z.err) z.err = kErrCode; return; }
        if (ds >= 30) { z.err = kErrSymbol; return; }
        const uint32_t d = dist_base(ds) + z_bits(z, dist_extra(ds));
        if (z.err) return;
        if (d > z.n) { z.err = kErrDistance; return; }
        if (len > z.cap - z.n) { z.err = kErrOutput; return; }
        if (d <= kRing) {
          // the source is in the ring; an overlapping copy (d < len) repeats the bytes just written
          for (uint32_t k = 0; k < len; k++) {
            ring[z.n & (kRing - 1)] = ring[(z.n - d) & (kRing - 1)];
            z.n++;
          }
        } else {
          // farther than the ring: flushed output, read 16 bytes at a time so the loads overlap
          const uint8_t* src = out + (z.n - d);
          uint32_t k = 0;
          for (; k + 16 <= len; k += 16) {
            uint8_t v[16];
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = src[k + j];
#pragma unroll
            for (int j = 0; j < 16; j++) ring[(z.n + j) & (kRing - 1)] = v[j];
            z.n += 16;
          }
          for (; k < len; k++) {
            ring[z.n & (kRing - 1)] = src[k];
            z.n++;
          }
        }
      }
    }
  }
}

// The decoder state is copied into a local for the run, so that it stays in registers.
BSQ_HD void z_run(Inflater& state, Tables& T, Codes& K, uint8_t* ring, const uint8_t* out) {
  Inflater z = state;
  z_run_body(z, T, K, ring, out);
  state = z;
}

// ----------------------------------------------------------------------------- one-lane decoder
// The same format decoded whole by one thread with its own small tables, so that a warp decodes 32
// blocks at once (one per lane) instead of one block on one lane.  Per thread: 9-bit and 6-bit
// lookup tables for literal/length and distance codes (a longer code falls back to the canonical
// decode from the code's counts and symbols), and a 64-byte output ring indexed by output address.
// Output goes to out[] in 16-byte aligned chunks, each stored once complete (the block's partial
// first and last chunks byte by byte: a neighbouring block's thread writes the rest of them); a
// back-reference of at most 64 bytes reads the ring, an older one reads out[], which by then holds
// it.  Input: a 64-bit bit buffer refilled four bytes at a time from aligned 32-bit loads.

constexpr int kLaneLitBits = 9, kLaneDistBits = 6;
constexpr uint32_t kLaneRing = 64;

// A canonical code: counts per length, symbols in (length, value) order (RFC 1951 §3.2.2).
struct LaneCode {
  uint16_t count[kMaxBits + 1];
  uint16_t symbol[288];
};
struct LaneDistCode {
  uint16_t count[kMaxBits + 1];
  uint16_t symbol[32];
};
// Per-thread tables (2.1 KB; the device keeps them in shared memory).
struct LaneTables {
  uint16_t lit[1 << kLaneLitBits];     // (length << 9) | symbol, 0 = not in the table
  uint16_t dist[1 << kLaneDistBits];
  LaneCode lc;                         // literal/length code; during a header, the code-length code
  LaneDistCode dc;
  uint8_t lengths[288 + 32];
  alignas(16) uint8_t ring[kLaneRing];   // the last 64 output bytes, at (address & 63)
};

struct LaneIn {
  const uint8_t* in;
  uint32_t len, pos;                   // bytes of the block; bytes moved into buf
  uint64_t buf;
  int cnt;
};

// Four bytes at in[pos] from the two aligned words that hold them (in[] is readable up to 3 bytes
// past the block, which the file's allocation guarantees); one byte at a time near the end.
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

// Counts and symbols of a canonical code from n code lengths; false when over-subscribed.
template <int kSyms>
BSQ_HD bool lane_code(uint16_t* count, uint16_t* symbol, const uint8_t* lengths, int n) {
  for (int l = 0; l <= kMaxBits; l++) count[l] = 0;
  for (int s = 0; s < n; s++) count[lengths[s]]++;
  int left = 1;
  for (int l = 1; l <= kMaxBits; l++) {
    left = (left << 1) - count[l];
    if (left < 0) return false;
  }
  uint16_t offs[kMaxBits + 1];
  offs[1] = 0;
  for (int l = 1; l < kMaxBits; l++) offs[l + 1] = offs[l] + count[l];
  for (int s = 0; s < n; s++)
    if (lengths[s] != 0 && offs[lengths[s]] < kSyms) symbol[offs[lengths[s]]++] = (uint16_t)s;
  return true;
}

// The k-bit lookup table of a code: each code of at most k bits, bit-reversed, fills its entries.
BSQ_HD void lane_table(uint16_t* table, int k, const uint8_t* lengths, int n, const uint16_t* count) {
  for (int i = 0; i < (1 << k); i++) table[i] = 0;
  uint32_t next[kMaxBits + 1];
  uint32_t code = 0;
  next[0] = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code = (code + (l > 1 ? count[l - 1] : 0u)) << 1;
    next[l] = code;
  }
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

// One symbol through the table, or the canonical decode for a code longer than it.  -1 on failure.
BSQ_HD int lane_symbol(LaneIn& b, const uint16_t* table, int k, const uint16_t* count, const uint16_t* symbol,
                       int nsym, int& err) {
  if (b.cnt < kMaxBits) lane_refill(b);
  const uint16_t e = table[b.buf & ((1u << k) - 1)];
  if (e) {
    const int l = e >> 9;
    if (l > b.cnt) { err = kErrInput; return -1; }
    b.buf >>= l;
    b.cnt -= l;
    return e & 511;
  }
  int code = 0, first = 0, index = 0;
  for (int l = 1; l <= kMaxBits; l++) {
    code |= (int)lane_bits(b, 1, err);
    if (err) return -1;
    const int c = count[l];
    if (code - first < c) {
      const int i = index + (code - first);
      if (i >= nsym) { err = kErrCode; return -1; }
      return symbol[i];
    }
    index += c;
    first += c;
    first <<= 1;
    code <<= 1;
  }
  err = kErrCode;
  return -1;
}

// Output of one block: bytes o[0, cap), the ring, the partial first chunk.
struct LaneOut {
  uint8_t* o;
  uint32_t n, cap;
};

// Stores the chunk that ends at output address a (16-byte aligned): whole when it lies inside the
// block, else the block's own bytes of it.
BSQ_HD void lane_store_chunk(LaneTables& T, const LaneOut& w, uintptr_t a) {
  const uintptr_t lo = a - 16, b0 = (uintptr_t)w.o, b1 = (uintptr_t)(w.o + w.n);
  const uint8_t* src = T.ring + (lo & (kLaneRing - 1));
  if (lo >= b0 && a <= b1) {
#ifdef __CUDA_ARCH__
    *reinterpret_cast<uint4*>(lo) = *reinterpret_cast<const uint4*>(src);
#else
    for (int j = 0; j < 16; j++) reinterpret_cast<uint8_t*>(lo)[j] = src[j];
#endif
  } else {
    for (uintptr_t x = lo < b0 ? b0 : lo; x < a && x < b1; x++) *reinterpret_cast<uint8_t*>(x) = src[x - lo];
  }
}

BSQ_HD void lane_emit(LaneTables& T, LaneOut& w, uint8_t v) {
  const uintptr_t a = (uintptr_t)(w.o + w.n);
  T.ring[a & (kLaneRing - 1)] = v;
  w.n++;
  if (((a + 1) & 15) == 0) lane_store_chunk(T, w, a + 1);
}

// The byte d back from the next output position (1 <= d <= n).
BSQ_HD uint8_t lane_back(const LaneTables& T, const LaneOut& w, uint32_t d) {
  const uintptr_t a = (uintptr_t)(w.o + w.n) - d;
  if (d <= kLaneRing) return T.ring[a & (kLaneRing - 1)];
  return *reinterpret_cast<const uint8_t*>(a);   // stored at least 48 bytes ago by this thread
}

// The decoder as a state machine of short steps, so that the 32 lanes of a warp, each in its own
// block, run the same loop iteration by iteration (the device loop reconverges the warp after every
// step): a block header with its tables, one Huffman symbol (a literal, or a length and distance
// that start a copy), up to 8 bytes of a copy, or up to 8 stored bytes.
enum : int { kLaneHeader = 0, kLaneStored = 1, kLaneSymbol = 2, kLaneCopy = 3, kLaneDone = 4 };
struct LaneState {
  LaneIn b;
  LaneOut w;
  int mode, last, err;
  uint32_t left, dist;      // stored or copy bytes left; copy distance
};

BSQ_HD void lane_start(LaneState& z, const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap) {
  z.b.in = in; z.b.len = in_len; z.b.pos = 0; z.b.buf = 0; z.b.cnt = 0;
  z.w.o = out; z.w.n = 0; z.w.cap = cap;
  z.mode = kLaneHeader; z.last = 0; z.err = kOk; z.left = 0; z.dist = 0;
}

// A block header: its type, and for Huffman blocks the code lengths and tables.
BSQ_HD void lane_header(LaneState& z, LaneTables& T) {
  LaneIn& b = z.b;
  int& err = z.err;
  z.last = (int)lane_bits(b, 1, err);
  const uint32_t type = lane_bits(b, 2, err);
  if (err) return;
  if (type == 0) {
    // stored: the rest of the current byte is skipped, then LEN, NLEN and the bytes
    const int drop = b.cnt & 7;
    b.buf >>= drop;
    b.cnt -= drop;
    const uint32_t len = lane_bits(b, 16, err), nlen = lane_bits(b, 16, err);
    if (err) return;
    if (len != (~nlen & 0xFFFFu)) { err = kErrStored; return; }
    if (len > z.w.cap - z.w.n) { err = kErrOutput; return; }
    z.left = len;
    z.mode = kLaneStored;
  } else if (type == 1) {
    for (int s = 0; s < 144; s++) T.lengths[s] = 8;
    for (int s = 144; s < 256; s++) T.lengths[s] = 9;
    for (int s = 256; s < 280; s++) T.lengths[s] = 7;
    for (int s = 280; s < 288; s++) T.lengths[s] = 8;
    for (int s = 0; s < 30; s++) T.lengths[288 + s] = 5;
    lane_code<288>(T.lc.count, T.lc.symbol, T.lengths, 288);
    lane_code<32>(T.dc.count, T.dc.symbol, T.lengths + 288, 30);
    lane_table(T.lit, kLaneLitBits, T.lengths, 288, T.lc.count);
    lane_table(T.dist, kLaneDistBits, T.lengths + 288, 30, T.dc.count);
    z.mode = kLaneSymbol;
  } else if (type == 2) {
    const int nlen = (int)lane_bits(b, 5, err) + 257, ndist = (int)lane_bits(b, 5, err) + 1;
    const int ncode = (int)lane_bits(b, 4, err) + 4;
    if (err) return;
    if (nlen > 286 || ndist > 30) { err = kErrCode; return; }
    const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    for (int k = 0; k < 19; k++) T.lengths[k] = 0;
    for (int k = 0; k < ncode; k++) T.lengths[order[k]] = (uint8_t)lane_bits(b, 3, err);
    if (err) return;
    // the code-length code, decoded through the distance table (codes of at most 7 bits)
    if (!lane_code<32>(T.dc.count, T.dc.symbol, T.lengths, 19)) { err = kErrCode; return; }
    lane_table(T.dist, kLaneDistBits, T.lengths, 19, T.dc.count);
    int k = 0;
    while (k < nlen + ndist) {
      const int sym = lane_symbol(b, T.dist, kLaneDistBits, T.dc.count, T.dc.symbol, 19, err);
      if (sym < 0) { if (!err) err = kErrCode; return; }
      if (sym < 16) { T.lengths[k++] = (uint8_t)sym; continue; }
      uint8_t v = 0;
      int rep;
      if (sym == 16) {
        if (k == 0) { err = kErrCode; return; }
        v = T.lengths[k - 1];
        rep = 3 + (int)lane_bits(b, 2, err);
      } else if (sym == 17) {
        rep = 3 + (int)lane_bits(b, 3, err);
      } else {
        rep = 11 + (int)lane_bits(b, 7, err);
      }
      if (err) return;
      if (k + rep > nlen + ndist) { err = kErrCode; return; }
      while (rep--) T.lengths[k++] = v;
    }
    if (T.lengths[256] == 0) { err = kErrCode; return; }
    if (!lane_code<288>(T.lc.count, T.lc.symbol, T.lengths, nlen) ||
        !lane_code<32>(T.dc.count, T.dc.symbol, T.lengths + nlen, ndist)) { err = kErrCode; return; }
    lane_table(T.lit, kLaneLitBits, T.lengths, nlen, T.lc.count);
    lane_table(T.dist, kLaneDistBits, T.lengths + nlen, ndist, T.dc.count);
    z.mode = kLaneSymbol;
  } else {
    err = kErrBlockType;
  }
}

// One step of the decoder; the stream ends in kLaneDone with err set on failure.
BSQ_HD void lane_step(LaneState& z, LaneTables& T) {
  if (z.mode == kLaneDone) return;
  if (z.mode == kLaneHeader) {
    lane_header(z, T);
  } else if (z.mode == kLaneSymbol) {
    const int sym = lane_symbol(z.b, T.lit, kLaneLitBits, T.lc.count, T.lc.symbol, 288, z.err);
    if (sym < 0) {
      if (!z.err) z.err = kErrCode;
    } else if (sym < 256) {
      if (z.w.n >= z.w.cap) z.err = kErrOutput;
      else lane_emit(T, z.w, (uint8_t)sym);
    } else if (sym == 256) {
      z.mode = z.last ? kLaneDone : kLaneHeader;
    } else {
      const int li = sym - 257;
      if (li >= 29) { z.err = kErrSymbol; }
      else {
        const uint32_t len = length_base(li) + lane_bits(z.b, length_extra(li), z.err);
        const int ds = lane_symbol(z.b, T.dist, kLaneDistBits, T.dc.count, T.dc.symbol, 32, z.err);
        if (ds < 0) { if (!z.err) z.err = kErrCode; }
        else if (ds >= 30) z.err = kErrSymbol;
        else {
          const uint32_t d = dist_base(ds) + lane_bits(z.b, dist_extra(ds), z.err);
          if (!z.err) {
            if (d > z.w.n) z.err = kErrDistance;
            else if (len > z.w.cap - z.w.n) z.err = kErrOutput;
            else { z.left = len; z.dist = d; z.mode = kLaneCopy; }
          }
        }
      }
    }
  } else if (z.mode == kLaneCopy) {
    // up to 8 bytes: independent loads when the source is older than the ring (d > 64 keeps them
    // clear of this copy's own bytes), else one at a time (an overlapping copy repeats its bytes)
    const uint32_t m = z.left < 8 ? z.left : 8;
    if (z.dist > kLaneRing && m == 8) {
      uint8_t v[8];
#pragma unroll
      for (int j = 0; j < 8; j++) v[j] = lane_back(T, z.w, z.dist - (uint32_t)j);
#pragma unroll
      for (int j = 0; j < 8; j++) lane_emit(T, z.w, v[j]);
    } else {
      for (uint32_t j = 0; j < m; j++) lane_emit(T, z.w, lane_back(T, z.w, z.dist));
    }
    z.left -= m;
    if (z.left == 0) z.mode = kLaneSymbol;
  } else {
    // stored bytes, up to 8
    const uint32_t m = z.left < 8 ? z.left : 8;
    for (uint32_t j = 0; j < m && !z.err; j++) lane_emit(T, z.w, (uint8_t)lane_bits(z.b, 8, z.err));
    z.left -= m;
    if (z.left == 0 && !z.err) z.mode = z.last ? kLaneDone : kLaneHeader;
  }
  if (z.err) z.mode = kLaneDone;
}

// The end of a block: its last partial chunk (the rest of that chunk is the next block's).
BSQ_HD void lane_finish(LaneState& z, LaneTables& T) {
  if (z.err) return;
  const uintptr_t end = (uintptr_t)(z.w.o + z.w.n);
  if (end & 15) lane_store_chunk(T, z.w, (end | 15) + 1);
}

// Inflates one block's raw DEFLATE data in[0, in_len) into out[0, cap) with one thread's tables;
// *out_len gets the bytes produced.
BSQ_HD int inflate_lane(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len,
                        LaneTables& T) {
  LaneState z;
  lane_start(z, in, in_len, out, cap);
  while (z.mode != kLaneDone) lane_step(z, T);
  lane_finish(z, T);
  *out_len = z.w.n;
  return z.err;
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

namespace bsq {
namespace inflate {

// Host-side driver of the resumable decoder: whenever it pauses the ring is flushed into out and a
// window of win_size input bytes from the current position is staged in win.
inline int inflate_ring_host(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len,
                             Tables& T, uint8_t* ring, uint8_t* win, uint32_t win_size) {
  Codes K;
  Inflater z;
  inflater_init(z, in_len, cap);
  z.win = win;
  while (z.err == kOk && z.state != 3) {
    if (z.win_hi < z.in_len && z.pos + kInMargin > z.win_hi) {
      z.win_lo = z.pos;
      z.win_hi = z.pos + win_size < in_len ? z.pos + win_size : in_len;
      for (uint32_t k = z.win_lo; k < z.win_hi; k++) win[k - z.win_lo] = in[k];
    }
    z_run(z, T, K, ring, out);
    for (uint32_t p = z.flushed; p < z.n; p++) out[p] = ring[p & (kRing - 1)];
    z.flushed = z.n;
  }
  *out_len = z.n;
  return z.err;
}

}  // namespace inflate
}  // namespace bsq
