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

// Length symbols 257..285 and distance symbols 0..29: base values and extra bits (RFC 1951 §3.2.5).
BSQ_HD uint32_t length_base(int i) {
  const uint16_t t[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59,
                          67, 83, 99, 115, 131, 163, 195, 227, 258};
  return t[i];
}
BSQ_HD int length_extra(int i) {
  const uint8_t t[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
  return t[i];
}
BSQ_HD uint32_t dist_base(int i) {
  const uint16_t t[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                          1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
  return t[i];
}
BSQ_HD int dist_extra(int i) {
  const uint8_t t[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
                         12, 12, 13, 13};
  return t[i];
}

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
