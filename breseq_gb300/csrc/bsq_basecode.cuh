// Class bytes of the column pass, four bases at a time in the bytes of a 32-bit word (host and device).
//
// A base's class byte is quality * 5 + observed base (A, C, G, T = 0..3) for a base A/C/G/T, 255 for
// N and 254 for any other 4-bit code (an IUPAC code, or the padding nibble after an odd-length read).
// The byte is exact for qualities up to kCodeMaxQ (50); the load flags a sample with an A/C/G/T base
// above that, and the column pass then keeps the packed bases and qualities for it.
#pragma once
#include <stdint.h>
#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace bsq {

constexpr uint32_t kCodeMaxQ = 50;

// __byte_perm(x, y, s) for selector nibbles 0..7 (bytes 0-3 of x, then of y)
__host__ __device__ inline uint32_t bc_perm(uint32_t x, uint32_t y, uint32_t s) {
#ifdef __CUDA_ARCH__
  return __byte_perm(x, y, s);
#else
  const uint64_t xy = (uint64_t)x | ((uint64_t)y << 32);
  uint32_t r = 0;
  for (int i = 0; i < 4; i++) r |= (uint32_t)((xy >> (8 * ((s >> (4 * i)) & 7u))) & 0xFFu) << (8 * i);
  return r;
#endif
}

// per-byte maximum
__host__ __device__ inline uint32_t bc_max4(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __vmaxu4(a, b);
#else
  uint32_t r = 0;
  for (int i = 0; i < 4; i++) {
    const uint32_t x = (a >> (8 * i)) & 0xFFu, y = (b >> (8 * i)) & 0xFFu;
    r |= (x > y ? x : y) << (8 * i);
  }
  return r;
#endif
}

// The class bytes of four bases.  q4: their quality bytes (byte k = base k); h: their two packed
// sequence bytes in the low 16 bits (the low byte first, its high nibble the earlier base).  *valid_q
// gets the quality bytes of the bases that are not N (A/C/G/T and other codes) and 0 for N.
__host__ __device__ inline uint32_t class_bytes4(uint32_t q4, uint32_t h, uint32_t* valid_q) {
  // the four nibbles into the four bytes: b0 >> 4, b0 & 15, b1 >> 4, b1 & 15
  const uint32_t t = bc_perm(h, 0u, 0x1100u);
  const uint32_t n4 = ((t >> 4) & 0x000F000Fu) | (t & 0x0F000F00u);
  // base index by a 16-entry byte table, addressed by each nibble's low three bits in a byte
  // permutation of the table half its bit 3 selects: 1, 2, 4, 8 -> 0..3, 15 -> 255, else 254
  const uint32_t v = n4 & 0x07070707u, w = v | (v >> 4);
  const uint32_t sel = (w & 0xFFu) | ((w >> 8) & 0xFF00u);
  const uint32_t lo = bc_perm(0xFE0100FEu, 0xFEFEFE02u, sel);    // nibbles 0..7
  const uint32_t hi = bc_perm(0xFEFEFE03u, 0xFFFEFEFEu, sel);    // nibbles 8..15
  const uint32_t m8 = ((n4 >> 3) & 0x01010101u) * 0xFFu;
  const uint32_t r = (hi & m8) | (lo & ~m8);
  const uint32_t bad = ((r >> 7) & 0x01010101u) * 0xFFu;         // 254 / 255: not A/C/G/T
  // quality * 5 + base in 16-bit lanes (no carry reaches the next byte)
  const uint32_t ce = (q4 & 0x00FF00FFu) * 5u + (r & 0x00FF00FFu);
  const uint32_t co = ((q4 >> 8) & 0x00FF00FFu) * 5u + ((r >> 8) & 0x00FF00FFu);
  const uint32_t code = ((ce & 0x00FF00FFu) | ((co & 0x00FF00FFu) << 8));
  const uint32_t n8 = (((r >> 7) & r) & 0x01010101u) * 0xFFu;  // 255: N
  *valid_q = q4 & ~n8;
  return (code & ~bad) | (r & bad);
}

// Pass 1's bases equal to the reference, eight at a time.  packed: four bytes of packed bases (eight
// bases, the earlier base of a byte in its high nibble); ref: the reference's eight 4-bit codes for the
// same columns, base k at nibble k (A, C, G, T one-hot, anything else 15).  Bit k of the result is set
// when base k equals its reference code and is not N (15).
__host__ __device__ inline uint32_t same_as_reference8(uint32_t packed, uint32_t ref) {
  const uint32_t s = ((packed >> 4) & 0x0F0F0F0Fu) | ((packed << 4) & 0xF0F0F0F0u);   // base k at nibble k
  const uint32_t x = s ^ ref;
  uint32_t z = x | (x >> 1);
  z |= z >> 2;                                      // bit 4k: nibble k differs from the reference
  uint32_t n = s & (s >> 1);
  n &= n >> 2;                                      // bit 4k: read nibble k is 15 (N)
  uint32_t m = ~(z | n) & 0x11111111u;
  m = (m | (m >> 3)) & 0x03030303u;                 // bit 4k -> bit k
  m = (m | (m >> 6)) & 0x000F000Fu;
  return (m | (m >> 12)) & 0xFFu;
}

}  // namespace bsq
