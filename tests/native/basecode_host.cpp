// The column pass's class-byte core (breseq_gb300/csrc/bsq_basecode.cuh) compiled for the host, checked
// against the per-base rule on every (nibble, quality) pair in every byte position and on random words.
#include <cstdio>
#include <cstdlib>
#include "../../breseq_gb300/csrc/bsq_basecode.cuh"

using namespace bsq;

// the per-base rule: quality * 5 + base for A/C/G/T (1, 2, 4, 8), 255 for N (15), 254 otherwise
static void rule(uint32_t nib, uint32_t q, uint32_t* code, uint32_t* vq) {
  const bool one_hot = nib == 1 || nib == 2 || nib == 4 || nib == 8;
  *vq = nib != 15 ? q : 0;
  if (nib == 15) *code = 255;
  else if (!one_hot) *code = 254;
  else *code = q * 5 + (nib == 1 ? 0 : nib == 2 ? 1 : nib == 4 ? 2 : 3);
}

static int check(uint32_t q4, uint32_t h) {
  uint32_t vq;
  const uint32_t code = class_bytes4(q4, h, &vq);
  for (int k = 0; k < 4; k++) {
    const uint32_t byte = (h >> (8 * (k >> 1))) & 0xFF;
    const uint32_t nib = (k & 1) ? (byte & 15) : (byte >> 4);
    const uint32_t q = (q4 >> (8 * k)) & 0xFF;
    uint32_t c, v;
    rule(nib, q, &c, &v);
    if (((vq >> (8 * k)) & 0xFF) != v) return 1;
    const bool acgt = nib == 1 || nib == 2 || nib == 4 || nib == 8;
    if (acgt && q > kCodeMaxQ) continue;     // A/C/G/T above kCodeMaxQ: not exact (the load flags the sample)
    if (((code >> (8 * k)) & 0xFF) != c) return 2;
  }
  return 0;
}

// the per-base rule of pass 1's combined count: read base equal to its reference code, and not N
static int check_same(uint32_t packed, uint32_t ref) {
  const uint32_t m = same_as_reference8(packed, ref);
  for (int k = 0; k < 8; k++) {
    const uint32_t byte = (packed >> (8 * (k >> 1))) & 0xFF;
    const uint32_t ob = (k & 1) ? (byte & 15) : (byte >> 4);
    const uint32_t rb = (ref >> (4 * k)) & 15;
    if (((m >> k) & 1) != (uint32_t)(ob == rb && ob != 15)) return 3;
  }
  return 0;
}

extern "C" int basecode_selftest(unsigned seed) {
  // every (nibble, quality) pair in every position, the other three bases varied
  for (int pos = 0; pos < 4; pos++)
    for (uint32_t nib = 0; nib < 16; nib++)
      for (uint32_t q = 0; q < 256; q++)
        for (uint32_t other = 0; other < 16; other += 5) {
          uint32_t h = 0, q4 = 0;
          for (int k = 0; k < 4; k++) {
            const uint32_t nk = k == pos ? nib : (other + 3 * k) & 15, qk = k == pos ? q : (q * 7 + 13 * k + other) & 0xFF;
            h |= nk << (8 * (k >> 1) + ((k & 1) ? 0 : 4));
            q4 |= qk << (8 * k);
          }
          if (int e = check(q4, h)) return e;
        }
  // reference match: every (read nibble, reference code) pair in every position, the others random
  static const uint32_t codes[] = {1, 2, 4, 8, 15};
  srand(seed);
  for (int pos = 0; pos < 8; pos++)
    for (uint32_t ob = 0; ob < 16; ob++)
      for (uint32_t rc : codes)
        for (int rep = 0; rep < 64; rep++) {
          uint32_t packed = ((uint32_t)rand() << 16) ^ (uint32_t)rand(), ref = 0;
          for (int k = 0; k < 8; k++) ref |= codes[rand() % 5] << (4 * k);
          const int sh = 8 * (pos >> 1) + ((pos & 1) ? 0 : 4);
          packed = (packed & ~(15u << sh)) | (ob << sh);
          ref = (ref & ~(15u << (4 * pos))) | (rc << (4 * pos));
          if (rep & 1) ref = 0;                       // also reference codes drawn from the read itself below
          if (rep & 1)
            for (int k = 0; k < 8; k++) {
              const uint32_t byte = (packed >> (8 * (k >> 1))) & 0xFF;
              ref |= ((k & 1) ? (byte & 15) : (byte >> 4)) << (4 * k);
            }
          if (int e = check_same(packed, ref)) return 20 + e;
        }
  for (int i = 0; i < 2000000; i++) {
    const uint32_t q4 = ((uint32_t)rand() << 16) ^ (uint32_t)rand();
    const uint32_t h = (uint32_t)rand() & 0xFFFF;
    if (int e = check(q4, h)) return 10 + e;
  }
  return 0;
}
