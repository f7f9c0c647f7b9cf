// Host build of the library's DEFLATE decoder (breseq_gb300/csrc/bsq_inflate.cuh) for the CPU tests.
#include "../../breseq_gb300/csrc/bsq_inflate.cuh"

extern "C" int host_inflate(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  return bsq::inflate::inflate_raw(in, in_len, out, cap, out_len);
}

// win_size: staged input window (at least kInMargin + 1 bytes)
extern "C" int host_inflate_ring(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len,
                                 uint32_t win_size) {
  static bsq::inflate::Tables T;
  static uint8_t ring[bsq::inflate::kRing];
  static uint8_t win[65536];
  if (win_size > sizeof win || win_size <= bsq::inflate::kInMargin) return -1;
  return bsq::inflate::inflate_ring_host(in, in_len, out, cap, out_len, T, ring, win, win_size);
}

extern "C" uint32_t host_crc_combine(uint32_t a, uint32_t b, uint64_t len_b) {
  return bsq::inflate::crc_combine(a, b, len_b);
}

// The one-lane decoder.  The input is copied into a buffer with 16 spare bytes on both sides (the
// decoder's aligned 32-bit loads may read up to 3 bytes beyond the block, as the file's allocation
// allows on the device); the output goes to out (any alignment).
extern "C" int host_inflate_lane(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  static bsq::inflate::LaneTables T;
  static uint8_t buf[16 + (1u << 20) + 16];
  if (in_len > (1u << 20)) return -1;
  for (uint32_t k = 0; k < in_len; k++) buf[16 + k] = in[k];
  return bsq::inflate::inflate_lane(buf + 16, in_len, out, cap, out_len, T);
}
