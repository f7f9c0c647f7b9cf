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
