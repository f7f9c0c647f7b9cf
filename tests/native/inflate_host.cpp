// Host build of the library's DEFLATE decoders (breseq_gb300/csrc/bsq_inflate.cuh) for the CPU tests.
#include "../../breseq_gb300/csrc/bsq_inflate.cuh"

extern "C" int host_inflate(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  return bsq::inflate::inflate_raw(in, in_len, out, cap, out_len);
}

// The device's two-phase form on one thread: tokens, then their bytes.  The input is copied into a
// buffer with 16 spare bytes on both sides (the decoder's aligned 32-bit loads may read up to 3 bytes
// beyond the block, as the file's allocation allows on the device).
extern "C" int host_inflate_tokens(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  static bsq::inflate::LaneTables T;
  static uint8_t buf[16 + (1u << 20) + 16];
  alignas(16) static uint32_t tok[65536 + 16];
  if (in_len > (1u << 20) || cap > 65536) return -1;
  for (uint32_t k = 0; k < in_len; k++) buf[16 + k] = in[k];
  uint32_t n = 0;
  return bsq::inflate::inflate_tokens(buf + 16, in_len, out, cap, out_len, tok, &n, T);
}

extern "C" uint32_t host_crc_combine(uint32_t a, uint32_t b, uint64_t len_b) {
  return bsq::inflate::crc_combine(a, b, len_b);
}
