// Host build of the library's DEFLATE decoder (breseq_gb300/csrc/bsq_inflate.cuh) for the CPU tests.
#include "../../breseq_gb300/csrc/bsq_inflate.cuh"

extern "C" int host_inflate(const uint8_t* in, uint32_t in_len, uint8_t* out, uint32_t cap, uint32_t* out_len) {
  return bsq::inflate::inflate_raw(in, in_len, out, cap, out_len);
}
