// Launch wrappers of the scoring kernels (bsq_kernels.cu) for the host orchestration (bsq_abi.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsq_basecode.cuh"
#include "bsq_common.h"

namespace bsq {

// Raw record arrays as uploaded from the caller's bsq_read_soa (device pointers).
struct RawSoA {
  const int32_t* tid;
  const int32_t* pos;
  const uint16_t* flag;
  const uint8_t* mapq;
  const uint32_t* x1;
  const int32_t* xl;
  const int32_t* xr;
  const uint8_t* read_file;
  const uint32_t* l_qseq;
  const uint64_t* seq_off;
  const uint64_t* cigar_off;
  const uint16_t* n_cigar;
  const uint32_t* cigar;
  const uint8_t* xj;         // XJ tag present (may be null: no record has one)
  const uint8_t* xp;         // BSQ_XP_* pair orientation (may be null: no record has an XP tag)
  const uint32_t* tpoff;     // padded target offsets
  const uint8_t* called;     // per target: in the pileup set
  uint32_t n;
  uint32_t n_targets;
  uint64_t n_bases;
  uint64_t n_cigar_total;
};

struct PackOut {
  DevRead* reads;
  QBounds* qb;
  uint32_t* rstart;
  uint8_t* mapq;
  uint32_t* err;
  uint32_t* maxspan;
  uint32_t* mapq_mask;       // [8] presence bits of MAPQ values
};

cudaError_t launch_pack(const RawSoA& in, const PackOut& out, cudaStream_t st);
// dst[0, bytes) = src[0, bytes) by a kernel reading page-locked host memory (bytes a multiple of 16,
// both 16-byte aligned): no copy engine, so no wait behind uploads on other streams.
cudaError_t launch_host_copy(const void* src, void* dst, size_t bytes, int sms, cudaStream_t st);
// Counts reference bytes outside A/C/G/T/N/separator into *bad and zero bytes into *zeros, and writes
// each column's 4-bit code (A,C,G,T = 1,2,4,8, anything else 15) into refnib.
// Words of the nibble-packed reference (column c at nibble c + 16), with one spare word after the last
// column a thread may read past.
// The per-base class bytes of the column pass (class_bytes4 in bsq_basecode.cuh).  code holds n_bases
// rounded up to 16 bytes; seq and qual have 16 bytes of slack.
// Lists the tiles whose read range holds more than thr reads into heavy (n_tiles + 16 entries) and sets
// their bits in heavy_bits (one word per 32 tiles); *n_heavy (zeroed by the caller) counts them.
cudaError_t launch_tile_heavy(const uint2* tile_range, uint32_t n_tiles, uint32_t thr, uint32_t* heavy,
                              uint32_t* heavy_bits, uint32_t* n_heavy, cudaStream_t st);
cudaError_t launch_base_code(const uint8_t* seq, const uint8_t* qual, uint64_t n_bases, uint8_t* code, uint32_t* flags,
                             int sms, cudaStream_t st);
inline uint32_t refnib_words(uint32_t n_cols) { return (n_cols + 16u) / 16u + 2u; }
cudaError_t launch_ref_check(const uint8_t* ref, unsigned long long* refnib, uint32_t n_cols, uint32_t* bad,
                             uint32_t* zeros, int sms, cudaStream_t st);
cudaError_t launch_mapq_index(DevRead* reads, const uint8_t* mapq, const uint8_t* map, uint32_t n, cudaStream_t st);
cudaError_t launch_tile_range(const uint32_t* rstart, uint32_t n_reads, uint32_t n_tiles, uint32_t maxspan,
                              uint2* tile_range, uint32_t* max_tile_reads, cudaStream_t st);
// Largest covariate table the pass-1 kernel keeps in shared memory (R*25*Q 32-bit bins, plus R*4*Q
// combined match counts).
constexpr size_t kEcMaxHistBytes = 200 * 1024;

// Grid sizes from the tuning knobs (resident blocks per SM, capped by the work).
int ec_grid(uint32_t n_chunks, int sms, uint32_t blocks_per_sm);
int column_grid(uint32_t total_tiles, int sms, uint32_t blocks_per_sm);
// Attribute setup that must precede a stream capture of launch_ec.
cudaError_t prepare_ec(uint32_t max_bins, uint32_t max_code_r);
cudaError_t launch_ec(const Batch& B, const uint4* chunks, uint32_t n_chunks, unsigned int* next, uint32_t max_bins,
                      uint32_t max_code_r, int grid, cudaStream_t st, cudaEvent_t main0, cudaEvent_t main1);
cudaError_t launch_im_column(const Batch& B, int precision, int grid, cudaStream_t st);
// Candidate columns in queue order (likely RA items first); total[0], total[1] = the two part sizes.
cudaError_t launch_compact(const ColCall* call, uint32_t n, uint32_t* block_counts, uint32_t* total, uint32_t* out,
                           cudaStream_t st);
cudaError_t launch_intervals(const Batch& B, const ColCov* cov, const ColCall* call, uint8_t* keep, uint32_t* block_counts,
                             uint32_t* total, uint32_t* out_col, ColCov* out_cov, ColCall* out_call, cudaStream_t st);
cudaError_t launch_candidates(const Batch& B, const CandArgs& A, uint32_t max_K, int n_warps, cudaStream_t st);
// The deferred frequency bounds the candidate kernel queued (no-op when A.bq is null).
cudaError_t launch_bounds(const Batch& B, const CandArgs& A, unsigned int* next, int sms, uint32_t warps_per_sm,
                          cudaStream_t st);

}  // namespace bsq
