// BAM2COV coverage columns on the device (bsq_covtable.cu), used by bsq_abi.cu.
//
// coverage_output::pileup_callback (src/breseq/coverage_output.cpp:307-470) for one region of one
// target:
//   1. read pass: each kept record overlapping the region adds +1/-1 per aligned block to a
//      difference array (unique or raw-redundant, per strand) and its first sequenced base, when
//      aligned, to a begin counter; the pileup's last column and the longest span are maxima;
//   2. scan: the difference arrays become counts (block sums, one sweep over them, apply);
//   3. redundant weights: at columns with redundant coverage a warp sums 1/X1 over the covering
//      records in record (BAM) order, as the pileup does, so the doubles are exact.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsq_common.h"

namespace bsq {

constexpr uint32_t kCtBlockCols = 2048;   // columns per scan block (256 threads x 8)

struct CovTabArgs {
  const DevRead* reads;
  const uint32_t* cigar;
  const uint32_t* x1;
  const uint32_t* rstart;      // record start columns (sorted)
  uint32_t n_reads;
  uint32_t c0;                 // first padded column of the region
  uint32_t n;                  // region columns
  uint32_t t0;                 // first padded column of the target (position 1)
  uint32_t n_blocks;           // scan blocks
  int32_t* diff;               // [4][stride]: unique top, unique bottom, raw redundant top, bottom
  uint64_t stride;             // n_blocks * kCtBlockCols (>= n + 1)
  long long* blk;              // [4][n_blocks]
  uint32_t* counts;            // [6][n]: the four counts, then begin top / bottom (read pass adds these)
  double* red;                 // [2][n]
  uint32_t* stat;              // [0] last column (1-based), [1] longest span, [2] error word,
                               // [3] [4] the records of the target that start before the region ends
  const uint16_t* rg;          // read group per record
  int32_t rg_only;             // >= 0: only this read group's records (--per-read-group columns)
  const uint8_t* seq;          // packed 4-bit bases (kCtIm* modes read them)
  uint32_t mode;               // kCtBam2cov, kCtImPileup or kCtImTabulate
  uint32_t dp_rg[8];           // kCtImPileup: read groups with a discordant-pair group (256-bit mask);
                               // their kDpCand records are left out of their first column, as the
                               // per-read loop's `continue` (identify_mutations.cpp:1399-1416) leaves
                               // them out of its tally
};

// Which pileup entries a column counts.
constexpr uint32_t kCtBam2cov = 0;     // coverage_output.cpp:373-376: every entry but deletions
constexpr uint32_t kCtImPileup = 1;    // identify_mutations.cpp:1560-1610 at insert_count 0: deletions
                                       // (read base '.') count, aligned N bases do not
constexpr uint32_t kCtImTabulate = 2;  // tabulate_position_coverage (identify_mutations.cpp:2218-2250):
                                       // neither deletions nor aligned N bases

// Read pass, scan and redundant weights.  counts[4..5], diff and stat must be zeroed first.
cudaError_t ct_launch(const CovTabArgs& A, int sms, cudaStream_t st);
// Region offsets first + k * step, k < m, of the counts and weights into [6][m] / [2][m] arrays.
cudaError_t ct_launch_gather(const CovTabArgs& A, uint32_t first, uint32_t step, uint32_t m, uint32_t* counts_out,
                             double* red_out, int sms, cudaStream_t st);

}  // namespace bsq
