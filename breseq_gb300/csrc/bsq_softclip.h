// Soft-clipping tabulation on the device (bsq_softclip.cu), used by bsq_abi.cu.
//
// tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666) over a resident sample:
//   1. read pass (count): per kept record, +1/-1 into a per-column difference array of spanning
//      reads (min bases aligned on both sides of the position) and one event per qualifying clip
//      into per-column counters, one array per direction;
//   2. column scan: spanning coverage, the testable totals, and the rows (columns with events) in
//      (direction, column) order with each row's slice of the tail array;
//   3. scatter: the reads the count pass listed (those with clip events) pack each tail (3 bits a
//      base, outward from the clip wall) into its row's slice;
//   4. consensus: one warp per row tallies the tails column by column and counts agreeing tails.
// The dispersion fit is O(rows) scalar arithmetic and runs on the host in the reference's row order.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsq_common.h"

namespace bsq {

constexpr uint32_t kScMaxConsensus = 21;     // soft_clipping.cpp:37 (3 bits a base in 64)
constexpr uint32_t kScBlockCols = 2048;      // columns per scan block (256 threads x 8)
constexpr uint32_t kScSmallRow = 4;          // rows with at most this many tails: one lane each

// A (position, direction) with clip events.
struct ScRowDev {
  uint32_t col;            // padded column: position = col - tpoff[target] + 1
  uint32_t clipped;        // clip events
  uint32_t read_through;   // spanning reads at the position
  uint32_t tail_off;       // first tail of the row in the tail array
};
// Consensus of a row's tails.
struct ScOutDev {
  unsigned long long cons; // consensus code per column, 3 bits each (4 = no A/C/G/T)
  uint32_t agree;          // tails agreeing with the consensus
  uint32_t informative;    // columns with a consensus base; 0 = no sequence
};

struct ScArgs {
  const DevRead* reads;
  const QBounds* qb;
  const uint8_t* seq;
  const uint32_t* tpoff;           // [n_targets + 1]
  uint32_t n_reads, n_targets, n_cols;
  uint32_t n_blocks;               // scan blocks of kScBlockCols columns
  uint64_t cstride;                // n_blocks * kScBlockCols: offset of the direction +1 counters
  uint32_t m;                      // minimum clipped bases
  uint32_t K;                      // consensus columns = min(m, 21)
  double base_fraction;            // consensus base fraction; <= 0 turns the consensus off
  int32_t* diff;                   // [cstride] spanning-read difference array
  uint32_t* cnt;                   // [2 * cstride] events per column; after the scan, tail cursors
  long long* blk;                  // [5 * n_blocks] per-block sums, then their exclusive scan
  unsigned long long* tot;         // [8]: rows(-1), tails(-1), rows(+1), tails(+1), spanning read bases, tested positions
  uint32_t* err;                   // kErrCigar: a kept record whose CIGAR does not fit
  // the count pass gives block b the reads [b * ev_per_block, (b + 1) * ev_per_block) and lists
  // those with clip events at ev[b * ev_per_block ..], ev_n[b] of them
  uint32_t* ev;                    // [n_reads]
  uint32_t* ev_n;                  // [ev_blocks]
  uint32_t ev_blocks, ev_per_block;
  ScRowDev* rows;                  // [rows(-1) + rows(+1)]
  ScOutDev* outs;
  unsigned long long* tails;       // [tails(-1) + tails(+1)]
};

// Grid shapes: n_blocks, cstride, ev_blocks and ev_per_block from n_reads and n_cols.
void sc_plan(ScArgs& A, int sms);
// Read pass (count), block sums and their scan: afterwards tot[0..3] hold the row and tail totals.
// main0 / main1 (may be null) are recorded around the read pass.
cudaError_t sc_launch_count(const ScArgs& A, int sms, cudaStream_t st, cudaEvent_t main0, cudaEvent_t main1);
// Rows and cursors, tail scatter and consensus, once rows / outs / tails are allocated.
cudaError_t sc_launch_rows(const ScArgs& A, uint32_t n_rows, int sms, cudaStream_t st);

}  // namespace bsq
