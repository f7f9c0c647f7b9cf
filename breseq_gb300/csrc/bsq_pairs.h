// Device side of the discordant-pair (DP), missing-pair (MP) and pair-distance (PD) candidate-region
// scans (bsq_pairs.cu), used by bsq_abi.cu.  The reads are classified in parallel; the few that enter
// a DP or MP window, and the start columns of the MP window totals, are compacted in BAM order for
// the host's sliding-window replay (bsq_pairs_host.cpp).  PD's gaps go into difference arrays whose
// scan evaluates every position on the device; the host assembles the regions and the calibration.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "bsq_common.h"

namespace bsq {

// classification code of a read, one byte
enum : uint8_t {
  kPairDpBinMask = 7,     // DP bin = strand * 3 + orientation (FR, RF, FF); 7 = not a DP read
  kPairMpAll = 8,         // counts toward the MP window total of its strand
  kPairMpUnmapped = 16,   // a mate-unmapped read of an MP window
  kPairRev = 32,          // focal strand reverse
  kPairXpSkip = 64,       // a DP-eligible read without a usable XP tag: breseq skips it at its start column
  kPairRead2 = 128,       // BAM flag 0x80
};
constexpr uint8_t kPairNoBin = 7;
constexpr int kPairNameSlot = 256;   // bytes per compacted read name (BAM names are at most 254)

// One read that enters a DP or MP window, in BAM order.
struct PairEvent {
  uint32_t rec;       // read index in the sample
  uint32_t start;     // padded column of the first aligned base
  uint32_t end;       // exclusive end column
  int32_t isize;
  uint8_t code;
  uint8_t group;      // DP group
  uint8_t redundant;  // X1 > 1
  uint8_t name_len;
};
static_assert(sizeof(PairEvent) == 20, "PairEvent layout");

#ifdef __CUDACC__
#define BSQ_PAIR_HD __host__ __device__ __forceinline__
#else
#define BSQ_PAIR_HD inline
#endif

// The tests breseq applies to a read at its start column (identify_mutations.cpp:1399-1493).
// dflags: the packed record's flags (kSkip, kRev); f: the BAM flag; xp: its XP code; gi: the DP
// group of its read group (-1 none).  Gives the code, the group, and whether the read is an event
// (sel) or an MP window-total member (mem).
BSQ_PAIR_HD void pair_classify_one(uint32_t dflags, uint32_t f, uint32_t xp, int32_t gi, bool mp, uint8_t& code,
                                   uint8_t& grp, uint32_t& sel, uint32_t& mem) {
  code = kPairNoBin;
  grp = 0xFF;
  sel = 0;
  mem = 0;
  if (dflags & kSkip) return;   // outside the scoring pileup
  const bool rev = (dflags & kRev) != 0;
  if (rev) code |= kPairRev;
  if (f & 0x80) code |= kPairRead2;
  if (gi < 0) return;
  grp = (uint8_t)gi;
  bool skip = false;
  // DP: paired, mapped, not proper, not secondary / supplementary / mate-unmapped
  if ((f & 0x1) && !(f & 0x4) && !(f & 0x2) && !(f & (0x100 | 0x800 | 0x8))) {
    if (xp <= 2) {
      code = (uint8_t)((code & ~kPairDpBinMask) | ((rev ? 3 : 0) + xp));
      sel = 1;
    } else {
      skip = true;             // `continue`: the rest of the read's processing at this column
      code |= kPairXpSkip;
    }
  }
  // MP: mapped, primary, not supplementary; the mate unmapped makes it an event
  if (mp && !skip && !(f & 0x4) && !(f & (0x100 | 0x800))) {
    code |= kPairMpAll;
    mem = 1;
    if ((f & 0x1) && (f & 0x8)) {
      code |= kPairMpUnmapped;
      sel = 1;
    }
  }
}

// ------------------------------------------------------------------ pair distance (PD)
constexpr int64_t kPdUScale = 1048576;          // quantiles in 2^20 fixed point
constexpr int kPdLadderSteps = 21;              // seed ladder |z| >= 1 + 0.25 k
constexpr int kPdHistPerUnit = 50, kPdHistLimit = 40;
constexpr int kPdHistBins = 2 * kPdHistLimit * kPdHistPerUnit + 1;
constexpr int32_t kPdHistMinCovering = 4;
constexpr int kPdBitLadder = 2;                 // mask bits: 0 above L, 1 above S, 2.. rungs L, 2 + 21.. rungs S

// The PD enter test of one read (identify_mutations.cpp:1514-1555): a normally oriented pair with
// both mates on this target, TLEN > 0, X1 <= 1, in a DP group whose null it matches; its unsequenced
// gap [lo, hi] (between-base positions, lo = the read's aligned end, hi = the mate's start - 1) is
// added with its distance quantile u and tail bin (0 long, 1 short, -1 neither).  bad: the interval
// breaks the reference's ring-buffer assertion (:2590-2593), where breseq stops.
struct PdInterval {
  int32_t lo, hi;
  int64_t u;
  int bin;
  bool ok, bad;
};
BSQ_PAIR_HD void pd_interval_one(uint32_t dflags, uint32_t f, bool xp_skip, int32_t gi, uint32_t x1, int32_t tid,
                                 int32_t mtid, int32_t isize, uint32_t start1, uint32_t end1, int32_t mpos,
                                 const int64_t* cdf, uint32_t cdf_len, uint32_t orient, int32_t max_span,
                                 int64_t lower_tail, PdInterval& out) {
  out.ok = false;
  out.bad = false;
  if ((dflags & kSkip) || xp_skip || gi < 0) return;
  if (!(f & 0x1) || (f & 0x4) || (f & (0x100 | 0x800 | 0x8))) return;
  const bool rev = (dflags & kRev) != 0, mrev = (f & 0x20) != 0;
  if (mtid != tid || isize <= 0 || rev == mrev || x1 > 1) return;
  if (orient == 0 && rev) return;                 // the group's null is FR
  if (orient == 1 && !rev) return;                // RF
  const int32_t lo = (int32_t)end1, hi = mpos;    // mate_start_1 - 1
  if (!(hi >= lo) || cdf_len == 0 || isize > max_span) return;
  const int64_t u = (uint32_t)isize < cdf_len ? cdf[isize] : kPdUScale;
  out.bin = (u >= kPdUScale - lower_tail) ? 0 : (u <= lower_tail ? 1 : -1);
  out.lo = lo;
  out.hi = hi;
  out.u = u;
  out.ok = true;
  out.bad = !(lo >= (int32_t)start1 && (int64_t)hi + 1 <= (int64_t)start1 + max_span);
}

// The per-position PD statistics (identify_mutations.cpp:2660-2706) from the covering counts: the
// rank-sum z, the z histogram bin (-1 when n < 4), and the mask of seed tests (above per direction,
// and each ladder rung per direction).  in_seq: the position is inside the target (not the flush).
BSQ_PAIR_HD void pd_eval_one(int64_t n, int64_t nlong, int64_t nshort, int64_t u, bool in_seq, double z_seed,
                             int32_t seed, double& z, int& hist_bin, uint64_t& mask) {
  z = 0.0;
  hist_bin = -1;
  if (n > 0) {
    const double mean_offset = ((double)u - (double)n * (double)kPdUScale / 2.0) / (double)kPdUScale;
    z = mean_offset * sqrt(12.0 / (double)n);
    if (n >= kPdHistMinCovering) {
      int b = (int)floor(z * kPdHistPerUnit) + kPdHistLimit * kPdHistPerUnit;
      if (b < 0) b = 0;
      if (b >= kPdHistBins) b = kPdHistBins - 1;
      hist_bin = b;
    }
  }
  mask = 0;
  for (int bin = 0; bin < 2; bin++) {
    const int64_t tail = bin == 0 ? nlong : nshort;
    const bool right_way = bin == 0 ? (z >= z_seed) : (z <= -z_seed);
    const bool tail_ok = (tail >= seed) && in_seq;
    if (tail_ok && right_way) mask |= 1ull << bin;
    const double directed = bin == 0 ? z : -z;
    if (tail_ok)
      for (int k = 0; k < kPdLadderSteps; k++)
        if (directed >= 1.0 + 0.25 * (double)k) mask |= 1ull << (kPdBitLadder + bin * kPdLadderSteps + k);
  }
}

// One position where a PD direction is above its seed, for the host's region assembly.
struct PdAbove {
  uint32_t col;
  uint32_t bits;     // bit 0: L, bit 1: S
  int32_t n, nlong, nshort, pad;
  double z;
};
static_assert(sizeof(PdAbove) == 32, "PdAbove layout");

struct PdArgs {
  const DevRead* reads;
  const uint16_t* flag;
  const uint8_t* code;        // pair classification (kPairXpSkip)
  const uint8_t* group;       // DP group per read (0xFF none)
  const uint32_t* x1;
  const int32_t* isize;
  const int32_t* mtid;
  const int32_t* mpos;
  const uint32_t* tpoff;      // [n_targets + 1]
  const uint8_t* piled;       // [n_targets]
  const int64_t* cdf;         // all groups' nulls, group g at cdf_off[g]
  const uint64_t* cdf_off;
  const uint32_t* cdf_len;
  const uint8_t* orient;
  uint32_t n, n_targets, n_cols;
  int32_t max_span, seed;
  int64_t lower_tail;
  double z_seed;
  long long* diff;            // [n_cols][4]: covering, long, short, quantile sum
  long long* blk;             // [blocks][4]
  uint64_t* mask;             // [n_cols]
  unsigned long long* hist;   // [kPdHistBins]
  unsigned long long* ladder; // [2][kPdLadderSteps]
  PdAbove* above;
  unsigned int* n_above;      // [0] count, [1] ring-assertion violations
  uint32_t above_cap;
};
constexpr int kPdScanCols = 2048;               // columns per scan block (256 threads x 8)

cudaError_t pd_launch(const PdArgs& a, int sms, cudaStream_t st);

struct PairArgs {
  const DevRead* reads;
  const uint16_t* flag;      // raw BAM flags
  const uint8_t* xp;
  const int32_t* isize;
  const uint64_t* qoff;
  const char* qname;
  const uint32_t* x1;
  const uint16_t* rg;
  const int32_t* rg_map;     // read group -> DP group, -1 none
  uint32_t n_rg;
  uint32_t n;
  int mp;                    // missing-pair scan enabled
  uint8_t* code;             // [n]
  uint8_t* group;            // [n]
  uint32_t* sel;             // [n] 1: DP or MP-unmapped event
  uint32_t* mem0;            // [n] 1: MP window-total member on the forward strand (mp only)
  uint32_t* mem1;            // [n] the same on the reverse strand
};

cudaError_t pair_classify(const PairArgs& a, int sms, cudaStream_t st);
// Writes the events at their scanned offsets (ev_off), names into names[e * kPairNameSlot], and per
// strand the MP members' start columns and DP groups at off0 / off1.
cudaError_t pair_scatter(const PairArgs& a, const uint64_t* ev_off, const uint64_t* off0, const uint64_t* off1,
                         PairEvent* ev, char* names, uint32_t* start0, uint32_t* start1, uint8_t* group0,
                         uint8_t* group1, int sms, cudaStream_t st);

}  // namespace bsq
