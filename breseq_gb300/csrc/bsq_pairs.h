// Device side of the discordant-pair (DP) and missing-pair (MP) candidate-region scans
// (bsq_pairs.cu), used by bsq_abi.cu.  The reads are classified in parallel; the few that enter a
// DP or MP window, and the start columns of the MP window totals, are compacted in BAM order for the
// host's sliding-window replay (bsq_pairs_host.cpp).
#pragma once
#include <cuda_runtime.h>
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
  uint32_t* mem;             // [n] 1: MP window-total member (mp only)
};

cudaError_t pair_classify(const PairArgs& a, int sms, cudaStream_t st);
// Writes the events at their scanned offsets (ev_off), names into names[e * kPairNameSlot], and the
// MP members' start columns and keys group * 2 + strand at mem_off.
cudaError_t pair_scatter(const PairArgs& a, const uint64_t* ev_off, const uint64_t* mem_off, PairEvent* ev, char* names,
                         uint32_t* mem_start, uint16_t* mem_key, int sms, cudaStream_t st);

}  // namespace bsq
