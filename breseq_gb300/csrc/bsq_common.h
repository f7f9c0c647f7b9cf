// Device-side layout of a resident sample and the argument blocks of the scoring kernels.
//
// Column space: every target t of a sample occupies padded columns [tpoff[t], tpoff[t] + len[t]),
// tpoff[t] = target_offset[t] + t, followed by one separator column holding '\0'.  The separator
// makes ref[c + 1] at a target's last base read as '\0', which is what breseq's NUL-terminated
// reference buffer yields there (src/breseq/pileup_base.cpp:80-85; error_count.cpp:937-940 reads
// one past the column), and it is never covered by a read.
//
// Tiles: 32 consecutive columns, one warp.  tile_range[t] = [lo, hi) is the range of (start-sorted)
// reads that can cover any column of the tile: start > c0 - maxspan and start < c0 + 32.
#pragma once
#include <stdint.h>

namespace bsq {

// 32-byte read record, coordinate-sorted; one broadcast load per (read, warp).
struct __align__(16) DevRead {
  uint32_t start;      // padded column of the first reference-consuming CIGAR op
  uint32_t end;        // exclusive end column
  uint64_t seq_off;    // nibble index into seq[] and byte index into qual[]
  uint32_t cigar_off;  // complex reads: offset into cigar[]
  uint16_t len;        // l_qseq
  uint16_t n_cigar;
  uint16_t xl;         // XL trim, 0xFFFF when absent
  uint16_t xr;         // XR trim, 0xFFFF when absent
  uint8_t mapq_idx;    // index of this read's MAPQ among the sample's distinct values
  uint8_t rfile;       // flat read-file index (k_read_set covariate)
  uint8_t flags;       // kRev | kSimple | kRedundant | kSkip | kScSkip | kBadCigar | kFiltered
  uint8_t clip;        // simple reads: leading soft clip
};
static_assert(sizeof(DevRead) == 32, "DevRead must stay 32 bytes");

// kSkip: the pileup of the scoring passes leaves the record out (flag filter, or a target outside
// the pileup set).  kFiltered: the flag filter alone (UNMAP | SECONDARY | QCFAIL | DUP), which the
// coverage table applies on every target.  kScSkip: the soft-clipping tabulation leaves it out
// (unmapped, XJ-tagged, or on an empty target).  kBadCigar: the CIGAR does not fit the read or the
// target; the load rejects such a record when the scoring pileup keeps it, the other passes report
// it when they keep it.  kDpCand: a primary, mapped, paired record that is not a proper pair, has a
// mapped mate and has no XP tag or one other than FR / RF / FF; pass 2 leaves it out of its first
// column when its read group is a discordant-pair group (identify_mutations.cpp:1399-1416).
enum : uint8_t { kRev = 1, kSimple = 2, kRedundant = 4, kSkip = 8, kScSkip = 16, kBadCigar = 32, kFiltered = 64,
                 kDpCand = 128 };
constexpr uint16_t kNoTag = 0xFFFF;

// Query bounds of complex reads (simple reads derive them from clip and span):
// qs0/qe0 = query_start_0/query_end_0 (alignment.cpp:219-256), qbe = query_bounds_0().second
// (alignment.cpp:113-196), qbs = its first.  Packed 4 x 16 bits.
struct QBounds { uint16_t qs0, qe0, qbs, qbe; };

struct DevSample {
  const uint8_t* ref;         // padded reference chars
  const unsigned long long* refnib;   // the same columns as 4-bit codes: column c at nibble c + 16,
                                      // A/C/G/T = 1/2/4/8, anything else 15
  const DevRead* reads;
  const uint32_t* x1;         // redundancy per read
  const uint16_t* rg;         // read group per read
  const QBounds* qb;          // per read (valid for complex reads)
  const uint32_t* cigar;
  const uint8_t* seq;         // packed 4-bit, high nibble first
  const uint8_t* qual;
  const uint8_t* code;        // per base: quality * 5 + observed base, 255 N, 254 other (null: not used)
  const uint2* tile_range;    // [n_tiles]
  const uint32_t* heavy;      // tiles with a long read range, run first by the column pass
  const uint32_t* heavy_bits; // bit per tile: listed in heavy
  const uint32_t* tpoff;      // padded target offsets [n_targets + 1]
  const uint32_t* tgt_group;  // coverage group per target
  const uint8_t* tgt_called;  // 1 when the target is in the pileup set
  const uint8_t* tgt_failed;  // pass 2: deletion propagation cutoff < 0 (coverage only)
  uint32_t n_cols;            // padded columns
  uint32_t n_tiles;
  uint32_t n_reads;
  uint32_t n_targets;
  uint32_t maxspan;
};

// ----------------------------------------------------------------------------- pass 1
struct EcArgs {
  unsigned long long* counts;       // [R*25*Q]
  unsigned long long* cov_hist;     // [G * hist_cap]
  unsigned long long* found;        // [n_targets * 2] preprocess read-start tallies
  uint32_t* err;                    // error word (bit set per kind)
  uint32_t R, Q, hist_cap;
  int do_errors, preprocess;
  uint32_t unmatched_min_len;
  float unmatched_factor;           // only used through floor(); double on host
  double unmatched_factor_d;
  uint32_t flush_tiles;             // shared histogram flush period (avoids u32 overflow)
  // read-parallel form: per-column difference arrays of unique / redundant coverage and the
  // preprocess read-start flags, turned into coverage by a scan afterwards
  int32_t* diff_u;                  // [n_cols + 1]
  int32_t* diff_r;                  // [n_cols + 1]
  uint8_t* qs_flag;                 // [2][n_cols]: a read starts at this column (forward, reverse)
  uint32_t* blk_u;                  // per 1024-column block: sums of diff_u / diff_r
  uint32_t* blk_r;
  // the sample's class bytes (quality * 5 + base) when they are exact, every quality of a base that is
  // not N is below Q and R <= kEcCodeMaxR; null otherwise (the pass reads the qualities)
  const uint8_t* code;
};
constexpr uint32_t kEcCodeMaxR = 16;

// ----------------------------------------------------------------------------- pass 2
// Likelihood class of a read base: (mapq_idx, read file, strand, quality, observed base).
// For each class the host precomputes, exactly as fill_read_base_likelihoods does per read
// (identify_mutations.cpp:3359-3384): log10 P(obs | b) for the five hypotheses, their maximum
// and r[b] = 10^(lp[b] - max).
struct ClassTable {
  const double* lp64;     // [K][5]
  const double* r64;      // [K][5]
  const double* lpmax64;  // [K]
  const float* lp32;      // [K + 1][8]: lp[0..4] as float, [5] (bits) bit r = the column pass's
                          // screen bound takes the base at reference base r; entry K all zeros
  uint32_t K;
  uint32_t R, Q, n_mapq;
};

// Per-column output of the column pass (insert position 0).
struct ColCov {               // 32 bytes
  uint32_t uniq_top, uniq_bot, rawred_top, rawred_bot;
  double red_top, red_bot;
};
struct ColCall {              // 16 bytes
  double score;               // consensus score (NaN when n == 0)
  uint32_t n;
  uint8_t best;               // 0..4, 5 = N
  uint8_t flags;              // kBasePredicted | kUniqueOnly | kCandidate | kSlots | kRecompute
  uint8_t pad[2];
};
enum : uint8_t { kBasePredicted = 1, kUniqueOnly = 2, kCandidate = 4, kSlots = 8, kRecompute = 16, kScored = 32,
                 kLikelyRa = 64 };   // best base differs from the reference: queued first (longest work)

struct ImArgs {
  ColCov* cov;
  ColCall* call;
  uint32_t* err;
  uint32_t base_quality_cutoff;
  int precision;              // 0 = FP64 everywhere, 1 = FP32 compensated + screen
  double log10_ref_len;
  double mutation_cutoff;
  double poly_cutoff;
  float screen_margin;        // log10 units subtracted from the polymorphism cutoff for the screen
  float guard;                // consensus guard band (log10 units) for FP64 recompute
  double precision_decimal;   // EM convergence tolerance (polymorphism_precision_decimal)
  uint32_t dp_rg[8];          // bit g: read group g is a discordant-pair group (groups 0..255)
};

// Pass 2 leaves a kDpCand record of a discordant-pair read group out of its first column, insert
// position 0 (identify_mutations.cpp:1399-1416).
__host__ __device__ inline bool dp_group_member(const uint32_t* dp_rg, uint32_t rg) {
  return rg < 256 && ((dp_rg[rg >> 5] >> (rg & 31)) & 1u);
}

// A scoring job for the candidate kernel: one reference column, all its insert slots.
struct CandArgs {
  const uint32_t* cand;       // candidate columns (batch column space)
  const uint32_t* n_cand_dev; // [2] candidates queued first (likely RA items) and the rest, from the compaction
  unsigned int* next;         // work counter (persistent warps)
  struct RaDev* ra;           // output records
  unsigned int* n_ra;
  uint32_t ra_cap;
  uint4* scratch;             // per-warp gather buffer: [n_warps][scratch_per_warp]
  uint32_t scratch_per_warp;
  uint32_t* err;
  uint32_t Qhist;             // quality histogram bins kept per RA (for the K-S test)
  uint32_t* qhist;            // [ra_cap][2][Qhist] major / minor qualities
  // deferred frequency bounds (may be null: bounds are then computed inline)
  struct BoundJob* bq;        // [bq_cap] one bisection each
  unsigned int* n_bq;
  uint32_t bq_cap;
  uint2* pool;                // [pool_cap] (class, multiplicity) lists the bound jobs read
  unsigned int* pool_used;
  uint32_t pool_cap;
};

// One deferred profile-likelihood bound of an RA item (write_RA_frequency_bounds,
// identify_mutations.cpp:3175-3217): the lower or the upper bisection, run on its own warp by the
// bounds kernel.  The two bisections of an item are independent (each test restarts from the free
// fit), so splitting them changes no arithmetic.
struct BoundJob {
  double full[5];             // free-fit frequencies
  double target, maxsum, fh, tol;
  uint32_t slot;              // RA record to complete
  uint32_t pool_off, m;       // the item's class list in the pool
  uint32_t n;                 // scored read bases
  uint32_t col;               // batch column (job lookup)
  uint8_t var, side, pad[2];  // variant allele; side 0 = lower, 1 = upper
};

// Raw RA values written by the candidate kernel (host adds Fisher / K-S and formats).
struct RaDev {
  uint32_t col;               // padded column
  uint32_t insert_position;
  double score, consensus_score;
  double f[5];
  double lower, upper;
  uint32_t pos_info[5][2];    // [base][top, bottom]
  uint32_t n;
  uint8_t ref_idx, var_idx, maj_idx, min_idx, passed_cons, passed_poly, pad[2];
};

// ----------------------------------------------------------------------------- batches
// One sample of a batch with everything its passes read and write.  Pass-2 per-column outputs of all
// jobs live in one array (the batch column space); I.cov / I.call point at this job's part of it.
struct DevJob {
  DevSample S;
  ClassTable T;
  EcArgs E;
  ImArgs I;
  const double* prop;       // per target deletion propagation cutoff (pass 2)
  const double* seed;       // per target deletion seed cutoff (pass 2)
  uint32_t col_begin;       // first column of this job in the batch column space
  uint32_t tile_begin;      // first tile of this job in the batch tile space
  uint32_t cblk_begin;      // first 1024-column coverage block of this job
  uint32_t pad;
};

// Kernel argument describing a batch: the jobs and the prefix sums that map a batch-wide tile /
// column / coverage block back to its job.  Passed by value as a __grid_constant__ parameter, so
// the job fields are read from the constant bank (and re-read there instead of being held in
// registers); 64 jobs keep it under the 32 KB kernel-parameter limit.  Larger batches run as
// consecutive groups of kBatchJobs.
constexpr uint32_t kBatchJobs = 64;
struct Batch {
  uint32_t n_jobs;
  uint32_t total_tiles;
  uint32_t total_cols;
  uint32_t total_cblk;
  uint32_t tile_begin[kBatchJobs + 1];
  uint32_t col_begin[kBatchJobs + 1];
  uint32_t cblk_begin[kBatchJobs + 1];
  uint32_t heavy_begin[kBatchJobs + 1];   // column pass: prefix of the jobs' heavy-tile counts
  uint32_t total_heavy;
  unsigned int* tile_next;                // column pass tile queue (zero before the launch)
  DevJob jobs[kBatchJobs];
};
static_assert(sizeof(Batch) <= 32764, "a Batch is passed as one kernel parameter");

// Per-warp scratch of the candidate kernels, in uint4 units: `cap` gather entries followed by `cap`
// (class, multiplicity) pairs.
inline __host__ __device__ uint64_t cand_warp_stride(uint32_t cap) { return (uint64_t)cap + (cap + 1) / 2; }

// error word bits
enum : uint32_t { kErrCovariate = 1, kErrBase = 2, kErrBounds = 4, kErrOrder = 8, kErrCigar = 16,
                  kErrScratch = 32, kErrRaOverflow = 64, kErrX1 = 128 };

}  // namespace bsq
