// Host-side steps around the scoring kernels (bsq_host.cpp).
#pragma once
#include <stdint.h>

#include <string>
#include <ostream>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "bsq_common.h"
#include "bsq_pairs.h"
#include "bsq_softclip.h"

namespace bsq {
namespace host {

// counts_to_log10_prob + the 6-significant-digit text round trip of error_rates.tab
// (src/breseq/error_count.cpp:629-690, 1005-1026).
void counts_to_log10_prob(const uint64_t* counts, uint32_t R, uint32_t Q, double* out);
// x as printf("%.6g") then strtod give it back (bit-exact).
double round_sig6(double x);

struct ClassTableHost {
  std::vector<double> lp64, r64, lpmax64;
  std::vector<float> lp32;
  uint32_t K = 0;
};
// Per likelihood class (mapq_idx, read file, strand, quality, observed base) the values that
// fill_read_base_likelihoods computes per read (src/breseq/identify_mutations.cpp:3359-3384).
void build_class_table(const double* log10_table, uint32_t R, uint32_t Q, const std::vector<uint8_t>& mapq_values,
                       ClassTableHost& out);

// fisher_exact_test_2x2 / ks_test_two_sample_less (src/breseq/stats.cpp:2144-2286)
double fisher_2x2(uint32_t a, uint32_t b, uint32_t c, uint32_t d);
// x, y given as quality histograms (value = bin index)
double ks_less_hist(const uint32_t* xh, const uint32_t* yh, uint32_t bins);

struct SampleLayout {
  const std::vector<uint32_t>* tpoff;
  const std::vector<uint64_t>* toff;
  const std::vector<uint32_t>* order;
};

void assemble_ra(const std::vector<RaDev>& ra, const std::vector<uint32_t>& qhist, uint32_t Qh, const SampleLayout& L,
                 std::vector<bsq_ra_record>& out);
// MC and UN state machines in pileup order (identify_mutations.cpp:2107-2164, 2262-2344, 2972-3007)
void intervals(const std::vector<ColCov>& cov, const std::vector<ColCall>& call, const SampleLayout& L,
               const bsq_im_params* p, std::vector<bsq_mc_record>& mc, std::vector<bsq_un_record>& un);
// The same state machines over the marked columns only (padded column indices, ascending).
void intervals_sparse(const std::vector<uint32_t>& cols, const std::vector<ColCov>& cov, const std::vector<ColCall>& call,
                      const SampleLayout& L, const bsq_im_params* p, std::vector<bsq_mc_record>& mc,
                      std::vector<bsq_un_record>& un);
void fill_positions(const std::vector<ColCov>& cov, const std::vector<ColCall>& call, const SampleLayout& L,
                    bsq_position_arrays* out);

// One region's coverage columns as bsq_covtable.cu produces them, at the positions first + k * step,
// k < m: counts [6][m] (unique top/bottom, raw redundant top/bottom, begin top/bottom), redundant
// weights [2][m]; the target's reference characters from position 1 to end, and the pileup's last
// column.
struct CoverageRegion {
  const uint32_t* counts;
  const double* red;
  const char* ref;
  uint32_t start, end, last;
  uint32_t first, step, m;
  // own(): copies the arrays out of the staging buffer the next call reuses
  std::vector<uint32_t> own_counts;
  std::vector<double> own_red;
  std::string own_ref;
  void own() {
    own_counts.assign(counts, counts + (size_t)6 * m);
    own_red.assign(red, red + (size_t)2 * m);
    own_ref.assign(ref, end);
    counts = own_counts.data();
    red = own_red.data();
    ref = own_ref.data();
  }
};
// <seq_id>.coverage.tsv of identify_mutations (identify_mutations.cpp:2028-2052, 2173-2204): the
// aggregate columns from pass 2's arrays, then each read group's (empty: none).  A BSQ_* status.
int write_im_coverage_table(const char* path, const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* pa,
                            const std::vector<CoverageRegion>& per_rg);
// The same table in parts: the header for n_groups read groups, then the rows of target offsets
// [lo, hi), each group's region holding exactly those positions.
void write_im_coverage_header(std::ostream& out, size_t n_groups);
int write_im_coverage_rows(std::ostream& out, const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* pa,
                           uint64_t lo, uint64_t hi, const std::vector<CoverageRegion>& per_rg);
// The table's downsampling for a region and --resolution (coverage_output.cpp:203-209) and the first
// position pileup_base::handle_position keeps, (position + start) % downsample == 0
// (pileup_base.cpp:130-133).
uint32_t coverage_downsample(uint32_t start, uint32_t end, uint32_t resolution);
uint32_t coverage_first_handled(uint32_t start, uint32_t downsample);
// coverage_output::table (src/breseq/coverage_output.cpp:190-284) with the rows the pileup driver
// produces for the region (pileup_base.cpp:130-133, 141-210, 308-355).  False if the file cannot be
// written.
// per_rg: with BSQ_COV_PER_READ_GROUP, each read group's columns at the same positions.
bool write_coverage_region(const char* path, const CoverageRegion& R, uint32_t resolution, uint32_t flags,
                           const double* reference_average, const std::vector<CoverageRegion>& per_rg);

// Soft-clipping rows in the reference's order (direction -1 then +1, targets in seq_id order,
// positions ascending; soft_clipping.cpp:500-545) and the genome-wide totals and dispersion fit
// (:547-623).  rows / outs hold the device's rows: direction -1 in column order, then direction +1.
// tested_spanning = 2 x the testable positions with spanning reads.
void sc_assemble(const ScRowDev* rows, const ScOutDev* outs, uint64_t rows_neg, uint64_t rows_pos,
                 const std::vector<uint32_t>& tpoff, const std::vector<uint32_t>& name_order, uint32_t K,
                 const bsq_sc_params& p, uint64_t total_clipped, uint64_t total_spanning, uint64_t tested_spanning,
                 std::vector<bsq_sc_position>& out, bsq_sc_summary& s);

// Discordant / missing-pair candidate regions (bsq_pairs_host.cpp) from the reads the device
// compacted: events in BAM order with their names in 256-byte slots, and per strand the MP
// window-total members' start columns (BAM order, so sorted) with their DP groups.  piled[t]: target t is in the pileup set and
// its deletion propagation cutoff is not below 0.
struct PairReplayInput {
  std::vector<uint32_t> tpoff, order;
  std::vector<uint8_t> piled;
  std::vector<double> window_width;
  std::vector<uint32_t> r1_prefix, r2_prefix;
  int32_t dp_seed = 3, mp_seed = 3;
  double mp_seed_fraction = 0.25;
  bool mp = false;
  const PairEvent* ev = nullptr;
  uint64_t n_ev = 0;
  const char* names = nullptr;
  const uint32_t* mem_start[2] = {nullptr, nullptr};
  const uint8_t* mem_group[2] = {nullptr, nullptr};
  uint64_t n_mem[2] = {0, 0};
};
struct PairReplayResult {
  std::vector<bsq_pair_region> dp, mp;
  std::string text;
};
int pair_replay(const PairReplayInput& in, PairReplayResult& out);

// Pair-distance regions and calibration (bsq_pairs_host.cpp) from the device's positions above a seed,
// its z histogram and ladder counts.
struct PdAssembleInput {
  std::vector<uint32_t> tpoff;
  std::vector<PdAbove> above;        // any order
  std::vector<uint64_t> hist;        // kPdHistBins; empty when the scan was not set up
  uint64_t ladder[2][kPdLadderSteps] = {};
  bool enabled = false;
  double z_seed = 0, mean_covering_gap = 0;
  uint64_t total_reference_length = 0;
};
struct PdResult {
  std::vector<bsq_pd_region> regions;   // capped and in the writer's order
  bsq_pd_summary summary;
};
void pd_assemble(PdAssembleInput& in, PdResult& out);

}  // namespace host
}  // namespace bsq
