// Output side of the scoring path, host only: breseq's text formats for the error tables and coverage
// distribution, the RA classification of test_RA_evidence, and the RA / MC / UN GenomeDiff lines.
// Every value goes through the same iostream formatting the reference uses, because the classification
// reads the formatted strings back (identify_mutations.cpp:187-229).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "bsq_host.h"

namespace {

const char kIdxChars[6] = {'A', 'C', 'G', 'T', '.', 'N'};

// to_string(double, precision, scientific) of src/breseq/common.h:845-870
std::string fmt_double(double v, int precision, bool scientific) {
  if (std::isnan(v)) return "NA";
  std::ostringstream o;
  o << (scientific ? std::scientific : std::fixed) << std::setprecision(precision) << v;
  std::string s = o.str();
  if (scientific && s.size() >= 3 && s[s.size() - 3] == '0') s.erase(s.size() - 3, 1);
  return s;
}
// default ostream formatting of a double (6 significant digits)
std::string fmt_default(double v) {
  std::ostringstream o;
  o << v;
  return o.str();
}
double double_from_string(const std::string& s) {   // common.h:939-950
  std::string u = s;
  for (auto& ch : u) ch = (char)toupper(ch);
  if (u == "NA" || u == "#NA" || u == "NAN") return std::numeric_limits<double>::quiet_NaN();
  if (u == "INF") return std::numeric_limits<double>::infinity();
  if (u == "-INF") return -std::numeric_limits<double>::infinity();
  std::istringstream i(s);
  double d = 0;
  i >> d;
  return d;
}
double num(const std::string& s) { std::istringstream i(s); double d = 0; i >> d; return d; }
std::vector<std::string> split(const std::string& s, char sep) {
  std::vector<std::string> out;
  std::string cur;
  for (char ch : s) { if (ch == sep) { out.push_back(cur); cur.clear(); } else cur += ch; }
  out.push_back(cur);
  return out;
}
std::string pair_str(int32_t top, int32_t bot) { return std::to_string(top) + "/" + std::to_string(bot); }

typedef std::map<std::string, std::string> Entry;

// RA fields as identify_mutations_pileup::pileup_callback fills them (identify_mutations.cpp:1836-1910)
Entry ra_entry(const bsq_ra_record& r, const char* seq_id, uint32_t places) {
  Entry e;
  auto reported = [&](double f) { return (r.n == 0 || f < 0.5 / (double)r.n) ? 0.0 : f; };
  e["seq_id"] = seq_id;
  e["position"] = std::to_string(r.position);
  e["insert_position"] = std::to_string(r.insert_position);
  e["score"] = fmt_double(r.score, 1, false);
  e["ref_base"] = std::string(1, r.ref_base);
  e["new_base"] = std::string(1, r.new_base);
  e["major_base"] = std::string(1, r.major_base);
  e["minor_base"] = std::string(1, r.minor_base);
  e["major_frequency"] = fmt_double(r.major_frequency, (int)places, true);
  e["frequency"] = fmt_double(r.frequency, (int)places, true);
  std::string spec;
  for (int b = 0; b < 5; b++) {
    const double fr = reported(r.f[b]);
    if (fr <= 0.0) continue;
    if (!spec.empty()) spec += ",";
    spec += std::string(1, kIdxChars[b]) + ":" + fmt_double(fr, (int)places, true);
  }
  e["allele_frequencies"] = spec;
  e["frequency_lower"] = fmt_double(r.frequency_lower, (int)places, true);
  e["frequency_upper"] = fmt_double(r.frequency_upper, (int)places, true);
  e["ks_quality_p_value"] = fmt_double(r.ks_quality_p, 5, true);
  e["fisher_strand_p_value"] = fmt_double(r.fisher_strand_p, 5, true);
  e["ref_cov"] = pair_str(r.ref_cov[0], r.ref_cov[1]);
  e["new_cov"] = pair_str(r.new_cov[0], r.new_cov[1]);
  e["major_cov"] = pair_str(r.major_cov[0], r.major_cov[1]);
  e["minor_cov"] = pair_str(r.minor_cov[0], r.minor_cov[1]);
  e["total_cov"] = pair_str(r.total_cov[0], r.total_cov[1]);
  return e;
}

bool has(const Entry& e, const char* k) { return e.count(k) != 0; }
void add_reject(Entry& e, const std::string& reason, const char* field = "reject") {
  if (!has(e, field)) { e[field] = reason; return; }
  for (const std::string& x : split(e[field], ',')) if (x == reason) return;
  e[field] = e[field] + "," + reason;
}

struct RefView {
  const bsq_reference* ref;
  uint32_t tid;
  uint32_t len() const { return (uint32_t)(ref->target_offset[tid + 1] - ref->target_offset[tid]); }
  std::string base1(int32_t p) const {   // get_sequence_1(p, p); empty outside the sequence
    if (p < 1 || (uint32_t)p > len()) return "";
    return std::string(1, ref->seq[ref->target_offset[tid] + p - 1]);
  }
};

bool rejected_bias(Entry& ra, const bsq_ra_settings& s) {        // identify_mutations.cpp:143-171
  bool rej = false;
  if (s.polymorphism_ks_quality_p_value_cutoff != 0 && has(ra, "ks_quality_p_value") &&
      num(ra["ks_quality_p_value"]) < s.polymorphism_ks_quality_p_value_cutoff) { rej = true; add_reject(ra, "KS_BASE_QUALITY"); }
  if (s.polymorphism_fisher_strand_p_value_cutoff != 0 && has(ra, "fisher_strand_p_value") &&
      num(ra["fisher_strand_p_value"]) < s.polymorphism_fisher_strand_p_value_cutoff) { rej = true; add_reject(ra, "FISHER_STRAND"); }
  return rej;
}

bool rejected_poly_coverage(Entry& ra, const bsq_ra_settings& s) {   // identify_mutations.cpp:231-327
  bool rej = false;
  if (s.polymorphism_minimum_variant_coverage_each_strand > 0) {
    bool passed = true;
    const std::string ref_base = has(ra, "ref_base") ? ra["ref_base"] : "";
    bool maj_var = has(ra, "major_base") && ra["major_base"] != ref_base;
    bool min_var = has(ra, "minor_base") && ra["minor_base"] != ref_base;
    if (!maj_var && !min_var) { maj_var = true; min_var = true; }
    if (maj_var && has(ra, "major_cov")) {
      auto tb = split(ra["major_cov"], '/');
      passed = passed && num(tb[0]) >= s.polymorphism_minimum_variant_coverage_each_strand;
      passed = passed && num(tb[1]) >= s.polymorphism_minimum_variant_coverage_each_strand;
    }
    if (min_var && has(ra, "minor_cov")) {
      auto tb = split(ra["minor_cov"], '/');
      passed = passed && num(tb[0]) >= s.polymorphism_minimum_variant_coverage_each_strand;
      passed = passed && num(tb[1]) >= s.polymorphism_minimum_variant_coverage_each_strand;
    }
    if (!passed) { rej = true; add_reject(ra, "VARIANT_STRAND_COVERAGE"); }
  }
  if (s.polymorphism_minimum_total_coverage_each_strand > 0) {
    auto tb = split(ra["total_cov"], '/');
    if (!(num(tb[0]) >= s.polymorphism_minimum_total_coverage_each_strand &&
          num(tb[1]) >= s.polymorphism_minimum_total_coverage_each_strand)) { rej = true; add_reject(ra, "TOTAL_STRAND_COVERAGE"); }
  }
  if (s.polymorphism_minimum_variant_coverage > 0) {
    auto a = split(ra["major_cov"], '/'), b = split(ra["minor_cov"], '/');
    bool passed = (num(a[0]) + num(a[1]) >= s.polymorphism_minimum_variant_coverage) &&
                  (num(b[0]) + num(b[1]) >= s.polymorphism_minimum_variant_coverage);
    if (!passed) { rej = true; add_reject(ra, "VARIANT_COVERAGE"); }
  }
  if (s.polymorphism_minimum_total_coverage > 0) {
    auto tb = split(ra["total_cov"], '/');
    if (num(tb[0]) + num(tb[1]) < s.polymorphism_minimum_total_coverage) { add_reject(ra, "TOTAL_COVERAGE"); rej = true; }
  }
  return rej;
}

bool rejected_cons_coverage(Entry& ra, const bsq_ra_settings& s) {   // identify_mutations.cpp:329-371
  bool rej = false;
  if (s.consensus_minimum_variant_coverage_each_strand > 0) {
    auto tb = split(ra["major_cov"], '/');
    if (num(tb[0]) < s.consensus_minimum_variant_coverage_each_strand || num(tb[1]) < s.consensus_minimum_variant_coverage_each_strand) {
      add_reject(ra, "VARIANT_STRAND_COVERAGE"); rej = true;
    }
  }
  if (s.consensus_minimum_total_coverage_each_strand > 0) {
    auto tb = split(ra["total_cov"], '/');
    if (num(tb[0]) < s.consensus_minimum_total_coverage_each_strand || num(tb[1]) < s.consensus_minimum_total_coverage_each_strand) {
      add_reject(ra, "TOTAL_STRAND_COVERAGE"); rej = true;
    }
  }
  if (s.consensus_minimum_variant_coverage > 0) {
    auto tb = split(ra["major_cov"], '/');
    if (num(tb[0]) + num(tb[1]) < s.consensus_minimum_variant_coverage) { add_reject(ra, "VARIANT_COVERAGE"); rej = true; }
  }
  if (s.consensus_minimum_total_coverage > 0) {
    auto tb = split(ra["total_cov"], '/');
    if (num(tb[0]) + num(tb[1]) < s.consensus_minimum_total_coverage) { add_reject(ra, "TOTAL_COVERAGE"); rej = true; }
  }
  return rej;
}

bool rejected_homopolymer(Entry& ra, const RefView& R, uint32_t indel_len, uint32_t surround_len, bool no_indels) {
  // identify_mutations.cpp:373-481
  bool rej = false;
  if (indel_len && (ra["ref_base"] == "." || ra["new_base"] == ".")) {
    int32_t mut_pos = (int32_t)num(ra["position"]);
    const bool is_ins = num(ra["insert_position"]) > 0;
    const std::string mut_base = (ra["ref_base"] == ".") ? ra["new_base"] : ra["ref_base"];
    int32_t hl = 0;
    bool no_match = false;
    if (is_ins && R.base1(mut_pos) != mut_base) {
      mut_pos++;
      if (mut_pos > (int32_t)R.len() || R.base1(mut_pos) != mut_base) no_match = true;
    }
    if (!no_match) {
      int32_t sp = mut_pos - 1;
      while (R.base1(sp) == mut_base && sp > 0) sp--;
      sp++;
      int32_t ep = mut_pos + 1;
      while (R.base1(ep) == mut_base && ep <= (int32_t)R.len()) ep++;
      ep--;
      hl = ep - sp + 1;
    }
    if (hl >= (int32_t)indel_len) { rej = true; add_reject(ra, "INDEL_HOMOPOLYMER"); }
  }
  if (surround_len && ra["ref_base"] != "." && ra["new_base"] != ".") {
    const int32_t mut_pos = (int32_t)num(ra["position"]);
    const std::string mut_base = ra["new_base"];
    int32_t sp = mut_pos - 1;
    while (sp >= 1 && R.base1(sp) == mut_base) sp--;
    sp++;
    int32_t ep = mut_pos + 1;
    while (ep <= (int32_t)R.len() && R.base1(ep) == mut_base) ep++;
    ep--;
    if (sp < mut_pos && ep > mut_pos && ep - sp + 1 >= (int32_t)surround_len) { rej = true; add_reject(ra, "SURROUNDING_HOMOPOLYMER"); }
  }
  if (no_indels && (ra["ref_base"] == "." || ra["new_base"] == ".")) { rej = true; add_reject(ra, "POLYMORPHIC_INDEL"); }
  return rej;
}

// Returns whether the entry is deleted (identify_mutations.cpp:522-684).
bool classify(Entry& ra, const RefView& R, const bsq_ra_settings& s) {
  const double score = has(ra, "score") ? double_from_string(ra["score"]) : std::numeric_limits<double>::quiet_NaN();
  double lower, upper;
  if (has(ra, "frequency_lower") && has(ra, "frequency_upper")) {
    lower = num(ra["frequency_lower"]);
    upper = num(ra["frequency_upper"]);
  } else {
    lower = upper = num(ra["frequency"]);
  }
  const bool poly_mode = s.polymorphism_prediction != 0;
  // 1. consensus
  if (score < s.mutation_log10_e_value_cutoff) add_reject(ra, "SCORE_CUTOFF");
  const double cons_bound = poly_mode ? upper : lower;
  if (s.consensus_frequency_cutoff > 0.0 && cons_bound < s.consensus_frequency_cutoff) add_reject(ra, "FREQUENCY_CUTOFF");
  rejected_cons_coverage(ra, s);
  rejected_homopolymer(ra, R, s.consensus_reject_indel_homopolymer_length, s.consensus_reject_surrounding_homopolymer_length, false);
  if (!has(ra, "reject")) {
    ra["prediction"] = "consensus";
    return ra["ref_base"] == ra["major_base"];
  }
  ra["consensus_reject"] = ra["reject"];
  ra.erase("reject");
  // 2. polymorphism
  if (score < s.polymorphism_log10_e_value_cutoff) add_reject(ra, "SCORE_CUTOFF");
  if (s.polymorphism_frequency_cutoff > 0.0 && lower < s.polymorphism_frequency_cutoff) add_reject(ra, "FREQUENCY_CUTOFF");
  rejected_bias(ra, s);
  rejected_poly_coverage(ra, s);
  rejected_homopolymer(ra, R, s.polymorphism_reject_indel_homopolymer_length,
                       s.polymorphism_reject_surrounding_homopolymer_length, s.polymorphism_no_indels != 0);
  if (!has(ra, "reject")) {
    ra["prediction"] = "polymorphism";
    return false;
  }
  if (!poly_mode) {
    ra["polymorphism_reject"] = ra["reject"];
    ra.erase("reject");
    return true;
  }
  // 3. polymorphism mode keeps the entry, marked rejected
  ra["prediction"] = "polymorphism";
  return false;
}

void copy_str(char* dst, size_t cap, const std::string& s) {
  const size_t n = std::min(cap - 1, s.size());
  memcpy(dst, s.data(), n);
  dst[n] = 0;
}

}  // namespace

namespace bsq {
namespace host {

uint32_t coverage_downsample(uint32_t start, uint32_t end, uint32_t resolution) {
  if (resolution == 0) return 1;
  return std::max<uint32_t>(1, (uint32_t)std::floor((double)(end - start + 1) / (double)resolution));
}
uint32_t coverage_first_handled(uint32_t start, uint32_t downsample) {
  return start + (uint32_t)((downsample - ((uint64_t)start * 2) % downsample) % downsample);
}

bool write_coverage_region(const char* path, const CoverageRegion& R, uint32_t resolution, uint32_t flags,
                           const double* reference_average, const std::vector<CoverageRegion>& per_rg) {
  const bool total_only = flags & BSQ_COV_TOTAL_ONLY;
  const char* d = (flags & BSQ_COV_CSV) ? "," : "\t";
  const uint32_t downsample = coverage_downsample(R.start, R.end, resolution);
  const uint32_t first_handled = coverage_first_handled(R.start, downsample);
  if (downsample % R.step != 0 || R.first > first_handled || (first_handled - R.first) % R.step != 0)
    return false;   // the columns do not include every handled position
  std::ofstream out(path);
  if (!out) return false;
  out << "position" << d << "ref_base";
  static const char* kFull[8] = {"unique_top_cov", "unique_bot_cov", "redundant_top_cov", "redundant_bot_cov",
                                 "raw_redundant_top_cov", "raw_redundant_bot_cov", "unique_top_begin", "unique_bot_begin"};
  static const char* kTotal[3] = {"unique_cov", "redundant_cov", "total_cov"};
  const int ncols = total_only ? 3 : 8;
  const bool by_rg = (flags & BSQ_COV_PER_READ_GROUP) != 0;
  const size_t n_rg = by_rg ? per_rg.size() : 0;
  for (int c = 0; c < ncols; c++) out << d << (total_only ? kTotal[c] : kFull[c]);
  // per read group, after the aggregate columns, prefixed "RG-<g>_" (coverage_output.cpp:236-247)
  for (size_t g = 0; g < n_rg; g++)
    for (int c = 0; c < ncols; c++) out << d << "RG-" << g << "_" << (total_only ? kTotal[c] : kFull[c]);
  out << "\n";
  double sum_unique = 0, sum_repeat = 0, sum_all = 0;
  std::vector<double> rg_unique(n_rg, 0.0), rg_repeat(n_rg, 0.0), rg_all(n_rg, 0.0);
  uint32_t rows = 0;
  // the columns of one region at position p: zero coverage outside its columns
  auto cells = [&](const CoverageRegion& X, uint32_t p, uint32_t (&c)[6], double& r0, double& r1) {
    for (int q = 0; q < 6; q++) c[q] = 0;
    r0 = r1 = 0;
    if (p >= X.first && p <= X.end && (p - X.first) % X.step == 0) {
      const uint32_t i = (p - X.first) / X.step;
      for (int q = 0; q < 6; q++) c[q] = X.counts[(size_t)q * X.m + i];
      r0 = X.red[i];
      r1 = X.red[(size_t)X.m + i];
    }
  };
  auto print = [&](const uint32_t (&c)[6], double r0, double r1) {
    if (total_only) out << (c[0] + c[1]) << d << fmt_default(r0 + r1) << d << fmt_default(c[0] + c[1] + r0 + r1);
    else out << c[0] << d << c[1] << d << fmt_default(r0) << d << fmt_default(r1) << d << c[2] << d << c[3] << d << c[4] << d << c[5];
  };
  // a row for position p (coverage_output.cpp:436-500)
  auto row = [&](uint32_t p) {
    uint32_t c[6];
    double r0, r1;
    cells(R, p, c, r0, r1);
    rows++;
    sum_unique += c[0] + c[1];
    sum_repeat += r0 + r1;
    sum_all += c[0] + c[1] + r0 + r1;
    out << p << d << R.ref[p - 1] << d;
    print(c, r0, r1);
    for (size_t g = 0; g < n_rg; g++) {
      cells(per_rg[g], p, c, r0, r1);
      out << d;
      print(c, r0, r1);
      rg_unique[g] += c[0] + c[1];
      rg_repeat[g] += r0 + r1;
      rg_all[g] += c[0] + c[1] + r0 + r1;
    }
    out << "\n";
  };
  // Up to the pileup's last column the driver moves its cursor through every position and the
  // handled ones get a row.  Past it only handled positions move the cursor, and each of them first
  // prints the positions skipped since the cursor as zero rows (coverage_output.cpp:318-327,
  // pileup_base.cpp:345-351).
  const uint32_t covered_end = std::min(R.last, R.end);
  uint64_t q = first_handled;
  for (; q <= covered_end; q += downsample) row((uint32_t)q);
  uint32_t cursor = R.last;
  for (; q <= R.end; q += downsample) {
    for (uint32_t i = cursor + 1; i < q; i++) {
      out << i << d << R.ref[i - 1];
      for (size_t c = 0; c < (size_t)ncols * (1 + n_rg); c++) out << d << 0;
      out << "\n";
      rows++;
    }
    row((uint32_t)q);
    cursor = (uint32_t)q;
  }
  if (reference_average) out << "#" << d << "reference_unique_average_cov" << d << fmt_default(*reference_average) << "\n";
  out << "#" << d << "region_unique_average_cov" << d << fmt_default(sum_unique / rows) << "\n";
  out << "#" << d << "region_repeat_average_cov" << d << fmt_default(sum_repeat / rows) << "\n";
  out << "#" << d << "region_average_cov" << d << fmt_default(sum_all / rows) << "\n";
  out << "#" << d << "number_of_positions" << d << rows << "\n";
  for (size_t g = 0; g < n_rg; g++) {
    out << "#" << d << "RG-" << g << "_region_unique_average_cov" << d << fmt_default(rg_unique[g] / rows) << "\n";
    out << "#" << d << "RG-" << g << "_region_repeat_average_cov" << d << fmt_default(rg_repeat[g] / rows) << "\n";
    out << "#" << d << "RG-" << g << "_region_average_cov" << d << fmt_default(rg_all[g] / rows) << "\n";
  }
  return (bool)out;
}

}  // namespace host
}  // namespace bsq

namespace bsq {
namespace host {

// <seq_id>.coverage.tsv: the header and rows of identify_mutations.cpp:2028-2052, 2173-2204.  The
// aggregate columns come from pass 2's per-position arrays (global columns); each read group's
// columns, when given, from its region tally over positions 1..len (region offsets).  position_coverage
// sums the strands bottom first (sum(), identify_mutations.h:99-126), and total_cov is the plain sum.
void write_im_coverage_header(std::ostream& out, size_t n_groups) {
  static const char* const kCols[3] = {"unique_cov", "redundant_cov", "total_cov"};
  out << "position\tref_base";
  for (const char* c : kCols) out << "\t" << c;
  for (size_t g = 0; g < n_groups; g++)      // group-major, as coverage_output::table
    for (const char* c : kCols) out << "\tRG-" << g << "_" << c;
  out << "\n";
}

int write_im_coverage_rows(std::ostream& out, const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* pa,
                           uint64_t lo, uint64_t hi, const std::vector<CoverageRegion>& per_rg) {
  if (!ref || !pa || tid >= ref->n_targets || !pa->unique_top || !pa->unique_bot || !pa->redundant_top ||
      !pa->redundant_bot)
    return BSQ_ERR_INVALID;
  const uint64_t b = ref->target_offset[tid], e = ref->target_offset[tid + 1];
  if (lo > hi || b + hi > e) return BSQ_ERR_INVALID;
  for (const CoverageRegion& R : per_rg)
    if (R.m != hi - lo) return BSQ_ERR_INVALID;
  auto cols = [&](uint32_t ut, uint32_t ub, double rt, double rb) {
    const double u = (double)ub + (double)ut;
    const double rr = rb + rt;
    out << "\t" << fmt_default(u) << "\t" << fmt_default(rr) << "\t" << fmt_default(u + rr);
  };
  for (uint64_t i = lo; i < hi; i++) {
    const uint64_t g = b + i;
    out << (i + 1) << "\t" << ref->seq[g];
    cols(pa->unique_top[g], pa->unique_bot[g], pa->redundant_top[g], pa->redundant_bot[g]);
    const uint64_t k = i - lo;
    for (const CoverageRegion& R : per_rg) cols(R.counts[k], R.counts[R.m + k], R.red[k], R.red[R.m + k]);
    out << "\n";
  }
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

int write_im_coverage_table(const char* path, const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* pa,
                            const std::vector<CoverageRegion>& per_rg) {
  if (!path || !ref || tid >= ref->n_targets) return BSQ_ERR_INVALID;
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  write_im_coverage_header(out, per_rg.size());
  return write_im_coverage_rows(out, ref, tid, pa, 0, ref->target_offset[tid + 1] - ref->target_offset[tid], per_rg);
}

}  // namespace host
}  // namespace bsq

extern "C" {

int bsq_default_ra_settings(int polymorphism_prediction, bsq_ra_settings* s) {
  if (!s) return BSQ_ERR_INVALID;
  memset(s, 0, sizeof *s);
  // src/breseq/settings.cpp:857-950
  s->polymorphism_prediction = polymorphism_prediction ? 1 : 0;
  s->mutation_log10_e_value_cutoff = 10;
  s->consensus_frequency_cutoff = polymorphism_prediction ? 0.95 : 0.50;
  s->polymorphism_log10_e_value_cutoff = polymorphism_prediction ? 2 : 10;
  s->polymorphism_frequency_cutoff = polymorphism_prediction ? 0.05 : 0.10;
  s->polymorphism_minimum_variant_coverage_each_strand = 2;
  s->polymorphism_fisher_strand_p_value_cutoff = 0.05;
  s->polymorphism_precision_places = polymorphism_prediction ? 8 : 3;
  return BSQ_OK;
}

int bsq_test_ra_evidence(const bsq_ra_record* ra, uint64_t n, const bsq_ra_settings* s, const bsq_reference* ref,
                         const char* const* target_names, bsq_ra_call* out) {
  if ((n && (!ra || !out)) || !s || !ref || !target_names) return BSQ_ERR_INVALID;
  for (uint64_t i = 0; i < n; i++) {
    if (ra[i].tid >= ref->n_targets) return BSQ_ERR_INVALID;
    Entry e = ra_entry(ra[i], target_names[ra[i].tid], s->polymorphism_precision_places);
    RefView R{ref, ra[i].tid};
    const bool del = classify(e, R, *s);
    memset(&out[i], 0, sizeof out[i]);
    out[i].deleted = del ? 1 : 0;
    copy_str(out[i].prediction, sizeof out[i].prediction, has(e, "prediction") ? e["prediction"] : "");
    copy_str(out[i].reject, sizeof out[i].reject, has(e, "reject") ? e["reject"] : "");
    copy_str(out[i].consensus_reject, sizeof out[i].consensus_reject, has(e, "consensus_reject") ? e["consensus_reject"] : "");
    copy_str(out[i].polymorphism_reject, sizeof out[i].polymorphism_reject,
             has(e, "polymorphism_reject") ? e["polymorphism_reject"] : "");
  }
  return BSQ_OK;
}

int bsq_format_ra(const bsq_ra_record* r, const char* seq_id, uint32_t precision_places, char* buf, uint64_t cap) {
  if (!r || !seq_id || !buf || cap == 0) return BSQ_ERR_INVALID;
  Entry e = ra_entry(*r, seq_id, precision_places);
  std::string line;
  for (const char* k : {"seq_id", "position", "insert_position", "ref_base", "new_base"}) { line += e[k]; line += "\t"; e.erase(k); }
  for (auto& kv : e) if (!kv.second.empty()) line += kv.first + "=" + kv.second + "\t";
  line.pop_back();
  if (line.size() + 1 > cap) return BSQ_ERR_SIZE;
  memcpy(buf, line.c_str(), line.size() + 1);
  return BSQ_OK;
}

int bsq_write_error_rates(const char* path, const uint64_t* counts, uint32_t R, uint32_t Q) {
  if (!path || !counts || !R || !Q) return BSQ_ERR_INVALID;
  std::vector<double> lp((size_t)R * 25 * Q);
  if (bsq_counts_to_log10_prob(counts, R, Q, lp.data()) != BSQ_OK) return BSQ_ERR_INVALID;
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  // error_count.cpp:660-690 (covariates in enum order; ref/obs base without a maximum)
  out << "read_set=" << R << ",ref_base,obs_base,quality=" << Q << "\n";
  out << "read_set\tref_base\tobs_base\tquality\tlog10_probability\n";
  for (size_t idx = 0; idx < lp.size(); idx++) {
    const uint32_t rs = idx % R, ref = (idx / R) % 5, obs = (idx / (5 * R)) % 5, q = (uint32_t)(idx / (25 * (size_t)R));
    out << rs << '\t' << kIdxChars[ref] << '\t' << kIdxChars[obs] << '\t' << q << '\t';
    // the parsed-back value prints as the value the reference printed
    out << fmt_default(lp[idx]) << "\n";
  }
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

int bsq_write_base_qual_error_prob(const char* path_pattern, const char* const* read_file_names, const uint64_t* counts,
                                   uint32_t R, uint32_t Q) {
  if (!path_pattern || !read_file_names || !counts || !R || !Q) return BSQ_ERR_INVALID;
  // error_count.cpp:697-785: counts summed to [read set][quality][obs][ref], each (obs) group of five
  // reference bases normalized, zeros printed as NA
  std::vector<double> t((size_t)R * Q * 25, 0.0);
  for (size_t idx = 0; idx < (size_t)R * 25 * Q; idx++) {
    const uint32_t rs = idx % R, ref = (idx / R) % 5, obs = (idx / (5 * R)) % 5, q = (uint32_t)(idx / (25 * (size_t)R));
    t[(size_t)rs * 25 * Q + (size_t)q * 25 + obs * 5 + ref] += (double)counts[idx];
  }
  double running = 0;
  for (uint32_t r = 0; r < R; r++) {
    for (uint32_t k = 0; k < 25 * Q; k++) {
      const size_t i = (size_t)r * 25 * Q + k;
      running += t[i];
      if (i % 5 == 4) {
        for (size_t j = i - 4; j <= i; j++) {
          if (running > 0) t[j] /= running;
          if (t[j] == 0) t[j] = std::numeric_limits<double>::quiet_NaN();
        }
        running = 0;
      }
    }
    std::string name(path_pattern);
    const size_t h = name.find('#');
    if (h != std::string::npos) name.replace(h, 1, read_file_names[r]);
    std::ofstream out(name.c_str());
    if (!out) return BSQ_ERR_INVALID;
    out << "quality";
    for (int b1 = 0; b1 < 5; b1++)
      for (int b2 = 0; b2 < 5; b2++) out << "\t" << kIdxChars[b1] << kIdxChars[b2];
    out << "\n";
    for (uint32_t q = 0; q < Q; q++) {
      out << q;
      for (int b1 = 0; b1 < 5; b1++)
        for (int b2 = 0; b2 < 5; b2++) {
          const double v = t[(size_t)r * 25 * Q + (size_t)q * 25 + b1 * 5 + b2];
          out << "\t";
          if (std::isnan(v)) out << "NA"; else out << fmt_default(v);
        }
      out << "\n";
    }
  }
  return BSQ_OK;
}

int bsq_write_coverage_distribution(const char* path, const uint64_t* hist, uint32_t size) {
  if (!path || (size && !hist)) return BSQ_ERR_INVALID;
  std::ofstream out(path);     // error_count.cpp:239-253
  if (!out) return BSQ_ERR_INVALID;
  out << "coverage\tn\n";
  for (uint32_t j = 1; j < size; j++) out << j << "\t" << hist[j] << "\n";
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

int bsq_write_coverage_table(const char* path, const char* seq_id, const bsq_reference* ref, uint32_t tid,
                             const bsq_position_arrays* pa) {
  (void)seq_id;
  return bsq::host::write_im_coverage_table(path, ref, tid, pa, {});
}

int bsq_write_gd(const char* path, const bsq_reference* ref, const char* const* target_names,
                 const double* deletion_propagation_cutoff, uint32_t precision_places,
                 const bsq_ra_record* ra, uint64_t n_ra, const bsq_ra_call* calls,
                 const bsq_mc_record* mc, uint64_t n_mc, const bsq_un_record* un, uint64_t n_un) {
  if (!path || !ref || !target_names || !deletion_propagation_cutoff) return BSQ_ERR_INVALID;
  std::vector<uint32_t> rank(ref->n_targets, 0);
  for (uint32_t i = 0; i < ref->n_target_order; i++) rank[ref->target_order[i]] = i;
  struct Item { int type; uint64_t idx; uint32_t tid; uint64_t add_pos; int phase; uint32_t ins; std::string id; Entry e; };
  std::vector<Item> items;
  // the order the pileup adds entries, which is the order ids are handed out in: per target, at each
  // position the MC ended there, then the UN ended there, then the position's RA items; at the
  // target's end the open MC / UN and a whole-target MC for a failed coverage fit
  for (uint64_t i = 0; i < n_ra; i++) {
    if (calls && calls[i].deleted) continue;
    Item it{0, i, ra[i].tid, ra[i].position, 2, ra[i].insert_position, "", ra_entry(ra[i], target_names[ra[i].tid], precision_places)};
    if (calls) {
      if (calls[i].prediction[0]) it.e["prediction"] = calls[i].prediction;
      if (calls[i].reject[0]) it.e["reject"] = calls[i].reject;
      if (calls[i].consensus_reject[0]) it.e["consensus_reject"] = calls[i].consensus_reject;
      if (calls[i].polymorphism_reject[0]) it.e["polymorphism_reject"] = calls[i].polymorphism_reject;
    }
    items.push_back(it);
  }
  for (uint64_t i = 0; i < n_mc; i++) {
    const bsq_mc_record& m = mc[i];
    if (m.tid >= ref->n_targets) return BSQ_ERR_INVALID;
    const uint32_t len = (uint32_t)(ref->target_offset[m.tid + 1] - ref->target_offset[m.tid]);
    const bool whole = deletion_propagation_cutoff[m.tid] < 0.0;
    Item it{1, i, m.tid, whole ? (uint64_t)len + 1 : (uint64_t)m.end + 1, whole ? 3 : 0, 0, "", Entry()};
    it.e["seq_id"] = target_names[m.tid];
    it.e["start"] = std::to_string(m.start);
    it.e["end"] = std::to_string(m.end);
    it.e["start_range"] = std::to_string(m.start_range);
    it.e["end_range"] = std::to_string(m.end_range);
    it.e["left_outside_cov"] = fmt_double(m.left_outside_cov, 0, false);
    it.e["left_inside_cov"] = fmt_double(m.left_inside_cov, 0, false);
    it.e["right_inside_cov"] = fmt_double(m.right_inside_cov, 0, false);
    it.e["right_outside_cov"] = fmt_double(m.right_outside_cov, 0, false);
    items.push_back(it);
  }
  for (uint64_t i = 0; i < n_un; i++) {
    if (un[i].tid >= ref->n_targets) return BSQ_ERR_INVALID;
    Item it{2, i, un[i].tid, (uint64_t)un[i].end + 1, 1, 0, "", Entry()};
    it.e["seq_id"] = target_names[un[i].tid];
    it.e["start"] = std::to_string(un[i].start);
    it.e["end"] = std::to_string(un[i].end);
    items.push_back(it);
  }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    const Item &x = items[a], &y = items[b];
    if (rank[x.tid] != rank[y.tid]) return rank[x.tid] < rank[y.tid];
    if (x.add_pos != y.add_pos) return x.add_pos < y.add_pos;
    if (x.phase != y.phase) return x.phase < y.phase;
    return x.ins < y.ins;
  });
  for (size_t k = 0; k < order.size(); k++) items[order[k]].id = std::to_string(k + 1);
  // cGenomeDiff::sort (genome_diff_entry.cpp:570-660): evidence group, seq_id, position, then the
  // line-specification fields; ties keep insertion order
  static const int group[3] = {3, 4, 7};
  auto key_pos = [](const Item& x) { return (uint32_t)num(x.type == 0 ? x.e.at("position") : x.e.at("start")); };
  std::vector<size_t> out_order(order);
  std::stable_sort(out_order.begin(), out_order.end(), [&](size_t a, size_t b) {
    const Item &x = items[a], &y = items[b];
    if (group[x.type] != group[y.type]) return group[x.type] < group[y.type];
    const std::string& sx = x.e.at("seq_id");
    const std::string& sy = y.e.at("seq_id");
    if (sx != sy) return sx < sy;
    if (key_pos(x) != key_pos(y)) return key_pos(x) < key_pos(y);
    if (x.type == 0) {
      const char* fields[] = {"insert_position", "ref_base", "new_base"};
      for (const char* f : fields) if (x.e.at(f) != y.e.at(f)) return x.e.at(f) < y.e.at(f);
    } else if (x.type == 1) {
      if (num(x.e.at("end")) != num(y.e.at("end"))) return num(x.e.at("end")) < num(y.e.at("end"));
      for (const char* f : {"start_range", "end_range"}) if (x.e.at(f) != y.e.at(f)) return x.e.at(f) < y.e.at(f);
    } else {
      if (num(x.e.at("end")) != num(y.e.at("end"))) return num(x.e.at("end")) < num(y.e.at("end"));
    }
    return false;
  });
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  out << "#=GENOME_DIFF\t1.0\n";
  static const char* tname[3] = {"RA", "MC", "UN"};
  static const std::vector<std::string> spec[3] = {
      {"seq_id", "position", "insert_position", "ref_base", "new_base"},
      {"seq_id", "start", "end", "start_range", "end_range"},
      {"seq_id", "start", "end"}};
  for (size_t k : out_order) {
    Item& x = items[k];
    out << tname[x.type] << "\t" << x.id << "\t.";
    Entry e = x.e;
    for (const std::string& f : spec[x.type]) { out << "\t" << e[f]; e.erase(f); }
    for (auto& kv : e) if (!kv.second.empty() && kv.first[0] != '_') out << "\t" << kv.first << "=" << kv.second;
    out << "\n";
  }
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

int bsq_default_sc_params(bsq_sc_params* p) {
  if (!p) return BSQ_ERR_INVALID;
  // Settings defaults (src/breseq/settings.cpp:1369-1374)
  p->minimum_clipped_bases = 12;
  p->consensus_base_fraction = 0.95;
  p->dispersion_trim_frequency = 0.25;
  p->maximum_dispersion = 0.005;
  p->minimum_rate = 1e-5;
  p->target_name_order = nullptr;
  return BSQ_OK;
}

int bsq_write_soft_clipping_counts(const char* path, const char* const* target_names, const bsq_sc_params* p,
                                   const bsq_sc_summary* s, const bsq_sc_position* rows, uint64_t n) {
  if (!path || !target_names || !p || !s || (n && !rows)) return BSQ_ERR_INVALID;
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  // soft_clipping.cpp:630-646: a parameter line (default ostream formatting of the doubles), the
  // column names, and one row per (position, direction) with clip events; "." for no sequence
  out << "#sc_format=2\tsoft_clipping_minimum_bases=" << p->minimum_clipped_bases
      << "\tconsensus_base_fraction=" << fmt_default(p->consensus_base_fraction)
      << "\tnull_rate=" << fmt_default(s->null_rate) << "\tdispersion=" << fmt_default(s->dispersion) << "\n";
  out << "seq_id\tposition\tdirection\tclipped_count\ttotal_count\tagree_count\tclipped_sequence\n";
  for (uint64_t i = 0; i < n; i++) {
    const bsq_sc_position& r = rows[i];
    out << target_names[r.target] << "\t" << r.position << "\t" << r.direction << "\t" << r.clipped_count << "\t"
        << r.total_count << "\t" << r.agree_count << "\t" << (r.clipped_sequence[0] ? r.clipped_sequence : ".") << "\n";
  }
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

}  // extern "C"
