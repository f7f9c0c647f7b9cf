/*
 * oracle.cpp -- CPU restatement of breseq's read-evidence scoring path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path: only tests/, the smoke test
 * and the CPU-baseline leg of bench.py load it.  Nothing in the breseq_gb300 package links or calls it.
 *
 * Parity status: UNPINNED against the reference binary.  breseq cannot be built here (it needs
 * htslib 1.23.1 and miniz 3.1.1, external libraries absent from the image, plus autotools), and its
 * tests' RA goldens need inputs that are not in the tree.  The statistics helpers are pinned to
 * R-equivalent implementations (scipy) by tests/test_oracle_stats.py, as the reference documents
 * them to be R-equivalent (src/breseq/stats.cpp:2130-2143, 2206-2219).
 *
 * What is restated, with the reference lines each part follows:
 *   - the pileup column iterator of htslib 1.23.1 (bam_plp_auto / resolve_cigar2, a third-party
 *     dependency not present under the reference tree), as breseq drives it from
 *     src/breseq/pileup_base.cpp:141-210, 308-385: per column, the covering reads in BAM order, with
 *     qpos, is_del (D and N ops) and indel (length of an I/D op that follows this aligned base).
 *     On a deletion column qpos is the query index of the next aligned base (htslib sets it to the
 *     query bases consumed so far);
 *   - error_count_pileup::pileup_callback      src/breseq/error_count.cpp:125-199
 *   - cErrorTable::count_alignment_position    src/breseq/error_count.cpp:854-986
 *   - covariates_to_index / counts_to_log10_prob  src/breseq/error_count.cpp:477-497, 1005-1026
 *   - identify_mutations_pileup::pileup_callback  src/breseq/identify_mutations.cpp:1309-2022
 *   - alignment_position_to_covariates         src/breseq/error_count.cpp:1049-1105
 *   - fill_read_base_likelihoods               src/breseq/identify_mutations.cpp:3359-3384
 *   - pure_genotype_call                       src/breseq/identify_mutations.cpp:3398-3433
 *   - fit_allele_frequencies / variant_presence_score   :3241-3318, :3329-3344
 *   - profile_log10_likelihood / write_RA_frequency_bounds  :3094-3143, :3175-3217
 *   - annotate_polymorphism_statistics          :3009-3033
 *   - fisher_exact_test_2x2 / ks_test_two_sample_less   src/breseq/stats.cpp:2144-2286
 *   - check_deletion_completion / update_unknown_intervals / at_target_end  :2262-2344, :2972-3007, :2107-2164
 *   - alignment accessors (query bounds, trims, redundancy)  src/breseq/alignment.cpp:44-290, alignment.h:355-411
 *   - tabulate_soft_clipping_counts / compute_clipped_tail_consensus / sc_position_is_testable
 *                                               src/breseq/soft_clipping.cpp:98-169, 285-666
 *     (pinned by hand-worked answers and the rules the reference states in its comments; see
 *     tests/test_softclip.py)
 *   - coverage_output::table / pileup_callback, with --per-read-group
 *                                               src/breseq/coverage_output.cpp:190-500
 *   - identify_mutations' coverage tally per read group and <seq_id>.coverage.tsv
 *                                               src/breseq/identify_mutations.cpp:1560-1610, 2028-2052,
 *                                               2173-2250
 *   - fit_censored_negative_binomial / fit_coverage_distribution and the Cephes functions they use
 *                                               src/breseq/coverage_distribution.cpp:115-396, stats.cpp
 *     (special functions pinned against scipy; see tests/test_coverage_fit.py)
 *   - the DP / MP / PD candidate-region scans walked position by position, and their writers
 *                                               src/breseq/identify_mutations.cpp:883-1006, 1395-1555, 2358-2967
 *
 * One deliberate divergence: where the reference would index a read past its end (a deletion that is
 * followed by a single aligned base, error_count.cpp:1073), it aborts on an assert; here the base is
 * treated as unusable.  The CUDA path does the same.
 */
#include "../include/breseq_gb300.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <iomanip>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

const double kNaN = std::numeric_limits<double>::quiet_NaN();
const uint32_t kUndef = 0xFFFFFFFFu;

// ----------------------------------------------------------------------------- encodings
// src/breseq/common.h:195-318
inline bool bam_is_N(uint8_t b) { return b == 0x0f; }
inline uint8_t compl_bam(uint8_t b) {
  switch (b) { case 1: return 8; case 2: return 4; case 4: return 2; case 8: return 1; default: return b; }
}
inline char compl_char(char c) {
  switch (c) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; case 'T': return 'A'; default: return c; }
}
inline int bam2index(uint8_t b) {  // '.' -> 4, unrecognised -> -1 (reference ASSERTs)
  switch (b) { case 1: return 0; case 2: return 1; case 4: return 2; case 8: return 3; case '.': return 4; default: return -1; }
}
inline int char2index(char c) {
  switch (c) { case 'A': return 0; case 'C': return 1; case 'G': return 2; case 'T': return 3; case '.': return 4; case 'N': return 5; default: return -1; }
}
inline int compl_index(int b) { return (b >= 0 && b <= 3) ? 3 - b : 4; }
const char kBaseChars[6] = {'A', 'C', 'G', 'T', '.', 'N'};

inline bool op_ref(uint32_t op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }
inline bool op_qmatch(uint32_t op) { return op == 0 || op == 7 || op == 8; }
enum { OP_M = 0, OP_I = 1, OP_D = 2, OP_N = 3, OP_S = 4, OP_H = 5, OP_P = 6, OP_EQ = 7, OP_X = 8 };

struct ReadInfo {
  int64_t pos, endpos;
  uint32_t len;
  int32_t qs0, qe0;    // query_start_0 / query_end_0       (alignment.cpp:219-256)
  int32_t qb0s, qb0e;  // query_bounds_0(min_qual = 0)       (alignment.cpp:113-196)
  uint32_t stranded_end1;  // query_stranded_end_1             (alignment.cpp:201-214)
  bool rev, skip;
};

struct Pile { int32_t qpos; bool is_del; int32_t indel; };

struct Data {
  const bsq_reference* ref;
  const bsq_read_soa* rd;
  std::vector<ReadInfo> info;
  std::vector<uint64_t> tgt_begin, tgt_end;  // read index range per target
  std::vector<int64_t> tgt_maxspan;
  std::string err;
};

inline uint8_t base_at(const bsq_read_soa* rd, uint64_t r, int64_t q) {
  uint64_t nib = rd->seq_off[r] + (uint64_t)q;
  uint8_t byte = rd->seq[nib >> 1];
  return (nib & 1) ? (byte & 0xf) : (byte >> 4);
}
inline uint8_t qual_at(const bsq_read_soa* rd, uint64_t r, int64_t q) { return rd->qual[rd->seq_off[r] + (uint64_t)q]; }

// htslib resolve_cigar2 restated from scratch for one column (see header comment).
bool resolve(const bsq_read_soa* rd, uint64_t r, int64_t col, Pile& e) {
  const uint32_t* cig = rd->cigar + rd->cigar_off[r];
  const int n = rd->n_cigar[r];
  int64_t x = rd->pos[r];
  int32_t y = 0;
  for (int k = 0; k < n; k++) {
    uint32_t op = cig[k] & 0xf, len = cig[k] >> 4;
    if (op_ref(op)) {
      if (col < x + (int64_t)len) {
        if (op_qmatch(op)) { e.qpos = y + (int32_t)(col - x); e.is_del = false; }
        else { e.qpos = y; e.is_del = true; }
        e.indel = 0;
        if (col == x + (int64_t)len - 1 && k + 1 < n) {
          uint32_t op2 = cig[k + 1] & 0xf, l2 = cig[k + 1] >> 4;
          if (op2 == OP_D && op != OP_D) {
            e.indel = -(int32_t)l2;
            for (int j = k + 2; j < n; j++) { if ((cig[j] & 0xf) == OP_D) e.indel -= (int32_t)(cig[j] >> 4); else break; }
          } else if (op2 == OP_I) {
            e.indel = (int32_t)l2;
            for (int j = k + 2; j < n; j++) {
              uint32_t o = cig[j] & 0xf;
              if (o == OP_I) e.indel += (int32_t)(cig[j] >> 4); else if (o != OP_P) break;
            }
          } else if (op2 == OP_P && k + 2 < n) {
            int32_t l3 = 0;
            for (int j = k + 2; j < n; j++) {
              uint32_t o = cig[j] & 0xf;
              if (o == OP_I) l3 += (int32_t)(cig[j] >> 4); else if (op_ref(o)) break;
            }
            if (l3 > 0) e.indel = l3;
          }
        }
        return true;
      }
      x += len;
      if (op_qmatch(op)) y += (int32_t)len;
    } else if (op == OP_I || op == OP_S) {
      y += (int32_t)len;
    }
  }
  return false;
}

int prepare(Data& d) {
  const bsq_read_soa* rd = d.rd;
  const bsq_reference* ref = d.ref;
  const uint64_t n = rd->n_reads;
  d.info.resize(n);
  d.tgt_begin.assign(ref->n_targets, 0);
  d.tgt_end.assign(ref->n_targets, 0);
  d.tgt_maxspan.assign(ref->n_targets, 1);
  int32_t last_tid = -1;
  int64_t last_pos = -1;
  for (uint64_t r = 0; r < n; r++) {
    ReadInfo& ri = d.info[r];
    int32_t tid = rd->tid[r];
    if (tid < 0 || (uint32_t)tid >= ref->n_targets) { d.err = "read with invalid tid"; return BSQ_ERR_INVALID; }
    if (tid < last_tid || (tid == last_tid && rd->pos[r] < last_pos)) { d.err = "records not coordinate-sorted"; return BSQ_ERR_INVALID; }
    last_tid = tid; last_pos = rd->pos[r];
    ri.skip = (rd->flag[r] & BSQ_PILEUP_SKIP_MASK) != 0;
    ri.rev = (rd->flag[r] & BSQ_FLAG_REVERSE) != 0;
    ri.pos = rd->pos[r];
    ri.len = rd->l_qseq[r];
    const uint32_t* cig = rd->cigar + rd->cigar_off[r];
    const int nc = rd->n_cigar[r];
    int64_t rlen = 0; uint32_t qlen = 0;
    for (int k = 0; k < nc; k++) {
      uint32_t op = cig[k] & 0xf, len = cig[k] >> 4;
      if (op_ref(op)) rlen += len;
      if (op == OP_M || op == OP_I || op == OP_S || op == OP_EQ || op == OP_X) qlen += len;
    }
    if (ri.skip) { ri.endpos = ri.pos + (rlen > 0 ? rlen : 1); continue; }
    if (nc == 0 || rlen == 0) { d.err = "mapped read without reference-consuming CIGAR op"; return BSQ_ERR_INVALID; }
    if (qlen != ri.len) { d.err = "CIGAR query length differs from read length"; return BSQ_ERR_INVALID; }
    ri.endpos = ri.pos + rlen;
    if ((uint64_t)ri.endpos > ref->target_offset[tid + 1] - ref->target_offset[tid]) { d.err = "read extends past target end"; return BSQ_ERR_INVALID; }
    d.tgt_maxspan[tid] = std::max<int64_t>(d.tgt_maxspan[tid], rlen);
    // query_start_1 (alignment.cpp:219-236)
    int32_t qs1 = 1;
    for (int k = 0; k < nc; k++) { if ((cig[k] & 0xf) != OP_S) break; qs1 += (int32_t)(cig[k] >> 4); }
    // query_end_1 (alignment.cpp:239-256)
    int32_t qe1 = (int32_t)qlen;
    for (int k = nc - 1; k > 0; k--) { if ((cig[k] & 0xf) != OP_S) break; qe1 -= (int32_t)(cig[k] >> 4); }
    ri.qs0 = qs1 - 1; ri.qe0 = qe1 - 1;
    // query_bounds_1 with min_qual = 0 (alignment.cpp:113-196): skips S/H/N, only S moves
    int32_t bs = 1, be = (int32_t)qlen;
    for (int k = 0; k < nc; k++) {
      uint32_t op = cig[k] & 0xf;
      if (op != OP_S && op != OP_H && op != OP_N) break;
      if (op == OP_S) bs += (int32_t)(cig[k] >> 4);
    }
    for (int k = nc - 1; k > 0; k--) {
      uint32_t op = cig[k] & 0xf;
      if (op != OP_S && op != OP_H && op != OP_N) break;
      if (op == OP_S) be -= (int32_t)(cig[k] >> 4);
    }
    ri.qb0s = bs - 1; ri.qb0e = be - 1;
    ri.stranded_end1 = ri.rev ? (uint32_t)((int32_t)ri.len - bs + 1) : (uint32_t)be;
  }
  // read index range of each target (records are sorted by tid)
  for (uint32_t t = 0; t < ref->n_targets; t++) {
    d.tgt_begin[t] = std::lower_bound(rd->tid, rd->tid + n, (int32_t)t) - rd->tid;
    d.tgt_end[t] = std::lower_bound(rd->tid, rd->tid + n, (int32_t)t + 1) - rd->tid;
  }
  return BSQ_OK;
}

// Active-window walk over columns [c0, c1) of target t: calls fn(col, active_reads) per column.
template <class F>
void walk_columns(const Data& d, uint32_t t, int64_t c0, int64_t c1, F&& fn) {
  const bsq_read_soa* rd = d.rd;
  uint64_t rb = d.tgt_begin[t], re = d.tgt_end[t];
  // first read that may still cover c0
  int64_t lo_pos = c0 - d.tgt_maxspan[t];
  uint64_t r = std::lower_bound(rd->pos + rb, rd->pos + re, (int32_t)std::max<int64_t>(lo_pos, -1)) - rd->pos;
  std::vector<uint64_t> active;
  for (; r < re && rd->pos[r] < c0; r++) {
    if (!d.info[r].skip && d.info[r].endpos > c0) active.push_back(r);
  }
  for (int64_t c = c0; c < c1; c++) {
    for (; r < re && rd->pos[r] <= c; r++) if (!d.info[r].skip) active.push_back(r);
    size_t w = 0;
    for (size_t i = 0; i < active.size(); i++) if (d.info[active[i]].endpos > c) active[w++] = active[i];
    active.resize(w);
    fn(c, active);
  }
}

template <class F>
void parallel_chunks(int64_t n, int n_threads, F&& fn) {
  if (n_threads <= 1 || n < 4096) { fn(0, n, 0); return; }
  int64_t chunk = std::max<int64_t>(1024, (n + n_threads * 4 - 1) / (n_threads * 4));
  std::atomic<int64_t> next(0);
  std::vector<std::thread> th;
  for (int i = 0; i < n_threads; i++) {
    th.emplace_back([&, i]() {
      for (;;) {
        int64_t s = next.fetch_add(chunk);
        if (s >= n) break;
        fn(s, std::min(n, s + chunk), i);
      }
    });
  }
  for (auto& x : th) x.join();
}

// ============================================================================ pass 1
struct EcPartial {
  std::vector<uint64_t> counts;
  std::vector<std::vector<uint64_t>> hist;   // per coverage group
  uint64_t found[2] = {0, 0};
  int err = 0;
};

// cErrorTable::count_alignment_position (error_count.cpp:854-986)
inline int count_events(const Data& d, uint64_t r, const Pile& e, int64_t ref_pos, const char* ref_seq, int64_t tlen,
                        uint32_t R, uint32_t Q, std::vector<uint64_t>& counts) {
  const bsq_read_soa* rd = d.rd;
  const ReadInfo& ri = d.info[r];
  const int rev = ri.rev ? 1 : 0;
  const uint32_t rs = rd->read_file[r];
  const int32_t qpos = e.qpos, qlen = (int32_t)ri.len;
  auto ref_at = [&](int64_t p) -> char { return (p >= 0 && p < tlen) ? ref_seq[p] : '\0'; };
  auto add = [&](uint32_t ref_i, uint32_t obs_i, uint32_t q) -> int {
    if (rs >= R || q >= Q) return BSQ_ERR_DATA;
    counts[rs + R * (ref_i + 5 * (obs_i + 5 * q))] += 1;
    return 0;
  };
  {  // (1) base substitution or match at this column
    uint8_t obs = base_at(rd, r, qpos);
    char refc = ref_at(ref_pos);
    if (!bam_is_N(obs) && refc != 'N') {
      if (rev) { obs = compl_bam(obs); refc = compl_char(refc); }
      int oi = bam2index(obs), ri2 = char2index(refc);
      if (oi < 0 || ri2 < 0 || ri2 > 4) return BSQ_ERR_DATA;
      if (add(ri2, oi, qual_at(rd, r, qpos))) return BSQ_ERR_DATA;
    }
  }
  if (e.indel == 0) {  // (2a) next base also aligned: '..'
    if (qpos < ri.qe0) {
      int32_t mq = qpos + 1 - rev;
      if (mq < 0 || mq >= qlen) return BSQ_ERR_DATA;
      uint8_t obs = base_at(rd, r, mq);
      char refc = ref_at(ref_pos + 1 - rev);
      if (!bam_is_N(obs) && refc != 'N') { if (add(4, 4, qual_at(rd, r, mq))) return BSQ_ERR_DATA; }
    }
  } else if (e.indel == -1) {  // (2b) exactly one deleted base follows
    int32_t mq = qpos + 1 - rev;
    if (mq < 0 || mq >= qlen) return BSQ_ERR_DATA;
    uint8_t obs = base_at(rd, r, mq);
    char refc = ref_at(ref_pos + 1);
    if (!bam_is_N(obs) && refc != 'N') {
      if (rev) refc = compl_char(refc);
      int ri2 = char2index(refc);
      if (ri2 < 0 || ri2 > 4) return BSQ_ERR_DATA;
      if (add(ri2, 4, qual_at(rd, r, mq))) return BSQ_ERR_DATA;
    }
  } else if (e.indel == 1) {  // (2c) exactly one inserted base follows
    int32_t mq = qpos + 1;
    if (mq >= qlen) return BSQ_ERR_DATA;
    if (mq <= ri.qe0 && mq >= ri.qs0) {
      uint8_t obs = base_at(rd, r, mq);
      if (!bam_is_N(obs)) {
        if (rev) obs = compl_bam(obs);
        int oi = bam2index(obs);
        if (oi < 0) return BSQ_ERR_DATA;
        if (add(4, oi, qual_at(rd, r, mq))) return BSQ_ERR_DATA;
      }
    }
  }
  return 0;
}

}  // namespace

// ============================================================================ exported: pass 1
extern "C" int oracle_error_count(const bsq_reference* ref, const bsq_read_soa* rd, const bsq_ec_params* p,
                                  bsq_ec_result* out, int n_threads, char* errbuf, int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  const uint32_t R = p->n_read_files, Q = p->n_quality;
  const uint32_t G = ref->n_coverage_groups;
  const size_t nbins = (size_t)R * 25 * Q;
  std::vector<uint64_t> counts(nbins, 0);
  std::vector<std::vector<uint64_t>> hist(G);
  if (out->no_pos_hash_pr) for (uint32_t t = 0; t < ref->n_targets; t++) out->no_pos_hash_pr[t] = 1.0;

  for (uint32_t oi = 0; oi < ref->n_target_order; oi++) {
    const uint32_t t = ref->target_order[oi];
    const char* tseq = ref->seq + ref->target_offset[t];
    const int64_t tlen = (int64_t)(ref->target_offset[t + 1] - ref->target_offset[t]);
    const uint32_t g = ref->coverage_group[t];
    int nth = std::max(1, n_threads);
    std::vector<EcPartial> parts(nth);
    for (auto& pp : parts) { pp.counts.assign(p->do_errors ? nbins : 0, 0); pp.hist.assign(1, {}); }
    parallel_chunks(tlen, nth, [&](int64_t c0, int64_t c1, int th) {
      EcPartial& P = parts[th];
      walk_columns(d, t, c0, c1, [&](int64_t c, const std::vector<uint64_t>& act) {
        size_t unique = 0;
        bool has_red = false;
        int hqs[2] = {0, 0};
        for (uint64_t r : act) {
          Pile e;
          if (!resolve(rd, r, c, e)) continue;
          if (e.is_del) continue;
          if (rd->x1[r] > 1) { has_red = true; continue; }
          ++unique;
          const ReadInfo& ri = d.info[r];
          if (p->preprocess_stage) {
            // Settings::required_junction_read_end_min_coordinate (settings.h:345-354)
            int32_t umax = (int32_t)std::floor((double)((int32_t)ri.len - (int32_t)p->unmatched_end_minimum_read_length) *
                                               p->unmatched_end_length_factor);
            uint32_t req = (umax <= 0) ? ri.len : ri.len - (uint32_t)umax;
            if (e.qpos + 1 == 1 && ri.stranded_end1 >= req) hqs[ri.rev ? 1 : 0] = 1;
          }
          if (!p->do_errors) continue;
          int er = count_events(d, r, e, c, tseq, tlen, R, Q, P.counts);
          if (er) P.err = er;
        }
        if (!has_red) {
          if (P.hist[0].size() <= unique) P.hist[0].resize(unique + 1, 0);
          P.hist[0][unique]++;
          if (p->preprocess_stage) { P.found[hqs[0]]++; P.found[hqs[1]]++; }
        }
      });
    });
    uint64_t found[2] = {0, 0};
    for (auto& P : parts) {
      if (P.err) { if (errbuf) snprintf(errbuf, errcap, "covariate outside the error table"); return P.err; }
      if (p->do_errors) for (size_t i = 0; i < nbins; i++) counts[i] += P.counts[i];
      if (hist[g].size() < P.hist[0].size()) hist[g].resize(P.hist[0].size(), 0);
      for (size_t i = 0; i < P.hist[0].size(); i++) hist[g][i] += P.hist[0][i];
      found[0] += P.found[0]; found[1] += P.found[1];
    }
    if (p->preprocess_stage && out->no_pos_hash_pr) {
      double total = (double)(found[0] + found[1]);
      out->no_pos_hash_pr[t] = (total != 0) ? (double)found[0] / total : 1.0;
    }
  }
  if (out->counts) for (size_t i = 0; i < nbins; i++) out->counts[i] = counts[i];
  for (uint32_t g = 0; g < G; g++) {
    if (out->hist_size) out->hist_size[g] = (uint32_t)hist[g].size();
    if (out->coverage_hist) {
      for (uint32_t i = 0; i < out->hist_capacity; i++)
        out->coverage_hist[(size_t)g * out->hist_capacity + i] = (i < hist[g].size()) ? hist[g][i] : 0;
      if (hist[g].size() > out->hist_capacity) { if (errbuf) snprintf(errbuf, errcap, "histogram capacity"); return BSQ_ERR_SIZE; }
    }
  }
  return BSQ_OK;
}

// counts_to_log10_prob (error_count.cpp:1005-1026) followed by the 6-significant-digit text round trip
// of write_log10_prob_table / read_log10_prob_table (error_count.cpp:629-690).
extern "C" int oracle_counts_to_log10_prob(const uint64_t* counts, uint32_t R, uint32_t Q, double* out) {
  for (uint32_t q = 0; q < Q; q++)
    for (uint32_t ref = 0; ref < 5; ref++)
      for (uint32_t rs = 0; rs < R; rs++) {
        double sum = 0;
        for (uint32_t obs = 0; obs < 5; obs++) sum += (double)counts[rs + R * (ref + 5 * (obs + 5 * q))];
        for (uint32_t obs = 0; obs < 5; obs++) {
          size_t i = rs + R * (ref + 5 * (obs + 5 * q));
          double v = log10((double)(counts[i] + 1)) - log10(sum + 1 * 5);
          char buf[64];
          snprintf(buf, sizeof buf, "%.6g", v);
          out[i] = strtod(buf, nullptr);
        }
      }
  return BSQ_OK;
}

// ============================================================================ pass 2
namespace {

struct PData {
  uint8_t obs;      // 0..4 (obs in top-strand space)
  uint8_t quality;
  int8_t strand;
  double lp[5], r[5], lpmax;
};

struct AlleleModel {
  double f[5] = {0, 0, 0, 0, 0};
  double log10_likelihood = 0;
  double sum_w[5] = {0, 0, 0, 0, 0};
  uint32_t n = 0, iterations = 0;
  double reported(int b) const {
    if (n == 0 || b < 0 || b >= 5) return 0.0;
    return (f[b] < 0.5 / (double)n) ? 0.0 : f[b];
  }
  int major() const {
    if (n == 0) return 5;
    int best = 0;
    for (int b = 1; b < 5; b++) if (f[b] > f[best]) best = b;
    return (f[best] > 0.0) ? best : 5;
  }
  int next(int excl) const {
    if (n == 0) return 5;
    double thr = 0.5 / (double)n;
    int best = 5;
    for (int b = 0; b < 5; b++) {
      if (b == excl) continue;
      if (f[b] < thr) continue;
      if (best == 5 || f[b] > f[best]) best = b;
    }
    return best;
  }
};

// The discordant-pair enter step of identify_mutations_pileup::pileup_callback
// (identify_mutations.cpp:1399-1416) ends the per-read loop (`continue`) for a read at its first
// column, insert position 0, when it is paired, mapped, not a proper pair, neither secondary nor
// supplementary, with a mapped mate, in a read group that has a DP group, and has no XP tag or an
// orientation other than FR / RF / FF.
inline bool dp_skip_at(const bsq_read_soa* rd, uint32_t n_read_groups, const int32_t* dp_group, uint64_t r,
                       int64_t col) {
  if ((int64_t)rd->pos[r] != col) return false;
  const uint16_t f = rd->flag[r];
  if (!(f & 0x1) || (f & 0x4) || (f & 0x2) || (f & (0x100 | 0x800 | 0x8))) return false;
  const uint32_t g = rd->read_group[r];
  if (!dp_group || g >= n_read_groups || dp_group[g] < 0) return false;   // dp_group_for(p, *i) < 0
  const uint8_t xp = rd->xp ? rd->xp[r] : (uint8_t)BSQ_XP_NONE;
  return xp != BSQ_XP_FR && xp != BSQ_XP_RF && xp != BSQ_XP_FF;
}

struct Pass2 {
  const Data& d;
  const bsq_im_params* p;
  std::vector<double> prob;  // pow(10, log10 table) (error_count.cpp:1032-1040)
  uint32_t R, Q;
  Pass2(const Data& dd, const bsq_im_params* pp, const double* table) : d(dd), p(pp) {
    R = p->n_read_files; Q = p->n_quality;
    prob.resize((size_t)R * 25 * Q);
    for (size_t i = 0; i < prob.size(); i++) prob[i] = pow(10, table[i]);
  }

  // fill_read_base_likelihoods (identify_mutations.cpp:3359-3384)
  void fill(PData& pd, uint32_t rs, int obs_idx, uint32_t q, int mapq) const {
    const double inc = pow(10, -(double)mapq / 10);
    const double cor = 1 - inc;
    const double uni = 1.0 / 5.0;
    const bool top = pd.strand == 1;
    int o = top ? obs_idx : compl_index(obs_idx);
    pd.lpmax = -std::numeric_limits<double>::max();
    for (int b = 0; b < 5; b++) {
      int refb = top ? b : compl_index(b);
      double pr = cor * prob[rs + R * (refb + 5 * (o + 5 * q))] + inc * uni;
      if (pr < 0.0) pr = 0.0;
      pd.lp[b] = log10(pr);
      pd.lpmax = std::max(pd.lpmax, pd.lp[b]);
    }
    for (int b = 0; b < 5; b++) pd.r[b] = pow(10, pd.lp[b] - pd.lpmax);
  }

  // fit_allele_frequencies (identify_mutations.cpp:3241-3318)
  AlleleModel fit(const std::vector<PData>& pd, const bool allowed[5]) const {
    AlleleModel m;
    m.n = (uint32_t)pd.size();
    if (m.n == 0) return m;
    uint32_t na = 0;
    for (int b = 0; b < 5; b++) if (allowed[b]) { na++; m.f[b] = 0.5; }
    if (na == 0) return m;
    for (auto& x : pd) if (x.obs < 5 && allowed[x.obs]) m.f[x.obs] += 1.0;
    double tot = 0;
    for (int b = 0; b < 5; b++) tot += m.f[b];
    for (int b = 0; b < 5; b++) m.f[b] /= tot;
    const double tol = p->polymorphism_precision_decimal;
    for (m.iterations = 1; m.iterations <= 50; m.iterations++) {
      double sw[5] = {0, 0, 0, 0, 0};
      double ll = 0;
      for (auto& x : pd) {
        double s = 0;
        for (int b = 0; b < 5; b++) if (allowed[b]) s += m.f[b] * x.r[b];
        if (s > 0.0) {
          ll += log10(s) + x.lpmax;
          for (int b = 0; b < 5; b++) if (allowed[b]) sw[b] += m.f[b] * x.r[b] / s;
        } else {
          for (int b = 0; b < 5; b++) if (allowed[b]) sw[b] += m.f[b];
        }
      }
      double md = 0;
      for (int b = 0; b < 5; b++) {
        if (!allowed[b]) continue;
        double fn = sw[b] / (double)m.n;
        md = std::max(md, fabs(fn - m.f[b]));
        m.f[b] = fn;
      }
      for (int b = 0; b < 5; b++) m.sum_w[b] = sw[b];
      m.log10_likelihood = ll;
      if (md < tol) break;
    }
    if (m.iterations > 50) m.iterations = 50;
    return m;
  }

  // variant_presence_score (identify_mutations.cpp:3329-3344)
  double presence(const std::vector<PData>& pd, const AlleleModel& full, int v) const {
    if (full.n == 0 || v >= 5) return kNaN;
    bool without[5];
    for (int b = 0; b < 5; b++) without[b] = (b != v);
    AlleleModel nf = fit(pd, without);
    return (full.log10_likelihood - nf.log10_likelihood) - p->log10_ref_length;
  }

  // profile_log10_likelihood (identify_mutations.cpp:3094-3143)
  double profile(const std::vector<PData>& pd, const AlleleModel& full, int v, double ff) const {
    if (full.n == 0 || v >= 5) return 0.0;
    double f[5], other = 0;
    for (int b = 0; b < 5; b++) if (b != v) other += full.f[b];
    for (int b = 0; b < 5; b++) {
      if (b == v) f[b] = ff;
      else f[b] = (other > 0.0) ? (1.0 - ff) * full.f[b] / other : (1.0 - ff) / 4.0;
    }
    double ll = 0;
    for (uint32_t it = 0; it < 50; it++) {
      double sw[5] = {0, 0, 0, 0, 0};
      ll = 0;
      for (auto& x : pd) {
        double s = 0;
        for (int b = 0; b < 5; b++) s += f[b] * x.r[b];
        if (s > 0.0) {
          ll += log10(s) + x.lpmax;
          for (int b = 0; b < 5; b++) sw[b] += f[b] * x.r[b] / s;
        } else {
          for (int b = 0; b < 5; b++) sw[b] += f[b];
        }
      }
      double others = 0;
      for (int b = 0; b < 5; b++) if (b != v) others += sw[b];
      double md = 0;
      for (int b = 0; b < 5; b++) {
        if (b == v) continue;
        double fn = (others > 0.0) ? (1.0 - ff) * sw[b] / others : (1.0 - ff) / 4.0;
        md = std::max(md, fabs(fn - f[b]));
        f[b] = fn;
      }
      if (md < p->polymorphism_precision_decimal) break;
    }
    return ll;
  }

  // write_RA_frequency_bounds (identify_mutations.cpp:3175-3217)
  void bounds(const std::vector<PData>& pd, const AlleleModel& am, int v, double& lower, double& upper) const {
    lower = 0.0; upper = 1.0;
    if (am.n > 0 && v < 5) {
      const double D = 0.587566;
      const double fh = am.f[v];
      const double plmax = profile(pd, am, v, fh);
      const double target = plmax - D;
      const double prec = p->polymorphism_precision_decimal;
      if (profile(pd, am, v, 0.0) >= target) lower = 0.0;
      else {
        double lo = 0.0, hi = fh;
        for (uint32_t i = 0; i < 40 && (hi - lo) > prec; i++) {
          double mid = 0.5 * (lo + hi);
          if (profile(pd, am, v, mid) >= target) hi = mid; else lo = mid;
        }
        lower = hi;
      }
      if (profile(pd, am, v, 1.0) >= target) upper = 1.0;
      else {
        double lo = fh, hi = 1.0;
        for (uint32_t i = 0; i < 40 && (hi - lo) > prec; i++) {
          double mid = 0.5 * (lo + hi);
          if (profile(pd, am, v, mid) >= target) lo = mid; else hi = mid;
        }
        upper = lo;
      }
    }
  }
};

// log-gamma based helpers for stats.cpp:2074-2078 (log_choose)
inline double log_choose(double n, double k) { return lgamma(n + 1) - lgamma(k + 1) - lgamma(n - k + 1); }

}  // namespace

// fisher_exact_test_2x2 (stats.cpp:2144-2169)
extern "C" double oracle_fisher_2x2(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  uint32_t row1 = a + b, row2 = c + d, col1 = a + c, col2 = b + d, n = row1 + row2;
  uint32_t amin = (row1 > col2) ? (row1 - col2) : 0;
  uint32_t amax = std::min(row1, col1);
  double ld = log_choose(n, row1);
  double lpo = log_choose(col1, a) + log_choose(col2, row1 - a) - ld;
  const double lre = log(1.0 + 1e-7);
  double tot = 0;
  for (uint32_t ai = amin; ai <= amax; ai++) {
    double lp = log_choose(col1, ai) + log_choose(col2, row1 - ai) - ld;
    if (lp <= lpo + lre) tot += exp(lp);
  }
  return std::min(tot, 1.0);
}

// ks_test_two_sample_less (stats.cpp:2180-2286)
extern "C" double oracle_ks_less(const double* x, uint32_t nx, const double* y, uint32_t ny) {
  if (nx == 0 || ny == 0) return kNaN;
  std::vector<std::pair<double, bool>> comb;
  comb.reserve(nx + ny);
  for (uint32_t i = 0; i < nx; i++) comb.push_back({x[i], true});
  for (uint32_t i = 0; i < ny; i++) comb.push_back({y[i], false});
  std::sort(comb.begin(), comb.end());
  uint32_t cx = 0, cy = 0, bx = 0, by = 0;
  double minz = 0; bool have = false;
  std::vector<char> boundary(nx + ny + 1, 1);
  size_t i = 0;
  while (i < comb.size()) {
    double v = comb[i].first;
    size_t gs = i;
    while (i < comb.size() && comb[i].first == v) { if (comb[i].second) cx++; else cy++; i++; }
    for (size_t k = gs + 1; k < i; k++) boundary[k] = 0;
    double z = (double)cx / nx - (double)cy / ny;
    if (!have || z < minz) { minz = z; have = true; bx = cx; by = cy; }
  }
  double stat = -minz;
  if ((double)nx * ny < 10000) {
    uint32_t m = ny, n = nx;
    int64_t thr = (int64_t)by * n - (int64_t)bx * m;
    std::vector<double> u((size_t)(m + 1) * (n + 1), 0.0);
    for (uint32_t a = 0; a <= m; a++)
      for (uint32_t b = 0; b <= n; b++) {
        double val;
        if (a == 0 && b == 0) val = 1.0;
        else val = (a > 0 ? u[(size_t)(a - 1) * (n + 1) + b] : 0.0) + (b > 0 ? u[(size_t)a * (n + 1) + b - 1] : 0.0);
        int64_t lev = (int64_t)a * n - (int64_t)b * m;
        if (boundary[a + b] && lev >= thr) val = 0.0;
        u[(size_t)a * (n + 1) + b] = val;
      }
    double allowed = u[(size_t)m * (n + 1) + n];
    double total = exp(log_choose(m + n, m));
    double pv = 1.0 - allowed / total;
    return std::min(std::max(pv, 0.0), 1.0);
  }
  double neff = ((double)nx * ny) / (nx + ny);
  return exp(-2.0 * stat * stat * neff);
}

namespace {

struct ColumnOut {   // insert position 0 of one reference column
  double unique[3], redundant[3];
  int raw_redundant[3];
  int total;
  bool base_predicted, unique_only;
  double consensus;
  uint8_t best;
  uint32_t n;
};

struct ImOut {
  std::vector<bsq_ra_record> ra;
  std::vector<bsq_mc_record> mc;
  std::vector<bsq_un_record> un;
};

// One (column, insert slot) of identify_mutations_pileup::pileup_callback (identify_mutations.cpp:1359-1910)
struct SlotScorer {
  const Pass2& P;
  const Data& d;
  SlotScorer(const Pass2& p, const Data& dd) : P(p), d(dd) {}

  // returns next_insert_count_exists
  bool score(uint32_t t, int64_t c, int insert_count, const std::vector<uint64_t>& act, const std::vector<Pile>& piles,
             char ref_base_char, ColumnOut* col, std::vector<bsq_ra_record>& ra_out, int& err) const {
    const bsq_read_soa* rd = d.rd;
    const bsq_im_params* p = P.p;
    bool next_exists = false;
    uint32_t pos_info[6][3];
    memset(pos_info, 0, sizeof pos_info);
    double cov_unique[3] = {0, 0, 0}, cov_red[3] = {0, 0, 0};
    int cov_raw[3] = {0, 0, 0};
    bool unique_only = true;
    std::vector<PData> pdata;
    double lps[5] = {0, 0, 0, 0, 0};
    for (size_t ii = 0; ii < act.size(); ii++) {
      const uint64_t r = act[ii];
      const Pile& e = piles[ii];
      const ReadInfo& ri = d.info[r];
      if (insert_count == 0 && dp_skip_at(rd, p->n_read_groups, p->dp_group, r, c)) continue;
      int indel = e.indel;
      if (indel < 0) indel = 0;
      if (e.is_del) indel = -1;
      uint8_t read_base = '.';
      bool past_base = true;
      if (indel >= insert_count) {
        int32_t qq = e.qpos + insert_count;
        if (qq < 0 || qq >= (int32_t)ri.len) { err = BSQ_ERR_DATA; return false; }
        read_base = base_at(rd, r, qq);
        past_base = false;
      }
      if (bam_is_N(read_base)) continue;
      const uint32_t red = rd->x1[r];
      const int strand = ri.rev ? -1 : 1;
      // is_trimmed (alignment.h:389-411), unsigned arithmetic as in the reference
      bool trimmed = false;
      {
        uint32_t qp1 = (uint32_t)(e.qpos + 1);
        if (rd->xl[r] >= 0 && qp1 <= (uint32_t)rd->xl[r]) trimmed = true;
        if (!trimmed && rd->xr[r] >= 0) {
          if (ri.len - qp1 + 1 <= (uint32_t)rd->xr[r]) trimmed = true;
          else if (past_base && (ri.len - qp1 == (uint32_t)rd->xr[r])) trimmed = true;
        }
      }
      if (red == 1) {
        ++cov_unique[1 + strand];
        if (indel > insert_count) next_exists = true;
      } else {
        unique_only = false;
        cov_red[1 + strand] += 1.0 / red;
        ++cov_raw[1 + strand];
      }
      if (red > 1) continue;
      if (trimmed) continue;
      // alignment_position_to_covariates (error_count.cpp:1049-1105)
      int obi = e.is_del ? -1 : std::max(e.indel, 0);
      uint8_t rb;
      {
        if (obi < insert_count) rb = '.';
        else rb = base_at(rd, r, e.qpos + insert_count);
      }
      if (bam_is_N(rb)) continue;
      int64_t qp = e.qpos;
      if (obi == -1) {
        qp += 1 - (ri.rev ? 1 : 0);
        if (qp < 0 || qp >= (int64_t)ri.len) continue;  // reference asserts here; treated as unusable
        if (bam_is_N(base_at(rd, r, qp))) continue;
      } else if (insert_count > 0) {
        int32_t mo = insert_count;
        if (obi < mo) mo = obi;
        qp += mo + 1 - (ri.rev ? 1 : 0);
        if (qp > ri.qb0e) continue;
        if (bam_is_N(base_at(rd, r, qp))) continue;
      }
      int oi = bam2index(rb);
      if (oi < 0) { err = BSQ_ERR_DATA; return false; }
      uint32_t q = qual_at(rd, r, qp);
      uint32_t rs = rd->read_file[r];
      if (q >= P.Q || rs >= P.R) { err = BSQ_ERR_DATA; return false; }
      if (q < p->base_quality_cutoff) continue;
      ++pos_info[oi][1 + strand];
      PData pd;
      pd.obs = (uint8_t)oi; pd.quality = (uint8_t)q; pd.strand = (int8_t)strand;
      P.fill(pd, rs, oi, q, rd->mapq[r]);
      for (int b = 0; b < 5; b++) lps[b] += pd.lp[b];
      pdata.push_back(pd);
    }
    cov_unique[1] = cov_unique[0] + cov_unique[2];
    cov_red[1] = cov_red[0] + cov_red[2];
    cov_raw[1] = cov_raw[0] + cov_raw[2];
    int total = (int)round(cov_unique[1]) + (int)round(cov_red[1]);

    // pure_genotype_call (identify_mutations.cpp:3398-3433)
    const uint32_t n = (uint32_t)pdata.size();
    uint8_t best = 5;
    double cscore = kNaN;
    if (n > 0) {
      int bb = 0;
      for (int b = 1; b < 5; b++) if (lps[b] > lps[bb]) bb = b;
      double off = -std::numeric_limits<double>::max();
      for (int b = 0; b < 5; b++) if (b != bb) off = std::max(off, lps[b]);
      double te = 0;
      for (int b = 0; b < 5; b++) if (b != bb) te += pow(10, lps[b] - off);
      double lte = log10(te) + off;
      best = (uint8_t)bb;
      cscore = (lps[bb] - lte) - p->log10_ref_length;
    }
    const char best_char = kBaseChars[best];
    const bool base_predicted = cscore >= p->mutation_cutoff;
    if (col) {
      for (int k = 0; k < 3; k++) { col->unique[k] = cov_unique[k]; col->redundant[k] = cov_red[k]; col->raw_redundant[k] = cov_raw[k]; }
      col->total = total; col->base_predicted = base_predicted; col->unique_only = unique_only;
      col->consensus = cscore; col->best = best; col->n = n;
    }
    int total_cov[3] = {0, 0, 0};
    for (int j = 0; j < 5; j++) { total_cov[2] += (int)pos_info[j][2]; total_cov[0] += (int)pos_info[j][0]; }

    const bool passed_cons = (best_char != ref_base_char) && !std::isnan(cscore) && cscore > 0;
    bool all[5] = {true, true, true, true, true};
    AlleleModel am = P.fit(pdata, all);
    const int ref_idx = (ref_base_char == 'N') ? 5 : char2index(ref_base_char);
    const int maj = am.major();
    const int minr = am.next(maj);
    const int var = am.next(ref_idx);
    double vscore = kNaN;
    bool passed_poly = false;
    if (var != 5) {
      vscore = P.presence(pdata, am, var);
      if (vscore >= p->polymorphism_cutoff) passed_poly = true;
    }
    if (passed_cons || passed_poly) {
      bsq_ra_record ra;
      memset(&ra, 0, sizeof ra);
      ra.tid = t; ra.position = (uint32_t)(c + 1); ra.insert_position = (uint32_t)insert_count;
      ra.ref_base = ref_base_char; ra.new_base = kBaseChars[var];
      ra.major_base = kBaseChars[maj]; ra.minor_base = kBaseChars[minr];
      ra.score = vscore; ra.consensus_score = cscore;
      for (int b = 0; b < 5; b++) ra.f[b] = am.f[b];
      ra.major_frequency = am.reported(maj);
      ra.frequency = am.reported(var);
      P.bounds(pdata, am, var, ra.frequency_lower, ra.frequency_upper);
      // annotate_polymorphism_statistics (identify_mutations.cpp:3009-3033)
      const int majc = maj, minc = minr;  // 5 == 'N': no reads carry it
      std::vector<double> mq, nq;
      for (auto& x : pdata) {
        if (x.obs == majc) mq.push_back(x.quality);
        if (x.obs == minc) nq.push_back(x.quality);
      }
      ra.ks_quality_p = 1.0;
      if (!mq.empty() && !nq.empty()) ra.ks_quality_p = oracle_ks_less(nq.data(), (uint32_t)nq.size(), mq.data(), (uint32_t)mq.size());
      ra.fisher_strand_p = oracle_fisher_2x2(pos_info[minc][2], pos_info[minc][0], pos_info[majc][2], pos_info[majc][0]);
      auto covpair = [&](int idx, int32_t out[2]) { out[0] = (int32_t)pos_info[idx][2]; out[1] = (int32_t)pos_info[idx][0]; };
      covpair(ref_idx, ra.ref_cov); covpair(var, ra.new_cov); covpair(maj, ra.major_cov); covpair(minr, ra.minor_cov);
      ra.total_cov[0] = total_cov[2]; ra.total_cov[1] = total_cov[0];
      ra.n = n;
      ra.passed_consensus = passed_cons; ra.passed_polymorphism = passed_poly;
      ra_out.push_back(ra);
    }
    return next_exists;
  }
};

}  // namespace

struct oracle_im_result { ImOut o; std::vector<ColumnOut> cols; std::vector<uint64_t> col_base; };

extern "C" int oracle_identify(const bsq_reference* ref, const bsq_read_soa* rd, const bsq_im_params* p,
                               const double* log10_table, oracle_im_result** res_out, int n_threads,
                               char* errbuf, int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  Pass2 P(d, p, log10_table);
  SlotScorer S(P, d);
  oracle_im_result* res = new oracle_im_result();
  const uint64_t total_len = ref->target_offset[ref->n_targets];
  res->cols.resize(total_len);
  int nth = std::max(1, n_threads);

  // MC / UN state (identify_mutations_pileup members; some persist across targets)
  uint32_t last_del_start = kUndef, last_del_end = kUndef, last_red_start = kUndef, last_red_end = kUndef;
  uint32_t last_un_start = kUndef;
  bool reaches_seed = false, red_zero = false;
  ColumnOut nan_col;
  for (int k = 0; k < 3; k++) { nan_col.unique[k] = kNaN; nan_col.redundant[k] = kNaN; nan_col.raw_redundant[k] = 0; }
  nan_col.total = 0;
  ColumnOut last_cov = nan_col, left_out = nan_col, left_in = nan_col;
  double prop_cut = 0, seed_cut = 0;

  auto check_deletion = [&](uint32_t t, uint32_t position, const ColumnOut& cov) {
    if (position == 1) last_cov = nan_col;
    if (cov.unique[1] <= prop_cut) {
      if (last_del_start == kUndef) { last_del_start = position; left_out = last_cov; left_in = cov; }
    }
    if (!std::isnan(cov.unique[1]) && (double)cov.total <= seed_cut) reaches_seed = true;
    if (last_del_start != kUndef && (std::isnan(cov.unique[1]) || cov.unique[1] > prop_cut)) {
      if (reaches_seed) {
        last_del_end = position - 1;
        if (last_red_end == kUndef) last_red_end = last_del_end;
        if (last_red_start == kUndef) last_red_start = last_del_start;
        bsq_mc_record mc;
        memset(&mc, 0, sizeof mc);
        mc.tid = t; mc.start = last_del_start; mc.end = last_del_end;
        mc.start_range = last_red_start - last_del_start; mc.end_range = last_del_end - last_red_end;
        mc.left_outside_cov = left_out.unique[1]; mc.left_inside_cov = left_in.unique[1];
        mc.right_inside_cov = last_cov.unique[1]; mc.right_outside_cov = cov.unique[1];
        res->o.mc.push_back(mc);
      }
      reaches_seed = false; red_zero = false;
      last_del_start = kUndef; last_del_end = kUndef; last_red_start = kUndef; last_red_end = kUndef;
    }
    if (last_del_start != kUndef) {
      if (cov.redundant[1] == 0) { red_zero = true; last_red_end = kUndef; }
      else if (cov.redundant[1] > 0) {
        if (!red_zero) last_red_start = position;
        else if (last_red_end == kUndef) last_red_end = position;
      }
    }
    last_cov = cov;
  };
  auto update_unknown = [&](uint32_t t, uint32_t position, bool base_predicted) {
    if (!base_predicted) {
      if (last_un_start == kUndef) last_un_start = position;
    } else if (last_un_start != kUndef) {
      bsq_un_record un; un.tid = t; un.start = last_un_start; un.end = position - 1;
      res->o.un.push_back(un);
      last_un_start = kUndef;
    }
  };

  for (uint32_t oi = 0; oi < ref->n_target_order; oi++) {
    const uint32_t t = ref->target_order[oi];
    const char* tseq = ref->seq + ref->target_offset[t];
    const int64_t tlen = (int64_t)(ref->target_offset[t + 1] - ref->target_offset[t]);
    const uint64_t cbase = ref->target_offset[t];
    const bool failed = p->deletion_propagation_cutoff[t] < 0.0;
    std::vector<std::vector<bsq_ra_record>> ra_parts((size_t)((tlen + 1023) / 1024) + 1);
    std::atomic<int> err(0);
    parallel_chunks(tlen, nth, [&](int64_t c0, int64_t c1, int) {
      std::vector<Pile> piles;
      std::vector<bsq_ra_record> local;
      walk_columns(d, t, c0, c1, [&](int64_t c, const std::vector<uint64_t>& act) {
        piles.resize(act.size());
        for (size_t i = 0; i < act.size(); i++) resolve(rd, act[i], c, piles[i]);
        ColumnOut& co = res->cols[cbase + c];
        int e = 0;
        if (failed) {
          // tabulate_position_coverage (identify_mutations.cpp:2218-2250): coverage only
          ColumnOut x;
          for (int k = 0; k < 3; k++) { x.unique[k] = 0; x.redundant[k] = 0; x.raw_redundant[k] = 0; }
          for (size_t i = 0; i < act.size(); i++) {
            if (piles[i].is_del) continue;
            if (bam_is_N(base_at(rd, act[i], piles[i].qpos))) continue;
            int strand = d.info[act[i]].rev ? -1 : 1;
            uint32_t red = rd->x1[act[i]];
            if (red == 1) ++x.unique[1 + strand];
            else { x.redundant[1 + strand] += 1.0 / red; ++x.raw_redundant[1 + strand]; }
          }
          x.unique[1] = x.unique[0] + x.unique[2]; x.redundant[1] = x.redundant[0] + x.redundant[2];
          x.raw_redundant[1] = x.raw_redundant[0] + x.raw_redundant[2];
          x.total = (int)round(x.unique[1]) + (int)round(x.redundant[1]);
          x.base_predicted = false; x.unique_only = true; x.consensus = kNaN; x.best = 5; x.n = 0;
          co = x;
          return;
        }
        int insert_count = -1;
        bool next = true;
        while (next) {
          ++insert_count;
          char refc = insert_count == 0 ? tseq[c] : '.';
          next = S.score(t, c, insert_count, act, piles, refc, insert_count == 0 ? &co : nullptr, local, e);
          if (e) { err = e; return; }
        }
      });
      // chunks are processed in any order; keep results keyed by chunk start
      if (!local.empty()) {
        std::vector<bsq_ra_record>& dst = ra_parts[(size_t)(c0 / 1024)];
        dst = std::move(local);
      }
    });
    if (err) { delete res; if (errbuf) snprintf(errbuf, errcap, "data outside the error table"); return err; }
    // RA items in column order
    for (auto& v : ra_parts) for (auto& x : v) res->o.ra.push_back(x);

    // sequential state machines in column order (at_target_start / per position / at_target_end)
    last_del_start = last_del_end = last_red_start = last_red_end = kUndef;
    last_un_start = kUndef;
    prop_cut = p->deletion_propagation_cutoff[t];
    seed_cut = p->deletion_seed_cutoff[t];
    if (!failed) {
      for (int64_t c = 0; c < tlen; c++) {
        const ColumnOut& co = res->cols[cbase + c];
        if (!p->skip_missing_coverage_prediction) check_deletion(t, (uint32_t)(c + 1), co);
        update_unknown(t, (uint32_t)(c + 1), co.base_predicted);
      }
    }
    if (!p->skip_missing_coverage_prediction) check_deletion(t, (uint32_t)(tlen + 1), nan_col);
    update_unknown(t, (uint32_t)(tlen + 1), true);
    if (!p->skip_missing_coverage_prediction && failed) {
      bsq_mc_record mc;
      memset(&mc, 0, sizeof mc);
      mc.tid = t; mc.start = 1; mc.end = (uint32_t)tlen; mc.start_range = 0; mc.end_range = 0;
      mc.left_outside_cov = kNaN; mc.left_inside_cov = 0.0; mc.right_inside_cov = 0.0; mc.right_outside_cov = kNaN;
      res->o.mc.push_back(mc);
    }
  }
  *res_out = res;
  return BSQ_OK;
}

extern "C" void oracle_im_counts(const oracle_im_result* r, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un) {
  *n_ra = r->o.ra.size(); *n_mc = r->o.mc.size(); *n_un = r->o.un.size();
}
extern "C" void oracle_im_copy(const oracle_im_result* r, bsq_ra_record* ra, bsq_mc_record* mc, bsq_un_record* un) {
  if (ra) std::copy(r->o.ra.begin(), r->o.ra.end(), ra);
  if (mc) std::copy(r->o.mc.begin(), r->o.mc.end(), mc);
  if (un) std::copy(r->o.un.begin(), r->o.un.end(), un);
}
extern "C" void oracle_im_positions(const oracle_im_result* r, bsq_position_arrays* pa) {
  const size_t n = r->cols.size();
  for (size_t i = 0; i < n; i++) {
    const ColumnOut& c = r->cols[i];
    if (pa->unique_top) pa->unique_top[i] = (uint32_t)c.unique[2];
    if (pa->unique_bot) pa->unique_bot[i] = (uint32_t)c.unique[0];
    if (pa->redundant_top) pa->redundant_top[i] = c.redundant[2];
    if (pa->redundant_bot) pa->redundant_bot[i] = c.redundant[0];
    if (pa->raw_redundant_top) pa->raw_redundant_top[i] = (uint32_t)c.raw_redundant[2];
    if (pa->raw_redundant_bot) pa->raw_redundant_bot[i] = (uint32_t)c.raw_redundant[0];
    if (pa->consensus_score) pa->consensus_score[i] = c.consensus;
    if (pa->best_base) pa->best_base[i] = c.best;
    if (pa->n_scored) pa->n_scored[i] = c.n;
  }
}
extern "C" void oracle_im_free(oracle_im_result* r) { delete r; }

// ============================================================================ soft-clipping tabulation
// tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666), restated over the decoded
// records with the reference's containers: tallies keyed by seq_id in std::map (which fixes the row
// order), tails packed 3 bits per base, the spanning denominator as a difference array.  Records the
// reference would walk past their own arrays (no CIGAR, no reference-consuming op, a CIGAR query
// length other than l_qseq, an alignment past the target's end) are reported as invalid instead.
namespace {

const uint32_t kScMaxConsensusBases = 21;   // soft_clipping.cpp:37

// base_to_code over BAM 4-bit codes (soft_clipping.cpp:41-50): only A/C/G/T get 0..3
inline uint32_t sc_code(uint8_t bam) {
  switch (bam) { case 1: return 0; case 2: return 1; case 4: return 2; case 8: return 3; default: return 4; }
}

// sc_position_is_testable (soft_clipping.cpp:162-169)
bool sc_testable(uint32_t p, uint32_t seq_length, uint32_t m) {
  if (seq_length == 0) return false;
  const uint32_t margin = m > 1 ? m : 1;
  if (p <= margin) return false;
  if ((uint64_t)p + margin > seq_length) return false;
  return true;
}

// compute_clipped_tail_consensus (soft_clipping.cpp:98-147)
void sc_consensus(const std::vector<uint64_t>& tails, uint32_t K, double base_fraction, std::string& cons,
                  uint32_t& agree) {
  cons.clear();
  agree = (uint32_t)tails.size();
  if (tails.empty() || base_fraction <= 0.0) return;
  cons.assign(K, 'N');
  std::vector<uint32_t> code(K, 4);
  uint32_t informative = 0;
  for (uint32_t col = 0; col < K; col++) {
    uint32_t tally[4] = {0, 0, 0, 0};
    for (uint64_t t : tails) { uint32_t c = (uint32_t)((t >> (3 * col)) & 7); if (c < 4) tally[c]++; }
    uint32_t best = 4, best_n = 0;
    for (uint32_t c = 0; c < 4; c++) if (tally[c] > best_n) { best_n = tally[c]; best = c; }
    code[col] = best;
    cons[col] = best < 4 ? "ACGT"[best] : 'N';
    if (best < 4) informative++;
  }
  if (informative == 0) { cons.clear(); agree = 0; return; }
  uint32_t required = (uint32_t)std::floor(base_fraction * (double)informative);
  if (required < 1) required = 1;
  agree = 0;
  for (uint64_t t : tails) {
    uint32_t matches = 0;
    for (uint32_t col = 0; col < K; col++) {
      if (code[col] >= 4) continue;
      if (((t >> (3 * col)) & 7) == code[col]) matches++;
    }
    if (matches >= required) agree++;
  }
}

struct ScRow { uint32_t target, position; int32_t direction; uint32_t clipped, total, agree; std::string tail; };

}  // namespace

struct oracle_sc_result { bsq_sc_summary s; std::vector<ScRow> rows; };

extern "C" int oracle_soft_clipping(const bsq_reference* ref, const bsq_read_soa* rd, const char* const* names,
                                    const bsq_sc_params* p, oracle_sc_result** res_out, char* errbuf, int errcap) {
  const uint32_t m = p->minimum_clipped_bases;
  const uint32_t T = ref->n_targets;
  std::map<std::string, uint32_t> seq_lengths, tid_of;      // soft_clipping.cpp:296-300
  for (uint32_t t = 0; t < T; t++) {
    seq_lengths[names[t]] = (uint32_t)(ref->target_offset[t + 1] - ref->target_offset[t]);
    tid_of[names[t]] = t;
  }
  std::map<std::string, std::map<uint32_t, uint32_t>> clipped_neg, clipped_pos;
  std::map<std::string, std::map<uint32_t, std::vector<uint64_t>>> tails_neg, tails_pos;
  std::map<std::string, std::vector<int32_t>> spanning_diff;
  const uint32_t K = std::min(m, kScMaxConsensusBases);
  uint64_t total_clipped = 0, total_agreeing = 0, total_tested = 0;
  for (uint64_t r = 0; r < rd->n_reads; r++) {                // soft_clipping.cpp:366-453
    if (rd->flag[r] & BSQ_FLAG_UNMAP) continue;
    if (rd->x1[r] > 1) continue;
    if (rd->xj && rd->xj[r]) continue;
    const std::string seq_id = names[rd->tid[r]];
    const uint32_t seq_length = seq_lengths[seq_id];
    if (seq_length == 0) continue;
    // bam_cigar2qlen / bam_endpos / query_start_1 / query_end_1 (alignment.cpp:248-290)
    const uint32_t* cg = rd->cigar + rd->cigar_off[r];
    const uint32_t nc = rd->n_cigar[r];
    uint64_t qlen = 0, rlen = 0;
    for (uint32_t k = 0; k < nc; k++) {
      const uint32_t op = cg[k] & 0xf, len = cg[k] >> 4;
      if (op == OP_M || op == OP_I || op == OP_S || op == OP_EQ || op == OP_X) qlen += len;
      if (op_ref(op)) rlen += len;
    }
    if (nc == 0 || rlen == 0 || qlen != rd->l_qseq[r] || (uint64_t)rd->pos[r] + rlen > seq_length) {
      if (errbuf) snprintf(errbuf, errcap, "record %llu: CIGAR does not match the read or runs past the target",
                           (unsigned long long)r);
      return BSQ_ERR_INVALID;
    }
    uint32_t qs1 = 1;
    for (uint32_t k = 0; k < nc; k++) { if ((cg[k] & 0xf) != OP_S) break; qs1 += cg[k] >> 4; }
    uint32_t qe1 = (uint32_t)qlen;
    for (uint32_t k = nc - 1; k > 0; k--) { if ((cg[k] & 0xf) != OP_S) break; qe1 -= cg[k] >> 4; }
    const uint32_t read_length = (uint32_t)qlen;
    const uint32_t lead = qs1 - 1, trail = read_length - qe1;
    const uint32_t ref_start = (uint32_t)rd->pos[r] + 1, ref_end = (uint32_t)(rd->pos[r] + rlen);
    std::vector<int32_t>& sd = spanning_diff[seq_id];
    if (sd.empty()) sd.resize(seq_length + 2, 0);
    if ((uint64_t)ref_end >= (uint64_t)ref_start + 2ull * m) {
      sd[ref_start + m] += 1;
      sd[ref_end - m + 1] -= 1;
    }
    if (lead >= m && sc_testable(ref_start, seq_length, m)) {
      clipped_neg[seq_id][ref_start]++;
      total_clipped++;
      uint64_t packed = 0;
      for (uint32_t col = 0; col < K; col++)
        packed |= (uint64_t)sc_code(base_at(rd, r, (int64_t)qs1 - 2 - col)) << (3 * col);
      tails_neg[seq_id][ref_start].push_back(packed);
    }
    if (trail >= m && sc_testable(ref_end, seq_length, m)) {
      clipped_pos[seq_id][ref_end]++;
      total_clipped++;
      uint64_t packed = 0;
      for (uint32_t col = 0; col < K; col++)
        packed |= (uint64_t)sc_code(base_at(rd, r, (int64_t)qe1 + col)) << (3 * col);
      tails_pos[seq_id][ref_end].push_back(packed);
    }
  }
  // prefix sums of the difference arrays (soft_clipping.cpp:455-490)
  std::map<std::string, std::vector<uint32_t>> spanning;
  uint64_t total_spanning = 0;
  for (auto& kv : seq_lengths) {
    auto it = spanning_diff.find(kv.first);
    if (it == spanning_diff.end()) continue;
    std::vector<int32_t>& sd = it->second;
    std::vector<uint32_t>& sp = spanning[kv.first];
    sp.assign(sd.size(), 0);
    int32_t running = 0;
    for (uint32_t q = 1; q < sd.size(); q++) {
      running += sd[q];
      sp[q] = running > 0 ? (uint32_t)running : 0;
      if (sc_testable(q, kv.second, m)) {
        total_spanning += 2ull * sp[q];
        if (sp[q] > 0) total_tested += 2;
      }
    }
  }
  // rows with their tail consensus (soft_clipping.cpp:500-545)
  oracle_sc_result* res = new oracle_sc_result();
  for (int32_t dir = -1; dir <= 1; dir += 2) {
    auto& clipped = dir < 0 ? clipped_neg : clipped_pos;
    auto& tails = dir < 0 ? tails_neg : tails_pos;
    for (auto& sk : clipped) {
      const std::vector<uint32_t>& cov = spanning[sk.first];
      for (auto& pk : sk.second) {
        ScRow row;
        row.target = tid_of[sk.first];
        row.position = pk.first;
        row.direction = dir;
        row.clipped = pk.second;
        const uint32_t read_through = pk.first < cov.size() ? cov[pk.first] : 0;
        row.total = row.clipped + read_through;
        sc_consensus(tails[sk.first][pk.first], K, p->consensus_base_fraction, row.tail, row.agree);
        if (dir < 0) std::reverse(row.tail.begin(), row.tail.end());
        total_agreeing += row.agree;
        if (read_through == 0) total_tested++;
        res->rows.push_back(row);
      }
    }
  }
  // genome-wide totals and the dispersion fit (soft_clipping.cpp:547-623)
  bsq_sc_summary& s = res->s;
  memset(&s, 0, sizeof s);
  const uint64_t total_opp = total_clipped + total_spanning;
  s.total_spanning_read_bases = total_spanning;
  s.total_clipped_read_ends = total_clipped;
  s.total_agreeing_clipped_read_ends = total_agreeing;
  s.soft_clipping_rate = total_opp > 0 ? (double)total_clipped / (double)total_opp : 0.0;
  const double p0_raw = total_opp > 0 ? (double)total_agreeing / (double)total_opp : 0.0;
  double p0 = p0_raw;
  if (p->minimum_rate > 0.0 && p0 < p->minimum_rate) p0 = p->minimum_rate;
  double S_k = 0.0, S_k2_over_n = 0.0, S_n_trimmed = 0.0;
  const double S_n = (double)total_opp;
  uint64_t trimmed = 0;
  for (const ScRow& row : res->rows) {
    if (row.total == 0) continue;
    const double k = (double)row.agree, n = (double)row.total;
    if (p->dispersion_trim_frequency > 0.0 && k / n >= p->dispersion_trim_frequency) {
      trimmed++;
      S_n_trimmed += n;
      continue;
    }
    S_k += k;
    S_k2_over_n += k * k / n;
  }
  const uint64_t N_prime = total_tested > trimmed ? total_tested - trimmed : 0;
  const double S_n_prime = S_n - S_n_trimmed;
  const double mean_n_prime = N_prime > 0 ? S_n_prime / (double)N_prime : 0.0;
  double phi = 0.0, rho = 0.0;
  if (N_prime > 1 && mean_n_prime > 1.0 && p0 > 0.0 && p0 < 1.0) {
    const double chi2 = (S_k2_over_n - 2.0 * p0 * S_k + p0 * p0 * S_n_prime) / (p0 * (1.0 - p0));
    phi = chi2 / (double)(N_prime - 1);
    rho = (phi - 1.0) / (mean_n_prime - 1.0);
  }
  const double rho_raw = rho;
  if (!std::isfinite(rho) || rho < 0.0) rho = 0.0;
  if (p->maximum_dispersion > 0.0 && rho > p->maximum_dispersion) rho = p->maximum_dispersion;
  if (rho < 1e-6) rho = 0.0;
  s.null_rate = p0;
  s.null_rate_raw = p0_raw;
  s.dispersion = rho;
  s.dispersion_raw = rho_raw;
  s.pearson_phi = phi;
  s.tested_positions = N_prime;
  s.trimmed_positions = trimmed;
  s.mean_tested_reads = mean_n_prime;
  s.n_positions = res->rows.size();
  *res_out = res;
  return BSQ_OK;
}

extern "C" void oracle_sc_summary(const oracle_sc_result* r, bsq_sc_summary* s) { *s = r->s; }
extern "C" void oracle_sc_rows(const oracle_sc_result* r, bsq_sc_position* out) {
  for (size_t i = 0; i < r->rows.size(); i++) {
    const ScRow& w = r->rows[i];
    bsq_sc_position& o = out[i];
    memset(&o, 0, sizeof o);
    o.target = w.target; o.position = w.position; o.direction = w.direction;
    o.clipped_count = w.clipped; o.total_count = w.total; o.agree_count = w.agree;
    snprintf(o.clipped_sequence, sizeof o.clipped_sequence, "%s", w.tail.c_str());
  }
}
extern "C" void oracle_sc_free(oracle_sc_result* r) { delete r; }

// ============================================================================ BAM2COV coverage table
// coverage_output::pileup_callback (src/breseq/coverage_output.cpp:307-470) over htslib's pileup of one
// region, as pileup_base::do_pileup drives it (src/breseq/pileup_base.cpp:130-133, 141-210, 308-355),
// and coverage_output::table (coverage_output.cpp:190-284).
namespace {

struct CovCol { uint32_t u[2] = {0, 0}, raw[2] = {0, 0}, beg[2] = {0, 0}; double red[2] = {0.0, 0.0}; };

int cov_columns(Data& d, uint32_t t, uint32_t start, uint32_t end, std::vector<CovCol>& cols, uint32_t& last,
                int32_t rg_only = -1) {
  const bsq_read_soa* rd = d.rd;
  cols.assign(end - start + 1, CovCol());
  // the pileup column entries in BAM order: deletions skipped, redundancy from X1
  walk_columns(d, t, (int64_t)start - 1, (int64_t)end, [&](int64_t c, const std::vector<uint64_t>& active) {
    CovCol& x = cols[c - ((int64_t)start - 1)];
    for (uint64_t r : active) {
      // --per-read-group: the entries of one read group (read_group_index, coverage_output.cpp:383)
      if (rg_only >= 0 && (int32_t)rd->read_group[r] != rg_only) continue;
      Pile e;
      if (!resolve(rd, r, c, e) || e.is_del) continue;
      const int rev = d.info[r].rev ? 1 : 0;
      const uint32_t redundancy = rd->x1[r];
      // first sequenced base: query position 1 on the top strand, read_length on the bottom
      const bool first = rev ? (e.qpos + 1 == (int32_t)d.info[r].len) : (e.qpos == 0);
      if (redundancy == 1) {
        x.u[rev]++;
        if (first) x.beg[rev]++;
      } else {
        x.raw[rev]++;
        x.red[rev] += 1.0 / redundancy;
      }
    }
  });
  // the pileup's last column: the furthest end of a kept record the region query returns
  last = 0;
  for (uint64_t r = d.tgt_begin[t]; r < d.tgt_end[t]; r++) {
    if (d.info[r].skip) continue;
    if (d.info[r].pos < (int64_t)end && d.info[r].endpos > (int64_t)start - 1)
      last = std::max<uint32_t>(last, (uint32_t)d.info[r].endpos);
  }
  return BSQ_OK;
}

std::string fmt_double(double v) {   // default ostream formatting, as the reference writes
  std::ostringstream o;
  o << v;
  return o.str();
}

}  // namespace

extern "C" int oracle_coverage_columns(const bsq_reference* ref, const bsq_read_soa* rd, uint32_t tid, uint32_t start,
                                       uint32_t end, bsq_cov_columns* out, uint32_t* last_out, char* errbuf, int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  std::vector<CovCol> cols;
  uint32_t last = 0;
  cov_columns(d, tid, start, end, cols, last);
  for (size_t i = 0; i < cols.size(); i++) {
    if (out->unique_top) out->unique_top[i] = cols[i].u[0];
    if (out->unique_bot) out->unique_bot[i] = cols[i].u[1];
    if (out->redundant_top) out->redundant_top[i] = cols[i].red[0];
    if (out->redundant_bot) out->redundant_bot[i] = cols[i].red[1];
    if (out->raw_redundant_top) out->raw_redundant_top[i] = cols[i].raw[0];
    if (out->raw_redundant_bot) out->raw_redundant_bot[i] = cols[i].raw[1];
    if (out->unique_top_begin) out->unique_top_begin[i] = cols[i].beg[0];
    if (out->unique_bot_begin) out->unique_bot_begin[i] = cols[i].beg[1];
  }
  if (last_out) *last_out = last;
  return BSQ_OK;
}

// identify_mutations' coverage tally of one read group's entries at insert position 0: the main loop
// (src/breseq/identify_mutations.cpp:1560-1610), where a deletion's read base is '.' and so counts, and an
// N read base does not; or tabulate_position_coverage (:2218-2250) for a target whose coverage fit failed,
// which skips deletions as well.  Per strand: unique count, Σ 1/X1 in pileup order, raw redundant count.
// The main loop's tally comes after the discordant-pair enter step, whose `continue` (:1399-1416) leaves
// a read out of its first column; tabulate_position_coverage has no such step.
static void im_cov_columns(Data& d, uint32_t t, uint32_t start, uint32_t end, int32_t rg_only, bool failed,
                           uint32_t n_read_groups, const int32_t* dp_group, std::vector<CovCol>& cols) {
  const bsq_read_soa* rd = d.rd;
  cols.assign(end - start + 1, CovCol());
  walk_columns(d, t, (int64_t)start - 1, (int64_t)end, [&](int64_t c, const std::vector<uint64_t>& active) {
    CovCol& x = cols[c - ((int64_t)start - 1)];
    for (uint64_t r : active) {
      if (rg_only >= 0 && (int32_t)rd->read_group[r] != rg_only) continue;   // p.read_group_index(*i)
      if (!failed && dp_skip_at(rd, n_read_groups, dp_group, r, c)) continue;
      Pile e;
      if (!resolve(rd, r, c, e)) continue;
      if (failed && e.is_del) continue;
      int indel = e.is_del ? -1 : std::max(e.indel, 0);
      uint8_t read_base = '.';
      if (indel >= 0) read_base = base_at(rd, r, e.qpos);
      if (bam_is_N(read_base)) continue;
      const int s = d.info[r].rev ? 1 : 0;
      const uint32_t redundancy = rd->x1[r];
      if (redundancy == 1) x.u[s]++;
      else { x.red[s] += 1.0 / redundancy; x.raw[s]++; }
    }
  });
}

extern "C" int oracle_im_coverage_columns(const bsq_reference* ref, const bsq_read_soa* rd, uint32_t tid,
                                          uint32_t start, uint32_t end, int32_t read_group, int coverage_fit_failed,
                                          uint32_t n_read_groups, const int32_t* dp_group,
                                          bsq_cov_columns* out, char* errbuf, int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  std::vector<CovCol> cols;
  im_cov_columns(d, tid, start, end, read_group, coverage_fit_failed != 0, n_read_groups, dp_group, cols);
  for (size_t i = 0; i < cols.size(); i++) {
    if (out->unique_top) out->unique_top[i] = cols[i].u[0];
    if (out->unique_bot) out->unique_bot[i] = cols[i].u[1];
    if (out->redundant_top) out->redundant_top[i] = cols[i].red[0];
    if (out->redundant_bot) out->redundant_bot[i] = cols[i].red[1];
    if (out->raw_redundant_top) out->raw_redundant_top[i] = cols[i].raw[0];
    if (out->raw_redundant_bot) out->raw_redundant_bot[i] = cols[i].raw[1];
    if (out->unique_top_begin) out->unique_top_begin[i] = 0;
    if (out->unique_bot_begin) out->unique_bot_begin[i] = 0;
  }
  return BSQ_OK;
}

// <seq_id>.coverage.tsv (identify_mutations.cpp:2028-2052, 2173-2216): the aggregate columns from the
// given per-position arrays (pass 2's), then, with more than one read group (:862), each group's three
// columns "RG-<g>_..." from im_cov_columns.  Strands are summed as position_coverage::sum does.
extern "C" int oracle_write_coverage_table_rg(const bsq_reference* ref, const bsq_read_soa* rd, const char* path,
                                              uint32_t tid, const bsq_position_arrays* pa, uint32_t n_read_groups,
                                              int coverage_fit_failed, const int32_t* dp_group, char* errbuf,
                                              int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  const uint64_t b = ref->target_offset[tid], len = ref->target_offset[tid + 1] - b;
  std::vector<std::vector<CovCol>> rg(n_read_groups > 1 && len ? n_read_groups : 0);
  for (uint32_t g = 0; g < rg.size(); g++)
    im_cov_columns(d, tid, 1, (uint32_t)len, (int32_t)g, coverage_fit_failed != 0, n_read_groups, dp_group, rg[g]);
  FILE* f = fopen(path, "w");
  if (!f) return BSQ_ERR_INVALID;
  const char* names[3] = {"unique_cov", "redundant_cov", "total_cov"};
  std::string line = "position\tref_base";
  for (const char* n : names) line += std::string("\t") + n;
  for (uint32_t g = 0; g < rg.size(); g++)
    for (const char* n : names) line += "\tRG-" + std::to_string(g) + "_" + n;
  fprintf(f, "%s\n", line.c_str());
  auto three = [&](std::string& l, double ut, double ub, double rt, double rb) {
    const double u = ub + ut, r = rb + rt;
    l += "\t" + fmt_double(u) + "\t" + fmt_double(r) + "\t" + fmt_double(u + r);
  };
  for (uint64_t i = 0; i < len; i++) {
    std::string l = std::to_string(i + 1) + "\t" + std::string(1, ref->seq[b + i]);
    three(l, pa->unique_top[b + i], pa->unique_bot[b + i], pa->redundant_top[b + i], pa->redundant_bot[b + i]);
    for (auto& cols : rg) three(l, cols[i].u[0], cols[i].u[1], cols[i].red[0], cols[i].red[1]);
    fprintf(f, "%s\n", l.c_str());
  }
  return fclose(f) == 0 ? BSQ_OK : BSQ_ERR_INVALID;
}

extern "C" int oracle_write_coverage_region_rg(const bsq_reference* ref, const bsq_read_soa* rd, const char* path,
                                               const char* seq_id, uint32_t tid, uint32_t start, uint32_t end,
                                               uint32_t resolution, uint32_t flags, const double* ref_average,
                                               uint32_t n_read_groups, char* errbuf, int errcap) {
  Data d; d.ref = ref; d.rd = rd;
  int rc = prepare(d);
  if (rc) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  (void)seq_id;
  std::vector<CovCol> cols;
  uint32_t last = 0;
  cov_columns(d, tid, start, end, cols, last);
  // --per-read-group: num_read_group_columns() = max(read groups, 1) (coverage_output.h:143-152)
  const uint32_t n_rg = (flags & BSQ_COV_PER_READ_GROUP) ? std::max<uint32_t>(n_read_groups, 1) : 0;
  std::vector<std::vector<CovCol>> rg_cols(n_rg);
  for (uint32_t g = 0; g < n_rg; g++) { uint32_t l2; cov_columns(d, tid, start, end, rg_cols[g], l2, (int32_t)g); }
  std::vector<double> rg_u(n_rg, 0.0), rg_r(n_rg, 0.0), rg_all(n_rg, 0.0);
  const char* refseq = ref->seq + ref->target_offset[tid];
  const bool total_only = flags & BSQ_COV_TOTAL_ONLY;
  const std::string dl = (flags & BSQ_COV_CSV) ? "," : "\t";
  // resolution -> downsampling (coverage_output.cpp:203-209) and the position filter of
  // pileup_base::handle_position (pileup_base.cpp:130-133)
  const uint32_t size = end - start + 1;
  uint32_t downsample = 1;
  if (resolution != 0) {
    downsample = (uint32_t)std::floor((double)size / (double)resolution);
    if (downsample < 1) downsample = 1;
  }
  auto handled = [&](uint32_t p) { return p >= start && p <= end && (p + start) % downsample == 0; };
  std::ostringstream o;
  o << "position" << dl << "ref_base";
  const char* names8[8] = {"unique_top_cov", "unique_bot_cov", "redundant_top_cov", "redundant_bot_cov",
                           "raw_redundant_top_cov", "raw_redundant_bot_cov", "unique_top_begin", "unique_bot_begin"};
  const char* names3[3] = {"unique_cov", "redundant_cov", "total_cov"};
  for (int c = 0; c < (total_only ? 3 : 8); c++) o << dl << (total_only ? names3[c] : names8[c]);
  for (uint32_t g = 0; g < n_rg; g++)
    for (int c = 0; c < (total_only ? 3 : 8); c++)
      o << dl << "RG-" << g << "_" << (total_only ? names3[c] : names8[c]);
  o << "\n";
  double sum_u = 0, sum_r = 0, sum_all = 0;
  uint32_t n_pos = 0;
  auto zero_row = [&](uint32_t i) {
    o << i << dl << refseq[i - 1];
    for (uint32_t c = 0; c < (total_only ? 3u : 8u) * (1 + n_rg); c++) o << dl << 0;
    o << "\n";
    n_pos++;
  };
  auto row = [&](uint32_t p) {
    CovCol x;
    if (p >= start && p <= end) x = cols[p - start];
    n_pos++;
    sum_u += x.u[0] + x.u[1];
    sum_r += x.red[0] + x.red[1];
    sum_all += x.u[0] + x.u[1] + x.red[0] + x.red[1];
    o << p << dl << refseq[p - 1] << dl;
    if (total_only) {
      o << (x.u[0] + x.u[1]) << dl << fmt_double(x.red[0] + x.red[1]) << dl
        << fmt_double(x.u[0] + x.u[1] + x.red[0] + x.red[1]);
    } else {
      o << x.u[0] << dl << x.u[1] << dl << fmt_double(x.red[0]) << dl << fmt_double(x.red[1]) << dl << x.raw[0] << dl
        << x.raw[1] << dl << x.beg[0] << dl << x.beg[1];
    }
    for (uint32_t g = 0; g < n_rg; g++) {
      CovCol y;
      if (p >= start && p <= end) y = rg_cols[g][p - start];
      if (total_only)
        o << dl << (y.u[0] + y.u[1]) << dl << fmt_double(y.red[0] + y.red[1]) << dl
          << fmt_double(y.u[0] + y.u[1] + y.red[0] + y.red[1]);
      else
        o << dl << y.u[0] << dl << y.u[1] << dl << fmt_double(y.red[0]) << dl << fmt_double(y.red[1]) << dl << y.raw[0]
          << dl << y.raw[1] << dl << y.beg[0] << dl << y.beg[1];
      rg_u[g] += y.u[0] + y.u[1];
      rg_r[g] += y.red[0] + y.red[1];
      rg_all[g] += y.u[0] + y.u[1] + y.red[0] + y.red[1];
    }
    o << "\n";
  };
  // the pileup's columns and the gaps between them: every position up to the last column is
  // visited, the handled ones print
  for (uint32_t p = 1; p <= last; p++) if (handled(p)) row(p);
  // past the last column only handled positions move the cursor, so each one first prints the
  // positions skipped since the previous one (coverage_output.cpp:318-327, pileup_base.cpp:345-351)
  uint32_t cursor = last;
  for (uint32_t q = last + 1; q <= end; q++) {
    if (!handled(q)) continue;
    for (uint32_t i = cursor + 1; i < q; i++) zero_row(i);
    row(q);
    cursor = q;
  }
  if (ref_average) o << "#" << dl << "reference_unique_average_cov" << dl << fmt_double(*ref_average) << "\n";
  o << "#" << dl << "region_unique_average_cov" << dl << fmt_double(sum_u / n_pos) << "\n";
  o << "#" << dl << "region_repeat_average_cov" << dl << fmt_double(sum_r / n_pos) << "\n";
  o << "#" << dl << "region_average_cov" << dl << fmt_double(sum_all / n_pos) << "\n";
  o << "#" << dl << "number_of_positions" << dl << n_pos << "\n";
  for (uint32_t g = 0; g < n_rg; g++) {
    const std::string pre = "RG-" + std::to_string(g) + "_";
    o << "#" << dl << pre << "region_unique_average_cov" << dl << fmt_double(rg_u[g] / n_pos) << "\n";
    o << "#" << dl << pre << "region_repeat_average_cov" << dl << fmt_double(rg_r[g] / n_pos) << "\n";
    o << "#" << dl << pre << "region_average_cov" << dl << fmt_double(rg_all[g] / n_pos) << "\n";
  }
  FILE* f = fopen(path, "w");
  if (!f) { if (errbuf) snprintf(errbuf, errcap, "cannot write %s", path); return BSQ_ERR_INVALID; }
  const std::string txt = o.str();
  fwrite(txt.data(), 1, txt.size(), f);
  fclose(f);
  return BSQ_OK;
}

// ======================================================================================= coverage fit
// The censored negative-binomial fit of a unique-only coverage histogram and its deletion-propagation
// cutoff, restated in the reference's own shape: per-bin dnbinom_mu calls, a std::function objective,
// vector vertices ordered by std::sort, the 48 restarts in sequence.
//   fit_censored_negative_binomial          src/breseq/coverage_distribution.cpp:115-319
//   fit_coverage_distribution               src/breseq/coverage_distribution.cpp:341-396
//   summary parameters                      src/breseq/coverage_distribution.cpp:566-588
//   nelder_mead_minimize                    src/breseq/stats.cpp:2289-2381
//   dnbinom_mu / qnbinom_mu / nbdtr         src/breseq/stats.h:92-100, stats.cpp:2047-2072, 982-990
//   lngamma (ALGLIB form of Cephes lgam)    src/breseq/stats.cpp:534-650
//   lgam / gamma / stirf / incbet / incbcf / incbd / pseries (Cephes 2.8)   stats.cpp:277-500, 1385-1700
namespace ofit {

const double MACHEP = 1.11022302462515654042E-16, MAXLOG = 7.09782712893383996732E2,
             MINLOG = -7.451332191019412076235E2, MAXGAM = 171.624376956302725, BIG = 4.503599627370496e15,
             BIGINV = 2.22044604925031308085e-16;

double polevl(double x, const double* c, int n) {
  double a = c[0];
  for (int i = 1; i <= n; i++) a = a * x + c[i];
  return a;
}
double p1evl(double x, const double* c, int n) {
  double a = x + c[0];
  for (int i = 1; i < n; i++) a = a * x + c[i];
  return a;
}

double lngamma(double x) {   // x > 0
  double z, p, u, q, a, b, c;
  if (x < 13) {
    z = 1; p = 0; u = x;
    while (u >= 3) { p = p - 1; u = x + p; z = z * u; }
    while (u < 2) { z = z / u; p = p + 1; u = x + p; }
    if (u == 2) return log(z);
    p = p - 2; x = x + p;
    b = -1378.25152569120859100;
    b = -38801.6315134637840924 + x * b;
    b = -331612.992738871184744 + x * b;
    b = -1162370.97492762307383 + x * b;
    b = -1721737.00820839662146 + x * b;
    b = -853555.664245765465627 + x * b;
    c = 1;
    c = -351.815701436523470549 + x * c;
    c = -17064.2106651881159223 + x * c;
    c = -220528.590553854454839 + x * c;
    c = -1139334.44367982507207 + x * c;
    c = -2532523.07177582951285 + x * c;
    c = -2018891.41433532773231 + x * c;
    p = x * b / c;
    return log(z) + p;
  }
  q = (x - 0.5) * log(x) - x + 0.91893853320467274178;
  if (x > 100000000) return q;
  p = 1 / (x * x);
  if (x >= 1000.0) return q + ((7.9365079365079365079365 * 0.0001 * p - 2.7777777777777777777778 * 0.001) * p +
                               0.0833333333333333333333) / x;
  a = 8.11614167470508450300 * 0.0001;
  a = -5.95061904284301438324 * 0.0001 + p * a;
  a = 7.93650340457716943945 * 0.0001 + p * a;
  a = -2.77777777730099687205 * 0.001 + p * a;
  a = 8.33333333333331927722 * 0.01 + p * a;
  return q + a / x;
}

const double LA[] = {8.11614167470508450300E-4, -5.95061904284301438324E-4, 7.93650340457716943945E-4,
                     -2.77777777730099687205E-3, 8.33333333333331927722E-2};
const double LB[] = {-1.37825152569120859100E3, -3.88016315134637840924E4, -3.31612992738871184744E5,
                     -1.16237097492762307383E6, -1.72173700820839662146E6, -8.53555664245765465627E5};
const double LC[] = {-3.51815701436523470549E2, -1.70642106651881159223E4, -2.20528590553854454839E5,
                     -1.13933444367982507207E6, -2.53252307177582951285E6, -2.01889141433532773231E6};
double lgam(double x) {   // x > 0
  double p, q, u, z;
  if (x < 13.0) {
    z = 1.0; p = 0.0; u = x;
    while (u >= 3.0) { p -= 1.0; u = x + p; z *= u; }
    while (u < 2.0) { z /= u; p += 1.0; u = x + p; }
    if (u == 2.0) return log(z);
    p -= 2.0; x = x + p;
    p = x * polevl(x, LB, 5) / p1evl(x, LC, 6);
    return log(z) + p;
  }
  if (x > 2.556348e305) return INFINITY;
  q = (x - 0.5) * log(x) - x + 0.91893853320467274178;
  if (x > 1.0e8) return q;
  p = 1.0 / (x * x);
  if (x >= 1000.0)
    q += ((7.9365079365079365079365e-4 * p - 2.7777777777777777777778e-3) * p + 0.0833333333333333333333) / x;
  else
    q += polevl(p, LA, 4) / x;
  return q;
}

const double GP[] = {1.60119522476751861407E-4, 1.19135147006586384913E-3, 1.04213797561761569935E-2,
                     4.76367800457137231464E-2, 2.07448227648435975150E-1, 4.94214826801497100753E-1,
                     9.99999999999999996796E-1};
const double GQ[] = {-2.31581873324120129819E-5, 5.39605580493303397842E-4, -4.45641913851797240494E-3,
                     1.18139785222060435552E-2, 3.58236398605498653373E-2, -2.34591795718243348568E-1,
                     7.14304917030273074085E-2, 1.00000000000000000320E0};
const double STIR[] = {7.87311395793093628397E-4, -2.29549961613378126380E-4, -2.68132617805781232825E-3,
                       3.47222221605458667310E-3, 8.33333333333482257126E-2};
double stirf(double x) {
  double w = 1.0 / x;
  w = 1.0 + w * polevl(w, STIR, 4);
  double y = exp(x);
  if (x > 143.01608) {
    double v = pow(x, 0.5 * x - 0.25);
    y = v * (v / y);
  } else {
    y = pow(x, x - 0.5) / y;
  }
  return 2.50662827463100050242E0 * y * w;
}
double gamma_(double x) {   // x > 0
  if (x > 33.0) return 1 * stirf(x);
  double z = 1.0;
  while (x >= 3.0) { x -= 1.0; z *= x; }
  while (x < 2.0) {
    if (x < 1.e-9) goto small;
    z /= x;
    x += 1.0;
  }
  if (x == 2.0) return z;
  x -= 2.0;
  return z * polevl(x, GP, 6) / polevl(x, GQ, 7);
small:
  if (x == 0.0) return INFINITY;
  return z / ((1.0 + 0.5772156649015329 * x) * x);
}

double incbcf(double a, double b, double x) {
  double xk, pk, pkm1, pkm2, qk, qkm1, qkm2, k1, k2, k3, k4, k5, k6, k7, k8, r, t, ans, thresh;
  int n;
  k1 = a; k2 = a + b; k3 = a; k4 = a + 1.0; k5 = 1.0; k6 = b - 1.0; k7 = k4; k8 = a + 2.0;
  pkm2 = 0.0; qkm2 = 1.0; pkm1 = 1.0; qkm1 = 1.0; ans = 1.0; r = 1.0; n = 0; thresh = 3.0 * MACHEP;
  do {
    xk = -(x * k1 * k2) / (k3 * k4);
    pk = pkm1 + pkm2 * xk; qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    xk = (x * k5 * k6) / (k7 * k8);
    pk = pkm1 + pkm2 * xk; qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    if (qk != 0) r = pk / qk;
    if (r != 0) { t = fabs((ans - r) / r); ans = r; } else t = 1.0;
    if (t < thresh) return ans;
    k1 += 1.0; k2 += 1.0; k3 += 2.0; k4 += 2.0; k5 += 1.0; k6 -= 1.0; k7 += 2.0; k8 += 2.0;
    if ((fabs(qk) + fabs(pk)) > BIG) { pkm2 *= BIGINV; pkm1 *= BIGINV; qkm2 *= BIGINV; qkm1 *= BIGINV; }
    if ((fabs(qk) < BIGINV) || (fabs(pk) < BIGINV)) { pkm2 *= BIG; pkm1 *= BIG; qkm2 *= BIG; qkm1 *= BIG; }
  } while (++n < 300);
  return ans;
}
double incbd(double a, double b, double x) {
  double xk, pk, pkm1, pkm2, qk, qkm1, qkm2, k1, k2, k3, k4, k5, k6, k7, k8, r, t, ans, z, thresh;
  int n;
  k1 = a; k2 = b - 1.0; k3 = a; k4 = a + 1.0; k5 = 1.0; k6 = a + b; k7 = a + 1.0; k8 = a + 2.0;
  pkm2 = 0.0; qkm2 = 1.0; pkm1 = 1.0; qkm1 = 1.0; z = x / (1.0 - x); ans = 1.0; r = 1.0; n = 0;
  thresh = 3.0 * MACHEP;
  do {
    xk = -(z * k1 * k2) / (k3 * k4);
    pk = pkm1 + pkm2 * xk; qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    xk = (z * k5 * k6) / (k7 * k8);
    pk = pkm1 + pkm2 * xk; qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    if (qk != 0) r = pk / qk;
    if (r != 0) { t = fabs((ans - r) / r); ans = r; } else t = 1.0;
    if (t < thresh) return ans;
    k1 += 1.0; k2 -= 1.0; k3 += 2.0; k4 += 2.0; k5 += 1.0; k6 += 1.0; k7 += 2.0; k8 += 2.0;
    if ((fabs(qk) + fabs(pk)) > BIG) { pkm2 *= BIGINV; pkm1 *= BIGINV; qkm2 *= BIGINV; qkm1 *= BIGINV; }
    if ((fabs(qk) < BIGINV) || (fabs(pk) < BIGINV)) { pkm2 *= BIG; pkm1 *= BIG; qkm2 *= BIG; qkm1 *= BIG; }
  } while (++n < 300);
  return ans;
}
double pseries(double a, double b, double x) {
  double s, t, u, v, n, t1, z, ai;
  ai = 1.0 / a; u = (1.0 - b) * x; v = u / (a + 1.0); t1 = v; t = u; n = 2.0; s = 0.0; z = MACHEP * ai;
  while (fabs(v) > z) { u = (n - b) * x / n; t *= u; v = t / (a + n); s += v; n += 1.0; }
  s += t1;
  s += ai;
  u = a * log(x);
  if ((a + b) < MAXGAM && fabs(u) < MAXLOG) {
    t = gamma_(a + b) / (gamma_(a) * gamma_(b));
    s = s * t * pow(x, a);
  } else {
    t = lgam(a + b) - lgam(a) - lgam(b) + u + log(s);
    if (t < MINLOG) s = 0.0; else s = exp(t);
  }
  return s;
}
double incbet(double aa, double bb, double xx) {
  double a, b, t, x, xc, w, y;
  int flag;
  if (aa <= 0.0 || bb <= 0.0) return 0.0;
  if ((xx <= 0.0) || (xx >= 1.0)) {
    if (xx == 0.0) return 0.0;
    if (xx == 1.0) return 1.0;
    return 0.0;
  }
  flag = 0;
  if ((bb * xx) <= 1.0 && xx <= 0.95) { t = pseries(aa, bb, xx); goto done; }
  w = 1.0 - xx;
  if (xx > (aa / (aa + bb))) { flag = 1; a = bb; b = aa; xc = xx; x = w; }
  else { a = aa; b = bb; xc = w; x = xx; }
  if (flag == 1 && (b * x) <= 1.0 && x <= 0.95) { t = pseries(a, b, x); goto done; }
  y = x * (a + b - 2.0) - (a - 1.0);
  if (y < 0.0) w = incbcf(a, b, x); else w = incbd(a, b, x) / xc;
  y = a * log(x);
  t = b * log(xc);
  if ((a + b) < MAXGAM && fabs(y) < MAXLOG && fabs(t) < MAXLOG) {
    t = pow(xc, b); t *= pow(x, a); t /= a; t *= w;
    t *= gamma_(a + b) / (gamma_(a) * gamma_(b));
    goto done;
  }
  y += t + lgam(a + b) - lgam(a) - lgam(b);
  y += log(w / a);
  if (y < MINLOG) t = 0.0; else t = exp(y);
done:
  if (flag == 1) { if (t <= MACHEP) t = 1.0 - MACHEP; else t = 1.0 - t; }
  return t;
}
double nbdtr(double k, double n, double p) { return incbet(n, k + 1, p); }
double dnbinom_mu(double k, double size, double mu) {
  double p = size / (size + mu);
  double log_pmf = lngamma(k + size) - lngamma(size) - lngamma(k + 1) + size * log(p) + k * log(1.0 - p);
  return exp(log_pmf);
}
uint32_t qnbinom_mu(double target_pr, double size, double mu) {
  double p = size / (size + mu);
  if (target_pr <= 0.0) return 0;
  uint64_t hi = 1;
  while (nbdtr((double)hi, size, p) < target_pr) hi *= 2;
  uint64_t lo = hi / 2;
  while (lo < hi) {
    uint64_t mid = lo + (hi - lo) / 2;
    if (nbdtr((double)mid, size, p) < target_pr) lo = mid + 1; else hi = mid;
  }
  return (uint32_t)lo;
}

struct NM { std::vector<double> estimate; bool converged; };
NM nelder_mead(const std::function<double(const std::vector<double>&)>& f, const std::vector<double>& init) {
  const size_t n = init.size();
  const uint32_t max_iterations = 1000;
  const double tolerance = 1e-8;
  std::vector<std::vector<double>> simplex(n + 1, init);
  for (size_t i = 0; i < n; i++) simplex[i + 1][i] += (init[i] != 0.0) ? 0.05 * fabs(init[i]) : 0.00025;
  std::vector<double> values(n + 1);
  for (size_t i = 0; i <= n; i++) values[i] = f(simplex[i]);
  bool converged = false;
  for (uint32_t iter = 0; iter < max_iterations; iter++) {
    std::vector<size_t> order(n + 1);
    for (size_t i = 0; i <= n; i++) order[i] = i;
    std::sort(order.begin(), order.end(), [&values](size_t l, size_t r) { return values[l] < values[r]; });
    std::vector<std::vector<double>> ss(n + 1);
    std::vector<double> sv(n + 1);
    for (size_t i = 0; i <= n; i++) { ss[i] = simplex[order[i]]; sv[i] = values[order[i]]; }
    simplex = ss;
    values = sv;
    if ((values[n] - values[0]) < tolerance) { converged = true; break; }
    std::vector<double> c(n, 0.0);
    for (size_t i = 0; i < n; i++) for (size_t j = 0; j < n; j++) c[j] += simplex[i][j];
    for (size_t j = 0; j < n; j++) c[j] /= (double)n;
    std::vector<double> r(n);
    for (size_t j = 0; j < n; j++) r[j] = c[j] + 1.0 * (c[j] - simplex[n][j]);
    double fr = f(r);
    if (fr < values[0]) {
      std::vector<double> e(n);
      for (size_t j = 0; j < n; j++) e[j] = c[j] + 2.0 * (r[j] - c[j]);
      double fe = f(e);
      if (fe < fr) { simplex[n] = e; values[n] = fe; } else { simplex[n] = r; values[n] = fr; }
    } else if (fr < values[n - 1]) {
      simplex[n] = r; values[n] = fr;
    } else {
      std::vector<double> k(n);
      for (size_t j = 0; j < n; j++) k[j] = c[j] + 0.5 * (simplex[n][j] - c[j]);
      double fk = f(k);
      if (fk < values[n]) { simplex[n] = k; values[n] = fk; }
      else {
        for (size_t i = 1; i <= n; i++) {
          for (size_t j = 0; j < n; j++) simplex[i][j] = simplex[0][j] + 0.5 * (simplex[i][j] - simplex[0][j]);
          values[i] = f(simplex[i]);
        }
      }
    }
  }
  size_t best = 0;
  for (size_t i = 1; i <= n; i++) if (values[i] < values[best]) best = i;
  return NM{simplex[best], converged && std::isfinite(values[best])};
}

}  // namespace ofit

extern "C" int oracle_fit_coverage_distribution(const uint64_t* hist, uint32_t hist_size, double cutoff_pr,
                                                bsq_coverage_fit* out) {
  using namespace ofit;
  memset(out, 0, sizeof(*out));
  const uint32_t N = hist_size ? hist_size - 1 : 0;
  std::vector<double> n((size_t)N + 1, 0.0);
  for (uint32_t i = 1; i <= N; i++) n[i] = (double)hist[i];
  double nb_mu = 0, nb_size = 0, m = 0, v = 0, scale = 0;
  uint32_t cs = 0, ce = 0, n_conv = 0;
  [&]() {
    double total_positions = 0;
    for (uint32_t i = 1; i <= N; i++) total_positions += n[i];
    if (total_positions == 0) return;
    for (uint32_t i = 1; i <= N; i++) m += i * n[i];
    m /= total_positions;
    if (total_positions > 1) {
      for (uint32_t i = 1; i <= N; i++) v += n[i] * (i - m) * (i - m);
      v /= (total_positions - 1);
    }
    std::vector<double> ma(N + 1, 0.0);
    std::vector<bool> ma_valid(N + 1, false);
    if (N >= 5) {
      for (uint32_t i = 3; i <= N - 2; i++) { ma[i] = (n[i - 2] + n[i - 1] + n[i] + n[i + 1] + n[i + 2]) / 5.0; ma_valid[i] = true; }
    } else {
      for (uint32_t i = 1; i <= N; i++) { ma[i] = n[i]; ma_valid[i] = true; }
    }
    uint32_t min_i = std::max((uint32_t)(m / 4.0), (uint32_t)1);
    double max_n = 0;
    uint32_t max_i = 0;
    for (uint32_t i = min_i; i <= N; i++) if (ma_valid[i] && ma[i] > max_n) { max_n = ma[i]; max_i = i; }
    uint32_t start_i = std::max((uint32_t)floor(max_i * 0.5), (uint32_t)1);
    uint32_t end_i = std::min((uint32_t)ceil(max_i * 1.5), N);
    if (start_i == end_i) return;
    cs = start_i;
    ce = end_i;
    uint32_t npb = (end_i - start_i) / 1000;
    std::vector<double> x;
    uint32_t s0, e0;
    if (npb > 1) {
      s0 = start_i / npb;
      e0 = (uint32_t)ceil((double)end_i / npb);
      x.assign(e0 + 1, 0.0);
      for (uint32_t i = s0; i <= e0; i++)
        for (uint32_t j = 1; j <= npb; j++) { uint32_t idx = i * npb + j; if (idx <= N) x[i] += n[idx]; }
    } else {
      npb = 1; s0 = start_i; e0 = end_i;
      x.assign(e0 + 1, 0.0);
      for (uint32_t i = 1; i <= e0; i++) x[i] = n[i];
    }
    double inner_total = 0;
    for (uint32_t i = s0; i <= e0; i++) inner_total += x[i];
    double num = 0, den = 0;
    for (uint32_t i = 1; i <= e0; i++) { num += i * x[i]; den += x[i]; }
    double mean_estimate = num / den;
    auto f_nb = [&](const std::vector<double>& par) -> double {
      double mu = exp(par[0]), size = exp(par[1]);
      if (!std::isfinite(mu) || !std::isfinite(size)) return 1e10;
      std::vector<double> dist(e0 + 1, 0.0);
      double total = 0;
      for (uint32_t i = s0; i <= e0; i++) { dist[i] = dnbinom_mu((double)i, size, mu); total += dist[i]; }
      if (!(total > 0) || !std::isfinite(total)) return 1e10;
      double l = 0;
      for (uint32_t i = s0; i <= e0; i++) { double d = (x[i] / inner_total) - (dist[i] / total); l += d * d; }
      return std::isfinite(l) ? l : 1e10;
    };
    std::vector<double> tm = {mean_estimate, (double)e0, (double)s0, 1.0 * (e0 + s0) / 4.0, 2.0 * (e0 + s0) / 4.0,
                              3.0 * (e0 + s0) / 4.0};
    double best = HUGE_VAL;
    for (double mean : tm) {
      double ts = 100000;
      for (int k = 0; k < 8; k++) {
        ts /= 10.0;
        NM r = nelder_mead(f_nb, {log(mean), log(ts)});
        if (!r.converged) continue;
        n_conv++;
        double obj = f_nb(r.estimate);
        if (obj < best) { best = obj; nb_mu = exp(r.estimate[0]); nb_size = exp(r.estimate[1]); }
      }
    }
    if (!(best < HUGE_VAL)) nb_mu = nb_size = 0;
    double inc = 0;
    if (nb_mu > 0) {
      double p = nb_size / (nb_size + nb_mu);
      inc = nbdtr((double)e0, nb_size, p) - nbdtr((double)s0, nb_size, p);
      if (inc >= 0.01 && npb > 1) nb_mu = nb_mu * npb;
    }
    if (inc < 0.01) nb_mu = nb_size = 0;
    if (nb_mu > 0) scale = inner_total / inc;
  }();
  double dpc;
  if (nb_mu > 0) {
    dpc = (double)qnbinom_mu(cutoff_pr, nb_size, nb_mu);
  } else {
    double se = (1.0 / (v - m)) * m * m;
    dpc = ((se > 0) && std::isfinite(se)) ? (double)qnbinom_mu(cutoff_pr, se, m) : -1;
    if (!(dpc >= 1)) dpc = m * 0.1;
  }
  if (dpc < 1) dpc = 1;
  if ((nb_mu <= 3) && (m <= 3)) dpc = -1;
  out->nbinom_size = nb_size;
  out->nbinom_mean = nb_mu;
  if (nb_mu != 0) {
    out->nbinom_prob = nb_size / (nb_mu + nb_size);
    out->nbinom_variance = nb_mu + pow(nb_mu, 2) / nb_size;
    out->nbinom_relative_variance = out->nbinom_variance / nb_mu;
  }
  out->average = m;
  out->variance = v;
  out->relative_variance = (m > 0) ? v / m : 0.0;
  out->deletion_coverage_propagation_cutoff = dpc;
  out->nbinom_scale = scale;
  out->censor_start = cs;
  out->censor_end = ce;
  out->restarts_converged = n_conv;
  return BSQ_OK;
}

extern "C" double oracle_nbinom_pmf(double k, double size, double mu) { return ofit::dnbinom_mu(k, size, mu); }
extern "C" double oracle_nbinom_cdf(double k, double size, double p) { return ofit::nbdtr(k, size, p); }
extern "C" double oracle_lgam(double x) { return ofit::lgam(x); }
extern "C" double oracle_lngamma(double x) { return ofit::lngamma(x); }
extern "C" double oracle_gamma(double x) { return ofit::gamma_(x); }

// ======================================================================================= pair scans
// The discordant-pair (DP) and missing-pair (MP) candidate-region scans, walked position by position
// as the identify_mutations pileup does:
//   groups / window widths                 src/breseq/identify_mutations.cpp:883-913
//   per-read enter steps (insert slot 0, at the read's start column)   :1395-1493
//   check_discordant_completion            :2358-2437
//   check_missing_pair_completion          :2439-2522
//   at_target_start / at_target_end        :2028-2100, :2117-2137
//   write_mp / write_dp_candidate_regions  :2524-2586
// A target whose deletion propagation cutoff is below 0 is not walked (pileup_callback returns at
// once, :1318-1329).
namespace opair {

struct DpRead { uint32_t start, end; std::string key; bool redundant; };
struct MpRead { uint32_t start, end; bool redundant; };
struct Group {
  double w;
  uint32_t r1, r2;
  std::deque<DpRead> reads[6];
  std::deque<MpRead> mp_reads[2];
  std::deque<uint32_t> mp_all[2];
};
struct DpRegion { std::string seq_id; uint32_t start, end; char strand; std::string orientation; uint32_t max_count; bool redundant; std::string pairs; };
struct MpRegion { std::string seq_id; uint32_t start, end; char strand; uint32_t max_count, max_total; bool redundant; std::string reads; };

std::string dp_desc(const DpRead& r) { return r.key + "__" + std::to_string(r.start) + "__" + std::to_string(r.end); }
std::string mp_desc(const MpRead& r) { return std::to_string(r.start) + "__" + std::to_string(r.end); }

}  // namespace opair

extern "C" int oracle_pair_candidates(const bsq_reference* ref, const bsq_read_soa* rd, const bsq_pair_params* prm,
                                      const char* const* target_names, const char* dp_path, const char* mp_path,
                                      const char* pd_path, char* errbuf, int errcap) {
  using namespace opair;
  Data d;
  d.ref = ref;
  d.rd = rd;
  int rc = prepare(d);
  if (rc != BSQ_OK) { if (errbuf) snprintf(errbuf, errcap, "%s", d.err.c_str()); return rc; }
  const uint32_t G = prm->n_dp_groups;
  std::vector<Group> groups(G);
  for (uint32_t g = 0; g < G; g++) { groups[g].w = prm->window_width[g]; groups[g].r1 = prm->r1_name_prefix[g]; groups[g].r2 = prm->r2_name_prefix[g]; }
  const bool dp_on = G > 0, mp_on = prm->predict_missing_pairs && G > 0;
  static const char* kOrientName[3] = {"FR", "RF", "FF"};
  int32_t dp_metric[6], mp_metric[2], mp_total[2];
  uint32_t dp_start[6], dp_max[6], dp_red[6], mp_start[2], mp_max[2], mp_maxt[2], mp_red[2];
  std::vector<std::string> dp_desc_v[6], mp_desc_v[2];
  std::vector<DpRegion> dp_regions;
  std::vector<MpRegion> mp_regions;
  // pair distance (identify_mutations.cpp:920-1006, 1514-1555, 2588-2757)
  const int64_t kS = 1048576;
  bool pd_usable = false;
  for (uint32_t g = 0; g < G && prm->predict_pair_distance; g++) if (prm->pd_cdf_len[g]) pd_usable = true;
  const bool pd_on = prm->predict_pair_distance && G > 0 && pd_usable && prm->pd_max_span > 0;
  const int32_t ring_w = prm->pd_max_span + 2;
  std::vector<int32_t> ring_n, ring_long, ring_short;
  std::vector<int64_t> ring_u;
  std::vector<uint64_t> z_hist;
  if (prm->predict_pair_distance && G > 0) z_hist.assign(4001, 0);
  int32_t pd_n = 0, pd_long = 0, pd_short = 0;
  int64_t pd_u = 0;
  uint32_t pd_last_b = 0;
  uint32_t pd_start[2];
  uint32_t pd_peak_pos[2];
  int32_t pd_peak_cov[2], pd_peak_tail[2];
  double pd_peak_z[2];
  bool ladder_open[2][21];
  uint64_t ladder_count[2][21] = {};
  struct PdRegion { std::string seq_id; uint32_t start, end; char direction; uint32_t peak_position; int32_t peak_covering, peak_tail; double peak_z; };
  std::vector<PdRegion> pd_regions;
  bool pd_bad = false;
  for (uint32_t oi = 0; oi < ref->n_target_order; oi++) {
    const uint32_t t = ref->target_order[oi];
    if (prm->deletion_propagation_cutoff[t] < 0.0) continue;
    const uint32_t len = (uint32_t)(ref->target_offset[t + 1] - ref->target_offset[t]);
    const std::string seq_id = target_names[t];
    // at_target_start
    for (int b = 0; b < 6; b++) {
      for (Group& g : groups) g.reads[b].clear();
      dp_metric[b] = 0; dp_start[b] = kUndef; dp_max[b] = 0; dp_red[b] = 0; dp_desc_v[b].clear();
    }
    for (int b = 0; b < 2; b++) {
      for (Group& g : groups) { g.mp_reads[b].clear(); g.mp_all[b].clear(); }
      mp_metric[b] = 0; mp_total[b] = 0; mp_start[b] = kUndef; mp_max[b] = 0; mp_maxt[b] = 0; mp_red[b] = 0;
      mp_desc_v[b].clear();
    }
    if (pd_on) {
      ring_n.assign(ring_w, 0); ring_long.assign(ring_w, 0); ring_short.assign(ring_w, 0); ring_u.assign(ring_w, 0);
      pd_n = pd_long = pd_short = 0; pd_u = 0; pd_last_b = 0;
      for (int b = 0; b < 2; b++) {
        pd_start[b] = kUndef; pd_peak_pos[b] = 0; pd_peak_cov[b] = 0; pd_peak_tail[b] = 0; pd_peak_z[b] = 0.0;
        for (int k = 0; k < 21; k++) ladder_open[b][k] = false;
      }
    }
    auto check_pd = [&](uint32_t position) {
      for (uint32_t b = pd_last_b + 1; b <= position; b++) {
        const int32_t i = (int32_t)(b % (uint32_t)ring_w);
        pd_n += ring_n[i]; ring_n[i] = 0;
        pd_long += ring_long[i]; ring_long[i] = 0;
        pd_short += ring_short[i]; ring_short[i] = 0;
        pd_u += ring_u[i]; ring_u[i] = 0;
      }
      pd_last_b = position;
      double z = 0.0;
      if (pd_n > 0) {
        double mean_offset = ((double)pd_u - (double)pd_n * (double)kS / 2.0) / (double)kS;
        z = mean_offset * sqrt(12.0 / (double)pd_n);
        if (pd_n >= 4) {
          int bin = (int)floor(z * 50) + 40 * 50;
          if (bin < 0) bin = 0;
          if (bin >= 4001) bin = 4000;
          z_hist[bin]++;
        }
      }
      for (int bin = 0; bin < 2; bin++) {
        const int32_t tail = bin == 0 ? pd_long : pd_short;
        const bool right_way = bin == 0 ? (z >= prm->pd_z_seed) : (z <= -prm->pd_z_seed);
        const bool above = (tail >= prm->pair_distance_seed) && right_way && (position <= len);
        const bool in_sequence = position <= len;
        const bool tail_ok = (tail >= prm->pair_distance_seed) && in_sequence;
        const double directed_z = bin == 0 ? z : -z;
        for (int step = 0; step < 21; step++) {
          const bool rung = tail_ok && (directed_z >= 1.0 + 0.25 * (double)step);
          if (rung) ladder_open[bin][step] = true;
          else if (ladder_open[bin][step]) { ladder_count[bin][step]++; ladder_open[bin][step] = false; }
        }
        if (above) {
          if (pd_start[bin] == kUndef) {
            pd_start[bin] = position; pd_peak_pos[bin] = position; pd_peak_cov[bin] = pd_n; pd_peak_tail[bin] = tail;
            pd_peak_z[bin] = z;
          } else if (fabs(z) > fabs(pd_peak_z[bin])) {
            pd_peak_pos[bin] = position; pd_peak_cov[bin] = pd_n; pd_peak_tail[bin] = tail; pd_peak_z[bin] = z;
          }
        } else if (pd_start[bin] != kUndef) {
          pd_regions.push_back(PdRegion{seq_id, pd_start[bin], position - 1, bin == 0 ? 'L' : 'S', pd_peak_pos[bin],
                                        pd_peak_cov[bin], pd_peak_tail[bin], pd_peak_z[bin]});
          pd_start[bin] = kUndef; pd_peak_pos[bin] = 0; pd_peak_cov[bin] = 0; pd_peak_tail[bin] = 0; pd_peak_z[bin] = 0.0;
        }
      }
    };
    auto check_dp = [&](uint32_t position) {
      for (int bin = 0; bin < 6; bin++) {
        for (Group& g : groups)
          while (!g.reads[bin].empty() && ((double)position - (double)g.reads[bin].front().start >= g.w)) {
            g.reads[bin].pop_front();
            --dp_metric[bin];
          }
        const bool above = (dp_metric[bin] >= prm->discordant_pair_seed) && (position <= len);
        if (above) {
          if (dp_start[bin] == kUndef) {
            dp_start[bin] = position;
            dp_max[bin] = (uint32_t)dp_metric[bin];
            dp_desc_v[bin].clear();
            dp_red[bin] = 0;
            for (Group& g : groups)
              for (const DpRead& r : g.reads[bin]) { dp_desc_v[bin].push_back(dp_desc(r)); if (r.redundant) ++dp_red[bin]; }
          } else if ((uint32_t)dp_metric[bin] > dp_max[bin]) {
            dp_max[bin] = (uint32_t)dp_metric[bin];
          }
        } else if (dp_start[bin] != kUndef) {
          DpRegion x;
          x.seq_id = seq_id; x.start = dp_start[bin]; x.end = position - 1;
          x.strand = (bin / 3 == 0) ? 'F' : 'R'; x.orientation = kOrientName[bin % 3]; x.max_count = dp_max[bin];
          x.redundant = (2 * dp_red[bin] > dp_desc_v[bin].size());
          for (size_t k = 0; k < dp_desc_v[bin].size(); k++) { if (k) x.pairs += ";"; x.pairs += dp_desc_v[bin][k]; }
          dp_regions.push_back(x);
          dp_start[bin] = kUndef; dp_max[bin] = 0; dp_desc_v[bin].clear(); dp_red[bin] = 0;
        }
      }
    };
    auto check_mp = [&](uint32_t position) {
      for (int bin = 0; bin < 2; bin++) {
        for (Group& g : groups) {
          while (!g.mp_reads[bin].empty() && ((double)position - (double)g.mp_reads[bin].front().start >= g.w)) {
            g.mp_reads[bin].pop_front();
            --mp_metric[bin];
          }
          while (!g.mp_all[bin].empty() && ((double)position - (double)g.mp_all[bin].front() >= g.w)) {
            g.mp_all[bin].pop_front();
            --mp_total[bin];
          }
        }
        const bool enriched = (mp_total[bin] > 0) &&
                              ((double)mp_metric[bin] >= prm->missing_pair_seed_fraction * (double)mp_total[bin]);
        const bool above = (mp_metric[bin] >= prm->missing_pair_seed) && enriched && (position <= len);
        if (above) {
          if (mp_start[bin] == kUndef) {
            mp_start[bin] = position;
            mp_max[bin] = (uint32_t)mp_metric[bin];
            mp_maxt[bin] = (uint32_t)mp_total[bin];
            mp_desc_v[bin].clear();
            mp_red[bin] = 0;
            for (Group& g : groups)
              for (const MpRead& r : g.mp_reads[bin]) { mp_desc_v[bin].push_back(mp_desc(r)); if (r.redundant) ++mp_red[bin]; }
          } else if ((uint32_t)mp_metric[bin] > mp_max[bin]) {
            mp_max[bin] = (uint32_t)mp_metric[bin];
            mp_maxt[bin] = (uint32_t)mp_total[bin];
          }
        } else if (mp_start[bin] != kUndef) {
          MpRegion x;
          x.seq_id = seq_id; x.start = mp_start[bin]; x.end = position - 1; x.strand = (bin == 0) ? 'F' : 'R';
          x.max_count = mp_max[bin]; x.max_total = mp_maxt[bin];
          x.redundant = (2 * mp_red[bin] > mp_desc_v[bin].size());
          for (size_t k = 0; k < mp_desc_v[bin].size(); k++) { if (k) x.reads += ";"; x.reads += mp_desc_v[bin][k]; }
          mp_regions.push_back(x);
          mp_start[bin] = kUndef; mp_max[bin] = 0; mp_maxt[bin] = 0; mp_desc_v[bin].clear(); mp_red[bin] = 0;
        }
      }
    };
    uint64_t r = d.tgt_begin[t];
    const uint64_t r_end = d.tgt_end[t];
    for (uint32_t position = 1; position <= len; position++) {
      // the pileup's reads that start at this column, in BAM order
      for (; r < r_end && (uint64_t)rd->pos[r] + 1 <= position; r++) {
        if ((uint64_t)rd->pos[r] + 1 < position) continue;
        const ReadInfo& ri = d.info[r];
        if (ri.skip) continue;
        const uint32_t f = rd->flag[r];
        const uint32_t rg = rd->read_group[r];
        const int gi = rg < prm->n_read_groups ? prm->dp_group[rg] : -1;
        const uint32_t end1 = (uint32_t)ri.endpos;
        const bool redundant = rd->x1[r] > 1;
        if (dp_on && (f & BSQ_FLAG_PAIRED) && !(f & BSQ_FLAG_UNMAP) && !(f & BSQ_FLAG_PROPER) &&
            !(f & (BSQ_FLAG_SECONDARY | BSQ_FLAG_SUPPLEMENTARY | BSQ_FLAG_MUNMAP)) && gi >= 0) {
          const Group& g = groups[gi];
          const int s = ri.rev ? 1 : 0;
          const int o = rd->xp[r] <= 2 ? rd->xp[r] : -1;
          if (o < 0) continue;   // no usable orientation: the rest of this read's processing is skipped
          const int bin = s * 3 + o;
          const bool focal_is_r1 = !(f & BSQ_FLAG_READ2);
          const std::string fname(rd->qname + rd->qname_off[r], rd->qname_off[r + 1] - rd->qname_off[r]);
          const size_t colon = fname.find(':');
          std::string read1_name, read2_name;
          if (colon != std::string::npos) {
            const std::string counter = fname.substr(colon + 1);
            read1_name = std::to_string(g.r1) + ":" + counter;
            read2_name = std::to_string(g.r2) + ":" + counter;
          } else {
            read1_name = focal_is_r1 ? fname : "";
            read2_name = focal_is_r1 ? "" : fname;
          }
          const int32_t r1_insert_size = focal_is_r1 ? rd->isize[r] : -rd->isize[r];
          DpRead dr{position, end1, read1_name + "__" + read2_name + "__" + std::to_string(r1_insert_size), redundant};
          groups[gi].reads[bin].push_back(dr);
          ++dp_metric[bin];
          if (dp_start[bin] != kUndef) { dp_desc_v[bin].push_back(dp_desc(dr)); if (dr.redundant) ++dp_red[bin]; }
        }
        if (mp_on && !(f & BSQ_FLAG_UNMAP) && !(f & (BSQ_FLAG_SECONDARY | BSQ_FLAG_SUPPLEMENTARY)) && gi >= 0) {
          const int bin = ri.rev ? 1 : 0;
          groups[gi].mp_all[bin].push_back(position);
          ++mp_total[bin];
          if ((f & BSQ_FLAG_PAIRED) && (f & BSQ_FLAG_MUNMAP)) {
            MpRead mr{position, end1, redundant};
            groups[gi].mp_reads[bin].push_back(mr);
            ++mp_metric[bin];
            if (mp_start[bin] != kUndef) { mp_desc_v[bin].push_back(mp_desc(mr)); if (mr.redundant) ++mp_red[bin]; }
          }
        }
        if (pd_on && (f & BSQ_FLAG_PAIRED) && !(f & BSQ_FLAG_UNMAP) &&
            !(f & (BSQ_FLAG_SECONDARY | BSQ_FLAG_SUPPLEMENTARY | BSQ_FLAG_MUNMAP)) && rd->mtid[r] == (int32_t)t &&
            rd->isize[r] > 0 && (ri.rev != ((f & BSQ_FLAG_MREVERSE) != 0)) && rd->x1[r] <= 1 && gi >= 0) {
          const uint8_t o = prm->pd_orientation[gi];
          const bool match = (o == BSQ_XP_FR) ? !ri.rev : (o == BSQ_XP_RF) ? ri.rev : true;
          if (match) {
            const int32_t d = rd->isize[r];
            const int32_t lo = (int32_t)end1, hi = rd->mpos[r] + 1 - 1;
            const uint32_t clen = prm->pd_cdf_len[gi];
            if ((hi >= lo) && clen && (d <= prm->pd_max_span)) {
              const int64_t u = ((uint32_t)d < clen) ? prm->pd_cdf[gi][d] : kS;
              const int64_t lower_tail = (int64_t)(prm->pair_distance_tail_quantile * (double)kS);
              int bin = -1;
              if (u >= kS - lower_tail) bin = 0;
              else if (u <= lower_tail) bin = 1;
              const int32_t next_b = (int32_t)pd_last_b + 1;
              if (!((lo >= next_b) && (hi + 1 <= next_b + prm->pd_max_span))) { pd_bad = true; continue; }
              const int32_t i_lo = lo % ring_w, i_hi = (hi + 1) % ring_w;
              ring_n[i_lo] += 1; ring_n[i_hi] -= 1;
              ring_u[i_lo] += u; ring_u[i_hi] -= u;
              if (bin == 0) { ring_long[i_lo] += 1; ring_long[i_hi] -= 1; }
              else if (bin == 1) { ring_short[i_lo] += 1; ring_short[i_hi] -= 1; }
            }
          }
        }
      }
      if (dp_on) check_dp(position);
      if (mp_on) check_mp(position);
      if (pd_on) check_pd(position);
    }
    if (dp_on) check_dp(len + 1);
    if (mp_on) check_mp(len + 1);
    if (pd_on) check_pd(len + 1);
  }
  if (pd_bad) { if (errbuf) snprintf(errbuf, errcap, "pair-distance ring write out of range"); return BSQ_ERR_DATA; }
  if (dp_path) {
    std::sort(dp_regions.begin(), dp_regions.end(), [](const DpRegion& a, const DpRegion& b) {
      if (a.seq_id != b.seq_id) return a.seq_id < b.seq_id;
      if (a.start != b.start) return a.start < b.start;
      if (a.strand != b.strand) return a.strand < b.strand;
      return a.orientation < b.orientation;
    });
    std::ostringstream o;
    o << "seq_id,start,end,strand,orientation,length,max_discordant_count,redundant,discordant_pairs\n";
    for (const DpRegion& x : dp_regions)
      o << x.seq_id << "," << x.start << "," << x.end << "," << x.strand << "," << x.orientation << ","
        << (x.end - x.start + 1) << "," << x.max_count << "," << (x.redundant ? 1 : 0) << "," << x.pairs << "\n";
    FILE* f = fopen(dp_path, "w");
    if (!f) return BSQ_ERR_INVALID;
    fwrite(o.str().data(), 1, o.str().size(), f);
    fclose(f);
  }
  if (pd_path) {
    // calibration (fill_pd_summary / pd_z_inflation / pd_fit_region_tail, :2758-2862), the rescan cap
    // and the file (:2864-2967)
    double infl = 1.0;
    if (!z_hist.empty()) {
      uint64_t total = 0;
      for (uint64_t h : z_hist) total += h;
      if (total >= 1000) {
        uint64_t want_lo = total / 4, want_hi = (total * 3) / 4, run = 0;
        double q_lo = 0, q_hi = 0;
        bool hl = false, hh = false;
        for (size_t i = 0; i < z_hist.size(); i++) {
          run += z_hist[i];
          double centre = ((double)i + 0.5) / 50 - 40;
          if (!hl && run >= want_lo) { q_lo = centre; hl = true; }
          if (!hh && run >= want_hi) { q_hi = centre; hh = true; break; }
        }
        if (hl && hh) { double sd = (q_hi - q_lo) / 1.34898038; if (sd > 1.0) infl = sd; }
      }
    }
    uint64_t ladder[21];
    for (int k = 0; k < 21; k++) ladder[k] = ladder_count[0][k] + ladder_count[1][k];
    bool fit_ok = false;
    double li = 0.0, sigma = 1.0, flo = 0.0, fhi = 0.0;
    if (pd_on) {
      uint64_t maxc = 0;
      for (int k = 0; k < 21; k++) maxc = std::max(maxc, ladder[k]);
      double sw = 0, swx = 0, swy = 0, swxx = 0, swxy = 0;
      int rungs = 0;
      double lo_t = 0, hi_t = 0;
      for (int k = 0; k < 21; k++) {
        if (ladder[k] < 20) continue;
        if (ladder[k] * 3 > maxc) continue;
        double t = 1.0 + 0.25 * (double)k, x = t * t, y = log((double)ladder[k]), w = (double)ladder[k];
        sw += w; swx += w * x; swy += w * y; swxx += w * x * x; swxy += w * x * y;
        if (rungs == 0) lo_t = t;
        hi_t = t;
        rungs++;
      }
      flo = lo_t; fhi = hi_t;
      if (rungs >= 3) {
        double denom = sw * swxx - swx * swx;
        if (fabs(denom) > 0.0) {
          double slope = (sw * swxy - swx * swy) / denom, intercept = (swy - slope * swx) / sw;
          if (slope < 0.0) {
            double sg = sqrt(-1.0 / (2.0 * slope));
            if (sg > 0.0 && std::isfinite(sg)) { fit_ok = true; li = intercept; sigma = sg; }
          }
        }
      }
    }
    double seed_z = prm->pd_z_seed, capped = seed_z;
    for (int k = 0; k < 21; k++) {
      double t = 1.0 + 0.25 * (double)k;
      if (t < seed_z) continue;
      capped = t;
      if (ladder[k] <= 3000) break;
    }
    if (capped > seed_z) {
      std::vector<PdRegion> kept;
      for (const PdRegion& x : pd_regions) if (fabs(x.peak_z) >= capped) kept.push_back(x);
      pd_regions.swap(kept);
      seed_z = capped;
    }
    std::sort(pd_regions.begin(), pd_regions.end(), [](const PdRegion& a, const PdRegion& b) {
      if (a.seq_id != b.seq_id) return a.seq_id < b.seq_id;
      if (a.start != b.start) return a.start < b.start;
      return a.direction < b.direction;
    });
    const double gap = prm->pd_mean_covering_gap;
    std::ostringstream o;
    o << std::fixed << std::setprecision(6);
    o << "#mean_covering_gap=" << gap << "\n";
    o << "#n_effective_tests=" << (gap > 0.0 ? (double)prm->total_reference_length / gap : 0.0) << "\n";
    o << "#seed_z=" << seed_z << "\n";
    o << "#z_iqr_inflation=" << infl << "\n";
    o << "#region_tail_fit_ok=" << (fit_ok ? 1 : 0) << "\n";
    o << "#region_tail_log_intercept=" << (fit_ok ? li : 0.0) << "\n";
    o << "#region_tail_sigma=" << (fit_ok ? sigma : 1.0) << "\n";
    o << "#region_tail_fit_lo=" << (pd_on ? flo : 0.0) << "\n";
    o << "#region_tail_fit_hi=" << (pd_on ? fhi : 0.0) << "\n";
    o << "#region_ladder=";
    for (int k = 0; k < 21; k++) { if (k) o << ";"; o << std::setprecision(2) << (1.0 + 0.25 * (double)k) << ":" << ladder[k]; }
    o << "\n";
    o << "seq_id,start,end,direction,length,peak_position,peak_covering_count,peak_tail_count,peak_z\n";
    o << std::setprecision(4);
    for (const PdRegion& x : pd_regions)
      o << x.seq_id << "," << x.start << "," << x.end << "," << x.direction << "," << (x.end - x.start + 1) << ","
        << x.peak_position << "," << x.peak_covering << "," << x.peak_tail << "," << x.peak_z << "\n";
    FILE* f = fopen(pd_path, "w");
    if (!f) return BSQ_ERR_INVALID;
    fwrite(o.str().data(), 1, o.str().size(), f);
    fclose(f);
  }
  if (mp_path) {
    std::sort(mp_regions.begin(), mp_regions.end(), [](const MpRegion& a, const MpRegion& b) {
      if (a.seq_id != b.seq_id) return a.seq_id < b.seq_id;
      if (a.start != b.start) return a.start < b.start;
      return a.strand < b.strand;
    });
    std::ostringstream o;
    o << "seq_id,start,end,strand,length,max_unpaired_count,max_window_total_count,redundant,unpaired_reads\n";
    for (const MpRegion& x : mp_regions)
      o << x.seq_id << "," << x.start << "," << x.end << "," << x.strand << "," << (x.end - x.start + 1) << ","
        << x.max_count << "," << x.max_total << "," << (x.redundant ? 1 : 0) << "," << x.reads << "\n";
    FILE* f = fopen(mp_path, "w");
    if (!f) return BSQ_ERR_INVALID;
    fwrite(o.str().data(), 1, o.str().size(), f);
    fclose(f);
  }
  return BSQ_OK;
}

extern "C" int oracle_write_coverage_region(const bsq_reference* ref, const bsq_read_soa* rd, const char* path,
                                            const char* seq_id, uint32_t tid, uint32_t start, uint32_t end,
                                            uint32_t resolution, uint32_t flags, const double* ref_average,
                                            char* errbuf, int errcap) {
  return oracle_write_coverage_region_rg(ref, rd, path, seq_id, tid, start, end, resolution,
                                         flags & ~(uint32_t)BSQ_COV_PER_READ_GROUP, ref_average, 0, errbuf, errcap);
}
