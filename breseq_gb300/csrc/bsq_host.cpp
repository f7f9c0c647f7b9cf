// Host-side steps around the scoring kernels: the error-table text round trip, the likelihood class
// table, RA assembly with the Fisher strand and K-S quality tests, and the MC / UN interval state
// machines, which are sequential over positions and run on the per-column arrays the kernels return.
#include "bsq_host.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>

namespace bsq {
namespace host {

static const double kNaN = std::numeric_limits<double>::quiet_NaN();
static const uint32_t kUndef = 0xFFFFFFFFu;
static const char kChars[6] = {'A', 'C', 'G', 'T', '.', 'N'};

// printf("%.6g") followed by strtod, without the text: for |x| in [1e-17, 1e6) the six significant
// digits are m = round(|x| * 10^k) with k = 5 - floor(log10|x|) and 10^k exact, and the parsed value is
// the correctly rounded quotient m / 10^k, which one IEEE division gives.  The product |x| * 10^k is
// within one ulp of exact, so a fraction within 1e-7 of one half (a possible tie or misrounding), an
// exponent estimate that lands outside [1e5, 1e6), and every other case take the text route.
static double round_sig6_text(double x) {
  char txt[48];
  snprintf(txt, sizeof txt, "%.6g", x);
  return strtod(txt, nullptr);
}
double round_sig6(double x) {
  static const double p10[23] = {1e0, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10, 1e11,
                                 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
  const double ax = fabs(x);
  if (!(ax >= 1e-17 && ax < 1e6)) return round_sig6_text(x);
  const int k = 5 - (int)floor(log10(ax));
  if (k < 0 || k > 22) return round_sig6_text(x);
  const double y = ax * p10[k];
  if (!(y >= 100000.0 && y < 999999.5)) return round_sig6_text(x);
  const double fl = floor(y), fr = y - fl;
  if (fabs(fr - 0.5) < 1e-7) return round_sig6_text(x);
  const double m = fr > 0.5 ? fl + 1.0 : fl;
  const double v = m / p10[k];
  return x < 0 ? -v : v;
}

void counts_to_log10_prob(const uint64_t* counts, uint32_t R, uint32_t Q, double* out) {
  for (uint32_t q = 0; q < Q; q++)
    for (uint32_t ref = 0; ref < 5; ref++)
      for (uint32_t rs = 0; rs < R; rs++) {
        const size_t base = rs + (size_t)R * ref + (size_t)R * 25 * q;
        double total = 0;
        for (uint32_t obs = 0; obs < 5; obs++) total += (double)counts[base + (size_t)R * 5 * obs];
        const double denom = log10(total + 5.0);
        for (uint32_t obs = 0; obs < 5; obs++) {
          const size_t i = base + (size_t)R * 5 * obs;
          out[i] = round_sig6(log10((double)(counts[i] + 1)) - denom);
        }
      }
}

void build_class_table(const double* tab, uint32_t R, uint32_t Q, const std::vector<uint8_t>& mapq_values,
                       ClassTableHost& o) {
  const uint32_t M = (uint32_t)mapq_values.size();
  o.K = M * R * 2 * Q * 5;
  o.lp64.assign((size_t)o.K * 5, 0);
  o.r64.assign((size_t)o.K * 5, 0);
  o.lpmax64.assign(o.K, 0);
  o.lp32.assign((size_t)(o.K + 1) * 8, 0);    // entry K: all zeros (a base the column pass does not score)
  std::vector<double> prob((size_t)R * 25 * Q);
  for (size_t i = 0; i < prob.size(); i++) prob[i] = pow(10, tab[i]);
  auto compl_idx = [](uint32_t b) -> uint32_t { return b < 4 ? 3 - b : 4; };
  for (uint32_t m = 0; m < M; m++) {
    const double inc = pow(10, -(double)mapq_values[m] / 10);
    const double cor = 1 - inc;
    const double uni = 1.0 / 5.0;
    for (uint32_t rs = 0; rs < R; rs++)
      for (uint32_t sb = 0; sb < 2; sb++)
        for (uint32_t q = 0; q < Q; q++)
          for (uint32_t obs = 0; obs < 5; obs++) {
            const uint32_t k = (((m * R + rs) * 2 + sb) * Q + q) * 5 + obs;
            const bool top = sb == 0;
            const uint32_t oc = top ? obs : compl_idx(obs);
            double lp[5], mx = -std::numeric_limits<double>::max();
            for (uint32_t b = 0; b < 5; b++) {
              const uint32_t rb = top ? b : compl_idx(b);
              double pr = cor * prob[rs + (size_t)R * (rb + 5 * (oc + 5 * (size_t)q))] + inc * uni;
              if (pr < 0.0) pr = 0.0;
              lp[b] = log10(pr);
              mx = std::max(mx, lp[b]);
            }
            for (uint32_t b = 0; b < 5; b++) {
              o.lp64[(size_t)k * 5 + b] = lp[b];
              o.r64[(size_t)k * 5 + b] = pow(10, lp[b] - mx);
              o.lp32[(size_t)k * 8 + b] = (float)lp[b];
            }
            o.lpmax64[k] = mx;
            // bit r: the column pass's screen bound takes this base at a column whose reference
            // base is r (0..4, 5 = none): its base is not r, or not its own most likely hypothesis
            uint32_t screen = 0;
            for (uint32_t r = 0; r < 6; r++)
              if (obs != r || lp[obs] < mx) screen |= 1u << r;
            memcpy(&o.lp32[(size_t)k * 8 + 5], &screen, 4);
          }
  }
}

// lgamma_r: the reentrant form (lgamma writes the global signgam), so batches assemble in parallel
static double lg(double x) { int sign; return lgamma_r(x, &sign); }
static double log_choose(double n, double k) { return lg(n + 1) - lg(k + 1) - lg(n - k + 1); }

double fisher_2x2(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  const uint32_t row1 = a + b, row2 = c + d, col1 = a + c, col2 = b + d, n = row1 + row2;
  const uint32_t lo = (row1 > col2) ? row1 - col2 : 0, hi = std::min(row1, col1);
  const double denom = log_choose(n, row1);
  const double obs = log_choose(col1, a) + log_choose(col2, row1 - a) - denom;
  const double slack = log(1.0 + 1e-7);
  double p = 0;
  for (uint32_t x = lo; x <= hi; x++) {
    const double lp = log_choose(col1, x) + log_choose(col2, row1 - x) - denom;
    if (lp <= obs + slack) p += exp(lp);
  }
  return std::min(p, 1.0);
}

double ks_less_hist(const uint32_t* xh, const uint32_t* yh, uint32_t bins) {
  uint32_t nx = 0, ny = 0;
  for (uint32_t q = 0; q < bins; q++) { nx += xh[q]; ny += yh[q]; }
  if (nx == 0 || ny == 0) return kNaN;
  // walk distinct values; positions inside a run of equal values are not checkpoints
  std::vector<char> boundary(nx + ny + 1, 1);
  uint32_t cx = 0, cy = 0, bx = 0, by = 0, consumed = 0;
  double minz = 0;
  bool have = false;
  for (uint32_t q = 0; q < bins; q++) {
    const uint32_t g = xh[q] + yh[q];
    if (!g) continue;
    for (uint32_t k = consumed + 1; k < consumed + g; k++) boundary[k] = 0;
    consumed += g;
    cx += xh[q]; cy += yh[q];
    const double z = (double)cx / nx - (double)cy / ny;
    if (!have || z < minz) { minz = z; have = true; bx = cx; by = cy; }
  }
  const double stat = -minz;
  if ((double)nx * ny < 10000) {
    const uint32_t m = ny, n = nx;
    const int64_t thr = (int64_t)by * n - (int64_t)bx * m;
    std::vector<double> row(n + 1, 0.0);
    for (uint32_t i = 0; i <= m; i++)
      for (uint32_t j = 0; j <= n; j++) {
        double v;
        if (i == 0 && j == 0) v = 1.0;
        else v = (i > 0 ? row[j] : 0.0) + (j > 0 ? row[j - 1] : 0.0);
        if (boundary[i + j] && (int64_t)i * n - (int64_t)j * m >= thr) v = 0.0;
        row[j] = v;
      }
    const double p = 1.0 - row[n] / exp(log_choose(m + n, m));
    return std::min(std::max(p, 0.0), 1.0);
  }
  const double neff = ((double)nx * ny) / (nx + ny);
  return exp(-2.0 * stat * stat * neff);
}

static void col_to_target(const SampleLayout& L, uint32_t col, uint32_t& tid, uint32_t& pos0) {
  const std::vector<uint32_t>& tp = *L.tpoff;
  uint32_t t = (uint32_t)(std::upper_bound(tp.begin(), tp.end(), col) - tp.begin()) - 1;
  tid = t;
  pos0 = col - tp[t];
}

void assemble_ra(const std::vector<RaDev>& ra, const std::vector<uint32_t>& qh, uint32_t Qh, const SampleLayout& L,
                 std::vector<bsq_ra_record>& out) {
  std::vector<uint32_t> idx(ra.size());
  for (uint32_t i = 0; i < idx.size(); i++) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (ra[a].col != ra[b].col) return ra[a].col < ra[b].col;
    return ra[a].insert_position < ra[b].insert_position;
  });
  // emit in pileup (target) order, column order within a target
  std::vector<uint32_t> rank(L.tpoff->size(), 0);
  for (uint32_t i = 0; i < L.order->size(); i++) rank[(*L.order)[i]] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    uint32_t ta, tb, pa, pb;
    col_to_target(L, ra[a].col, ta, pa);
    col_to_target(L, ra[b].col, tb, pb);
    return rank[ta] < rank[tb];
  });
  out.clear();
  out.reserve(ra.size());
  for (uint32_t i : idx) {
    const RaDev& d = ra[i];
    bsq_ra_record r;
    memset(&r, 0, sizeof r);
    uint32_t tid, pos0;
    col_to_target(L, d.col, tid, pos0);
    r.tid = tid; r.position = pos0 + 1; r.insert_position = d.insert_position;
    r.ref_base = kChars[d.ref_idx]; r.new_base = kChars[d.var_idx];
    r.major_base = kChars[d.maj_idx]; r.minor_base = kChars[d.min_idx];
    r.score = d.score; r.consensus_score = d.consensus_score;
    for (int b = 0; b < 5; b++) r.f[b] = d.f[b];
    auto reported = [&](int b) -> double {
      if (d.n == 0 || b >= 5) return 0.0;
      return (d.f[b] < 0.5 / (double)d.n) ? 0.0 : d.f[b];
    };
    r.major_frequency = reported(d.maj_idx);
    r.frequency = reported(d.var_idx);
    r.frequency_lower = d.lower; r.frequency_upper = d.upper;
    auto cov = [&](int b, int32_t o[2]) {
      if (b < 5) { o[0] = (int32_t)d.pos_info[b][0]; o[1] = (int32_t)d.pos_info[b][1]; }
      else { o[0] = 0; o[1] = 0; }
    };
    cov(d.ref_idx, r.ref_cov); cov(d.var_idx, r.new_cov); cov(d.maj_idx, r.major_cov); cov(d.min_idx, r.minor_cov);
    for (int b = 0; b < 5; b++) { r.total_cov[0] += (int32_t)d.pos_info[b][0]; r.total_cov[1] += (int32_t)d.pos_info[b][1]; }
    // annotate_polymorphism_statistics (identify_mutations.cpp:3009-3033)
    uint32_t mt = 0, mb = 0, nt = 0, nb = 0;
    if (d.maj_idx < 5) { mt = d.pos_info[d.maj_idx][0]; mb = d.pos_info[d.maj_idx][1]; }
    if (d.min_idx < 5) { nt = d.pos_info[d.min_idx][0]; nb = d.pos_info[d.min_idx][1]; }
    const uint32_t* maj_q = qh.data() + (size_t)i * 2 * Qh;
    const uint32_t* min_q = maj_q + Qh;
    uint32_t nmaj = 0, nmin = 0;
    for (uint32_t q = 0; q < Qh; q++) { nmaj += maj_q[q]; nmin += min_q[q]; }
    r.ks_quality_p = (nmaj && nmin && d.maj_idx < 5 && d.min_idx < 5) ? ks_less_hist(min_q, maj_q, Qh) : 1.0;
    r.fisher_strand_p = fisher_2x2(nt, nb, mt, mb);
    r.n = d.n;
    r.passed_consensus = d.passed_cons; r.passed_polymorphism = d.passed_poly;
    out.push_back(r);
  }
}

namespace {
struct Cov1 { double unique1, red1; int total; };

// check_deletion_completion / update_unknown_intervals / at_target_end of identify_mutations_pileup
// (identify_mutations.cpp:2107-2164, 2262-2344, 2972-3007).  Some of the state deliberately carries
// over from one target to the next, as it does there.
struct IntervalMachine {
  const bsq_im_params* p;
  std::vector<bsq_mc_record>& mc;
  std::vector<bsq_un_record>& un;
  uint32_t del_start = kUndef, del_end = kUndef, red_start = kUndef, red_end = kUndef, un_start = kUndef;
  bool reaches_seed = false, red_zero = false;
  Cov1 nan_cov = {kNaN, kNaN, 0};
  Cov1 last = nan_cov, left_out = nan_cov, left_in = nan_cov;
  double prop = 0, seed = 0;

  IntervalMachine(const bsq_im_params* pp, std::vector<bsq_mc_record>& m, std::vector<bsq_un_record>& u) : p(pp), mc(m), un(u) {}

  void check(uint32_t t, uint32_t position, const Cov1& c) {
    if (position == 1) last = nan_cov;
    if (c.unique1 <= prop && del_start == kUndef) { del_start = position; left_out = last; left_in = c; }
    if (!std::isnan(c.unique1) && (double)c.total <= seed) reaches_seed = true;
    if (del_start != kUndef && (std::isnan(c.unique1) || c.unique1 > prop)) {
      if (reaches_seed) {
        del_end = position - 1;
        if (red_end == kUndef) red_end = del_end;
        if (red_start == kUndef) red_start = del_start;
        bsq_mc_record m;
        memset(&m, 0, sizeof m);
        m.tid = t; m.start = del_start; m.end = del_end;
        m.start_range = red_start - del_start; m.end_range = del_end - red_end;
        m.left_outside_cov = left_out.unique1; m.left_inside_cov = left_in.unique1;
        m.right_inside_cov = last.unique1; m.right_outside_cov = c.unique1;
        mc.push_back(m);
      }
      reaches_seed = false; red_zero = false;
      del_start = del_end = red_start = red_end = kUndef;
    }
    if (del_start != kUndef) {
      if (c.red1 == 0) { red_zero = true; red_end = kUndef; }
      else if (c.red1 > 0) {
        if (!red_zero) red_start = position;
        else if (red_end == kUndef) red_end = position;
      }
    }
    last = c;
  }
  void unknown(uint32_t t, uint32_t position, bool predicted) {
    if (!predicted) {
      if (un_start == kUndef) un_start = position;
    } else if (un_start != kUndef) {
      bsq_un_record u; u.tid = t; u.start = un_start; u.end = position - 1;
      un.push_back(u);
      un_start = kUndef;
    }
  }
  void target_start(uint32_t t) {
    del_start = del_end = red_start = red_end = kUndef;
    un_start = kUndef;
    prop = p->deletion_propagation_cutoff[t];
    seed = p->deletion_seed_cutoff[t];
  }
  void position(uint32_t t, uint32_t pos1, const ColCov& cv, const ColCall& cl) {
    Cov1 c;
    c.unique1 = (double)cv.uniq_bot + (double)cv.uniq_top;
    c.red1 = cv.red_bot + cv.red_top;
    c.total = (int)std::round(c.unique1) + (int)std::round(c.red1);
    if (!p->skip_missing_coverage_prediction) check(t, pos1, c);
    unknown(t, pos1, (cl.flags & kBasePredicted) != 0);
  }
  void target_end(uint32_t t, uint32_t len, bool failed) {
    if (!p->skip_missing_coverage_prediction) check(t, len + 1, nan_cov);
    unknown(t, len + 1, true);
    if (!p->skip_missing_coverage_prediction && failed) {
      bsq_mc_record m;
      memset(&m, 0, sizeof m);
      m.tid = t; m.start = 1; m.end = len;
      m.left_outside_cov = kNaN; m.left_inside_cov = 0.0; m.right_inside_cov = 0.0; m.right_outside_cov = kNaN;
      mc.push_back(m);
    }
  }
};
}  // namespace

void intervals(const std::vector<ColCov>& cov, const std::vector<ColCall>& call, const SampleLayout& L,
               const bsq_im_params* p, std::vector<bsq_mc_record>& mc, std::vector<bsq_un_record>& un) {
  IntervalMachine M(p, mc, un);
  const std::vector<uint32_t>& tp = *L.tpoff;
  for (uint32_t t : *L.order) {
    const uint32_t len = tp[t + 1] - tp[t] - 1;
    const bool failed = p->deletion_propagation_cutoff[t] < 0.0;
    M.target_start(t);
    if (!failed)
      for (uint32_t i = 0; i < len; i++) M.position(t, i + 1, cov[tp[t] + i], call[tp[t] + i]);
    M.target_end(t, len, failed);
  }
}

void intervals_sparse(const std::vector<uint32_t>& cols, const std::vector<ColCov>& cov, const std::vector<ColCall>& call,
                      const SampleLayout& L, const bsq_im_params* p, std::vector<bsq_mc_record>& mc,
                      std::vector<bsq_un_record>& un) {
  IntervalMachine M(p, mc, un);
  const std::vector<uint32_t>& tp = *L.tpoff;
  for (uint32_t t : *L.order) {
    const uint32_t len = tp[t + 1] - tp[t] - 1;
    const bool failed = p->deletion_propagation_cutoff[t] < 0.0;
    M.target_start(t);
    if (!failed) {
      auto it = std::lower_bound(cols.begin(), cols.end(), tp[t]);
      for (; it != cols.end() && *it < tp[t] + len; ++it) {
        const size_t k = (size_t)(it - cols.begin());
        M.position(t, *it - tp[t] + 1, cov[k], call[k]);
      }
    }
    M.target_end(t, len, failed);
  }
}

void fill_positions(const std::vector<ColCov>& cov, const std::vector<ColCall>& call, const SampleLayout& L,
                    bsq_position_arrays* o) {
  const std::vector<uint32_t>& tp = *L.tpoff;
  const std::vector<uint64_t>& to = *L.toff;
  for (size_t t = 0; t + 1 < tp.size(); t++) {
    const uint32_t len = tp[t + 1] - tp[t] - 1;
    for (uint32_t i = 0; i < len; i++) {
      const ColCov& cv = cov[tp[t] + i];
      const ColCall& cl = call[tp[t] + i];
      const uint64_t g = to[t] + i;
      if (o->unique_top) o->unique_top[g] = cv.uniq_top;
      if (o->unique_bot) o->unique_bot[g] = cv.uniq_bot;
      if (o->redundant_top) o->redundant_top[g] = cv.red_top;
      if (o->redundant_bot) o->redundant_bot[g] = cv.red_bot;
      if (o->raw_redundant_top) o->raw_redundant_top[g] = cv.rawred_top;
      if (o->raw_redundant_bot) o->raw_redundant_bot[g] = cv.rawred_bot;
      if (o->consensus_score) o->consensus_score[g] = cl.score;
      if (o->best_base) o->best_base[g] = cl.best;
      if (o->n_scored) o->n_scored[g] = cl.n;
    }
  }
}

void sc_assemble(const ScRowDev* rows, const ScOutDev* outs, uint64_t rows_neg, uint64_t rows_pos,
                 const std::vector<uint32_t>& tpoff, const std::vector<uint32_t>& name_order, uint32_t K,
                 const bsq_sc_params& p, uint64_t total_clipped, uint64_t total_spanning, uint64_t tested_spanning,
                 std::vector<bsq_sc_position>& out, bsq_sc_summary& s) {
  out.clear();
  out.reserve(rows_neg + rows_pos);
  uint64_t total_agreeing = 0, tested = tested_spanning;
  for (int dir = -1; dir <= 1; dir += 2) {
    const ScRowDev* R = dir < 0 ? rows : rows + rows_neg;
    const ScOutDev* O = dir < 0 ? outs : outs + rows_neg;
    const uint64_t n = dir < 0 ? rows_neg : rows_pos;
    for (uint32_t t : name_order) {
      const uint32_t c0 = tpoff[t], c1 = tpoff[t + 1];
      uint64_t i = std::lower_bound(R, R + n, c0, [](const ScRowDev& r, uint32_t c) { return r.col < c; }) - R;
      for (; i < n && R[i].col < c1; i++) {
        bsq_sc_position w;
        memset(&w, 0, sizeof w);
        w.target = t;
        w.position = R[i].col - c0 + 1;
        w.direction = dir;
        w.clipped_count = R[i].clipped;
        w.total_count = R[i].clipped + R[i].read_through;
        w.agree_count = O[i].agree;
        if (O[i].informative > 0) {
          // columns run outward from the clip wall; a leading clip's tail is stored reference-forward
          for (uint32_t k = 0; k < K; k++) {
            const uint32_t code = (uint32_t)(O[i].cons >> (3 * k)) & 7u;
            w.clipped_sequence[dir < 0 ? K - 1 - k : k] = code < 4 ? "ACGT"[code] : 'N';
          }
        }
        total_agreeing += w.agree_count;
        if (R[i].read_through == 0) tested++;
        out.push_back(w);
      }
    }
  }
  memset(&s, 0, sizeof s);
  const uint64_t total_opp = total_clipped + total_spanning;
  s.total_spanning_read_bases = total_spanning;
  s.total_clipped_read_ends = total_clipped;
  s.total_agreeing_clipped_read_ends = total_agreeing;
  s.soft_clipping_rate = total_opp > 0 ? (double)total_clipped / (double)total_opp : 0.0;
  const double p0_raw = total_opp > 0 ? (double)total_agreeing / (double)total_opp : 0.0;
  double p0 = p0_raw;
  if (p.minimum_rate > 0.0 && p0 < p.minimum_rate) p0 = p.minimum_rate;
  // Pearson chi-square of the quasi-binomial over the untrimmed rows, in row order
  double S_k = 0.0, S_k2_over_n = 0.0, S_n_trimmed = 0.0;
  uint64_t trimmed = 0;
  for (const bsq_sc_position& w : out) {
    if (w.total_count == 0) continue;
    const double k = (double)w.agree_count, n = (double)w.total_count;
    if (p.dispersion_trim_frequency > 0.0 && k / n >= p.dispersion_trim_frequency) {
      trimmed++;
      S_n_trimmed += n;
      continue;
    }
    S_k += k;
    S_k2_over_n += k * k / n;
  }
  const uint64_t N_prime = tested > trimmed ? tested - trimmed : 0;
  const double S_n_prime = (double)total_opp - S_n_trimmed;
  const double mean_n = N_prime > 0 ? S_n_prime / (double)N_prime : 0.0;
  double phi = 0.0, rho = 0.0;
  if (N_prime > 1 && mean_n > 1.0 && p0 > 0.0 && p0 < 1.0) {
    const double chi2 = (S_k2_over_n - 2.0 * p0 * S_k + p0 * p0 * S_n_prime) / (p0 * (1.0 - p0));
    phi = chi2 / (double)(N_prime - 1);
    rho = (phi - 1.0) / (mean_n - 1.0);
  }
  const double rho_raw = rho;
  if (!std::isfinite(rho) || rho < 0.0) rho = 0.0;   // degenerate: plain binomial
  if (p.maximum_dispersion > 0.0 && rho > p.maximum_dispersion) rho = p.maximum_dispersion;
  if (rho < 1e-6) rho = 0.0;
  s.null_rate = p0;
  s.null_rate_raw = p0_raw;
  s.dispersion = rho;
  s.dispersion_raw = rho_raw;
  s.pearson_phi = phi;
  s.tested_positions = N_prime;
  s.trimmed_positions = trimmed;
  s.mean_tested_reads = mean_n;
  s.n_positions = out.size();
}

}  // namespace host
}  // namespace bsq
