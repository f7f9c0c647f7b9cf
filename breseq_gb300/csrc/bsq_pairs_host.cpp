// Discordant-pair (DP) and missing-pair (MP) candidate regions: the sliding-window replay on the host
// over the reads the device compacted (bsq_pairs.cu), and the two CSV writers.
//
// breseq advances every window at every reference position of a piled-up target
// (check_discordant_completion / check_missing_pair_completion, src/breseq/identify_mutations.cpp:
// 2358-2437, 2439-2522, called per column at :1758-1767 and once past the end at :2131-2137).  A DP
// window count only changes where a read enters (its start) or leaves (start + ceil(width)), so the
// replay visits those positions only; an MP region also depends on the window total of all reads of
// the strand, which changes almost everywhere, so where the MP count reaches the seed every position
// is evaluated, the total coming from binary searches over the members' start positions.  Region
// contents, their order and every count are those of the per-position walk.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <deque>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "bsq_host.h"
#include "bsq_pairs.h"

namespace bsq {
namespace host {
namespace {

constexpr uint32_t kUndefPos = 0xFFFFFFFFu;
const char* const kOrient[3] = {"FR", "RF", "FF"};

struct Ev {
  uint32_t start1, end1;   // 1-based aligned extent
  uint32_t group;
  bool redundant;
  uint64_t idx;            // index into the compacted events
};

std::string dp_key(const PairEvent& e, const char* name, uint32_t r1_prefix, uint32_t r2_prefix) {
  // <read1_name>__<read2_name>__<r1_insert_size> (identify_mutations.cpp:1418-1436)
  const std::string fname(name, e.name_len);
  const bool focal_is_r1 = !(e.code & kPairRead2);
  const size_t colon = fname.find(':');
  std::string r1, r2;
  if (colon != std::string::npos) {
    const std::string counter = fname.substr(colon + 1);
    r1 = std::to_string(r1_prefix) + ":" + counter;
    r2 = std::to_string(r2_prefix) + ":" + counter;
  } else {
    r1 = focal_is_r1 ? fname : "";
    r2 = focal_is_r1 ? "" : fname;
  }
  const int32_t r1_insert = focal_is_r1 ? e.isize : (int32_t)(0u - (uint32_t)e.isize);
  return r1 + "__" + r2 + "__" + std::to_string(r1_insert);
}

// One bin's open region.
struct Region {
  uint32_t start = kUndefPos, max_count = 0, max_total = 0, redundant = 0;
  std::vector<uint64_t> reads;   // indices into the descriptor strings, in region order
};

// Descriptors are built when a region that lists the read closes: most compacted reads never make one
// (a read can be listed by more than one region of its bin, so each is kept once built).  A read
// belongs to one bin, and one task replays a bin, so tasks fill disjoint entries.
struct Descriptors {
  const PairReplayInput& in;
  std::vector<std::string> text;
  const std::string& get(uint64_t k) {
    std::string& d = text[k];
    if (!d.empty()) return d;
    const PairEvent& e = in.ev[k];
    const uint32_t t = (uint32_t)(std::upper_bound(in.tpoff.begin(), in.tpoff.end(), e.start) - in.tpoff.begin()) - 1;
    const uint32_t s1 = e.start - in.tpoff[t] + 1, e1 = e.end - in.tpoff[t];
    if ((e.code & kPairDpBinMask) != kPairNoBin)
      d = dp_key(e, in.names + k * kPairNameSlot, in.r1_prefix[e.group], in.r2_prefix[e.group]) + "__" +
          std::to_string(s1) + "__" + std::to_string(e1);
    else
      d = std::to_string(s1) + "__" + std::to_string(e1);
    return d;
  }
};

struct Ctx {
  const PairReplayInput& in;
  PairReplayResult& out;
  Descriptors& desc;
};

void close_region(Ctx& c, Region& r, uint32_t tid, uint32_t end, char strand, const char* orient, bool mp) {
  bsq_pair_region x;
  memset(&x, 0, sizeof x);
  x.target = tid;
  x.start = r.start;
  x.end = end;
  x.strand = strand;
  if (orient) { x.orientation[0] = orient[0]; x.orientation[1] = orient[1]; }
  x.max_count = r.max_count;
  x.max_total = mp ? r.max_total : 0;
  x.redundant = (2 * (uint64_t)r.redundant > r.reads.size()) ? 1 : 0;
  x.text_off = c.out.text.size();
  for (size_t k = 0; k < r.reads.size(); k++) {
    if (k) c.out.text += ';';
    c.out.text += c.desc.get(r.reads[k]);
  }
  x.text_len = c.out.text.size() - x.text_off;
  (mp ? c.out.mp : c.out.dp).push_back(x);
  r = Region();
}

// Start columns of one strand's MP window-total members on one target, per DP group: group g's sorted
// columns are col[off[g] .. off[g + 1]).  With one group col points at the device's array itself.
struct Members {
  const uint32_t* col = nullptr;
  std::vector<uint64_t> off;
  std::vector<uint32_t> own;
};

// The first index at or after i (below end) whose column is above v: a galloping search, so a cursor
// that catches up over a long stretch (between the runs of positions an MP bin evaluates) costs a
// logarithm rather than a scan.
inline uint64_t advance_past(const uint32_t* col, uint64_t i, uint64_t end, int64_t v) {
  if (i >= end || (int64_t)col[i] > v) return i;
  uint64_t lo = i, step = 1;
  while (lo + step < end && (int64_t)col[lo + step] <= v) {
    lo += step;
    step <<= 1;
  }
  const uint64_t hi = std::min(lo + step, end);
  return (uint64_t)(std::upper_bound(col + lo + 1, col + hi, v,
                                     [](int64_t x, uint32_t c) { return x < (int64_t)c; }) - col);
}

// The windows of one bin over one target.  ev: the bin's reads in BAM order.  members: MP only.
void replay_bin(Ctx& c, uint32_t tid, uint32_t len, const std::vector<Ev>& ev, int bin, bool mp,
                const Members* members) {
  const PairReplayInput& in = c.in;
  const uint32_t G = (uint32_t)in.window_width.size();
  const int32_t seed = mp ? in.mp_seed : in.dp_seed;
  // positions where the window count can change: entries, exits inside the target, and the flush
  std::vector<uint32_t> pos;
  pos.reserve(2 * ev.size() + 1);
  for (const Ev& e : ev) {
    pos.push_back(e.start1);
    const double w = ceil(in.window_width[e.group]);
    if ((double)e.start1 + w <= (double)len) pos.push_back(e.start1 + (uint32_t)w);
  }
  if (len >= 1) pos.push_back(1);   // a seed of 0 is reached before any read enters
  pos.push_back(len + 1);
  std::sort(pos.begin(), pos.end());
  pos.erase(std::unique(pos.begin(), pos.end()), pos.end());

  std::vector<std::deque<size_t>> win(G);
  int32_t metric = 0;
  size_t next = 0;
  Region r;
  const char strand = mp ? (bin == 0 ? 'F' : 'R') : (bin / 3 == 0 ? 'F' : 'R');
  const char* orient = mp ? nullptr : kOrient[bin % 3];

  // the window total at p: members with p - ceil(width) < start <= p, compared as columns (position
  // p is column c0 + p - 1).  Positions only increase within a bin, so two cursors per group advance
  // through the sorted columns.
  const int64_t c0m1 = (int64_t)in.tpoff[tid] - 1;
  std::vector<uint64_t> lo_i(G), hi_i(G);
  std::vector<int64_t> wceil(G);
  for (uint32_t g = 0; g < G; g++) {
    wceil[g] = (int64_t)ceil(in.window_width[g]);
    if (members) lo_i[g] = hi_i[g] = members->off[g];
  }
  auto total_at = [&](uint32_t p) -> int64_t {
    int64_t t = 0;
    const int64_t cp = c0m1 + p;
    for (uint32_t g = 0; g < G; g++) {
      hi_i[g] = advance_past(members->col, hi_i[g], members->off[g + 1], cp);
      lo_i[g] = advance_past(members->col, lo_i[g], hi_i[g], cp - wceil[g]);
      t += (int64_t)(hi_i[g] - lo_i[g]);
    }
    return t;
  };
  // the per-position test and region bookkeeping, after the position's entries and exits
  // a region opens at p with the reads in the windows as its snapshot
  auto open_region = [&](uint32_t p, int64_t total) {
    r.start = p;
    r.max_count = (uint32_t)metric;
    r.max_total = (uint32_t)total;
    r.reads.clear();
    r.redundant = 0;
    for (uint32_t g = 0; g < G; g++)
      for (size_t k : win[g]) {
        r.reads.push_back(ev[k].idx);
        if (ev[k].redundant) r.redundant++;
      }
  };
  auto check = [&](uint32_t p) {
    bool above;
    int64_t total = 0;
    if (mp) {
      total = total_at(p);
      const bool enriched = (total > 0) && ((double)metric >= in.mp_seed_fraction * (double)total);
      above = (metric >= seed) && enriched && (p <= len);
    } else {
      above = (metric >= seed) && (p <= len);
    }
    if (above) {
      if (r.start == kUndefPos) {
        open_region(p, total);
      } else if ((uint32_t)metric > r.max_count) {
        r.max_count = (uint32_t)metric;
        r.max_total = (uint32_t)total;
      }
    } else if (r.start != kUndefPos) {
      close_region(c, r, tid, p - 1, strand, orient, mp);
    }
  };

  for (size_t pi = 0; pi < pos.size(); pi++) {
    const uint32_t p = pos[pi];
    // entries at p, in BAM order; an open region takes them at once
    while (next < ev.size() && ev[next].start1 == p) {
      win[ev[next].group].push_back(next);
      metric++;
      if (r.start != kUndefPos) {
        r.reads.push_back(ev[next].idx);
        if (ev[next].redundant) r.redundant++;
      }
      next++;
    }
    // exits
    for (uint32_t g = 0; g < G; g++)
      while (!win[g].empty() && ((double)p - (double)ev[win[g].front()].start1 >= in.window_width[g])) {
        win[g].pop_front();
        metric--;
      }
    check(p);
    // MP: between this position and the next event the count is fixed (so the region's maximum
    // cannot move), but the total is not: only the enrichment test can open or close a region
    if (mp && metric >= seed && pi + 1 < pos.size()) {
      const uint32_t q_end = std::min<uint32_t>(pos[pi + 1] - 1, len);
      const double m = (double)metric;
      // one DP group: the two cursors in registers
      const bool one = G == 1;
      const uint32_t* col = one ? members->col : nullptr;
      uint64_t lo1 = one ? lo_i[0] : 0, hi1 = one ? hi_i[0] : 0;
      const uint64_t end1 = one ? members->off[1] : 0;
      const int64_t wc1 = one ? wceil[0] : 0;
      for (uint32_t q = p + 1; q <= q_end; q++) {
        int64_t total;
        if (one) {
          const int64_t cp = c0m1 + q;
          hi1 = advance_past(col, hi1, end1, cp);
          lo1 = advance_past(col, lo1, hi1, cp - wc1);
          total = (int64_t)(hi1 - lo1);
        } else {
          total = total_at(q);
        }
        const bool above = (total > 0) && (m >= in.mp_seed_fraction * (double)total);
        if (above) {
          if (r.start == kUndefPos) open_region(q, total);
        } else if (r.start != kUndefPos) {
          close_region(c, r, tid, q - 1, strand, orient, mp);
        }
      }
      if (one) {
        lo_i[0] = lo1;
        hi_i[0] = hi1;
      }
    }
  }
}

}  // namespace

int pair_replay(const PairReplayInput& in, PairReplayResult& out) {
  const uint32_t G = (uint32_t)in.window_width.size();
  for (uint64_t k = 0; k < in.n_ev; k++)
    if ((in.ev[k].code & kPairDpBinMask) != kPairNoBin && in.ev[k].group >= G) return BSQ_ERR_INVALID;
  Descriptors desc{in, std::vector<std::string>(in.n_ev)};
  for (int b = 0; b < 2; b++)
    for (uint64_t k = 0; k < in.n_mem[b]; k++)
      if (in.mem_group[b][k] >= G) return BSQ_ERR_INVALID;
  if (!G) return BSQ_OK;
  // independent tasks: per piled target, the six DP bins, and each MP strand; merged in this order
  struct Task { uint32_t t; int kind; PairReplayResult res; };
  std::vector<Task> tasks;
  // MP window-total members of each piled target and strand; with several DP groups they are split by
  // group with a counting pass (BAM order keeps each group's columns sorted)
  std::vector<Members> members(in.mp ? 2 * (size_t)in.tpoff.size() : 0);
  for (uint32_t t : in.order) {
    if (!in.piled[t]) continue;
    tasks.push_back({t, 0, {}});
    if (!in.mp) continue;
    tasks.push_back({t, 1, {}});
    tasks.push_back({t, 2, {}});
    const uint32_t c0 = in.tpoff[t], c1 = in.tpoff[t + 1] - 1;
    for (int b = 0; b < 2; b++) {
      const uint32_t* ms = in.mem_start[b];
      const uint64_t lo = std::lower_bound(ms, ms + in.n_mem[b], c0) - ms;
      const uint64_t hi = std::lower_bound(ms + lo, ms + in.n_mem[b], c1) - ms;
      Members& m = members[2 * t + b];
      if (G == 1) {
        m.col = ms;
        m.off = {lo, hi};
        continue;
      }
      m.off.assign(G + 1, 0);
      for (uint64_t k = lo; k < hi; k++) m.off[in.mem_group[b][k] + 1]++;
      for (uint32_t g = 0; g < G; g++) m.off[g + 1] += m.off[g];
      m.own.resize(m.off[G]);
      std::vector<uint64_t> fill(m.off.begin(), m.off.end() - 1);
      for (uint64_t k = lo; k < hi; k++) m.own[fill[in.mem_group[b][k]]++] = ms[k];
      m.col = m.own.data();
    }
  }
  auto run = [&](Task& task) {
    const uint32_t t = task.t;
    const uint32_t len = in.tpoff[t + 1] - in.tpoff[t] - 1;
    const uint32_t c0 = in.tpoff[t], c1 = in.tpoff[t] + len;
    Ctx c{in, task.res, desc};
    // this target's events and members (both in BAM order, so contiguous and start-sorted)
    auto ev_lo = std::lower_bound(in.ev, in.ev + in.n_ev, c0, [](const PairEvent& e, uint32_t v) { return e.start < v; });
    auto ev_hi = std::lower_bound(ev_lo, in.ev + in.n_ev, c1 + 1, [](const PairEvent& e, uint32_t v) { return e.start < v; });
    if (task.kind == 0) {
      std::vector<Ev> dp[6];
      for (auto it = ev_lo; it != ev_hi; ++it) {
        const int bin = it->code & kPairDpBinMask;
        if (bin != kPairNoBin) dp[bin].push_back(Ev{it->start - c0 + 1, it->end - c0, it->group, it->redundant != 0,
                                                    (uint64_t)(it - in.ev)});
      }
      for (int b = 0; b < 6; b++) replay_bin(c, t, len, dp[b], b, false, nullptr);
      return;
    }
    const int b = task.kind - 1;
    std::vector<Ev> mpe;
    for (auto it = ev_lo; it != ev_hi; ++it)
      if ((it->code & kPairMpUnmapped) && ((it->code & kPairRev) ? 1 : 0) == b)
        mpe.push_back(Ev{it->start - c0 + 1, it->end - c0, it->group, it->redundant != 0, (uint64_t)(it - in.ev)});
    replay_bin(c, t, len, mpe, b, true, &members[2 * t + b]);
  };
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t n_threads = std::min<size_t>(tasks.size(), hw ? hw : 1);
  if (n_threads <= 1) {
    for (Task& task : tasks) run(task);
  } else {
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (size_t i = 0; i < n_threads; i++)
      pool.emplace_back([&]() {
        for (size_t k; (k = next.fetch_add(1)) < tasks.size();) run(tasks[k]);
      });
    for (std::thread& th : pool) th.join();
  }
  for (Task& task : tasks) {
    const uint64_t base = out.text.size();
    out.text += task.res.text;
    for (bsq_pair_region r : task.res.dp) { r.text_off += base; out.dp.push_back(r); }
    for (bsq_pair_region r : task.res.mp) { r.text_off += base; out.mp.push_back(r); }
  }
  return BSQ_OK;
}

// identify_mutations_pileup::pd_z_inflation (identify_mutations.cpp:2758-2786): the spread of the
// per-position z over the genome, as the interquartile range of its histogram over 1.34898038.
static double pd_z_inflation(const std::vector<uint64_t>& hist) {
  if (hist.empty()) return 1.0;
  uint64_t total = 0;
  for (uint64_t h : hist) total += h;
  if (total < 1000) return 1.0;
  const uint64_t want_lo = total / 4, want_hi = (total * 3) / 4;
  double q_lo = 0.0, q_hi = 0.0;
  uint64_t run = 0;
  bool have_lo = false, have_hi = false;
  for (size_t i = 0; i < hist.size(); i++) {
    run += hist[i];
    const double centre = (static_cast<double>(i) + 0.5) / kPdHistPerUnit - kPdHistLimit;
    if (!have_lo && (run >= want_lo)) { q_lo = centre; have_lo = true; }
    if (!have_hi && (run >= want_hi)) { q_hi = centre; have_hi = true; break; }
  }
  if (!have_lo || !have_hi) return 1.0;
  const double sd = (q_hi - q_lo) / 1.34898038;
  if (!(sd > 1.0)) return 1.0;
  return sd;
}

static double pd_ladder_z(int i) { return 1.0 + 0.25 * static_cast<double>(i); }

// pd_fit_region_tail (identify_mutations.cpp:2788-2850): a weighted least-squares fit of
// log(count) against t^2 over the ladder rungs with enough regions and past the bulk.
static bool pd_fit_region_tail(const uint64_t (&ladder)[2][kPdLadderSteps], bool enabled, double& out_log_intercept,
                               double& out_sigma, double& out_fit_lo, double& out_fit_hi) {
  out_log_intercept = 0.0;
  out_sigma = 1.0;
  out_fit_lo = 0.0;
  out_fit_hi = 0.0;
  if (!enabled) return false;
  const uint64_t kMinRegions = 20, kTailFactor = 3;
  const int kMinRungs = 3;
  uint64_t max_count = 0;
  for (int step = 0; step < kPdLadderSteps; step++) max_count = std::max(max_count, ladder[0][step] + ladder[1][step]);
  double sw = 0.0, swx = 0.0, swy = 0.0, swxx = 0.0, swxy = 0.0;
  int rungs = 0;
  for (int step = 0; step < kPdLadderSteps; step++) {
    const uint64_t count = ladder[0][step] + ladder[1][step];
    if (count < kMinRegions) continue;
    if (count * kTailFactor > max_count) continue;
    const double t = pd_ladder_z(step);
    const double x = t * t;
    const double y = log(static_cast<double>(count));
    const double w = static_cast<double>(count);
    sw += w; swx += w * x; swy += w * y; swxx += w * x * x; swxy += w * x * y;
    if (rungs == 0) out_fit_lo = t;
    out_fit_hi = t;
    rungs++;
  }
  if (rungs < kMinRungs) return false;
  const double denom = sw * swxx - swx * swx;
  if (!(fabs(denom) > 0.0)) return false;
  const double slope = (sw * swxy - swx * swy) / denom;
  const double intercept = (swy - slope * swx) / sw;
  if (!(slope < 0.0)) return false;
  const double sigma = sqrt(-1.0 / (2.0 * slope));
  if (!(sigma > 0.0) || !std::isfinite(sigma)) return false;
  out_log_intercept = intercept;
  out_sigma = sigma;
  return true;
}

void pd_assemble(PdAssembleInput& in, PdResult& out) {
  // regions: maximal runs of consecutive positions above a direction's seed; the peak is the first
  // position of largest |z| (identify_mutations.cpp:2708-2742)
  std::sort(in.above.begin(), in.above.end(), [](const PdAbove& a, const PdAbove& b) { return a.col < b.col; });
  std::vector<bsq_pd_region> regions;
  for (int bin = 0; bin < 2; bin++) {
    bool open = false;
    uint32_t last = 0;
    bsq_pd_region r;
    auto close = [&]() {
      const uint32_t t = (uint32_t)(std::upper_bound(in.tpoff.begin(), in.tpoff.end(), last) - in.tpoff.begin()) - 1;
      r.end = last - in.tpoff[t] + 1;
      regions.push_back(r);
      open = false;
    };
    for (const PdAbove& a : in.above) {
      if (!(a.bits & (1u << bin))) continue;
      if (open && a.col != last + 1) close();
      if (!open) {
        const uint32_t t = (uint32_t)(std::upper_bound(in.tpoff.begin(), in.tpoff.end(), a.col) - in.tpoff.begin()) - 1;
        memset(&r, 0, sizeof r);
        r.target = t;
        r.start = a.col - in.tpoff[t] + 1;
        r.direction = bin == 0 ? 'L' : 'S';
        r.peak_position = r.start;
        r.peak_covering = a.n;
        r.peak_tail = bin == 0 ? a.nlong : a.nshort;
        r.peak_z = a.z;
        open = true;
      } else if (fabs(a.z) > fabs(r.peak_z)) {
        r.peak_position = a.col - in.tpoff[r.target] + 1;
        r.peak_covering = a.n;
        r.peak_tail = bin == 0 ? a.nlong : a.nshort;
        r.peak_z = a.z;
      }
      last = a.col;
    }
    if (open) close();
  }
  // calibration (fill_pd_summary, :2852-2862)
  bsq_pd_summary& c = out.summary;
  memset(&c, 0, sizeof c);
  c.mean_covering_gap = in.mean_covering_gap;
  c.n_effective_tests =
      (in.mean_covering_gap > 0.0) ? static_cast<double>(in.total_reference_length) / in.mean_covering_gap : 0.0;
  c.seed_z_used = in.z_seed;
  c.z_iqr_inflation = pd_z_inflation(in.hist);
  c.regions_seeded = regions.size();
  c.region_tail_fit_ok = pd_fit_region_tail(in.ladder, in.enabled, c.region_tail_log_intercept, c.region_tail_sigma,
                                            c.region_tail_fit_lo, c.region_tail_fit_hi) ? 1 : 0;
  for (int step = 0; step < kPdLadderSteps; step++) c.ladder[step] = in.ladder[0][step] + in.ladder[1][step];
  // the rescan budget: raise the seed to the first rung at or above it with at most 3000 regions
  // (write_pd_candidate_regions, :2875-2904)
  const uint64_t kMaxCandidateRegions = 3000;
  double capped_z = c.seed_z_used;
  for (int step = 0; step < kPdLadderSteps; step++) {
    const double t = pd_ladder_z(step);
    if (t < c.seed_z_used) continue;
    capped_z = t;
    if (c.ladder[step] <= kMaxCandidateRegions) break;
  }
  if (capped_z > c.seed_z_used) {
    std::vector<bsq_pd_region> kept;
    for (const bsq_pd_region& r : regions)
      if (fabs(r.peak_z) >= capped_z) kept.push_back(r);
    regions.swap(kept);
    c.seed_z_used = capped_z;
    c.regions_seeded = regions.size();
  }
  out.regions = std::move(regions);
}

}  // namespace host
}  // namespace bsq

namespace {

template <class Less>
int write_regions(const char* path, const char* const* names, const bsq_pair_region* regions, uint64_t n,
                  const char* text, bool mp, Less less) {
  if (!path || (n && (!regions || !names || !text))) return BSQ_ERR_INVALID;
  std::vector<const bsq_pair_region*> v(n);
  for (uint64_t i = 0; i < n; i++) v[i] = regions + i;
  std::sort(v.begin(), v.end(), [&](const bsq_pair_region* a, const bsq_pair_region* b) { return less(*a, *b); });
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  if (mp)
    out << "seq_id,start,end,strand,length,max_unpaired_count,max_window_total_count,redundant,unpaired_reads\n";
  else
    out << "seq_id,start,end,strand,orientation,length,max_discordant_count,redundant,discordant_pairs\n";
  for (const bsq_pair_region* r : v) {
    out << names[r->target] << "," << r->start << "," << r->end << "," << r->strand << ",";
    if (!mp) out << std::string(r->orientation, strnlen(r->orientation, 3)) << ",";
    out << (r->end - r->start + 1) << "," << r->max_count << ",";
    if (mp) out << r->max_total << ",";
    out << (r->redundant ? 1 : 0) << "," << std::string(text + r->text_off, r->text_len) << "\n";
  }
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

}  // namespace

extern "C" int bsq_write_dp_candidate_regions(const char* path, const char* const* target_names,
                                              const bsq_pair_region* regions, uint64_t n, const char* text) {
  // sorted by (seq_id, start, strand, orientation): identify_mutations.cpp:2553-2560
  return write_regions(path, target_names, regions, n, text, false,
                       [&](const bsq_pair_region& a, const bsq_pair_region& b) {
                         const std::string sa = target_names[a.target], sb = target_names[b.target];
                         if (sa != sb) return sa < sb;
                         if (a.start != b.start) return a.start < b.start;
                         if (a.strand != b.strand) return a.strand < b.strand;
                         return std::string(a.orientation, strnlen(a.orientation, 3)) <
                                std::string(b.orientation, strnlen(b.orientation, 3));
                       });
}

extern "C" int bsq_write_mp_candidate_regions(const char* path, const char* const* target_names,
                                              const bsq_pair_region* regions, uint64_t n, const char* text) {
  // sorted by (seq_id, start, strand): identify_mutations.cpp:2527-2533
  return write_regions(path, target_names, regions, n, text, true,
                       [&](const bsq_pair_region& a, const bsq_pair_region& b) {
                         const std::string sa = target_names[a.target], sb = target_names[b.target];
                         if (sa != sb) return sa < sb;
                         if (a.start != b.start) return a.start < b.start;
                         return a.strand < b.strand;
                       });
}

extern "C" int bsq_write_pd_candidate_regions(const char* path, const char* const* target_names,
                                              const bsq_pd_region* regions, uint64_t n, const bsq_pd_summary* c) {
  // identify_mutations.cpp:2906-2957: calibration lines, the ladder, then the regions sorted by
  // (seq_id, start, direction)
  if (!path || !c || (n && (!regions || !target_names))) return BSQ_ERR_INVALID;
  std::vector<const bsq_pd_region*> v(n);
  for (uint64_t i = 0; i < n; i++) v[i] = regions + i;
  std::sort(v.begin(), v.end(), [&](const bsq_pd_region* a, const bsq_pd_region* b) {
    const std::string sa = target_names[a->target], sb = target_names[b->target];
    if (sa != sb) return sa < sb;
    if (a->start != b->start) return a->start < b->start;
    return a->direction < b->direction;
  });
  std::ofstream out(path);
  if (!out) return BSQ_ERR_INVALID;
  out << std::fixed << std::setprecision(6);
  out << "#mean_covering_gap=" << c->mean_covering_gap << "\n";
  out << "#n_effective_tests=" << c->n_effective_tests << "\n";
  out << "#seed_z=" << c->seed_z_used << "\n";
  out << "#z_iqr_inflation=" << c->z_iqr_inflation << "\n";
  out << "#region_tail_fit_ok=" << (c->region_tail_fit_ok ? 1 : 0) << "\n";
  out << "#region_tail_log_intercept=" << c->region_tail_log_intercept << "\n";
  out << "#region_tail_sigma=" << c->region_tail_sigma << "\n";
  out << "#region_tail_fit_lo=" << c->region_tail_fit_lo << "\n";
  out << "#region_tail_fit_hi=" << c->region_tail_fit_hi << "\n";
  out << "#region_ladder=";
  for (int step = 0; step < bsq::kPdLadderSteps; step++) {
    if (step) out << ";";
    out << std::setprecision(2) << (1.0 + 0.25 * static_cast<double>(step)) << ":" << c->ladder[step];
  }
  out << "\n";
  out << "seq_id,start,end,direction,length,peak_position,peak_covering_count,peak_tail_count,peak_z\n";
  out << std::setprecision(4);
  for (const bsq_pd_region* r : v)
    out << target_names[r->target] << "," << r->start << "," << r->end << "," << r->direction << ","
        << (r->end - r->start + 1) << "," << r->peak_position << "," << r->peak_covering << "," << r->peak_tail
        << "," << r->peak_z << "\n";
  return out ? BSQ_OK : BSQ_ERR_INVALID;
}

// ------------------------------------------------------------------ pair-distance setup (host)
namespace {

// Cephes ndtri (S. L. Moshier, Cephes Math Library 2.8; src/breseq/stats.cpp:1747-1791): the inverse
// of the standard normal CDF, with breseq's coefficients and order of operations.
const double kNdP0[5] = {-5.99633501014107895267E1, 9.80010754185999661536E1, -5.66762857469070293439E1,
                         1.39312609387279679503E1, -1.23916583867381258016E0};
const double kNdQ0[8] = {1.95448858338141759834E0, 4.67627912898881538453E0, 8.63602421390890590575E1,
                         -2.25462687854119370527E2, 2.00260212380060660359E2, -8.20372256168333339912E1,
                         1.59056225126211695515E1, -1.18331621121330003142E0};
const double kNdP1[9] = {4.05544892305962419923E0, 3.15251094599893866154E1, 5.71628192246421288162E1,
                         4.40805073893200834700E1, 1.46849561928858024014E1, 2.18663306850790267539E0,
                         -1.40256079171354495875E-1, -3.50424626827848203418E-2, -8.57456785154685413611E-4};
const double kNdQ1[8] = {1.57799883256466749731E1, 4.53907635128879210584E1, 4.13172038254672030440E1,
                         1.50425385692907503408E1, 2.50464946208309415979E0, -1.42182922854787788574E-1,
                         -3.80806407691578277194E-2, -9.33259480895457427372E-4};
const double kNdP2[9] = {3.23774891776946035970E0, 6.91522889068984211695E0, 3.93881025292474443415E0,
                         1.33303460815807542389E0, 2.01485389549179081538E-1, 1.23716634817820021358E-2,
                         3.01581553508235416007E-4, 2.65806974686737550832E-6, 6.23974539184983293730E-9};
const double kNdQ2[8] = {6.02427039364742014255E0, 3.67983563856160859403E0, 1.37702099489081330271E0,
                         2.16236993594496635890E-1, 1.34204006088543189037E-2, 3.28014464682127739104E-4,
                         2.89247864745380683936E-6, 6.79019408009981274425E-9};

double horner(double x, const double* c, int n) {     // c[0] x^n + ... + c[n]
  double r = c[0];
  for (int i = 1; i <= n; i++) r = r * x + c[i];
  return r;
}
double horner1(double x, const double* c, int n) {    // x^n + c[0] x^(n-1) + ... + c[n-1]
  double r = x + c[0];
  for (int i = 1; i < n; i++) r = r * x + c[i];
  return r;
}

double ndtri(double y0) {
  const double kMaxNum = 1.79769313486231570815E308, kS2Pi = 2.50662827463100050242E0;
  if (y0 <= 0.0) return -kMaxNum;
  if (y0 >= 1.0) return kMaxNum;
  int code = 1;
  double y = y0;
  if (y > (1.0 - 0.13533528323661269189)) {   // exp(-2)
    y = 1.0 - y;
    code = 0;
  }
  if (y > 0.13533528323661269189) {
    y = y - 0.5;
    const double y2 = y * y;
    double x = y + y * (y2 * horner(y2, kNdP0, 4) / horner1(y2, kNdQ0, 8));
    x = x * kS2Pi;
    return x;
  }
  double x = sqrt(-2.0 * log(y));
  const double x0 = x - log(x) / x;
  const double z = 1.0 / x;
  const double x1 = x < 8.0 ? z * horner(z, kNdP1, 8) / horner1(z, kNdQ1, 8)
                            : z * horner(z, kNdP2, 8) / horner1(z, kNdQ2, 8);
  x = x0 - x1;
  if (code != 0) x = -x;
  return x;
}

}  // namespace

extern "C" int bsq_pd_build_null(const int32_t* distance, const double* count, uint64_t n_rows, int32_t trunc,
                                 int32_t max_distance, int64_t* cdf, uint32_t capacity, uint32_t* cdf_len,
                                 double* mean_covering_gap) {
  if ((n_rows && (!distance || !count)) || !cdf_len || !mean_covering_gap) return BSQ_ERR_INVALID;
  // pd_load_weighted_histogram (src/breseq/pd_evidence.cpp:56-97): each distance weighted by its gap
  // d - trunc, rows past max_distance (when > 0) and gapless rows dropped; a repeated distance keeps
  // its last row's weight while the total takes every row
  std::vector<double> weighted;
  double total = 0.0;
  for (uint64_t i = 0; i < n_rows; i++) {
    const int32_t d = distance[i];
    const double n = count[i];
    if ((d < 0) || (n <= 0.0)) continue;
    if ((max_distance > 0) && (d > max_distance)) continue;
    const double weight = static_cast<double>(d - trunc);
    if (weight <= 0.0) continue;
    if (static_cast<int32_t>(weighted.size()) <= d) weighted.resize((size_t)d + 1, 0.0);
    weighted[d] = n * weight;
    total += weighted[d];
  }
  *cdf_len = 0;
  *mean_covering_gap = 0.0;
  if (total <= 0.0) return BSQ_OK;   // no usable weight: no null, PD skips the group
  if (weighted.size() > capacity) {
    *cdf_len = (uint32_t)weighted.size();
    return BSQ_ERR_SIZE;
  }
  // pd_build_cdf (src/breseq/identify_mutations.cpp:112-141): the mid-CDF in 2^20 fixed point and the
  // mean gap of a covering pair
  double below = 0.0, gap_sum = 0.0;
  for (size_t d = 0; d < weighted.size(); d++) {
    const double mid = (below + 0.5 * weighted[d]) / total;
    below += weighted[d];
    gap_sum += weighted[d] * (static_cast<double>(d) - static_cast<double>(trunc));
    int64_t scaled = static_cast<int64_t>(mid * static_cast<double>(bsq::kPdUScale) + 0.5);
    if (scaled < 0) scaled = 0;
    if (scaled > bsq::kPdUScale) scaled = bsq::kPdUScale;
    cdf[d] = scaled;
  }
  *cdf_len = (uint32_t)weighted.size();
  *mean_covering_gap = gap_sum / total;
  return BSQ_OK;
}

extern "C" int32_t bsq_pd_max_span(int32_t pair_distance_maximum_span, const double* distance_cutoff,
                                   uint32_t n_groups) {
  // identify_mutations.cpp:928-941: twice the largest paired-mapping distance cutoff, unless given
  double derived = 0.0;
  for (uint32_t g = 0; g < n_groups; g++) derived = std::max(derived, 2.0 * distance_cutoff[g]);
  return pair_distance_maximum_span > 0 ? pair_distance_maximum_span : static_cast<int32_t>(derived + 0.5);
}

extern "C" double bsq_pd_seed_z(double pair_distance_seed_z, double mean_covering_gap, uint64_t total_reference_length) {
  // identify_mutations.cpp:979-994: the analytic one-sided threshold with the effective number of
  // tests (reference length / covering gap), never above 2.5 nor below 1, unless given
  if (pair_distance_seed_z > 0.0) return pair_distance_seed_z;
  double alpha_half = 0.005;
  if ((mean_covering_gap > 0.0) && (total_reference_length > 0))
    alpha_half *= mean_covering_gap / static_cast<double>(total_reference_length);
  if (alpha_half > 0.5) alpha_half = 0.5;
  if (alpha_half < 1e-12) alpha_half = 1e-12;
  const double analytic_z = ndtri(1.0 - alpha_half);
  double z = std::min(analytic_z, 2.5);
  if (z < 1.0) z = 1.0;
  return z;
}

extern "C" double bsq_ndtri(double y) { return ndtri(y); }
