// Test driver: the library's discordant / missing-pair scan with the device steps done on the host.
// pair_classify_one (bsq_pairs.h, shared with the classification kernel) classifies every read; the
// window entries and MP window-total members are compacted in BAM order exactly as the scatter
// kernel lays them out; host::pair_replay (bsq_pairs_host.cpp, the library's own replay) and the
// library's CSV writers produce the files.  Compared with the oracle's position-by-position walk by
// tests/test_pairs.py.
#include <cuda_runtime.h>   // vector types and alignment macros of the shared headers; nothing is called
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../breseq_gb300/csrc/bsq_host.h"
#include "../../breseq_gb300/csrc/bsq_pairs.h"

using namespace bsq;

extern "C" int host_pair_candidates(const bsq_reference* ref, const bsq_read_soa* rd, const bsq_pair_params* p,
                                    const char* const* target_names, const char* dp_path, const char* mp_path,
                                    const char* pd_path) {
  const uint32_t T = ref->n_targets;
  std::vector<uint32_t> tpoff(T + 1);
  for (uint32_t t = 0; t <= T; t++) tpoff[t] = (uint32_t)(ref->target_offset[t] + t);
  std::vector<uint8_t> called(T, 0);
  for (uint32_t i = 0; i < ref->n_target_order; i++) called[ref->target_order[i]] = 1;
  const bool mp = p->predict_missing_pairs && p->n_dp_groups > 0;
  std::vector<PairEvent> ev;
  std::vector<uint8_t> codes(rd->n_reads), groups(rd->n_reads);
  std::vector<char> names;
  std::vector<uint32_t> mem_start[2];
  std::vector<uint8_t> mem_group[2];
  for (uint64_t i = 0; i < rd->n_reads; i++) {
    const uint32_t t = (uint32_t)rd->tid[i];
    uint32_t rlen = 0;
    for (uint32_t k = 0; k < rd->n_cigar[i]; k++) {
      const uint32_t w = rd->cigar[rd->cigar_off[i] + k], op = w & 0xF;
      if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rlen += w >> 4;
    }
    uint32_t dflags = 0;
    if ((rd->flag[i] & BSQ_PILEUP_SKIP_MASK) || !called[t]) dflags |= kSkip;
    if (rd->flag[i] & BSQ_FLAG_REVERSE) dflags |= kRev;
    const uint32_t g = rd->read_group[i];
    const int32_t gi = g < p->n_read_groups ? p->dp_group[g] : -1;
    uint8_t code, grp;
    uint32_t sel, mem;
    pair_classify_one(dflags, rd->flag[i], rd->xp[i], gi, mp, code, grp, sel, mem);
    codes[i] = code;
    groups[i] = grp;
    const uint32_t start = tpoff[t] + (uint32_t)rd->pos[i];
    if (sel) {
      PairEvent x;
      x.rec = (uint32_t)i;
      x.start = start;
      x.end = start + rlen;
      x.isize = rd->isize[i];
      x.code = code;
      x.group = grp;
      x.redundant = rd->x1[i] > 1;
      const uint64_t len = rd->qname_off[i + 1] - rd->qname_off[i];
      x.name_len = (uint8_t)len;
      ev.push_back(x);
      names.resize(ev.size() * kPairNameSlot, 0);
      memcpy(names.data() + (ev.size() - 1) * kPairNameSlot, rd->qname + rd->qname_off[i], len);
    }
    if (mem) {
      const int b = (code & kPairRev) ? 1 : 0;
      mem_start[b].push_back(start);
      mem_group[b].push_back(grp);
    }
  }
  host::PairReplayInput in;
  in.tpoff = tpoff;
  in.order.assign(ref->target_order, ref->target_order + ref->n_target_order);
  in.piled.assign(T, 0);
  for (uint32_t t : in.order) in.piled[t] = p->deletion_propagation_cutoff[t] >= 0.0 ? 1 : 0;
  in.window_width.assign(p->window_width, p->window_width + p->n_dp_groups);
  in.r1_prefix.assign(p->r1_name_prefix, p->r1_name_prefix + p->n_dp_groups);
  in.r2_prefix.assign(p->r2_name_prefix, p->r2_name_prefix + p->n_dp_groups);
  in.dp_seed = p->discordant_pair_seed;
  in.mp_seed = p->missing_pair_seed;
  in.mp_seed_fraction = p->missing_pair_seed_fraction;
  in.mp = mp;
  in.ev = ev.data();
  in.n_ev = ev.size();
  in.names = names.data();
  for (int b = 0; b < 2; b++) {
    in.mem_start[b] = mem_start[b].data();
    in.mem_group[b] = mem_group[b].data();
    in.n_mem[b] = mem_start[b].size();
  }
  host::PairReplayResult out;
  int rc = host::pair_replay(in, out);
  if (rc != BSQ_OK) return rc;
  // pair distance: the device's difference arrays, scan, per-position evaluation and ladder edges
  if (pd_path && p->predict_pair_distance) {
    const uint32_t G = p->n_dp_groups;
    bool usable = false;
    for (uint32_t g = 0; g < G; g++) if (p->pd_cdf_len[g]) usable = true;
    host::PdAssembleInput pin;
    pin.tpoff = tpoff;
    pin.enabled = usable && p->pd_max_span > 0 && G > 0;
    pin.z_seed = p->pd_z_seed;
    pin.mean_covering_gap = p->pd_mean_covering_gap;
    pin.total_reference_length = p->total_reference_length;
    if (G) pin.hist.assign(kPdHistBins, 0);
    if (pin.enabled) {
      std::vector<uint8_t> piled(T, 0);
      for (uint32_t t : in.order) piled[t] = p->deletion_propagation_cutoff[t] >= 0.0 ? 1 : 0;
      const uint32_t cols = tpoff[T];
      std::vector<int64_t> diff(4ull * cols + 4, 0);
      const int64_t lower_tail = static_cast<int64_t>(p->pair_distance_tail_quantile * static_cast<double>(kPdUScale));
      for (uint64_t i = 0; i < rd->n_reads; i++) {
        const uint32_t t = (uint32_t)rd->tid[i];
        if (!piled[t] || groups[i] == 0xFF) continue;
        uint32_t dflags = 0;
        if ((rd->flag[i] & BSQ_PILEUP_SKIP_MASK) || !called[t]) dflags |= kSkip;
        if (rd->flag[i] & BSQ_FLAG_REVERSE) dflags |= kRev;
        uint32_t rlen = 0;
        for (uint32_t k = 0; k < rd->n_cigar[i]; k++) {
          const uint32_t w = rd->cigar[rd->cigar_off[i] + k], op = w & 0xF;
          if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) rlen += w >> 4;
        }
        const uint32_t g = groups[i], len = tpoff[t + 1] - tpoff[t] - 1;
        PdInterval iv;
        pd_interval_one(dflags, rd->flag[i], (codes[i] & kPairXpSkip) != 0, (int32_t)g, rd->x1[i], (int32_t)t,
                        rd->mtid[i], rd->isize[i], (uint32_t)rd->pos[i] + 1, (uint32_t)rd->pos[i] + rlen, rd->mpos[i],
                        p->pd_cdf[g], p->pd_cdf_len[g], p->pd_orientation[g], p->pd_max_span, lower_tail, iv);
        if (!iv.ok) continue;
        if (iv.bad || iv.lo < 1 || (uint32_t)iv.hi > len) return BSQ_ERR_DATA;
        int64_t* d0 = &diff[4ull * (tpoff[t] + (uint32_t)iv.lo - 1)];
        int64_t* d1 = &diff[4ull * (tpoff[t] + (uint32_t)iv.hi)];
        d0[0]++; d1[0]--;
        if (iv.bin >= 0) { d0[1 + iv.bin]++; d1[1 + iv.bin]--; }
        d0[3] += iv.u; d1[3] -= iv.u;
      }
      int64_t run[4] = {0, 0, 0, 0};
      uint64_t prev = 0;
      uint32_t t = 0;
      for (uint32_t c = 0; c < cols; c++) {
        for (int j = 0; j < 4; j++) run[j] += diff[4ull * c + j];
        while (c >= tpoff[t + 1]) t++;
        uint64_t m = 0;
        if (piled[t]) {
          const uint32_t pp = c - tpoff[t] + 1, len = tpoff[t + 1] - tpoff[t] - 1;
          double z;
          int hb;
          pd_eval_one(run[0], run[1], run[2], run[3], pp <= len, p->pd_z_seed, p->pair_distance_seed, z, hb, m);
          if (hb >= 0) pin.hist[hb]++;
          if (m & 3) {
            PdAbove a;
            a.col = c; a.bits = (uint32_t)(m & 3); a.n = (int32_t)run[0]; a.nlong = (int32_t)run[1];
            a.nshort = (int32_t)run[2]; a.pad = 0; a.z = z;
            pin.above.push_back(a);
          }
        }
        uint64_t rise = (m & ~prev) >> kPdBitLadder;
        for (int b = 0; b < 2 * kPdLadderSteps; b++)
          if (rise & (1ull << b)) pin.ladder[b / kPdLadderSteps][b % kPdLadderSteps]++;
        prev = m;
      }
    }
    host::PdResult pr;
    host::pd_assemble(pin, pr);
    rc = bsq_write_pd_candidate_regions(pd_path, target_names, pr.regions.data(), pr.regions.size(), &pr.summary);
    if (rc != BSQ_OK) return rc;
  }
  if (dp_path) rc = bsq_write_dp_candidate_regions(dp_path, target_names, out.dp.data(), out.dp.size(), out.text.data());
  if (rc == BSQ_OK && mp_path)
    rc = bsq_write_mp_candidate_regions(mp_path, target_names, out.mp.data(), out.mp.size(), out.text.data());
  return rc;
}
