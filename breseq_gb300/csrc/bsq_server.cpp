// Scoring server: HBM-budget admission, uploads (several at once) beside the running GPU round,
// and continuous batching of both passes over the resident jobs.  Built only on the library's C ABI.
//
// breseq scores one sample per process, one pass after the other (error_count at
// src/breseq/breseq_cmdline.cpp:2293, identify_mutations at :2471); a job here is that sequence for
// one sample, with the error table converted between the passes exactly as error_rates.tab
// round-trips it (bsq_counts_to_log10_prob).  The deletion cutoffs that breseq derives from the
// coverage fit between the passes come with the job.
#include <stdint.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/breseq_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  uint64_t id = 0;
  bsq_job desc;
  int32_t state = BSQ_JOB_QUEUED;
  int32_t sample = -1;
  uint64_t footprint = 0;
  bool charged = false;             // footprint counted in in_use
  uint64_t read_bases = 0;
  uint32_t round_jobs = 0;
  Clock::time_point t_submit, t_admit, t_ready, t_start, t_done;
  std::string err;
  std::vector<uint64_t> counts, hist;
  std::vector<uint32_t> hist_size;
  std::vector<double> table;
  std::vector<bsq_ra_record> ra;
  std::vector<bsq_mc_record> mc;
  std::vector<bsq_un_record> un;
};

// Aligned read bases of a sample, the unit of the throughput figures: M/=/X and I lengths of the
// records the pileup keeps.
uint64_t aligned_read_bases(const bsq_read_soa* r) {
  uint64_t n = 0;
  for (uint64_t i = 0; i < r->n_reads; i++) {
    if (r->flag[i] & BSQ_PILEUP_SKIP_MASK) continue;
    const uint32_t* cg = r->cigar + r->cigar_off[i];
    for (uint32_t k = 0; k < r->n_cigar[i]; k++) {
      const uint32_t op = cg[k] & 0xF;
      if (op == 0 || op == 1 || op == 7 || op == 8) n += cg[k] >> 4;
    }
  }
  return n;
}

}  // namespace

struct bsq_server {
  bsq_ctx* ctx = nullptr;
  uint64_t budget = 0;
  uint32_t max_batch = 64;
  int32_t precision = BSQ_PRECISION_FP32C;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable cv_admit, cv_ready, cv_done;
  std::deque<Job*> queued;          // submitted, waiting for budget
  std::deque<Job*> ready;           // resident, waiting for a GPU round
  std::map<uint64_t, std::unique_ptr<Job>> jobs;
  uint64_t next_id = 1;
  uint64_t in_use = 0, peak_in_use = 0;
  uint64_t jobs_done = 0, rounds = 0;
  uint32_t max_round_jobs = 0, resident = 0, max_resident = 0;
  uint32_t pending = 0;             // submitted and not finished
  uint32_t loading = 0;             // admitted, upload in progress
  double gpu_busy_ms = 0;
  bool tune_pending = false;
  bsq_tuning tune{};                      // applied by the GPU thread before its next round
  double phase_ms[5] = {0, 0, 0, 0, 0};   // pass 1, tables, pass 2, result copies, frees (summed over rounds)
  bool stop = false;
  std::string err;
  static constexpr int kLoaders = 8;   // uploads in flight at once (each on its own load stream)
  static constexpr size_t kMinRound = 4;   // a round waits (at most kJoinMs) for this many ready jobs
  static constexpr int kJoinMs = 2;        // while uploads are in progress
  std::vector<std::thread> admitters;
  std::thread gpu;

  double ms(Clock::time_point t) const { return std::chrono::duration<double, std::milli>(t - t0).count(); }

  void finish(Job* j, int32_t state, const std::string& e) {   // mu held
    j->state = state;
    j->err = e;
    j->t_done = Clock::now();
    if (j->charged) { in_use -= j->footprint; j->charged = false; }
    pending--;
    jobs_done++;
    cv_done.notify_all();
    cv_admit.notify_all();
  }

  // ---------------------------------------------------------------- admission + upload
  void admit_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      // a stopping server still admits what was submitted before the stop
      cv_admit.wait(lk, [&] {
        return (!queued.empty() && in_use + queued.front()->footprint <= budget) || (stop && queued.empty());
      });
      if (queued.empty()) return;
      Job* j = queued.front();
      queued.pop_front();
      in_use += j->footprint;
      j->charged = true;
      if (in_use > peak_in_use) peak_in_use = in_use;
      j->state = BSQ_JOB_LOADING;
      j->t_admit = Clock::now();
      loading++;
      lk.unlock();
      j->read_bases = aligned_read_bases(j->desc.reads);
      int32_t sid = -1;
      const int rc = bsq_load_sample(ctx, j->desc.ref, j->desc.reads, &sid);
      const std::string e = rc == BSQ_OK ? std::string() : std::string(bsq_last_error(ctx));
      lk.lock();
      loading--;
      if (rc != BSQ_OK) {
        finish(j, rc, "load: " + e);
        cv_ready.notify_all();
        continue;
      }
      j->sample = sid;
      j->state = BSQ_JOB_READY;
      j->t_ready = Clock::now();
      ready.push_back(j);
      resident++;
      if (resident > max_resident) max_resident = resident;
      cv_ready.notify_all();
    }
  }

  // ---------------------------------------------------------------- GPU rounds
  // Both passes for a list of jobs; on a batch failure each job is rerun alone so that one bad
  // job does not fail the others.
  int run_round(std::vector<Job*>& js, std::string& e) {
    const uint32_t n = (uint32_t)js.size();
    std::vector<int32_t> ids(n);
    std::vector<bsq_ec_params> ep(n);
    std::vector<bsq_ec_result> eo(n);
    for (uint32_t i = 0; i < n; i++) {
      Job* j = js[i];
      ids[i] = j->sample;
      ep[i] = j->desc.ec;
      const uint32_t R = ep[i].n_read_files, Q = ep[i].n_quality;
      const uint32_t G = j->desc.ref->n_coverage_groups;
      j->counts.assign((size_t)R * 25 * Q, 0);
      j->hist.assign((size_t)G * j->desc.hist_capacity, 0);
      j->hist_size.assign(G, 0);
      memset(&eo[i], 0, sizeof eo[i]);
      eo[i].counts = j->counts.data();
      eo[i].coverage_hist = j->hist.data();
      eo[i].hist_capacity = j->desc.hist_capacity;
      eo[i].hist_size = j->hist_size.data();
    }
    auto tick = [](Clock::time_point& t) {
      const Clock::time_point now = Clock::now();
      const double d = std::chrono::duration<double, std::milli>(now - t).count();
      t = now;
      return d;
    };
    Clock::time_point tp = Clock::now();
    double ph[4] = {0, 0, 0, 0};
    int rc = bsq_error_count_batch(ctx, n, ids.data(), ep.data(), eo.data());
    if (rc != BSQ_OK) { e = std::string("error_count: ") + bsq_last_error(ctx); return rc; }
    ph[0] = tick(tp);
    std::vector<bsq_im_params> ip(n);
    std::vector<const double*> tabs(n);
    std::vector<const uint64_t*> cptr(n);
    std::vector<double*> tptr(n);
    std::vector<uint32_t> Rs(n), Qs(n);
    for (uint32_t i = 0; i < n; i++) {
      Job* j = js[i];
      const uint32_t R = j->desc.im.n_read_files, Q = j->desc.im.n_quality;
      if (R != ep[i].n_read_files || Q != ep[i].n_quality) { e = "error table dimensions differ between passes"; return BSQ_ERR_INVALID; }
      j->table.assign((size_t)R * 25 * Q, 0.0);
      cptr[i] = j->counts.data(); tptr[i] = j->table.data(); Rs[i] = R; Qs[i] = Q;
      ip[i] = j->desc.im;
      ip[i].precision = precision;
      tabs[i] = j->table.data();
    }
    rc = bsq_counts_to_log10_prob_batch(n, cptr.data(), Rs.data(), Qs.data(), tptr.data());
    if (rc != BSQ_OK) { e = "counts_to_log10_prob failed"; return rc; }
    ph[1] = tick(tp);
    rc = bsq_identify_mutations_batch(ctx, n, ids.data(), ip.data(), tabs.data(), nullptr);
    if (rc != BSQ_OK) { e = std::string("identify_mutations: ") + bsq_last_error(ctx); return rc; }
    ph[2] = tick(tp);
    for (uint32_t i = 0; i < n; i++) {
      Job* j = js[i];
      uint64_t a = 0, b = 0, c = 0;
      bsq_im_batch_result_counts(ctx, i, &a, &b, &c);
      j->ra.resize(a); j->mc.resize(b); j->un.resize(c);
      rc = bsq_im_batch_result_copy(ctx, i, j->ra.data(), a, j->mc.data(), b, j->un.data(), c);
      if (rc != BSQ_OK) { e = "result copy failed"; return rc; }
    }
    ph[3] = tick(tp);
    std::lock_guard<std::mutex> lk(mu);
    for (int k = 0; k < 4; k++) phase_ms[k] += ph[k];
    return BSQ_OK;
  }

  void gpu_loop() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      cv_ready.wait(lk, [&] { return !ready.empty() || (stop && pending == 0); });
      if (ready.empty()) return;
      // A round of one or two jobs while others are still uploading pays a round's fixed costs (and
      // the wait of passes beside uploads) for little work: give the uploads up to kJoinMs to join it.
      if (ready.size() < kMinRound && loading > 0)
        cv_ready.wait_for(lk, std::chrono::milliseconds(kJoinMs),
                          [&] { return ready.size() >= kMinRound || loading == 0 || stop; });
      if (tune_pending) {
        // passes run without graph capture here: captures were measured to wait behind the
        // admission threads' uploads (tens of ms), and rounds are large enough not to need graphs
        bsq_tuning t = tune;
        t.use_graphs = 0;
        bsq_set_tuning(ctx, &t);
        tune_pending = false;
      }
      std::vector<Job*> js;
      while (!ready.empty() && js.size() < max_batch) { js.push_back(ready.front()); ready.pop_front(); }
      const Clock::time_point ts = Clock::now();
      for (Job* j : js) { j->state = BSQ_JOB_RUNNING; j->t_start = ts; j->round_jobs = (uint32_t)js.size(); }
      if (js.size() > max_round_jobs) max_round_jobs = (uint32_t)js.size();
      lk.unlock();
      std::string e;
      int rc = run_round(js, e);
      std::vector<int> rcs(js.size(), rc);
      std::vector<std::string> es(js.size(), e);
      if (rc != BSQ_OK && js.size() > 1) {
        for (size_t i = 0; i < js.size(); i++) {
          std::vector<Job*> one{js[i]};
          rcs[i] = run_round(one, es[i]);
        }
      }
      const Clock::time_point tf = Clock::now();
      for (Job* j : js) bsq_free_sample(ctx, j->sample);
      const Clock::time_point te = Clock::now();
      lk.lock();
      phase_ms[4] += std::chrono::duration<double, std::milli>(te - tf).count();
      gpu_busy_ms += std::chrono::duration<double, std::milli>(te - ts).count();
      rounds++;
      for (size_t i = 0; i < js.size(); i++) {
        resident--;
        finish(js[i], rcs[i] == BSQ_OK ? BSQ_JOB_DONE : rcs[i], rcs[i] == BSQ_OK ? std::string() : es[i]);
      }
    }
  }

  Job* find(uint64_t id) {   // mu held
    auto it = jobs.find(id);
    return it == jobs.end() ? nullptr : it->second.get();
  }

  void info(const Job* j, bsq_job_info* o) const {
    memset(o, 0, sizeof *o);
    o->state = j->state;
    o->round_jobs = j->round_jobs;
    o->footprint = j->footprint;
    o->n_ra = j->ra.size(); o->n_mc = j->mc.size(); o->n_un = j->un.size();
    o->read_bases = j->read_bases;
    o->submit_ms = ms(j->t_submit);
    if (j->state >= BSQ_JOB_LOADING || j->state < 0) o->admit_ms = ms(j->t_admit);
    if (j->state >= BSQ_JOB_READY) o->ready_ms = ms(j->t_ready);
    if (j->state >= BSQ_JOB_RUNNING) o->start_ms = ms(j->t_start);
    if (j->state == BSQ_JOB_DONE || j->state < 0) o->done_ms = ms(j->t_done);
  }
};

extern "C" {

uint64_t bsq_job_footprint(const bsq_reference* ref, const bsq_read_soa* reads) {
  if (!ref || !reads) return 0;
  const uint64_t cols = ref->target_offset[ref->n_targets] + ref->n_targets;
  // pass buffers per column: coverage (32 B) + call (16 B) records, candidate list, interval marks
  // and their compacted copies (1 + 4 + 32 + 16 B), pass-1 difference arrays and read-start flags
  return bsq_sample_footprint(ref, reads) + cols * (32 + 16 + 4 + 1 + 4 + 32 + 16 + 8 + 2) + (1u << 20);
}

int bsq_server_create(bsq_server** out, int device, uint64_t budget, uint32_t max_batch_jobs, int32_t precision) {
  if (!out || budget == 0 || (precision != BSQ_PRECISION_FP64 && precision != BSQ_PRECISION_FP32C))
    return BSQ_ERR_INVALID;
  *out = nullptr;
  std::unique_ptr<bsq_server> s(new bsq_server());
  const int rc = bsq_create(&s->ctx, device);
  if (rc != BSQ_OK) return rc;
  s->budget = budget;
  s->max_batch = max_batch_jobs ? max_batch_jobs : 64;
  s->precision = precision;
  s->t0 = Clock::now();
  bsq_get_tuning(s->ctx, &s->tune);
  s->tune_pending = true;   // graph capture off from the first round (see gpu_loop)
  bsq_server* p = s.get();
  for (int i = 0; i < bsq_server::kLoaders; i++) s->admitters.emplace_back([p] { p->admit_loop(); });
  s->gpu = std::thread([p] { p->gpu_loop(); });
  *out = s.release();
  return BSQ_OK;
}

void bsq_server_destroy(bsq_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_admit.notify_all();
  s->cv_ready.notify_all();
  {
    // queued jobs still run: wait until nothing is pending
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->pending == 0; });
  }
  s->cv_admit.notify_all();
  s->cv_ready.notify_all();
  for (std::thread& t : s->admitters) t.join();
  s->gpu.join();
  bsq_destroy(s->ctx);
  delete s;
}

const char* bsq_server_last_error(const bsq_server* s) { return s ? s->err.c_str() : "null server"; }

int bsq_server_submit(bsq_server* s, const bsq_job* job, uint64_t* id) {
  if (!s || !job || !id || !job->ref || !job->reads || !job->im.deletion_propagation_cutoff ||
      !job->im.deletion_seed_cutoff || job->hist_capacity == 0)
    return BSQ_ERR_INVALID;
  std::unique_ptr<Job> j(new Job());
  j->desc = *job;
  j->footprint = bsq_job_footprint(job->ref, job->reads);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) { s->err = "server is stopping"; return BSQ_ERR_INVALID; }
  if (j->footprint > s->budget) { s->err = "job footprint exceeds the HBM budget"; return BSQ_ERR_NOMEM; }
  j->id = s->next_id++;
  j->t_submit = Clock::now();
  *id = j->id;
  s->queued.push_back(j.get());
  s->jobs[j->id] = std::move(j);
  s->pending++;
  s->cv_admit.notify_all();
  return BSQ_OK;
}

int bsq_server_wait(bsq_server* s, uint64_t id, int64_t timeout_ms, bsq_job_info* info) {
  if (!s) return BSQ_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  if (!j) return BSQ_ERR_INVALID;
  auto done = [&] { return j->state == BSQ_JOB_DONE || j->state < 0; };
  if (timeout_ms < 0) s->cv_done.wait(lk, done);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) return BSQ_ERR_TIMEOUT;
  if (info) s->info(j, info);
  return BSQ_OK;
}

int bsq_server_job_info(bsq_server* s, uint64_t id, bsq_job_info* info) {
  if (!s || !info) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  if (!j) return BSQ_ERR_INVALID;
  s->info(j, info);
  return BSQ_OK;
}

const char* bsq_server_job_error(bsq_server* s, uint64_t id) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  return j ? j->err.c_str() : "unknown job";
}

int bsq_server_error_counts(bsq_server* s, uint64_t id, uint64_t* counts, uint64_t* hist, uint32_t* hist_size) {
  if (!s) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  if (!j || j->state != BSQ_JOB_DONE) return BSQ_ERR_INVALID;
  if (counts) memcpy(counts, j->counts.data(), j->counts.size() * 8);
  if (hist) memcpy(hist, j->hist.data(), j->hist.size() * 8);
  if (hist_size) memcpy(hist_size, j->hist_size.data(), j->hist_size.size() * 4);
  return BSQ_OK;
}

int bsq_server_results(bsq_server* s, uint64_t id, bsq_ra_record* ra, uint64_t ra_cap, bsq_mc_record* mc,
                       uint64_t mc_cap, bsq_un_record* un, uint64_t un_cap) {
  if (!s) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  if (!j || j->state != BSQ_JOB_DONE) return BSQ_ERR_INVALID;
  if ((ra && ra_cap < j->ra.size()) || (mc && mc_cap < j->mc.size()) || (un && un_cap < j->un.size()))
    return BSQ_ERR_SIZE;
  if (ra) std::copy(j->ra.begin(), j->ra.end(), ra);
  if (mc) std::copy(j->mc.begin(), j->mc.end(), mc);
  if (un) std::copy(j->un.begin(), j->un.end(), un);
  return BSQ_OK;
}

int bsq_server_release(bsq_server* s, uint64_t id) {
  if (!s) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  Job* j = s->find(id);
  if (!j || !(j->state == BSQ_JOB_DONE || j->state < 0)) return BSQ_ERR_INVALID;
  s->jobs.erase(id);
  return BSQ_OK;
}

int bsq_server_set_tuning(bsq_server* s, const bsq_tuning* t) {
  if (!s || !t) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->tune = *t;
  s->tune_pending = true;
  return BSQ_OK;
}

int bsq_server_get_stats(bsq_server* s, bsq_server_stats* o) {
  if (!s || !o) return BSQ_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(o, 0, sizeof *o);
  o->jobs_done = s->jobs_done; o->rounds = s->rounds; o->budget = s->budget; o->in_use = s->in_use;
  o->peak_in_use = s->peak_in_use; o->max_round_jobs = s->max_round_jobs; o->max_resident_jobs = s->max_resident;
  o->gpu_busy_ms = s->gpu_busy_ms;
  for (int k = 0; k < 5; k++) o->phase_ms[k] = s->phase_ms[k];
  return BSQ_OK;
}

}  // extern "C"
