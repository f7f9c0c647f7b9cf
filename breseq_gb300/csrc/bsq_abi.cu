// C ABI of libbsq_gb300.so (include/breseq_gb300.h): sample residency, the two passes, and the
// host-side steps that follow the kernels (RA assembly with Fisher / K-S, MC and UN intervals).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "bsq_common.h"
#include "bsq_host.h"
#include "bsq_kernels.h"
#include "bsq_noalloc.h"
#include "bsq_softclip.h"
#include "bsq_covtable.h"
#include "bsq_bam.h"
#include "bsq_pairs.h"

using namespace bsq;

namespace {

// Device buffer from the device's stream-ordered pool: the context keeps the pool's memory instead of
// returning it to the driver, so loading and freeing samples per job costs no cudaMalloc/cudaFree.
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() { if (p) cudaFreeAsync(p, st); p = nullptr; bytes = 0; }
  cudaError_t alloc(size_t n, cudaStream_t stream) {
    if (n == 0) n = 16;
    if (p && bytes >= n) return cudaSuccess;
    release();
    st = stream;
    cudaError_t e = cudaMallocAsync(&p, n, stream);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

struct SampleDev {
  DevMem ref, refnib, reads, x1, rg, qb, cigar, seq, qual, tile_range, d_tpoff, tgt_group, tgt_called, tgt_failed, rstart,
      mapq;
  // pair annotations for the discordant / missing-pair scans: raw flags, XP codes, TLEN, names
  DevMem pflag, pxp, pisize, pqoff, pqname, pmtid, pmpos;
  bool has_pairs = false, has_mates = false;
  // per-base class bytes (base_code_kernel); usable by the passes when no base but N has a quality
  // above kCodeMaxQ (code_ok), and for a call whose quality range is above max_q (the largest such)
  DevMem code;
  bool code_ok = false;
  uint32_t max_q = 0;
  // tiles with long read ranges, which the column pass runs first
  DevMem heavy, heavy_bits;
  uint32_t n_heavy = 0;
  uint32_t n_targets = 0, n_cols = 0, n_tiles = 0, n_reads = 0, maxspan = 1, max_tile_reads = 0;
  uint32_t n_groups = 0;
  std::vector<uint64_t> toff;       // caller's target offsets
  std::vector<uint32_t> tpoff;      // padded offsets
  std::vector<uint32_t> order;      // pileup order
  std::vector<uint32_t> group;
  std::vector<uint8_t> mapq_values; // distinct MAPQ values, index = mapq_idx
};

// Page-locked host staging: a pass's inputs go to the device in one copy and its small results come
// back in one copy, both graph-capturable.
struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() { if (p) cudaFreeHost(p); }
  cudaError_t reserve(size_t n) {
    if (p && bytes >= n) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    // geometric growth: a pinned allocation can wait behind other threads' transfers, so it
    // should happen rarely
    const size_t want = std::max<size_t>(n + n / 4 + 4096, std::max<size_t>(2 * bytes, size_t(8) << 20));
    cudaError_t e = cudaMallocHost(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  unsigned char* at(size_t off) const { return static_cast<unsigned char*>(p) + off; }
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

struct bsq_ctx {
  int device = 0;
  int sms = 1;
  cudaStream_t stream = nullptr;        // the passes
  // sample uploads run on their own streams, beside the passes; concurrent loads (loader threads)
  // take the streams round robin
  static constexpr int kLoadStreams = 8;
  cudaStream_t load_streams[kLoadStreams] = {};
  std::atomic<uint32_t> load_rr{0};
  std::mutex mu;                        // guards `samples` and `next_id`
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm0 = nullptr, evm1 = nullptr, evt0 = nullptr, evt1 = nullptr;
  std::map<int32_t, std::unique_ptr<SampleDev>> samples;
  int32_t next_id = 1;
  // working memory reused across calls
  DevMem cov, call, blk, cand, next, ra, qhist, scratch, bq, pool;
  DevMem keep, kcol, kcov, kcall;
  DevMem d_chunks, ec_arena, im_arena, ctl;
  PinnedBuf pin_in, pin_out;
  // page-locked landing areas of device-to-host reads that run beside other threads' work: a read into
  // pageable memory is staged by the CUDA driver, and such reads wait for one another across streams (an
  // upload's check would hold up a pass's results until the upload ends)
  PinnedBuf pin_res;                    // pass 2's RA items, quality histograms and kept columns
  static constexpr uint32_t kStatSlots = 64;
  PinnedBuf pin_stats;                  // kStatSlots x 64 bytes: a load's packing statistics
  std::atomic<uint32_t> stat_rr{0};
  bsq_tuning tune = {1024, 8, 8, 16, 4, 1};
  cudaGraphExec_t exec_ec = nullptr, exec_im = nullptr;
  uint64_t graph_instantiations = 0, graph_updates = 0;
  std::vector<std::vector<bsq_ra_record>> res_ra;
  std::vector<std::vector<bsq_mc_record>> res_mc;
  std::vector<std::vector<bsq_un_record>> res_un;
  // soft-clipping tabulation: working buffers and the rows of the last call
  DevMem sc_diff, sc_cnt, sc_blk, sc_tot, sc_rows, sc_outs, sc_tails, sc_ev, sc_ev_n;
  // coverage table of a region
  DevMem ct_diff, ct_blk, ct_counts, ct_red, ct_stat, ct_gather;
  // discordant / missing-pair scans
  DevMem pr_code, pr_group, pr_sel, pr_mem, pr_evoff, pr_memoff, pr_tmp, pr_tot, pr_map, pr_ev, pr_names, pr_mstart,
      pr_mkey;
  host::PairReplayResult pair_res;
  DevMem pd_diff, pd_blk, pd_mask, pd_hist, pd_ladder, pd_above, pd_cnt, pd_cdf, pd_cdfoff, pd_cdflen, pd_orient,
      pd_piled;
  host::PdResult pd_res;
  std::vector<bsq_sc_position> sc_res;
  double last_ms = 0, main_ms = 0;
  uint32_t launches = 0;
  uint64_t last_h2d = 0, last_d2h = 0;   // bytes the last pass call copied each way
  uint64_t last_candidates = 0;
};

// The message of the last failed call, per calling thread: a loader thread and the pass thread can
// share one context without overwriting each other's message.
static thread_local std::string t_err;

static int fail(bsq_ctx*, int code, const std::string& msg) {
  t_err = msg;
  return code;
}
#define CK(call)                                                                                          \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) return fail(ctx, BSQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static std::string err_text(uint32_t e) {
  std::string s;
  if (e & kErrCovariate) s += "covariate value exceeds the error table (quality >= Q or read file >= R); ";
  if (e & kErrBase) s += "unrecognised base code; ";
  if (e & kErrBounds) s += "read offsets / lengths / trims out of range; ";
  if (e & kErrOrder) s += "records not coordinate-sorted or invalid tid/pos; ";
  if (e & kErrCigar) s += "CIGAR does not match the read or runs past the target; ";
  if (e & kErrScratch) s += "candidate gather buffer overflow; ";
  if (e & kErrRaOverflow) s += "RA buffer overflow; ";
  if (e & kErrX1) s += "X1 redundancy of 0; ";
  return s;
}

template <class T>
static cudaError_t upload(DevMem& m, const T* src, uint64_t n, cudaStream_t st) {
  cudaError_t e = m.alloc(n * sizeof(T) + 16, st);
  if (e != cudaSuccess) return e;
  if (n) e = cudaMemcpyAsync(m.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st);
  return e;
}

static DevSample make_dev_sample(const SampleDev& s) {
  DevSample S;
  S.ref = s.ref.as<uint8_t>();
  S.refnib = s.refnib.as<unsigned long long>();
  S.reads = s.reads.as<DevRead>();
  S.x1 = s.x1.as<uint32_t>();
  S.rg = s.rg.as<uint16_t>();
  S.qb = s.qb.as<QBounds>();
  S.cigar = s.cigar.as<uint32_t>();
  S.seq = s.seq.as<uint8_t>();
  S.qual = s.qual.as<uint8_t>();
  S.code = nullptr;                 // set per call by the column pass's job setup
  S.tile_range = s.tile_range.as<uint2>();
  S.heavy = s.heavy.as<uint32_t>();
  S.heavy_bits = s.heavy_bits.as<uint32_t>();
  S.tpoff = s.d_tpoff.as<uint32_t>();
  S.tgt_group = s.tgt_group.as<uint32_t>();
  S.tgt_called = s.tgt_called.as<uint8_t>();
  S.tgt_failed = s.tgt_failed.as<uint8_t>();
  S.n_cols = s.n_cols;
  S.n_tiles = s.n_tiles;
  S.n_reads = s.n_reads;
  S.n_targets = s.n_targets;
  S.maxspan = s.maxspan;
  return S;
}

static SampleDev* find_sample(bsq_ctx* ctx, int32_t id) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto it = ctx->samples.find(id);
  return it == ctx->samples.end() ? nullptr : it->second.get();
}

// Runs `enqueue` on the context's stream.  With graphs on, the work is captured and launched as one
// CUDA graph; the executable graph is kept and updated in place for the next call of the same shape
// (the node list of a pass does not depend on the number of jobs), else instantiated anew.
// f(0..n-1) on up to 16 host threads (the calling thread included); items are independent.
template <class F>
static void parallel_for(uint32_t n, F&& f) {
  const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
  const uint32_t nt = std::min<uint32_t>(n, std::min<uint32_t>(hw, 16));
  if (nt <= 1) {
    for (uint32_t i = 0; i < n; i++) f(i);
    return;
  }
  std::atomic<uint32_t> next{0};
  auto work = [&]() { for (uint32_t i; (i = next.fetch_add(1)) < n;) f(i); };
  std::vector<std::thread> th;
  for (uint32_t t = 1; t < nt; t++) th.emplace_back(work);
  work();
  for (std::thread& t : th) t.join();
}

// Timing event inside a pass: recorded as an event node when the pass is captured (a plain record
// in a capture only orders the capture and is never recorded).
static cudaError_t record(cudaEvent_t ev, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
    return cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
  return cudaEventRecord(ev, st);
}

// Device time between two events of the last pass, 0 when unavailable.
static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) { cudaGetLastError(); ms = 0; }
  return ms;
}

template <class F>
static cudaError_t run_pass(bsq_ctx* ctx, cudaGraphExec_t& exec, F&& enqueue, std::string& where) {
  cudaGetLastError();   // a launch reports through cudaGetLastError: start from a clean slate
  if (!ctx->tune.use_graphs) { where = "launch"; return enqueue(); }
  cudaStream_t st = ctx->stream;
  where = "begin capture";
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  const cudaError_t ee = enqueue();
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(st, &g);
  if (ee != cudaSuccess || e != cudaSuccess) {
    where = ee != cudaSuccess ? "capture" : "end capture";
    if (g) cudaGraphDestroy(g);
    return ee != cudaSuccess ? ee : e;
  }
  if (exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(exec, g, &info) == cudaSuccess) {
      ctx->graph_updates++;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
  }
  if (!exec) {
    where = "instantiate";
    e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) { exec = nullptr; cudaGraphDestroy(g); return e; }
    ctx->graph_instantiations++;
  }
  cudaGraphDestroy(g);
  where = "graph launch";
  return cudaGraphLaunch(exec, st);
}

extern "C" {

const char* bsq_version(void) { return "breseq_gb300 0.1 (sm_103a)"; }

int bsq_create(bsq_ctx** out, int device) {
  if (!out) return BSQ_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return BSQ_ERR_CUDA;
  if (device < 0 || device >= n) return BSQ_ERR_INVALID;
  std::unique_ptr<bsq_ctx> c(new bsq_ctx());
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) return BSQ_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BSQ_ERR_CUDA;
  c->sms = prop.multiProcessorCount;
  // the passes' stream first in line for SMs; uploads (copies plus small packing kernels) behind it
  int prio_low = 0, prio_high = 0;
  if (cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess) prio_low = prio_high = 0;
  if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_high) != cudaSuccess) return BSQ_ERR_CUDA;
  for (cudaStream_t& ls : c->load_streams)
    if (cudaStreamCreateWithPriority(&ls, cudaStreamNonBlocking, prio_low) != cudaSuccess) return BSQ_ERR_CUDA;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;   // keep freed blocks in this process's pool for the next sample
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  // pinned staging reserved now, before any upload runs beside it (see PinnedBuf::reserve)
  if (c->pin_in.reserve(8u << 20) != cudaSuccess || c->pin_out.reserve(8u << 20) != cudaSuccess ||
      c->pin_res.reserve(16u << 20) != cudaSuccess || c->pin_stats.reserve(bsq_ctx::kStatSlots * 64) != cudaSuccess)
    return BSQ_ERR_CUDA;
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->evm0) != cudaSuccess || cudaEventCreate(&c->evm1) != cudaSuccess ||
      cudaEventCreate(&c->evt0) != cudaSuccess || cudaEventCreate(&c->evt1) != cudaSuccess)
    return BSQ_ERR_CUDA;
  *out = c.release();
  return BSQ_OK;
}

void bsq_destroy(bsq_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (cudaStream_t ls : ctx->load_streams) if (ls) cudaStreamSynchronize(ls);
  ctx->samples.clear();
  // pool blocks are returned on the context's stream, so before it goes
  for (DevMem* m : {&ctx->cov, &ctx->call, &ctx->blk, &ctx->cand, &ctx->next, &ctx->ra, &ctx->bq, &ctx->pool,
                    &ctx->qhist, &ctx->scratch, &ctx->keep, &ctx->kcol, &ctx->kcov, &ctx->kcall,
                    &ctx->d_chunks, &ctx->ec_arena, &ctx->im_arena, &ctx->ctl, &ctx->sc_diff, &ctx->sc_cnt,
                    &ctx->sc_blk, &ctx->sc_tot, &ctx->sc_rows, &ctx->sc_outs, &ctx->sc_tails, &ctx->sc_ev,
                    &ctx->sc_ev_n, &ctx->ct_diff, &ctx->ct_blk, &ctx->ct_counts, &ctx->ct_red, &ctx->ct_stat,
                    &ctx->ct_gather, &ctx->pr_code, &ctx->pr_group, &ctx->pr_sel, &ctx->pr_mem, &ctx->pr_evoff,
                    &ctx->pr_memoff, &ctx->pr_tmp, &ctx->pr_tot, &ctx->pr_map, &ctx->pr_ev, &ctx->pr_names,
                    &ctx->pr_mstart, &ctx->pr_mkey, &ctx->pd_diff, &ctx->pd_blk, &ctx->pd_mask, &ctx->pd_hist,
                    &ctx->pd_ladder, &ctx->pd_above, &ctx->pd_cnt, &ctx->pd_cdf, &ctx->pd_cdfoff, &ctx->pd_cdflen,
                    &ctx->pd_orient, &ctx->pd_piled})
    m->release();
  if (ctx->exec_ec) cudaGraphExecDestroy(ctx->exec_ec);
  if (ctx->exec_im) cudaGraphExecDestroy(ctx->exec_im);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaEventDestroy(ctx->ev0); cudaEventDestroy(ctx->ev1); cudaEventDestroy(ctx->evm0); cudaEventDestroy(ctx->evm1);
  cudaEventDestroy(ctx->evt0); cudaEventDestroy(ctx->evt1);
  for (cudaStream_t ls : ctx->load_streams) if (ls) cudaStreamSynchronize(ls);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  for (cudaStream_t ls : ctx->load_streams) if (ls) cudaStreamDestroy(ls);
  delete ctx;
}

const char* bsq_last_error(const bsq_ctx* ctx) { return ctx ? t_err.c_str() : "null context"; }

uint64_t bsq_sample_footprint(const bsq_reference* ref, const bsq_read_soa* rd) {
  if (!ref || !rd) return 0;
  const uint64_t cols = ref->target_offset[ref->n_targets] + ref->n_targets;
  const uint64_t tiles = (cols + 31) / 32;
  const uint64_t per_read = sizeof(DevRead) + 4 + 2 + sizeof(QBounds) + 4 + 1;
  const uint64_t upload_tmp = rd->n_reads * 48;  // raw arrays, freed after packing
  // pair annotations stay resident: flag, XP, TLEN, name offsets and names
  const uint64_t pairs = (rd->xp && rd->isize && rd->qname_off && rd->qname)
                             ? rd->n_reads * 15 + 8 + (rd->n_reads ? rd->qname_off[rd->n_reads] : 0)
                             : 0;
  // bases: packed nibbles, qualities and the column pass's class bytes
  return 2 * (cols + 64) + rd->n_reads * per_read + rd->n_cigar_total * 4 + rd->n_bases_total / 2 + 16 +
         2 * rd->n_bases_total + 48 + tiles * 13 + 192 + upload_tmp + pairs;   // tiles: range, heavy list and bits
}

}  // extern "C"

// The record arrays of a sample on the device, in the bsq_read_soa layout, before packing.
struct RecordsDev {
  DevMem tid, pos, flag, mapq, x1, xl, xr, rfile, rg, lq, soff, coff, nc, cigar, seq, qual, xj;
  DevMem isize, xp, qoff, qname;   // pair annotations (has_pairs)
  DevMem mtid, mpos;               // mate positions (has_mates)
  uint64_t n = 0, n_cigar_total = 0, n_bases_total = 0;
  bool has_xj = false, has_pairs = false, has_mates = false;
};

static void take(DevMem& to, DevMem& from) {
  to.release();
  to.p = from.p; to.bytes = from.bytes; to.st = from.st;
  from.p = nullptr; from.bytes = 0;
}

// A new sample's reference side: target offsets, coverage groups, the pileup set, and the padded
// reference uploaded on stream st.
static int new_sample(bsq_ctx* ctx, const bsq_reference* ref, uint64_t n_reads, std::unique_ptr<SampleDev>& out,
                      cudaStream_t st) {
  const uint32_t T = ref->n_targets;
  if (T == 0 || !ref->target_offset || !ref->seq || !ref->coverage_group || !ref->target_order)
    return fail(ctx, BSQ_ERR_INVALID, "reference without targets");
  const uint64_t total = ref->target_offset[T];
  if (total + T >= 0xFFFFFF00ull) return fail(ctx, BSQ_ERR_INVALID, "reference longer than 2^32 - 256 columns");
  if (n_reads >= 0xFFFFFFFFull) return fail(ctx, BSQ_ERR_INVALID, "more than 2^32 - 1 records in one sample");
  std::unique_ptr<SampleDev> s(new SampleDev());
  s->n_targets = T;
  s->toff.assign(ref->target_offset, ref->target_offset + T + 1);
  s->tpoff.resize(T + 1);
  for (uint32_t t = 0; t <= T; t++) {
    if (t > 0 && s->toff[t] < s->toff[t - 1]) return fail(ctx, BSQ_ERR_INVALID, "target offsets not increasing");
    s->tpoff[t] = (uint32_t)(s->toff[t] + t);
  }
  s->n_cols = s->tpoff[T];
  s->n_tiles = (s->n_cols + 31) / 32;
  s->n_reads = (uint32_t)n_reads;
  s->group.assign(ref->coverage_group, ref->coverage_group + T);
  s->n_groups = ref->n_coverage_groups;
  for (uint32_t t = 0; t < T; t++)
    if (s->group[t] >= s->n_groups) return fail(ctx, BSQ_ERR_INVALID, "coverage group out of range");
  s->order.assign(ref->target_order, ref->target_order + ref->n_target_order);
  std::vector<uint8_t> called(T, 0);
  for (uint32_t t : s->order) {
    if (t >= T) return fail(ctx, BSQ_ERR_INVALID, "target_order entry out of range");
    called[t] = 1;
  }
  // reference, one '\0' separator after each target
  CK(s->ref.alloc(s->n_cols + 64, st));
  CK(cudaMemsetAsync(s->ref.p, 0, s->n_cols + 64, st));
  for (uint32_t t = 0; t < T; t++) {
    const uint64_t len = s->toff[t + 1] - s->toff[t];
    if (len) CK(cudaMemcpyAsync(s->ref.as<uint8_t>() + s->tpoff[t], ref->seq + s->toff[t], len, cudaMemcpyHostToDevice, st));
  }
  CK(upload(s->d_tpoff, s->tpoff.data(), T + 1, st));
  CK(upload(s->tgt_group, s->group.data(), T, st));
  CK(upload(s->tgt_called, called.data(), T, st));
  CK(s->tgt_failed.alloc(T + 16, st));
  CK(cudaMemsetAsync(s->tgt_failed.p, 0, T, st));
  out = std::move(s);
  return BSQ_OK;
}

// Packs and validates the records (sorted, CIGAR consumes the reference, offsets inside the arrays),
// checks the reference characters, builds the MAPQ classes and tile read ranges, and registers the
// sample.  The arrays the passes keep move into the sample.
static int pack_sample(bsq_ctx* ctx, std::unique_ptr<SampleDev>& s, RecordsDev& R, cudaStream_t st, int32_t* sample_id) {
  const uint32_t T = s->n_targets;
  const uint64_t n = R.n;
  take(s->mapq, R.mapq);
  take(s->x1, R.x1);
  take(s->rg, R.rg);
  take(s->cigar, R.cigar);
  take(s->seq, R.seq);
  take(s->qual, R.qual);
  CK(s->reads.alloc(n * sizeof(DevRead) + 64, st));
  CK(s->qb.alloc(n * sizeof(QBounds) + 64, st));
  CK(s->rstart.alloc(n * 4 + 64, st));
  DevMem dstats;
  CK(dstats.alloc(64, st));
  CK(cudaMemsetAsync(dstats.p, 0, 64, st));
  uint32_t* stats = dstats.as<uint32_t>();  // [0] err, [1] maxspan, [2..9] mapq mask, [10] max tile reads
  RawSoA in;
  in.tid = R.tid.as<int32_t>(); in.pos = R.pos.as<int32_t>(); in.flag = R.flag.as<uint16_t>(); in.mapq = s->mapq.as<uint8_t>();
  in.x1 = s->x1.as<uint32_t>(); in.xl = R.xl.as<int32_t>(); in.xr = R.xr.as<int32_t>(); in.read_file = R.rfile.as<uint8_t>();
  in.l_qseq = R.lq.as<uint32_t>(); in.seq_off = R.soff.as<uint64_t>(); in.cigar_off = R.coff.as<uint64_t>();
  in.n_cigar = R.nc.as<uint16_t>(); in.cigar = s->cigar.as<uint32_t>(); in.tpoff = s->d_tpoff.as<uint32_t>(); in.called = s->tgt_called.as<uint8_t>();
  in.xj = R.has_xj ? R.xj.as<uint8_t>() : nullptr;
  in.xp = R.has_pairs ? R.xp.as<uint8_t>() : nullptr;
  in.n = (uint32_t)n; in.n_targets = T; in.n_bases = R.n_bases_total; in.n_cigar_total = R.n_cigar_total;
  PackOut po;
  po.reads = s->reads.as<DevRead>(); po.qb = s->qb.as<QBounds>(); po.rstart = s->rstart.as<uint32_t>();
  po.mapq = s->mapq.as<uint8_t>(); po.err = stats; po.maxspan = stats + 1; po.mapq_mask = stats + 2;
  CK(launch_pack(in, po, st));
  // the column pass's per-base class bytes: [13] a quality too large for them, [14] the largest quality
  CK(s->code.alloc((R.n_bases_total + 15) / 16 * 16 + 16, st));
  CK(launch_base_code(s->seq.as<uint8_t>(), s->qual.as<uint8_t>(), R.n_bases_total, s->code.as<uint8_t>(), stats + 13,
                      ctx->sms, st));
  // the reference checked on the device: [11] bytes outside A/C/G/T/N, [12] zero bytes (separators)
  CK(s->refnib.alloc((size_t)refnib_words(s->n_cols) * 8, st));
  CK(launch_ref_check(s->ref.as<uint8_t>(), s->refnib.as<unsigned long long>(), s->n_cols, stats + 11, stats + 12,
                      ctx->sms, st));
  uint32_t* h = reinterpret_cast<uint32_t*>(ctx->pin_stats.at(64 * (ctx->stat_rr.fetch_add(1) % bsq_ctx::kStatSlots)));
  CK(cudaMemcpyAsync(h, stats, 16 * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h[11] || h[12] != T) return fail(ctx, BSQ_ERR_DATA, "reference base outside A/C/G/T/N");
  if (h[0]) return fail(ctx, (h[0] & (kErrOrder | kErrCigar | kErrBounds | kErrX1)) ? BSQ_ERR_INVALID : BSQ_ERR_DATA,
                        "invalid records: " + err_text(h[0]));
  s->maxspan = std::max<uint32_t>(1, h[1]);
  s->code_ok = h[13] == 0 && R.n_bases_total + 64 < (1ull << 32);   // 32-bit class-byte indices
  s->max_q = h[14];
  uint8_t map[256];
  memset(map, 0, sizeof map);
  for (int v = 0; v < 256; v++) {
    if (h[2 + (v >> 5)] & (1u << (v & 31))) { map[v] = (uint8_t)s->mapq_values.size(); s->mapq_values.push_back((uint8_t)v); }
  }
  if (s->mapq_values.empty()) s->mapq_values.push_back(0);
  DevMem dmap;
  CK(upload(dmap, map, 256, st));
  CK(launch_mapq_index(s->reads.as<DevRead>(), s->mapq.as<uint8_t>(), dmap.as<uint8_t>(), (uint32_t)n, st));
  CK(s->tile_range.alloc((size_t)s->n_tiles * sizeof(uint2) + 16, st));
  CK(cudaMemsetAsync(stats + 10, 0, 4, st));
  CK(launch_tile_range(s->rstart.as<uint32_t>(), (uint32_t)n, s->n_tiles, s->maxspan, s->tile_range.as<uint2>(), stats + 10, st));
  // heavy tiles: a read range above twice the expected n * (maxspan + 31) / columns reads ([15] counts)
  CK(s->heavy.alloc(((size_t)s->n_tiles + 16) * 4, st));
  CK(s->heavy_bits.alloc(((size_t)s->n_tiles / 32 + 16) * 4, st));
  const uint64_t expect = s->n_cols ? (uint64_t)n * (s->maxspan + 31) / s->n_cols : 0;
  CK(launch_tile_heavy(s->tile_range.as<uint2>(), s->n_tiles, (uint32_t)std::min<uint64_t>(2 * expect + 8, UINT32_MAX - 1),
                       s->heavy.as<uint32_t>(), s->heavy_bits.as<uint32_t>(), stats + 15, st));
  CK(cudaMemcpyAsync(h + 10, stats + 10, 6 * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  s->max_tile_reads = h[10];
  s->n_heavy = h[15];
  if (R.has_pairs) {
    take(s->pflag, R.flag);
    take(s->pxp, R.xp);
    take(s->pisize, R.isize);
    take(s->pqoff, R.qoff);
    take(s->pqname, R.qname);
    s->has_pairs = true;
  }
  if (R.has_mates) {
    take(s->pmtid, R.mtid);
    take(s->pmpos, R.mpos);
    s->has_mates = true;
  }
  std::lock_guard<std::mutex> lk(ctx->mu);
  const int32_t id = ctx->next_id++;
  ctx->samples[id] = std::move(s);
  *sample_id = id;
  return BSQ_OK;
}

extern "C" {

int bsq_load_sample(bsq_ctx* ctx, const bsq_reference* ref, const bsq_read_soa* rd, int32_t* sample_id) {
  if (!ctx || !ref || !rd || !sample_id) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  if (rd->n_reads && (!rd->tid || !rd->pos || !rd->flag || !rd->mapq || !rd->x1 || !rd->xl || !rd->xr ||
                      !rd->read_file || !rd->read_group || !rd->l_qseq || !rd->seq_off || !rd->cigar_off ||
                      !rd->n_cigar || !rd->cigar || !rd->seq || !rd->qual))
    return fail(ctx, BSQ_ERR_INVALID, "null record array");
  cudaStream_t st = ctx->load_streams[ctx->load_rr.fetch_add(1) % bsq_ctx::kLoadStreams];
  std::unique_ptr<SampleDev> s;
  int rc = new_sample(ctx, ref, rd->n_reads, s, st);
  if (rc != BSQ_OK) return rc;
  // records: raw arrays -> packed 32-byte records on the device
  const uint64_t n = rd->n_reads;
  RecordsDev R;
  R.n = n;
  R.n_cigar_total = rd->n_cigar_total;
  R.n_bases_total = rd->n_bases_total;
  CK(upload(R.tid, rd->tid, n, st));
  CK(upload(R.pos, rd->pos, n, st));
  CK(upload(R.flag, rd->flag, n, st));
  CK(upload(R.mapq, rd->mapq, n, st));
  CK(upload(R.x1, rd->x1, n, st));
  CK(upload(R.xl, rd->xl, n, st));
  CK(upload(R.xr, rd->xr, n, st));
  CK(upload(R.rfile, rd->read_file, n, st));
  CK(upload(R.rg, rd->read_group, n, st));
  CK(upload(R.lq, rd->l_qseq, n, st));
  CK(upload(R.soff, rd->seq_off, n, st));
  CK(upload(R.coff, rd->cigar_off, n, st));
  CK(upload(R.nc, rd->n_cigar, n, st));
  CK(upload(R.cigar, rd->cigar, rd->n_cigar_total, st));
  CK(upload(R.seq, rd->seq, (rd->n_bases_total + 1) / 2, st));
  CK(upload(R.qual, rd->qual, rd->n_bases_total, st));
  if (rd->xj) {
    CK(upload(R.xj, rd->xj, n, st));
    R.has_xj = true;
  }
  if (rd->isize || rd->xp || rd->qname_off || rd->qname) {
    if (!rd->isize || !rd->xp || !rd->qname_off || !rd->qname)
      return fail(ctx, BSQ_ERR_INVALID, "pair annotations need isize, xp, qname_off and qname together");
    for (uint64_t i = 0; i < n; i++)
      if (rd->qname_off[i + 1] < rd->qname_off[i] || rd->qname_off[i + 1] - rd->qname_off[i] > 254)
        return fail(ctx, BSQ_ERR_INVALID, "read name offsets decreasing or a name longer than 254 bytes");
    CK(upload(R.isize, rd->isize, n, st));
    CK(upload(R.xp, rd->xp, n, st));
    CK(upload(R.qoff, rd->qname_off, n + 1, st));
    CK(upload(R.qname, rd->qname, rd->qname_off[n], st));
    R.has_pairs = true;
  }
  if (rd->mtid || rd->mpos) {
    if (!rd->mtid || !rd->mpos) return fail(ctx, BSQ_ERR_INVALID, "mate positions need mtid and mpos together");
    CK(upload(R.mtid, rd->mtid, n, st));
    CK(upload(R.mpos, rd->mpos, n, st));
    R.has_mates = true;
  }
  return pack_sample(ctx, s, R, st, sample_id);
}

int bsq_free_sample(bsq_ctx* ctx, int32_t id) {
  if (!ctx) return BSQ_ERR_INVALID;
  std::unique_ptr<SampleDev> victim;
  {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->samples.find(id);
    if (it == ctx->samples.end()) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
    victim = std::move(it->second);
    ctx->samples.erase(it);
  }
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);   // no pass still reads it; its blocks go back on the load stream
  victim.reset();
  return BSQ_OK;
}

// ============================================================================ pass 1
// How many of the next samples form one launch group: at most kBatchJobs, and at most 2^31 columns
// and 2^31 reads in total so that batch-wide column, tile and read indices stay 32-bit.  A single
// sample is always a group of its own (its sizes were checked at load).  0 for an unknown id.
static uint32_t group_size(bsq_ctx* ctx, uint32_t left, const int32_t* ids) {
  uint64_t cols = 0, reads = 0;
  uint32_t k = 0;
  while (k < left && k < kBatchJobs) {
    const SampleDev* s = find_sample(ctx, ids[k]);
    if (!s) return k;   // the group stops before it; the pass reports the unknown id
    if (k > 0 && (cols + s->n_cols > (1ull << 31) || reads + s->n_reads > (1ull << 31))) break;
    cols += s->n_cols;
    reads += s->n_reads;
    k++;
  }
  return k;
}

// One group of at most kBatchJobs samples: one launch per kernel of pass 1.
//   device arena: [results of every job: counts | coverage hist | read-start tallies | error word]
//                 [work of every job: coverage difference arrays, read-start flags, block sums]
// zeroed by one memset; the result part comes back in one copy.
static int ec_group(bsq_ctx* ctx, uint32_t n, const int32_t* ids, const bsq_ec_params* P, bsq_ec_result* out) {
  std::vector<SampleDev*> smp(n);
  for (uint32_t j = 0; j < n; j++) {
    smp[j] = find_sample(ctx, ids[j]);
    if (!smp[j]) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
    if (P[j].n_read_files == 0 || P[j].n_read_files > 255 || P[j].n_quality == 0 || P[j].n_quality > 256)
      return fail(ctx, BSQ_ERR_INVALID, "covariate dimensions out of range");
    if ((size_t)P[j].n_read_files * 29 * P[j].n_quality * 4 > kEcMaxHistBytes)   // histogram + combined counts
      return fail(ctx, BSQ_ERR_SIZE, "covariate table larger than the shared-memory histogram of the pass-1 kernel");
  }
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const bsq_tuning& tn = ctx->tune;
  struct Lay { size_t counts, hist, found, err, diff_u, diff_r, qs, blk_u, blk_r; uint32_t cap; };
  std::vector<Lay> lay(n);
  std::vector<uint32_t> cblk(n + 1, 0);
  size_t off = 0;
  uint32_t max_bins = 0, max_code_r = 0;
  for (uint32_t j = 0; j < n; j++) {
    const SampleDev* s = smp[j];
    const size_t nbins = (size_t)P[j].n_read_files * 25 * P[j].n_quality;
    max_bins = std::max<uint32_t>(max_bins, (uint32_t)nbins);
    lay[j].cap = s->max_tile_reads + 2;
    lay[j].counts = off; off = align256(off + nbins * 8);
    lay[j].hist = off; off = align256(off + (size_t)s->n_groups * lay[j].cap * 8);
    lay[j].found = off; off = align256(off + (size_t)s->n_targets * 16);
    lay[j].err = off; off = align256(off + 8);
  }
  const size_t res_bytes = off;
  for (uint32_t j = 0; j < n; j++) {
    const SampleDev* s = smp[j];
    const uint32_t ncb = (s->n_cols + 1023) / 1024;
    lay[j].diff_u = off; off = align256(off + (size_t)(s->n_cols + 16) * 4);
    lay[j].diff_r = off; off = align256(off + (size_t)(s->n_cols + 16) * 4);
    lay[j].qs = off; off = align256(off + (size_t)2 * s->n_cols + 16);
    lay[j].blk_u = off; off = align256(off + (size_t)(ncb + 16) * 4);
    lay[j].blk_r = off; off = align256(off + (size_t)(ncb + 16) * 4);
    cblk[j + 1] = cblk[j] + ncb;
  }
  const size_t arena_bytes = off;
  CK(ctx->ec_arena.alloc(arena_bytes, st));
  unsigned char* A0 = ctx->ec_arena.as<unsigned char>();
  // work units: chunks of reads, tuned size
  const uint32_t chunk = std::max<uint32_t>(64, tn.ec_read_chunk);
  size_t n_chunks = 0;
  for (uint32_t j = 0; j < n; j++) n_chunks += (smp[j]->n_reads + chunk - 1) / chunk;
  CK(ctx->pin_in.reserve(std::max<size_t>(16, n_chunks * sizeof(uint4))));
  CK(ctx->pin_out.reserve(res_bytes));
  CK(ctx->d_chunks.alloc(std::max<size_t>(16, n_chunks * sizeof(uint4)), st));
  CK(ctx->next.alloc(16, st));
  uint4* ch = reinterpret_cast<uint4*>(ctx->pin_in.p);
  size_t c = 0;
  std::unique_ptr<Batch> Bp(new Batch());
  Batch& B = *Bp;
  memset(&B, 0, sizeof B);
  B.n_jobs = n;
  B.total_cblk = cblk[n];
  for (uint32_t j = 0; j < n; j++) {
    const SampleDev* s = smp[j];
    for (uint32_t r0 = 0; r0 < s->n_reads; r0 += chunk) ch[c++] = make_uint4(j, r0, std::min<uint32_t>(s->n_reads, r0 + chunk), 0);
    DevJob& J = B.jobs[j];
    J.S = make_dev_sample(*s);
    EcArgs& E = J.E;
    E.counts = reinterpret_cast<unsigned long long*>(A0 + lay[j].counts);
    E.cov_hist = reinterpret_cast<unsigned long long*>(A0 + lay[j].hist);
    E.found = reinterpret_cast<unsigned long long*>(A0 + lay[j].found);
    E.err = reinterpret_cast<uint32_t*>(A0 + lay[j].err);
    E.R = P[j].n_read_files; E.Q = P[j].n_quality; E.hist_cap = lay[j].cap;
    E.do_errors = P[j].do_errors; E.preprocess = P[j].preprocess_stage;
    E.unmatched_min_len = P[j].unmatched_end_minimum_read_length;
    E.unmatched_factor = (float)P[j].unmatched_end_length_factor;
    E.unmatched_factor_d = P[j].unmatched_end_length_factor;
    E.flush_tiles = 1;
    E.diff_u = reinterpret_cast<int32_t*>(A0 + lay[j].diff_u);
    E.diff_r = reinterpret_cast<int32_t*>(A0 + lay[j].diff_r);
    E.qs_flag = A0 + lay[j].qs;
    E.blk_u = reinterpret_cast<uint32_t*>(A0 + lay[j].blk_u);
    E.blk_r = reinterpret_cast<uint32_t*>(A0 + lay[j].blk_r);
    // class bytes: exact, every quality of a base that is not N below Q, and room for the counters
    E.code = nullptr;
    const uint32_t R = P[j].n_read_files, Q = P[j].n_quality;
    if (s->code_ok && s->max_q < Q && R <= kEcCodeMaxR && ((size_t)R * 29 * Q + 512u * R) * 4 <= kEcMaxHistBytes) {
      E.code = s->code.as<uint8_t>();
      max_code_r = std::max(max_code_r, R);
    }
  }
  for (uint32_t j = 0; j <= n; j++) B.cblk_begin[j] = cblk[j];
  CK(prepare_ec(max_bins, max_code_r));
  const int grid = ec_grid((uint32_t)n_chunks, ctx->sms, tn.ec_blocks_per_sm);
  std::string where, step;
  const cudaError_t pe = run_pass(ctx, ctx->exec_ec, [&]() -> cudaError_t {
    cudaError_t e;
    if ((e = record(ctx->ev0, st)) != cudaSuccess) return e;
    if ((e = launch_host_copy(ctx->pin_in.p, ctx->d_chunks.p, std::max<size_t>(16, n_chunks * sizeof(uint4)), ctx->sms,
                              st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(A0, 0, arena_bytes, st)) != cudaSuccess) return e;
    if ((e = launch_ec(B, ctx->d_chunks.as<uint4>(), (uint32_t)n_chunks, ctx->next.as<unsigned int>(), max_bins,
                       max_code_r, grid, st, ctx->evm0, ctx->evm1)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(ctx->pin_out.p, A0, res_bytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    return record(ctx->ev1, st);
  }, where);
  if (pe != cudaSuccess) return fail(ctx, BSQ_ERR_CUDA, "error_count pass (" + where + "): " + cudaGetErrorString(pe));
  CK(cudaStreamSynchronize(st));
  const float ms = elapsed(ctx->ev0, ctx->ev1), mms = elapsed(ctx->evm0, ctx->evm1);
  ctx->last_ms += ms; ctx->main_ms += mms; ctx->launches += 5;     // staging copy, read pass, 3 coverage kernels
  ctx->last_h2d += std::max<size_t>(16, n_chunks * sizeof(uint4));
  ctx->last_d2h += res_bytes;
  int rc = BSQ_OK;
  for (uint32_t j = 0; j < n; j++) {
    const uint32_t err = *reinterpret_cast<const uint32_t*>(ctx->pin_out.at(lay[j].err));
    if (err) return fail(ctx, BSQ_ERR_DATA, "error_count: " + err_text(err));
    const SampleDev* s = smp[j];
    const uint64_t* counts = reinterpret_cast<const uint64_t*>(ctx->pin_out.at(lay[j].counts));
    const uint64_t* hist = reinterpret_cast<const uint64_t*>(ctx->pin_out.at(lay[j].hist));
    const uint64_t* found = reinterpret_cast<const uint64_t*>(ctx->pin_out.at(lay[j].found));
    bsq_ec_result* o = &out[j];
    const size_t nbins = (size_t)P[j].n_read_files * 25 * P[j].n_quality;
    if (o->counts) for (size_t i = 0; i < nbins; i++) o->counts[i] = P[j].do_errors ? counts[i] : 0;
    const uint32_t cap = lay[j].cap;
    for (uint32_t g = 0; g < s->n_groups; g++) {
      uint32_t size = 0;
      for (uint32_t i = 0; i < cap; i++) if (hist[(size_t)g * cap + i]) size = i + 1;
      if (!P[j].do_coverage) size = 0;
      if (o->hist_size) o->hist_size[g] = size;
      if (o->coverage_hist) {
        for (uint32_t i = 0; i < o->hist_capacity; i++)
          o->coverage_hist[(size_t)g * o->hist_capacity + i] = (i < size) ? hist[(size_t)g * cap + i] : 0;
        if (size > o->hist_capacity) rc = BSQ_ERR_SIZE;
      }
    }
    if (o->no_pos_hash_pr) {
      for (uint32_t t = 0; t < s->n_targets; t++) o->no_pos_hash_pr[t] = 1.0;
      if (P[j].preprocess_stage)
        for (uint32_t t : s->order) {
          const double tot = (double)(found[2 * t] + found[2 * t + 1]);
          o->no_pos_hash_pr[t] = (tot != 0) ? (double)found[2 * t] / tot : 1.0;
        }
    }
  }
  if (rc == BSQ_ERR_SIZE) return fail(ctx, rc, "coverage histogram larger than hist_capacity; see hist_size");
  return BSQ_OK;
}

int bsq_error_count_batch(bsq_ctx* ctx, uint32_t n, const int32_t* ids, const bsq_ec_params* P, bsq_ec_result* out) {
  if (!ctx || !ids || !P || !out || n == 0) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  ctx->last_ms = 0; ctx->main_ms = 0; ctx->launches = 0; ctx->last_h2d = 0; ctx->last_d2h = 0;
  for (uint32_t g = 0; g < n;) {
    const uint32_t k = group_size(ctx, n - g, ids + g);
    if (k == 0) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
    const int rc = ec_group(ctx, k, ids + g, P + g, out + g);
    if (rc != BSQ_OK) return rc;
    g += k;
  }
  return BSQ_OK;
}

int bsq_error_count(bsq_ctx* ctx, int32_t sid, const bsq_ec_params* p, bsq_ec_result* out) {
  return bsq_error_count_batch(ctx, 1, &sid, p, out);
}

int bsq_counts_to_log10_prob(const uint64_t* counts, uint32_t R, uint32_t Q, double* out) {
  if (!counts || !out || R == 0 || Q == 0) return BSQ_ERR_INVALID;
  host::counts_to_log10_prob(counts, R, Q, out);
  return BSQ_OK;
}

int bsq_counts_to_log10_prob_batch(uint32_t n, const uint64_t* const* counts, const uint32_t* R, const uint32_t* Q,
                                   double* const* out) {
  if (!counts || !R || !Q || !out) return BSQ_ERR_INVALID;
  for (uint32_t j = 0; j < n; j++)
    if (!counts[j] || !out[j] || R[j] == 0 || Q[j] == 0) return BSQ_ERR_INVALID;
  parallel_for(n, [&](uint32_t j) { host::counts_to_log10_prob(counts[j], R[j], Q[j], out[j]); });
  return BSQ_OK;
}

// ============================================================================ pass 2
// Control words of pass 2, written on the device and read back in one copy.
enum : uint32_t { kCtlCand = 0, kCtlCand2 = 1, kCtlKept = 2, kCtlRa = 3, kCtlCandErr = 4, kCtlBq = 5, kCtlPool = 6,
                  kCtlBqNext = 7, kCtlJobErr = 8, kCtlColNext = 8 + kBatchJobs, kCtlWords = 9 + kBatchJobs };
constexpr uint32_t kBoundPool = 4u << 20;   // (class, multiplicity) entries for deferred bounds: 32 MiB

// One group of at most kBatchJobs samples; results go to res_*[job0 + j].
//   device arena: per job the likelihood-class table (lp64 | r64 | lpmax64 | lp32) and the per-target
//   deletion cutoffs and failed-fit flags, staged on the host and sent in one copy.
// The discordant-pair read groups of pass-2 parameters as a 256-bit mask (identify_mutations.cpp:883-911).
static int dp_mask(bsq_ctx* ctx, const bsq_im_params& p, uint32_t out[8]) {
  for (int i = 0; i < 8; i++) out[i] = 0;
  if (p.n_read_groups && !p.dp_group) return fail(ctx, BSQ_ERR_INVALID, "n_read_groups without dp_group");
  for (uint32_t g = 0; g < p.n_read_groups; g++) {
    if (p.dp_group[g] < -1) return fail(ctx, BSQ_ERR_INVALID, "DP group out of range");
    if (p.dp_group[g] < 0) continue;
    if (g >= 256) return fail(ctx, BSQ_ERR_INVALID, "discordant-pair groups on read groups beyond the first 256");
    out[g >> 5] |= 1u << (g & 31);
  }
  return BSQ_OK;
}

static int im_group(bsq_ctx* ctx, uint32_t n, const int32_t* ids, const bsq_im_params* P,
                    const double* const* tables, bsq_position_arrays* const* pos_out, uint32_t job0) {
  std::vector<SampleDev*> smp(n);
  for (uint32_t j = 0; j < n; j++) {
    smp[j] = find_sample(ctx, ids[j]);
    if (!smp[j]) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
    if (!tables[j] || !P[j].deletion_propagation_cutoff || !P[j].deletion_seed_cutoff)
      return fail(ctx, BSQ_ERR_INVALID, "missing error table or deletion cutoffs");
    if (P[j].n_read_files == 0 || P[j].n_read_files > 255 || P[j].n_quality == 0 || P[j].n_quality > 256)
      return fail(ctx, BSQ_ERR_INVALID, "error table dimensions out of range");
    if (P[j].precision != P[0].precision) return fail(ctx, BSQ_ERR_INVALID, "one precision per batch");
    uint32_t m[8];
    const int rc = dp_mask(ctx, P[j], m);
    if (rc != BSQ_OK) return rc;
  }
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const bsq_tuning& tn = ctx->tune;
  // likelihood classes, computed on the host exactly as fill_read_base_likelihoods does
  std::vector<host::ClassTableHost> ct(n);
  struct Lay { size_t lp64, r64, lpmax64, lp32, prop, seed, failed; };
  std::vector<Lay> lay(n);
  std::vector<uint32_t> tile_b(n + 1, 0), col_b(n + 1, 0);
  uint32_t max_K = 0, per_warp = 32, Qh = 0;
  size_t off = 0;
  parallel_for(n, [&](uint32_t j) {
    host::build_class_table(tables[j], P[j].n_read_files, P[j].n_quality, smp[j]->mapq_values, ct[j]);
  });
  for (uint32_t j = 0; j < n; j++) {
    const SampleDev* s = smp[j];
    lay[j].lp64 = off; off = align256(off + ct[j].lp64.size() * 8);
    lay[j].r64 = off; off = align256(off + ct[j].r64.size() * 8);
    lay[j].lpmax64 = off; off = align256(off + ct[j].lpmax64.size() * 8);
    lay[j].lp32 = off; off = align256(off + ct[j].lp32.size() * 4);
    lay[j].prop = off; off = align256(off + (size_t)s->n_targets * 8);
    lay[j].seed = off; off = align256(off + (size_t)s->n_targets * 8);
    lay[j].failed = off; off = align256(off + s->n_targets);
    col_b[j + 1] = col_b[j] + s->n_cols;
    tile_b[j + 1] = tile_b[j] + s->n_tiles;
    max_K = std::max(max_K, ct[j].K);
    per_warp = std::max<uint32_t>(per_warp, s->max_tile_reads);
    Qh = std::max(Qh, P[j].n_quality);
  }
  const size_t arena_bytes = std::max<size_t>(off, 256);
  const uint32_t total_cols = col_b[n];
  // ---- every device buffer before anything is enqueued (nothing allocates inside a capture)
  CK(ctx->pin_in.reserve(arena_bytes));
  CK(ctx->pin_out.reserve(kCtlWords * 4));
  CK(ctx->im_arena.alloc(arena_bytes, st));
  CK(ctx->ctl.alloc(kCtlWords * 4, st));
  CK(ctx->cov.alloc((size_t)total_cols * sizeof(ColCov), st));
  CK(ctx->call.alloc((size_t)total_cols * sizeof(ColCall), st));
  const uint32_t nblk = (total_cols + 255) / 256;
  CK(ctx->blk.alloc((size_t)nblk * 4 + 16, st));
  CK(ctx->cand.alloc((size_t)total_cols * 4 + 16, st));
  CK(ctx->next.alloc(16, st));
  const int n_warps = ctx->sms * (int)std::max<uint32_t>(1, tn.cand_warps_per_sm);
  CK(ctx->scratch.alloc((size_t)n_warps * cand_warp_stride(per_warp) * sizeof(uint4), st));
  uint32_t ra_cap = 4096 + total_cols / 64;
  CK(ctx->ra.alloc((size_t)ra_cap * sizeof(RaDev), st));
  CK(ctx->qhist.alloc((size_t)ra_cap * 2 * Qh * 4, st));
  CK(ctx->bq.alloc((size_t)2 * ra_cap * sizeof(BoundJob), st));
  CK(ctx->pool.alloc((size_t)kBoundPool * sizeof(uint2), st));
  CK(ctx->keep.alloc(total_cols + 16, st));
  CK(ctx->kcol.alloc((size_t)total_cols * 4 + 16, st));
  CK(ctx->kcov.alloc((size_t)total_cols * sizeof(ColCov) + 16, st));
  CK(ctx->kcall.alloc((size_t)total_cols * sizeof(ColCall) + 16, st));
  unsigned char* A0 = ctx->im_arena.as<unsigned char>();
  uint32_t* ctl = ctx->ctl.as<uint32_t>();
  std::unique_ptr<Batch> Bp(new Batch());
  Batch& B = *Bp;
  memset(&B, 0, sizeof B);
  B.n_jobs = n;
  B.total_tiles = tile_b[n]; B.total_cols = total_cols;
  for (uint32_t j = 0; j <= n; j++) { B.tile_begin[j] = tile_b[j]; B.col_begin[j] = col_b[j]; }
  for (uint32_t j = 0; j < n; j++) B.heavy_begin[j + 1] = B.heavy_begin[j] + smp[j]->n_heavy;
  B.total_heavy = B.heavy_begin[n];
  B.tile_next = ctl + kCtlColNext;
  for (uint32_t j = 0; j < n; j++) {
    const SampleDev* s = smp[j];
    memcpy(ctx->pin_in.at(lay[j].lp64), ct[j].lp64.data(), ct[j].lp64.size() * 8);
    memcpy(ctx->pin_in.at(lay[j].r64), ct[j].r64.data(), ct[j].r64.size() * 8);
    memcpy(ctx->pin_in.at(lay[j].lpmax64), ct[j].lpmax64.data(), ct[j].lpmax64.size() * 8);
    memcpy(ctx->pin_in.at(lay[j].lp32), ct[j].lp32.data(), ct[j].lp32.size() * 4);
    memcpy(ctx->pin_in.at(lay[j].prop), P[j].deletion_propagation_cutoff, (size_t)s->n_targets * 8);
    memcpy(ctx->pin_in.at(lay[j].seed), P[j].deletion_seed_cutoff, (size_t)s->n_targets * 8);
    // per job, not per sample: one sample may sit in a batch twice with different cutoffs
    for (uint32_t t = 0; t < s->n_targets; t++) ctx->pin_in.at(lay[j].failed)[t] = P[j].deletion_propagation_cutoff[t] < 0.0;
    DevJob& J = B.jobs[j];
    J.S = make_dev_sample(*s);
    J.S.tgt_failed = A0 + lay[j].failed;
    if (s->code_ok && s->max_q < P[j].n_quality) J.S.code = s->code.as<uint8_t>();
    J.T.lp64 = reinterpret_cast<const double*>(A0 + lay[j].lp64);
    J.T.r64 = reinterpret_cast<const double*>(A0 + lay[j].r64);
    J.T.lpmax64 = reinterpret_cast<const double*>(A0 + lay[j].lpmax64);
    J.T.lp32 = reinterpret_cast<const float*>(A0 + lay[j].lp32);
    J.T.K = ct[j].K; J.T.R = P[j].n_read_files; J.T.Q = P[j].n_quality;
    J.T.n_mapq = (uint32_t)s->mapq_values.size();
    J.prop = reinterpret_cast<const double*>(A0 + lay[j].prop);
    J.seed = reinterpret_cast<const double*>(A0 + lay[j].seed);
    J.col_begin = col_b[j]; J.tile_begin = tile_b[j];
    ImArgs& A = J.I;
    A.cov = ctx->cov.as<ColCov>() + col_b[j]; A.call = ctx->call.as<ColCall>() + col_b[j];
    A.err = ctl + kCtlJobErr + j;
    A.base_quality_cutoff = P[j].base_quality_cutoff;
    A.precision = P[j].precision;
    A.log10_ref_len = P[j].log10_ref_length;
    A.mutation_cutoff = P[j].mutation_cutoff;
    A.poly_cutoff = P[j].polymorphism_cutoff;
    A.screen_margin = 1.0f;
    A.guard = 2e-6f;
    A.precision_decimal = P[j].polymorphism_precision_decimal;
    dp_mask(ctx, P[j], A.dp_rg);      // checked above
  }
  CandArgs C;
  memset(&C, 0, sizeof C);
  C.cand = ctx->cand.as<uint32_t>(); C.n_cand_dev = ctl + kCtlCand; C.next = ctx->next.as<unsigned int>();
  C.ra = ctx->ra.as<RaDev>(); C.n_ra = ctl + kCtlRa; C.ra_cap = ra_cap;
  C.scratch = ctx->scratch.as<uint4>(); C.scratch_per_warp = per_warp; C.err = ctl + kCtlCandErr;
  C.Qhist = Qh; C.qhist = ctx->qhist.as<uint32_t>();
  C.bq = ctx->bq.as<BoundJob>(); C.n_bq = ctl + kCtlBq; C.bq_cap = 2 * ra_cap;
  C.pool = ctx->pool.as<uint2>(); C.pool_used = ctl + kCtlPool; C.pool_cap = kBoundPool;
  const int col_grid = column_grid(B.total_tiles, ctx->sms, tn.col_blocks_per_sm);
  const uint32_t* ctl_host = reinterpret_cast<const uint32_t*>(ctx->pin_out.p);
  // ---- the device part of the pass: column scores -> candidates -> EM -> interval marks
  std::string where, step;
  const cudaError_t pe = run_pass(ctx, ctx->exec_im, [&]() -> cudaError_t {
    cudaError_t e;
    step = "ev0";
    if ((e = record(ctx->ev0, st)) != cudaSuccess) return e;
    step = "arena copy";
    if ((e = launch_host_copy(ctx->pin_in.p, A0, arena_bytes, ctx->sms, st)) != cudaSuccess) return e;
    step = "control words";
    if ((e = cudaMemsetAsync(ctl, 0, kCtlWords * 4, st)) != cudaSuccess) return e;
    if ((e = record(ctx->evm0, st)) != cudaSuccess) return e;
    step = "column kernel";
    if ((e = launch_im_column(B, P[0].precision, col_grid, st)) != cudaSuccess) return e;
    if ((e = record(ctx->evm1, st)) != cudaSuccess) return e;
    step = "compaction";
    if ((e = launch_compact(ctx->call.as<ColCall>(), total_cols, ctx->blk.as<uint32_t>(), ctl + kCtlCand,
                            ctx->cand.as<uint32_t>(), st)) != cudaSuccess) return e;
    step = "candidate kernel";
    if ((e = launch_candidates(B, C, max_K, n_warps, st)) != cudaSuccess) return e;
    step = "bounds kernel";
    if ((e = launch_bounds(B, C, ctl + kCtlBqNext, ctx->sms, tn.bound_warps_per_sm, st)) != cudaSuccess) return e;
    step = "interval kernels";
    if ((e = launch_intervals(B, ctx->cov.as<ColCov>(), ctx->call.as<ColCall>(), ctx->keep.as<uint8_t>(),
                              ctx->blk.as<uint32_t>(), ctl + kCtlKept, ctx->kcol.as<uint32_t>(), ctx->kcov.as<ColCov>(),
                              ctx->kcall.as<ColCall>(), st)) != cudaSuccess) return e;
    step = "control copy";
    if ((e = cudaMemcpyAsync(ctx->pin_out.p, ctl, kCtlWords * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    step = "ev1";
    return record(ctx->ev1, st);
  }, where);
  if (pe != cudaSuccess)
    return fail(ctx, BSQ_ERR_CUDA, "identify_mutations pass (" + where + (where == "capture" ? ": " + step : "") +
                                       "): " + cudaGetErrorString(pe));
  CK(cudaStreamSynchronize(st));
  const float ms = elapsed(ctx->ev0, ctx->ev1), mms = elapsed(ctx->evm0, ctx->evm1);
  // more RA items than the buffer holds: rerun the candidate kernel alone with room for all
  for (int attempt = 0; attempt < 3 && ctl_host[kCtlRa] > ra_cap; attempt++) {
    ra_cap = ctl_host[kCtlRa] + 1024;
    CK(ctx->ra.alloc((size_t)ra_cap * sizeof(RaDev), st));
    CK(ctx->qhist.alloc((size_t)ra_cap * 2 * Qh * 4, st));
    CK(ctx->bq.alloc((size_t)2 * ra_cap * sizeof(BoundJob), st));
    C.ra = ctx->ra.as<RaDev>(); C.ra_cap = ra_cap; C.qhist = ctx->qhist.as<uint32_t>();
    C.bq = ctx->bq.as<BoundJob>(); C.bq_cap = 2 * ra_cap;
    CK(cudaMemsetAsync(ctl + kCtlRa, 0, (kCtlBqNext + 1 - kCtlRa) * 4, st));   // RA, error, bound-job counters
    CK(launch_candidates(B, C, max_K, n_warps, st));
    CK(launch_bounds(B, C, ctl + kCtlBqNext, ctx->sms, tn.bound_warps_per_sm, st));
    CK(cudaMemcpyAsync(ctx->pin_out.p, ctl, kCtlWords * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  const uint32_t n_cand = ctl_host[kCtlCand] + ctl_host[kCtlCand2], nk = ctl_host[kCtlKept], n_ra = ctl_host[kCtlRa];
  const uint32_t cerr = ctl_host[kCtlCandErr];
  ctx->last_ms += ms; ctx->main_ms += mms; ctx->launches += 14;    // staging copy + 13 (launch list of the step)
  ctx->last_h2d += arena_bytes;
  ctx->last_d2h += (uint64_t)kCtlWords * 4 + (uint64_t)n_ra * (sizeof(RaDev) + 2 * Qh * 4) +
                   (uint64_t)nk * (4 + sizeof(ColCov) + sizeof(ColCall));
  for (uint32_t j = 0; j < n; j++)
    if (pos_out && pos_out[j]) ctx->last_d2h += (uint64_t)smp[j]->n_cols * (sizeof(ColCov) + sizeof(ColCall));
  ctx->last_candidates += n_cand;
  if (n_ra > ra_cap) return fail(ctx, BSQ_ERR_NOMEM, "identify_mutations: RA buffer overflow");
  if (cerr & ~kErrRaOverflow) return fail(ctx, BSQ_ERR_DATA, "identify_mutations: " + err_text(cerr));
  for (uint32_t j = 0; j < n; j++)
    if (ctl_host[kCtlJobErr + j]) return fail(ctx, BSQ_ERR_DATA, "identify_mutations: " + err_text(ctl_host[kCtlJobErr + j]));
  // ---- variable-size results, through page-locked memory
  std::vector<RaDev> ra(n_ra);
  std::vector<uint32_t> qh((size_t)n_ra * 2 * Qh);
  std::vector<uint32_t> kept(nk);
  std::vector<ColCov> kcov(nk);
  std::vector<ColCall> kcall(nk);
  const size_t r_ra = 0, r_qh = align256(r_ra + ra.size() * sizeof(RaDev)), r_kept = align256(r_qh + qh.size() * 4),
               r_kcov = align256(r_kept + (size_t)nk * 4), r_kcall = align256(r_kcov + (size_t)nk * sizeof(ColCov)),
               r_end = r_kcall + (size_t)nk * sizeof(ColCall);
  CK(ctx->pin_res.reserve(r_end + 16));
  if (n_ra) {
    CK(cudaMemcpyAsync(ctx->pin_res.at(r_ra), ctx->ra.p, (size_t)n_ra * sizeof(RaDev), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ctx->pin_res.at(r_qh), ctx->qhist.p, qh.size() * 4, cudaMemcpyDeviceToHost, st));
  }
  if (nk) {
    CK(cudaMemcpyAsync(ctx->pin_res.at(r_kept), ctx->kcol.p, (size_t)nk * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ctx->pin_res.at(r_kcov), ctx->kcov.p, (size_t)nk * sizeof(ColCov), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ctx->pin_res.at(r_kcall), ctx->kcall.p, (size_t)nk * sizeof(ColCall), cudaMemcpyDeviceToHost, st));
  }
  // per-position arrays only where they were asked for
  std::vector<std::vector<ColCov>> pcov(n);
  std::vector<std::vector<ColCall>> pcall(n);
  for (uint32_t j = 0; j < n; j++) {
    if (!pos_out || !pos_out[j]) continue;
    const uint32_t nc = smp[j]->n_cols;
    pcov[j].resize(nc);
    pcall[j].resize(nc);
    CK(cudaMemcpyAsync(pcov[j].data(), ctx->cov.as<ColCov>() + col_b[j], (size_t)nc * sizeof(ColCov), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(pcall[j].data(), ctx->call.as<ColCall>() + col_b[j], (size_t)nc * sizeof(ColCall), cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  if (n_ra) {
    memcpy(ra.data(), ctx->pin_res.at(r_ra), (size_t)n_ra * sizeof(RaDev));
    memcpy(qh.data(), ctx->pin_res.at(r_qh), qh.size() * 4);
  }
  if (nk) {
    memcpy(kept.data(), ctx->pin_res.at(r_kept), (size_t)nk * 4);
    memcpy(kcov.data(), ctx->pin_res.at(r_kcov), (size_t)nk * sizeof(ColCov));
    memcpy(kcall.data(), ctx->pin_res.at(r_kcall), (size_t)nk * sizeof(ColCall));
  }
  // ---- host assembly, per job
  std::vector<std::vector<RaDev>> jra(n);
  std::vector<std::vector<uint32_t>> jqh(n);
  for (uint32_t i = 0; i < n_ra; i++) {
    const uint32_t j = (uint32_t)(std::upper_bound(col_b.begin(), col_b.end(), ra[i].col) - col_b.begin()) - 1;
    RaDev d = ra[i];
    d.col -= col_b[j];
    jra[j].push_back(d);
    jqh[j].insert(jqh[j].end(), qh.begin() + (size_t)i * 2 * Qh, qh.begin() + (size_t)(i + 1) * 2 * Qh);
  }
  // the kept columns of each job: a range of the (column-sorted) compacted list
  std::vector<size_t> kb(n + 1, 0);
  for (uint32_t j = 0; j < n; j++)
    kb[j + 1] = (size_t)(std::lower_bound(kept.begin(), kept.end(), col_b[j + 1]) - kept.begin());
  parallel_for(n, [&](uint32_t j) {
    SampleDev* s = smp[j];
    host::SampleLayout L;
    L.tpoff = &s->tpoff; L.toff = &s->toff; L.order = &s->order;
    host::assemble_ra(jra[j], jqh[j], Qh, L, ctx->res_ra[job0 + j]);
    if (pos_out && pos_out[j]) {   // dense arrays fetched anyway: run the state machines over every column
      host::intervals(pcov[j], pcall[j], L, &P[j], ctx->res_mc[job0 + j], ctx->res_un[job0 + j]);
      host::fill_positions(pcov[j], pcall[j], L, pos_out[j]);
    } else {
      std::vector<uint32_t> kc;
      kc.reserve(kb[j + 1] - kb[j]);
      for (size_t i = kb[j]; i < kb[j + 1]; i++) kc.push_back(kept[i] - col_b[j]);
      const std::vector<ColCov> kv(kcov.begin() + kb[j], kcov.begin() + kb[j + 1]);
      const std::vector<ColCall> kl(kcall.begin() + kb[j], kcall.begin() + kb[j + 1]);
      host::intervals_sparse(kc, kv, kl, L, &P[j], ctx->res_mc[job0 + j], ctx->res_un[job0 + j]);
    }
  });
  return BSQ_OK;
}

int bsq_identify_mutations_batch(bsq_ctx* ctx, uint32_t n, const int32_t* ids, const bsq_im_params* P,
                                 const double* const* tables, bsq_position_arrays* const* pos_out) {
  if (!ctx || !ids || !P || !tables || n == 0) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  ctx->res_ra.assign(n, {}); ctx->res_mc.assign(n, {}); ctx->res_un.assign(n, {});
  ctx->last_ms = 0; ctx->main_ms = 0; ctx->launches = 0; ctx->last_candidates = 0; ctx->last_h2d = 0; ctx->last_d2h = 0;
  for (uint32_t g = 0; g < n;) {
    const uint32_t k = group_size(ctx, n - g, ids + g);
    if (k == 0) { ctx->res_ra.clear(); ctx->res_mc.clear(); ctx->res_un.clear(); return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id"); }
    const int rc = im_group(ctx, k, ids + g, P + g, tables + g, pos_out ? pos_out + g : nullptr, g);
    if (rc != BSQ_OK) { ctx->res_ra.clear(); ctx->res_mc.clear(); ctx->res_un.clear(); return rc; }
    g += k;
  }
  return BSQ_OK;
}

int bsq_identify_mutations(bsq_ctx* ctx, int32_t sid, const bsq_im_params* p, const double* table,
                           bsq_position_arrays* pos_out) {
  bsq_position_arrays* po[1] = {pos_out};
  return bsq_identify_mutations_batch(ctx, 1, &sid, p, &table, pos_out ? po : nullptr);
}

int bsq_im_batch_result_counts(const bsq_ctx* ctx, uint32_t job, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un) {
  if (!ctx || job >= ctx->res_ra.size()) return BSQ_ERR_INVALID;
  if (n_ra) *n_ra = ctx->res_ra[job].size();
  if (n_mc) *n_mc = ctx->res_mc[job].size();
  if (n_un) *n_un = ctx->res_un[job].size();
  return BSQ_OK;
}

int bsq_im_batch_result_copy(const bsq_ctx* ctx, uint32_t job, bsq_ra_record* ra, uint64_t ra_cap, bsq_mc_record* mc,
                             uint64_t mc_cap, bsq_un_record* un, uint64_t un_cap) {
  if (!ctx || job >= ctx->res_ra.size()) return BSQ_ERR_INVALID;
  const auto &R = ctx->res_ra[job];
  const auto &M = ctx->res_mc[job];
  const auto &U = ctx->res_un[job];
  if ((ra && ra_cap < R.size()) || (mc && mc_cap < M.size()) || (un && un_cap < U.size())) return BSQ_ERR_SIZE;
  if (ra) std::copy(R.begin(), R.end(), ra);
  if (mc) std::copy(M.begin(), M.end(), mc);
  if (un) std::copy(U.begin(), U.end(), un);
  return BSQ_OK;
}

int bsq_im_result_counts(const bsq_ctx* ctx, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un) {
  return bsq_im_batch_result_counts(ctx, 0, n_ra, n_mc, n_un);
}

int bsq_intervals_from_positions(const bsq_reference* ref, const bsq_position_arrays* pa, const bsq_im_params* p,
                                 bsq_mc_record* mc, uint64_t mc_cap, uint64_t* n_mc, bsq_un_record* un, uint64_t un_cap,
                                 uint64_t* n_un) {
  if (!ref || !pa || !p || !n_mc || !n_un || !ref->target_offset || !p->deletion_propagation_cutoff ||
      !p->deletion_seed_cutoff || !pa->unique_top || !pa->unique_bot || !pa->redundant_top || !pa->redundant_bot ||
      !pa->consensus_score || (mc_cap && !mc) || (un_cap && !un))
    return BSQ_ERR_INVALID;
  const uint32_t T = ref->n_targets;
  std::vector<uint64_t> toff(ref->target_offset, ref->target_offset + T + 1);
  std::vector<uint32_t> tpoff(T + 1), order;
  for (uint32_t t = 0; t <= T; t++) tpoff[t] = (uint32_t)(toff[t] + t);
  for (uint32_t i = 0; i < ref->n_target_order; i++) {
    if (ref->target_order[i] >= T) return BSQ_ERR_INVALID;
    order.push_back(ref->target_order[i]);
  }
  std::vector<ColCov> cov(tpoff[T]);
  std::vector<ColCall> call(tpoff[T]);
  for (uint32_t t = 0; t < T; t++)
    for (uint64_t g = toff[t]; g < toff[t + 1]; g++) {
      ColCov& cv = cov[tpoff[t] + (g - toff[t])];
      cv.uniq_top = pa->unique_top[g]; cv.uniq_bot = pa->unique_bot[g];
      cv.red_top = pa->redundant_top[g]; cv.red_bot = pa->redundant_bot[g];
      ColCall& cl = call[tpoff[t] + (g - toff[t])];
      cl.flags = (pa->consensus_score[g] >= p->mutation_cutoff) ? kBasePredicted : 0;
    }
  host::SampleLayout L;
  L.tpoff = &tpoff; L.toff = &toff; L.order = &order;
  std::vector<bsq_mc_record> m;
  std::vector<bsq_un_record> u;
  host::intervals(cov, call, L, p, m, u);
  *n_mc = m.size();
  *n_un = u.size();
  if (m.size() > mc_cap || u.size() > un_cap) return BSQ_ERR_SIZE;
  std::copy(m.begin(), m.end(), mc);
  std::copy(u.begin(), u.end(), un);
  return BSQ_OK;
}

int bsq_im_result_copy(const bsq_ctx* ctx, bsq_ra_record* ra, uint64_t ra_cap, bsq_mc_record* mc, uint64_t mc_cap,
                       bsq_un_record* un, uint64_t un_cap) {
  return bsq_im_batch_result_copy(ctx, 0, ra, ra_cap, mc, mc_cap, un, un_cap);
}

// tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666): the device walks the records
// and the columns (bsq_softclip.cu); the rows come back in (direction, column) order and the host
// puts them in the reference's order and fits the null model.
int bsq_soft_clipping(bsq_ctx* ctx, int32_t sample_id, const bsq_sc_params* p, bsq_sc_summary* summary) {
  if (!ctx || !p || !summary) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  // the ranges Settings enforces when it parses the options (src/breseq/settings.cpp:766-779)
  if (!(p->consensus_base_fraction >= 0.0 && p->consensus_base_fraction <= 1.0) ||
      !(p->dispersion_trim_frequency >= 0.0 && p->dispersion_trim_frequency <= 1.0) ||
      !(p->maximum_dispersion >= 0.0 && p->maximum_dispersion < 1.0) ||
      !(p->minimum_rate >= 0.0 && p->minimum_rate < 1.0))
    return fail(ctx, BSQ_ERR_INVALID, "soft-clipping setting out of range");
  SampleDev* s = find_sample(ctx, sample_id);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  CK(cudaSetDevice(ctx->device));
  const uint32_t T = s->n_targets;
  std::vector<uint32_t> order(T);
  if (p->target_name_order) {
    std::vector<uint8_t> seen(T, 0);
    for (uint32_t i = 0; i < T; i++) {
      const uint32_t t = p->target_name_order[i];
      if (t >= T || seen[t]) return fail(ctx, BSQ_ERR_INVALID, "target_name_order is not a permutation of the targets");
      seen[t] = 1;
      order[i] = t;
    }
  } else {
    for (uint32_t i = 0; i < T; i++) order[i] = i;
  }
  cudaStream_t st = ctx->stream;
  cudaGetLastError();
  ScArgs A;
  memset(&A, 0, sizeof A);
  A.reads = s->reads.as<DevRead>();
  A.qb = s->qb.as<QBounds>();
  A.seq = s->seq.as<uint8_t>();
  A.tpoff = s->d_tpoff.as<uint32_t>();
  A.n_reads = s->n_reads;
  A.n_targets = T;
  A.n_cols = s->n_cols;
  sc_plan(A, ctx->sms);
  const uint32_t nb = A.n_blocks;
  const uint64_t cstride = A.cstride;
  CK(ctx->sc_diff.alloc(cstride * 4, st));
  CK(ctx->sc_cnt.alloc(cstride * 8, st));
  CK(ctx->sc_blk.alloc((uint64_t)nb * 5 * 8, st));
  CK(ctx->sc_tot.alloc(128, st));
  CK(ctx->sc_ev.alloc((uint64_t)s->n_reads * 4, st));
  CK(ctx->sc_ev_n.alloc((uint64_t)A.ev_blocks * 4, st));
  CK(record(ctx->ev0, st));
  CK(cudaMemsetAsync(ctx->sc_diff.p, 0, cstride * 4, st));
  CK(cudaMemsetAsync(ctx->sc_cnt.p, 0, cstride * 8, st));
  CK(cudaMemsetAsync(ctx->sc_tot.p, 0, 128, st));
  A.ev = ctx->sc_ev.as<uint32_t>();
  A.ev_n = ctx->sc_ev_n.as<uint32_t>();
  A.m = p->minimum_clipped_bases;
  A.K = std::min(p->minimum_clipped_bases, kScMaxConsensus);
  A.base_fraction = p->consensus_base_fraction;
  A.diff = ctx->sc_diff.as<int32_t>();
  A.cnt = ctx->sc_cnt.as<uint32_t>();
  A.blk = ctx->sc_blk.as<long long>();
  A.tot = ctx->sc_tot.as<unsigned long long>();
  A.err = reinterpret_cast<uint32_t*>(ctx->sc_tot.as<unsigned char>() + 64);
  CK(sc_launch_count(A, ctx->sms, st, ctx->evm0, ctx->evm1));
  CK(ctx->pin_out.reserve(128));
  CK(cudaMemcpyAsync(ctx->pin_out.p, ctx->sc_tot.p, 128, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  uint64_t tot[8];
  memcpy(tot, ctx->pin_out.p, sizeof tot);
  const uint32_t err = *reinterpret_cast<const uint32_t*>(ctx->pin_out.at(64));
  if (err) return fail(ctx, BSQ_ERR_INVALID, "invalid records: " + err_text(err));
  const uint64_t n_rows = tot[0] + tot[2], n_tails = tot[1] + tot[3];
  if (n_tails >= 0xFFFFFFFFull) return fail(ctx, BSQ_ERR_SIZE, "more than 2^32 - 1 clip events in one sample");
  CK(ctx->sc_rows.alloc(n_rows * sizeof(ScRowDev), st));
  CK(ctx->sc_outs.alloc(n_rows * sizeof(ScOutDev), st));
  CK(ctx->sc_tails.alloc(n_tails * 8, st));
  A.rows = ctx->sc_rows.as<ScRowDev>();
  A.outs = ctx->sc_outs.as<ScOutDev>();
  A.tails = ctx->sc_tails.as<unsigned long long>();
  CK(sc_launch_rows(A, (uint32_t)n_rows, ctx->sms, st));
  const size_t rows_bytes = n_rows * sizeof(ScRowDev), outs_bytes = n_rows * sizeof(ScOutDev);
  CK(ctx->pin_out.reserve(128 + rows_bytes + outs_bytes));
  unsigned char* h = ctx->pin_out.at(0);
  CK(cudaMemcpyAsync(h, ctx->sc_tot.p, 64, cudaMemcpyDeviceToHost, st));
  if (n_rows) {
    CK(cudaMemcpyAsync(h + 128, ctx->sc_rows.p, rows_bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h + 128 + rows_bytes, ctx->sc_outs.p, outs_bytes, cudaMemcpyDeviceToHost, st));
  }
  CK(record(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_ms = elapsed(ctx->ev0, ctx->ev1);
  ctx->main_ms = elapsed(ctx->evm0, ctx->evm1);   // the read pass that counts the events
  ctx->launches = n_rows ? 7 : 4;
  ctx->last_h2d = 0;
  ctx->last_d2h = 128 + 64 + rows_bytes + outs_bytes;
  memcpy(tot, h, 64);
  host::sc_assemble(reinterpret_cast<const ScRowDev*>(h + 128), reinterpret_cast<const ScOutDev*>(h + 128 + rows_bytes),
                    tot[0], tot[2], s->tpoff, order, A.K, *p, n_tails, tot[4], tot[5], ctx->sc_res, *summary);
  return BSQ_OK;
}

// Discordant-pair / missing-pair candidate regions: the reads are classified and the window entries
// compacted on the device (bsq_pairs.cu); the sliding windows are replayed on the host over the
// compacted reads (bsq_pairs_host.cpp).
int bsq_pair_candidates(bsq_ctx* ctx, int32_t sample_id, const bsq_pair_params* p, uint64_t* n_dp, uint64_t* n_mp,
                        uint64_t* text_bytes) {
  if (!ctx || !p || !n_dp || !n_mp || !text_bytes) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  SampleDev* s = find_sample(ctx, sample_id);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  if (!s->has_pairs) return fail(ctx, BSQ_ERR_INVALID, "sample loaded without pair annotations (isize, xp, qname)");
  const uint32_t T = s->n_targets, G = p->n_dp_groups, NRG = p->n_read_groups;
  if (G > 255) return fail(ctx, BSQ_ERR_INVALID, "more than 255 DP groups");
  if ((NRG && !p->dp_group) || (G && (!p->window_width || !p->r1_name_prefix || !p->r2_name_prefix)) ||
      !p->deletion_propagation_cutoff)
    return fail(ctx, BSQ_ERR_INVALID, "null parameter array");
  for (uint32_t r = 0; r < NRG; r++)
    if (p->dp_group[r] < -1 || p->dp_group[r] >= (int32_t)G) return fail(ctx, BSQ_ERR_INVALID, "DP group out of range");
  for (uint32_t g = 0; g < G; g++)
    if (!(p->window_width[g] > 0.0) || !std::isfinite(p->window_width[g]))
      return fail(ctx, BSQ_ERR_INVALID, "window width must be positive and finite");
  // the ranges Settings enforces (src/breseq/settings.cpp:719-735)
  if (p->discordant_pair_seed < 0 || (p->predict_missing_pairs && (p->missing_pair_seed < 0 ||
      !(p->missing_pair_seed_fraction >= 0.0 && p->missing_pair_seed_fraction <= 1.0))))
    return fail(ctx, BSQ_ERR_INVALID, "seed setting out of range");
  const bool pd = p->predict_pair_distance != 0;
  if (pd) {
    if (!s->has_mates) return fail(ctx, BSQ_ERR_INVALID, "pair-distance scan needs the records' mtid and mpos");
    if (G && (!p->pd_cdf || !p->pd_cdf_len || !p->pd_orientation))
      return fail(ctx, BSQ_ERR_INVALID, "null pair-distance parameter array");
    if (!(p->pair_distance_tail_quantile >= 0.0 && p->pair_distance_tail_quantile <= 1.0) || !std::isfinite(p->pd_z_seed))
      return fail(ctx, BSQ_ERR_INVALID, "pair-distance setting out of range");
    for (uint32_t g = 0; g < G; g++)
      if (p->pd_cdf_len[g] && !p->pd_cdf[g]) return fail(ctx, BSQ_ERR_INVALID, "null pair-distance null");
  }
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  cudaGetLastError();
  const uint64_t n = s->n_reads;
  const bool mp = p->predict_missing_pairs && G > 0;
  host::PairReplayInput in;
  in.tpoff = s->tpoff;
  in.order = s->order;
  in.piled.assign(T, 0);
  for (uint32_t t : s->order) in.piled[t] = p->deletion_propagation_cutoff[t] >= 0.0 ? 1 : 0;
  in.window_width.assign(p->window_width, p->window_width + G);
  in.r1_prefix.assign(p->r1_name_prefix, p->r1_name_prefix + G);
  in.r2_prefix.assign(p->r2_name_prefix, p->r2_name_prefix + G);
  in.dp_seed = p->discordant_pair_seed;
  in.mp_seed = p->missing_pair_seed;
  in.mp_seed_fraction = p->missing_pair_seed_fraction;
  in.mp = mp;
  CK(record(ctx->ev0, st));
  CK(ctx->pr_code.alloc(n + 16, st));
  CK(ctx->pr_group.alloc(n + 16, st));
  CK(ctx->pr_sel.alloc(n * 4 + 16, st));
  CK(ctx->pr_evoff.alloc(n * 8 + 16, st));
  if (mp) {
    CK(ctx->pr_mem.alloc(2 * n * 4 + 16, st));
    CK(ctx->pr_memoff.alloc(2 * n * 8 + 16, st));
  }
  CK(ctx->pr_tmp.alloc((n / 1024 + 4) * 8 + 64, st));
  CK(ctx->pr_tot.alloc(64, st));
  CK(upload(ctx->pr_map, p->dp_group, NRG, st));
  PairArgs A;
  memset(&A, 0, sizeof A);
  A.reads = s->reads.as<DevRead>();
  A.flag = s->pflag.as<uint16_t>();
  A.xp = s->pxp.as<uint8_t>();
  A.isize = s->pisize.as<int32_t>();
  A.qoff = s->pqoff.as<uint64_t>();
  A.qname = s->pqname.as<char>();
  A.x1 = s->x1.as<uint32_t>();
  A.rg = s->rg.as<uint16_t>();
  A.rg_map = ctx->pr_map.as<int32_t>();
  A.n_rg = NRG;
  A.n = (uint32_t)n;
  A.mp = mp ? 1 : 0;
  A.code = ctx->pr_code.as<uint8_t>();
  A.group = ctx->pr_group.as<uint8_t>();
  A.sel = ctx->pr_sel.as<uint32_t>();
  A.mem0 = mp ? ctx->pr_mem.as<uint32_t>() : nullptr;
  A.mem1 = mp ? ctx->pr_mem.as<uint32_t>() + n : nullptr;
  uint64_t* tot = ctx->pr_tot.as<uint64_t>();
  CK(record(ctx->evm0, st));
  CK(pair_classify(A, ctx->sms, st));
  CK(record(ctx->evm1, st));
  CK(scan_u32(A.sel, ctx->pr_evoff.as<uint64_t>(), n, ctx->pr_tmp.as<uint64_t>(), tot, st));
  uint64_t* off0 = mp ? ctx->pr_memoff.as<uint64_t>() : nullptr;
  uint64_t* off1 = mp ? off0 + n : nullptr;
  if (mp) {
    CK(scan_u32(A.mem0, off0, n, ctx->pr_tmp.as<uint64_t>(), tot + 1, st));
    CK(scan_u32(A.mem1, off1, n, ctx->pr_tmp.as<uint64_t>(), tot + 2, st));
  }
  CK(ctx->pin_out.reserve(64));
  CK(cudaMemcpyAsync(ctx->pin_out.p, tot, 24, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  uint64_t counts[3];
  memcpy(counts, ctx->pin_out.p, 24);
  const uint64_t n_ev = counts[0], n_m0 = mp ? counts[1] : 0, n_m1 = mp ? counts[2] : 0, n_mem = n_m0 + n_m1;
  CK(ctx->pr_ev.alloc(n_ev * sizeof(PairEvent) + 16, st));
  CK(ctx->pr_names.alloc(n_ev * kPairNameSlot + 16, st));
  CK(ctx->pr_mstart.alloc(n_mem * 4 + 16, st));
  CK(ctx->pr_mkey.alloc(n_mem + 16, st));
  uint32_t* ms = ctx->pr_mstart.as<uint32_t>();
  uint8_t* mg = ctx->pr_mkey.as<uint8_t>();
  CK(pair_scatter(A, ctx->pr_evoff.as<uint64_t>(), mp ? off0 : nullptr, mp ? off1 : nullptr, ctx->pr_ev.as<PairEvent>(),
                  ctx->pr_names.as<char>(), ms, ms + n_m0, mg, mg + n_m0, ctx->sms, st));
  // pair distance: gaps into difference arrays, every position's statistics, the ladder edges
  bool pd_on = false;
  uint32_t pd_launches = 0;
  host::PdAssembleInput pdin;
  if (pd) {
    std::vector<int64_t> cdf;
    std::vector<uint64_t> cdf_off(G + 1, 0);
    std::vector<uint32_t> cdf_len(G + 1, 0);
    std::vector<uint8_t> orient(G + 1, 3);
    bool usable = false;
    for (uint32_t g = 0; g < G; g++) {
      cdf_off[g] = cdf.size();
      cdf_len[g] = p->pd_cdf_len[g];
      orient[g] = p->pd_orientation[g];
      if (cdf_len[g]) { cdf.insert(cdf.end(), p->pd_cdf[g], p->pd_cdf[g] + cdf_len[g]); usable = true; }
    }
    pd_on = usable && p->pd_max_span > 0 && G > 0;
    pdin.tpoff = s->tpoff;
    pdin.enabled = pd_on;
    pdin.z_seed = p->pd_z_seed;
    pdin.mean_covering_gap = p->pd_mean_covering_gap;
    pdin.total_reference_length = p->total_reference_length;
    if (G) pdin.hist.assign(kPdHistBins, 0);
    if (pd_on) {
      const uint64_t cols = s->n_cols;
      const uint32_t nb = (uint32_t)((cols + kPdScanCols - 1) / kPdScanCols);
      std::vector<uint8_t> piled(T, 0);
      for (uint32_t t : s->order) piled[t] = p->deletion_propagation_cutoff[t] >= 0.0 ? 1 : 0;
      CK(upload(ctx->pd_cdf, cdf.data(), cdf.size(), st));
      CK(upload(ctx->pd_cdfoff, cdf_off.data(), G + 1, st));
      CK(upload(ctx->pd_cdflen, cdf_len.data(), G + 1, st));
      CK(upload(ctx->pd_orient, orient.data(), G + 1, st));
      CK(upload(ctx->pd_piled, piled.data(), T, st));
      CK(ctx->pd_diff.alloc(cols * 32 + 64, st));
      CK(ctx->pd_blk.alloc((uint64_t)nb * 32 + 64, st));
      CK(ctx->pd_mask.alloc(cols * 8 + 64, st));
      CK(ctx->pd_hist.alloc(kPdHistBins * 8 + 64, st));
      CK(ctx->pd_ladder.alloc(2 * kPdLadderSteps * 8 + 64, st));
      CK(ctx->pd_above.alloc(cols * sizeof(PdAbove) + 64, st));
      CK(ctx->pd_cnt.alloc(64, st));
      CK(cudaMemsetAsync(ctx->pd_diff.p, 0, cols * 32, st));
      CK(cudaMemsetAsync(ctx->pd_hist.p, 0, kPdHistBins * 8, st));
      CK(cudaMemsetAsync(ctx->pd_ladder.p, 0, 2 * kPdLadderSteps * 8, st));
      CK(cudaMemsetAsync(ctx->pd_cnt.p, 0, 16, st));
      PdArgs D;
      memset(&D, 0, sizeof D);
      D.reads = s->reads.as<DevRead>(); D.flag = s->pflag.as<uint16_t>(); D.code = A.code; D.group = A.group;
      D.x1 = A.x1; D.isize = A.isize; D.mtid = s->pmtid.as<int32_t>(); D.mpos = s->pmpos.as<int32_t>();
      D.tpoff = s->d_tpoff.as<uint32_t>(); D.piled = ctx->pd_piled.as<uint8_t>(); D.cdf = ctx->pd_cdf.as<int64_t>();
      D.cdf_off = ctx->pd_cdfoff.as<uint64_t>(); D.cdf_len = ctx->pd_cdflen.as<uint32_t>();
      D.orient = ctx->pd_orient.as<uint8_t>(); D.n = (uint32_t)n; D.n_targets = T; D.n_cols = (uint32_t)cols;
      D.max_span = p->pd_max_span; D.seed = p->pair_distance_seed;
      D.lower_tail = static_cast<int64_t>(p->pair_distance_tail_quantile * static_cast<double>(kPdUScale));
      D.z_seed = p->pd_z_seed; D.diff = ctx->pd_diff.as<long long>(); D.blk = ctx->pd_blk.as<long long>();
      D.mask = ctx->pd_mask.as<uint64_t>(); D.hist = ctx->pd_hist.as<unsigned long long>();
      D.ladder = ctx->pd_ladder.as<unsigned long long>(); D.above = ctx->pd_above.as<PdAbove>();
      D.n_above = ctx->pd_cnt.as<unsigned int>(); D.above_cap = (uint32_t)cols;
      CK(pd_launch(D, ctx->sms, st));
      pd_launches = 5;
    }
  }
  const uint64_t b_ev = n_ev * sizeof(PairEvent), b_nm = n_ev * kPairNameSlot, b_ms = n_mem * 4, b_mk = n_mem;
  const uint64_t o_nm = align256(b_ev), o_ms = o_nm + align256(b_nm), o_mk = o_ms + align256(b_ms);
  const uint64_t o_pd = align256(o_mk + b_mk), b_pd = 64 + (kPdHistBins + 2 * kPdLadderSteps) * 8;
  CK(ctx->pin_out.reserve(o_pd + b_pd + 64));
  unsigned char* h = ctx->pin_out.at(0);
  if (pd_on) {
    CK(cudaMemcpyAsync(h + o_pd, ctx->pd_cnt.p, 16, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h + o_pd + 64, ctx->pd_hist.p, kPdHistBins * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h + o_pd + 64 + kPdHistBins * 8, ctx->pd_ladder.p, 2 * kPdLadderSteps * 8,
                       cudaMemcpyDeviceToHost, st));
  }
  if (b_ev) CK(cudaMemcpyAsync(h, ctx->pr_ev.p, b_ev, cudaMemcpyDeviceToHost, st));
  if (b_nm) CK(cudaMemcpyAsync(h + o_nm, ctx->pr_names.p, b_nm, cudaMemcpyDeviceToHost, st));
  if (b_ms) CK(cudaMemcpyAsync(h + o_ms, ctx->pr_mstart.p, b_ms, cudaMemcpyDeviceToHost, st));
  if (b_mk) CK(cudaMemcpyAsync(h + o_mk, ctx->pr_mkey.p, b_mk, cudaMemcpyDeviceToHost, st));
  uint64_t b_above = 0;
  if (pd_on) {
    CK(cudaStreamSynchronize(st));
    uint32_t cnt[2];
    memcpy(cnt, h + o_pd, 8);
    if (cnt[1])
      return fail(ctx, BSQ_ERR_DATA, "a pair's gap runs outside the pair-distance window (TLEN shorter than the gap, "
                                     "or the mate outside its target)");
    pdin.above.resize(cnt[0]);
    b_above = (uint64_t)cnt[0] * sizeof(PdAbove);
    if (cnt[0]) CK(cudaMemcpyAsync(pdin.above.data(), ctx->pd_above.p, b_above, cudaMemcpyDeviceToHost, st));
    memcpy(pdin.hist.data(), h + o_pd + 64, kPdHistBins * 8);
    memcpy(pdin.ladder, h + o_pd + 64 + kPdHistBins * 8, 2 * kPdLadderSteps * 8);
  }
  CK(record(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_ms = elapsed(ctx->ev0, ctx->ev1);
  ctx->main_ms = elapsed(ctx->evm0, ctx->evm1);   // the classification pass over every read
  ctx->launches = 1 + 3 + (mp ? 6 : 0) + 1 + pd_launches;
  ctx->last_h2d = (uint64_t)NRG * 4;
  ctx->last_d2h = 16 + b_ev + b_nm + b_ms + b_mk + (pd_on ? b_pd + b_above : 0);
  ctx->pd_res = host::PdResult();
  if (pd) host::pd_assemble(pdin, ctx->pd_res);
  in.ev = reinterpret_cast<const PairEvent*>(h);
  in.n_ev = n_ev;
  in.names = reinterpret_cast<const char*>(h + o_nm);
  in.mem_start[0] = reinterpret_cast<const uint32_t*>(h + o_ms);
  in.mem_start[1] = in.mem_start[0] + n_m0;
  in.mem_group[0] = reinterpret_cast<const uint8_t*>(h + o_mk);
  in.mem_group[1] = in.mem_group[0] + n_m0;
  in.n_mem[0] = n_m0;
  in.n_mem[1] = n_m1;
  ctx->pair_res = host::PairReplayResult();
  const int rc = host::pair_replay(in, ctx->pair_res);
  if (rc != BSQ_OK) return fail(ctx, rc, "inconsistent pair events");
  *n_dp = ctx->pair_res.dp.size();
  *n_mp = ctx->pair_res.mp.size();
  *text_bytes = ctx->pair_res.text.size();
  return BSQ_OK;
}

int bsq_pd_result(bsq_ctx* ctx, uint64_t* n_regions, bsq_pd_region* regions, uint64_t capacity, bsq_pd_summary* summary) {
  if (!ctx || !n_regions) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  const host::PdResult& r = ctx->pd_res;
  *n_regions = r.regions.size();
  if (summary) *summary = r.summary;
  if (!regions) return BSQ_OK;
  if (capacity < r.regions.size()) return fail(ctx, BSQ_ERR_SIZE, "region buffer too small");
  if (r.regions.size()) memcpy(regions, r.regions.data(), r.regions.size() * sizeof(bsq_pd_region));
  return BSQ_OK;
}

int bsq_pair_result_copy(bsq_ctx* ctx, bsq_pair_region* dp, uint64_t n_dp, bsq_pair_region* mp, uint64_t n_mp,
                         char* text, uint64_t text_bytes) {
  if (!ctx) return BSQ_ERR_INVALID;
  const host::PairReplayResult& r = ctx->pair_res;
  if (n_dp < r.dp.size() || n_mp < r.mp.size() || text_bytes < r.text.size())
    return fail(ctx, BSQ_ERR_SIZE, "result buffers too small");
  if ((r.dp.size() && !dp) || (r.mp.size() && !mp) || (r.text.size() && !text))
    return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (r.dp.size()) memcpy(dp, r.dp.data(), r.dp.size() * sizeof(bsq_pair_region));
  if (r.mp.size()) memcpy(mp, r.mp.data(), r.mp.size() * sizeof(bsq_pair_region));
  if (r.text.size()) memcpy(text, r.text.data(), r.text.size());
  return BSQ_OK;
}

// Coverage columns of one region (coverage_output::pileup_callback, coverage_output.cpp:307-470):
// bsq_covtable.cu on the device.  The columns at positions start + k * step (k < m; step 1 = every
// position) come back in one pinned buffer with the reference characters: [6][m] u32 counts |
// [2][m] f64 weights | stat | the target's reference characters up to end_1.
static int coverage_region(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start, uint32_t end,
                           uint32_t first, uint32_t step, host::CoverageRegion& out, int32_t rg_only = -1,
                           uint32_t mode = kCtBam2cov, const uint32_t* dp_rg = nullptr) {
  SampleDev* s = find_sample(ctx, sample_id);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  if (tid >= s->n_targets) return fail(ctx, BSQ_ERR_INVALID, "target index out of range");
  const uint32_t tlen = s->tpoff[tid + 1] - s->tpoff[tid] - 1;
  if (start < 1 || start > end || end > tlen) return fail(ctx, BSQ_ERR_INVALID, "region outside the target");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  cudaGetLastError();
  const uint32_t n = end - start + 1;
  CovTabArgs A;
  memset(&A, 0, sizeof A);
  A.reads = s->reads.as<DevRead>();
  A.cigar = s->cigar.as<uint32_t>();
  A.x1 = s->x1.as<uint32_t>();
  A.rstart = s->rstart.as<uint32_t>();
  A.rg = s->rg.as<uint16_t>();
  A.rg_only = rg_only;
  A.seq = s->seq.as<uint8_t>();
  A.mode = mode;
  if (dp_rg) memcpy(A.dp_rg, dp_rg, sizeof A.dp_rg);
  A.n_reads = s->n_reads;
  A.t0 = s->tpoff[tid];
  A.c0 = A.t0 + start - 1;
  A.n = n;
  A.n_blocks = (uint32_t)(((uint64_t)n + 1 + kCtBlockCols - 1) / kCtBlockCols);
  A.stride = (uint64_t)A.n_blocks * kCtBlockCols;
  CK(ctx->ct_diff.alloc(A.stride * 16, st));
  CK(ctx->ct_blk.alloc((uint64_t)A.n_blocks * 32, st));
  CK(ctx->ct_counts.alloc((uint64_t)n * 24, st));
  CK(ctx->ct_red.alloc((uint64_t)n * 16, st));
  CK(ctx->ct_stat.alloc(64, st));
  const uint32_t m = first <= end ? (end - first) / step + 1 : 0;
  if (step > 1) CK(ctx->ct_gather.alloc((uint64_t)m * 40 + 16, st));
  A.diff = ctx->ct_diff.as<int32_t>();
  A.blk = ctx->ct_blk.as<long long>();
  A.counts = ctx->ct_counts.as<uint32_t>();
  A.red = ctx->ct_red.as<double>();
  A.stat = ctx->ct_stat.as<uint32_t>();
  CK(record(ctx->ev0, st));
  CK(cudaMemsetAsync(A.diff, 0, A.stride * 16, st));
  CK(cudaMemsetAsync(A.counts + 4ull * n, 0, (uint64_t)n * 8, st));
  CK(cudaMemsetAsync(A.stat, 0, 64, st));
  CK(record(ctx->evm0, st));
  CK(ct_launch(A, ctx->sms, st));
  const uint32_t* counts_src = A.counts;
  const double* red_src = A.red;
  if (step > 1) {
    uint32_t* gc = ctx->ct_gather.as<uint32_t>();
    double* gr = reinterpret_cast<double*>(ctx->ct_gather.as<unsigned char>() + (size_t)m * 24);
    CK(ct_launch_gather(A, first - start, step, m, gc, gr, ctx->sms, st));
    counts_src = gc;
    red_src = gr;
  }
  CK(record(ctx->evm1, st));
  const size_t cbytes = (size_t)m * 24, rbytes = (size_t)m * 16;
  CK(ctx->pin_out.reserve(cbytes + rbytes + 64 + end + 16));
  unsigned char* h = ctx->pin_out.at(0);
  if (m) {
    CK(cudaMemcpyAsync(h, counts_src, cbytes, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(h + cbytes, red_src, rbytes, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaMemcpyAsync(h + cbytes + rbytes, A.stat, 64, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(h + cbytes + rbytes + 64, s->ref.as<uint8_t>() + A.t0, end, cudaMemcpyDeviceToHost, st));
  CK(record(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_ms = elapsed(ctx->ev0, ctx->ev1);
  ctx->main_ms = elapsed(ctx->evm0, ctx->evm1);
  ctx->launches = step > 1 && m ? 7 : 6;
  ctx->last_h2d = 0;
  ctx->last_d2h = cbytes + rbytes + 64 + end;
  const uint32_t* stat = reinterpret_cast<const uint32_t*>(h + cbytes + rbytes);
  if (stat[2]) return fail(ctx, BSQ_ERR_INVALID, "invalid records: " + err_text(stat[2]));
  out.counts = reinterpret_cast<const uint32_t*>(h);
  out.red = reinterpret_cast<const double*>(h + cbytes);
  out.ref = reinterpret_cast<const char*>(h + cbytes + rbytes + 64);
  out.start = start;
  out.end = end;
  out.last = stat[0];
  out.first = first;
  out.step = step;
  out.m = m;
  return BSQ_OK;
}

int bsq_coverage_columns(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                         bsq_cov_columns* out, uint32_t* last_column_1) {
  return bsq_coverage_columns_rg(ctx, sample_id, tid, start_1, end_1, -1, out, last_column_1);
}

int bsq_coverage_columns_rg(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                            int32_t read_group, bsq_cov_columns* out, uint32_t* last_column_1) {
  if (!ctx || !out) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  host::CoverageRegion R;
  const int rc = coverage_region(ctx, sample_id, tid, start_1, end_1, start_1, 1, R, read_group < 0 ? -1 : read_group);
  if (rc != BSQ_OK) return rc;
  uint32_t* const u32[6] = {out->unique_top, out->unique_bot, out->raw_redundant_top, out->raw_redundant_bot,
                            out->unique_top_begin, out->unique_bot_begin};
  for (int q = 0; q < 6; q++)
    if (u32[q]) memcpy(u32[q], R.counts + (size_t)q * R.m, (size_t)R.m * 4);
  if (out->redundant_top) memcpy(out->redundant_top, R.red, (size_t)R.m * 8);
  if (out->redundant_bot) memcpy(out->redundant_bot, R.red + R.m, (size_t)R.m * 8);
  if (last_column_1) *last_column_1 = R.last;
  return BSQ_OK;
}

int bsq_write_coverage_region(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id, uint32_t tid,
                              uint32_t start_1, uint32_t end_1, uint32_t resolution, uint32_t flags,
                              const double* reference_average) {
  return bsq_write_coverage_region_rg(ctx, sample_id, path, seq_id, tid, start_1, end_1, resolution,
                                      flags & ~(uint32_t)BSQ_COV_PER_READ_GROUP, reference_average, 0);
}

int bsq_write_coverage_region_rg(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id, uint32_t tid,
                                 uint32_t start_1, uint32_t end_1, uint32_t resolution, uint32_t flags,
                                 const double* reference_average, uint32_t n_read_groups) {
  if (!ctx || !path) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (start_1 < 1 || start_1 > end_1) return fail(ctx, BSQ_ERR_INVALID, "region outside the target");
  if (n_read_groups > 0xFFFF) return fail(ctx, BSQ_ERR_INVALID, "more read groups than a record can name");
  // only the positions the table can show a count for come back: the handled ones
  const uint32_t ds = host::coverage_downsample(start_1, end_1, resolution);
  const uint32_t first = host::coverage_first_handled(start_1, ds);
  host::CoverageRegion R;
  int rc = coverage_region(ctx, sample_id, tid, start_1, end_1, first, ds, R);
  if (rc != BSQ_OK) return rc;
  R.own();
  // --per-read-group: the same columns over each group's records (num_read_group_columns() =
  // max(read groups, 1), coverage_output.h:143-152)
  std::vector<host::CoverageRegion> per_rg;
  if (flags & BSQ_COV_PER_READ_GROUP) {
    per_rg.resize(std::max<uint32_t>(n_read_groups, 1));
    for (uint32_t g = 0; g < per_rg.size(); g++) {
      rc = coverage_region(ctx, sample_id, tid, start_1, end_1, first, ds, per_rg[g], (int32_t)g);
      if (rc != BSQ_OK) return rc;
      per_rg[g].own();
    }
  }
  (void)seq_id;   // the table has no seq_id column; the name is part of the caller's file name
  if (!host::write_coverage_region(path, R, resolution, flags, reference_average, per_rg))
    return fail(ctx, BSQ_ERR_INVALID, std::string("cannot write ") + path);
  return BSQ_OK;
}

// The discordant-pair read groups as the 256-bit mask the kernels take (identify_mutations.cpp:883-911).
static int dp_mask_groups(bsq_ctx* ctx, uint32_t n_read_groups, const int32_t* dp_group, uint32_t out[8]) {
  bsq_im_params p;
  memset(&p, 0, sizeof p);
  p.n_read_groups = dp_group ? n_read_groups : 0;
  p.dp_group = dp_group;
  return dp_mask(ctx, p, out);
}

int bsq_im_coverage_columns_rg(bsq_ctx* ctx, int32_t sample_id, uint32_t tid, uint32_t start_1, uint32_t end_1,
                               int32_t read_group, int coverage_fit_failed, uint32_t n_read_groups,
                               const int32_t* dp_group, bsq_cov_columns* out) {
  if (!ctx || !out) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  uint32_t dp[8];
  int rc = dp_mask_groups(ctx, n_read_groups, dp_group, dp);
  if (rc != BSQ_OK) return rc;
  host::CoverageRegion R;
  rc = coverage_region(ctx, sample_id, tid, start_1, end_1, start_1, 1, R, read_group < 0 ? -1 : read_group,
                       coverage_fit_failed ? kCtImTabulate : kCtImPileup, dp);
  if (rc != BSQ_OK) return rc;
  uint32_t* const u32[4] = {out->unique_top, out->unique_bot, out->raw_redundant_top, out->raw_redundant_bot};
  for (int q = 0; q < 4; q++)
    if (u32[q]) memcpy(u32[q], R.counts + (size_t)q * R.m, (size_t)R.m * 4);
  if (out->unique_top_begin) memset(out->unique_top_begin, 0, (size_t)R.m * 4);
  if (out->unique_bot_begin) memset(out->unique_bot_begin, 0, (size_t)R.m * 4);
  if (out->redundant_top) memcpy(out->redundant_top, R.red, (size_t)R.m * 8);
  if (out->redundant_bot) memcpy(out->redundant_bot, R.red + R.m, (size_t)R.m * 8);
  return BSQ_OK;
}

int bsq_write_coverage_table_rg(bsq_ctx* ctx, int32_t sample_id, const char* path, const char* seq_id,
                                const bsq_reference* ref, uint32_t tid, const bsq_position_arrays* positions,
                                uint32_t n_read_groups, int coverage_fit_failed, const int32_t* dp_group) {
  if (!ctx || !path || !ref || !positions) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (tid >= ref->n_targets) return fail(ctx, BSQ_ERR_INVALID, "target index out of range");
  if (n_read_groups > 0xFFFF) return fail(ctx, BSQ_ERR_INVALID, "more read groups than a record can name");
  uint32_t dp[8];
  int rc = dp_mask_groups(ctx, n_read_groups, dp_group, dp);
  if (rc != BSQ_OK) return rc;
  const uint32_t len = (uint32_t)(ref->target_offset[tid + 1] - ref->target_offset[tid]);
  // _print_read_group_coverage: only with more than one read group (identify_mutations.cpp:862)
  const uint32_t groups = n_read_groups > 1 && len > 0 ? n_read_groups : 0;
  std::ofstream out(path);
  if (!out) return fail(ctx, BSQ_ERR_INVALID, std::string("cannot write ") + path);
  host::write_im_coverage_header(out, groups);
  // the groups' columns come chunk by chunk, so host memory stays at one chunk per group
  constexpr uint32_t kChunk = 1u << 20;
  std::vector<host::CoverageRegion> per_rg(groups);
  for (uint32_t a = 1; a <= len || (a == 1 && len == 0); a += kChunk) {
    const uint32_t b = std::min<uint64_t>((uint64_t)a + kChunk - 1, len);
    for (uint32_t g = 0; g < groups; g++) {
      rc = coverage_region(ctx, sample_id, tid, a, b, a, 1, per_rg[g], (int32_t)g,
                           coverage_fit_failed ? kCtImTabulate : kCtImPileup, dp);
      if (rc != BSQ_OK) return rc;
      per_rg[g].own();
    }
    rc = host::write_im_coverage_rows(out, ref, tid, positions, a - 1, b, per_rg);
    if (rc != BSQ_OK) return fail(ctx, rc, std::string("cannot write ") + path);
    if (len == 0) break;
  }
  (void)seq_id;
  if (!out.flush()) return fail(ctx, BSQ_ERR_INVALID, std::string("cannot write ") + path);
  return BSQ_OK;
}

int bsq_sc_result_copy(const bsq_ctx* ctx, bsq_sc_position* rows, uint64_t capacity) {
  if (!ctx || (!rows && capacity)) return BSQ_ERR_INVALID;
  if (capacity < ctx->sc_res.size()) return BSQ_ERR_SIZE;
  std::copy(ctx->sc_res.begin(), ctx->sc_res.end(), rows);
  return BSQ_OK;
}

int bsq_last_pass_stats(const bsq_ctx* ctx, double* device_ms, uint32_t* kernel_launches, double* main_kernel_ms) {
  if (!ctx) return BSQ_ERR_INVALID;
  if (device_ms) *device_ms = ctx->last_ms;
  if (kernel_launches) *kernel_launches = ctx->launches;
  if (main_kernel_ms) *main_kernel_ms = ctx->main_ms;
  return BSQ_OK;
}

int bsq_last_pass_bytes(const bsq_ctx* ctx, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
  if (!ctx) return BSQ_ERR_INVALID;
  if (h2d_bytes) *h2d_bytes = ctx->last_h2d;
  if (d2h_bytes) *d2h_bytes = ctx->last_d2h;
  return BSQ_OK;
}

int bsq_get_tuning(const bsq_ctx* ctx, bsq_tuning* out) {
  if (!ctx || !out) return BSQ_ERR_INVALID;
  *out = ctx->tune;
  return BSQ_OK;
}

int bsq_set_tuning(bsq_ctx* ctx, const bsq_tuning* t) {
  if (!ctx || !t) return BSQ_ERR_INVALID;
  if (t->ec_read_chunk < 64 || t->ec_read_chunk > (1u << 20) || t->ec_blocks_per_sm < 1 || t->ec_blocks_per_sm > 64 ||
      t->col_blocks_per_sm < 1 || t->col_blocks_per_sm > 64 || t->cand_warps_per_sm < 1 || t->cand_warps_per_sm > 64 ||
      t->bound_warps_per_sm < 1 || t->bound_warps_per_sm > 8)
    return fail(ctx, BSQ_ERR_INVALID, "tuning value out of range");
  ctx->tune = *t;
  return BSQ_OK;
}

int bsq_autotune(bsq_ctx* ctx, uint32_t n, const int32_t* ids, const bsq_ec_params* ec, const bsq_im_params* im,
                 const double* const* tables, bsq_tuning* chosen) {
  if (!ctx || !ids || !ec || !im || !tables || n == 0) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  std::vector<bsq_ec_result> eo(n);
  memset(eo.data(), 0, n * sizeof(bsq_ec_result));
  auto time_ec = [&](double& ms) -> int {
    const int rc = bsq_error_count_batch(ctx, n, ids, ec, eo.data());
    ms = ctx->last_ms;
    return rc;
  };
  auto time_im = [&](double& ms) -> int {
    const int rc = bsq_identify_mutations_batch(ctx, n, ids, im, tables, nullptr);
    ms = ctx->last_ms;
    return rc;
  };
  // coordinate search: each knob over its candidates with the others held, fastest kept
  auto search = [&](uint32_t bsq_tuning::*knob, std::initializer_list<uint32_t> values, bool pass1) -> int {
    bsq_tuning best = ctx->tune;
    double best_ms = 1e300;
    for (uint32_t v : values) {
      bsq_tuning t = best;
      t.*knob = v;
      ctx->tune = t;
      double ms = 0;
      const int rc = pass1 ? time_ec(ms) : time_im(ms);
      if (rc != BSQ_OK) return rc;
      if (ms < best_ms) { best_ms = ms; best = t; }
    }
    ctx->tune = best;
    return BSQ_OK;
  };
  const bsq_tuning start = ctx->tune;
  double warm = 0;
  int rc = time_ec(warm);                           // first use: allocations and graph instantiation
  if (rc == BSQ_OK) rc = time_im(warm);
  if (rc == BSQ_OK) rc = search(&bsq_tuning::ec_read_chunk, {256, 512, 1024, 2048, 4096}, true);
  if (rc == BSQ_OK) rc = search(&bsq_tuning::ec_blocks_per_sm, {2, 4, 6, 8, 12}, true);
  if (rc == BSQ_OK) rc = search(&bsq_tuning::col_blocks_per_sm, {2, 3, 4, 6, 8, 12}, false);
  if (rc == BSQ_OK) rc = search(&bsq_tuning::cand_warps_per_sm, {4, 8, 16, 32}, false);
  if (rc == BSQ_OK) rc = search(&bsq_tuning::bound_warps_per_sm, {1, 2, 3, 4, 6, 8}, false);
  if (rc != BSQ_OK) { ctx->tune = start; return rc; }
  if (chosen) *chosen = ctx->tune;
  return BSQ_OK;
}

int bsq_score_positions_noalloc(bsq_ctx* ctx, int32_t sid, const bsq_im_params* p, const double* table,
                                const uint32_t* d_tid, const uint32_t* d_pos0, uint32_t n_positions, bsq_ra_raw* d_ra,
                                uint32_t ra_capacity, uint32_t* d_n_ra, uint32_t* d_qhist) {
  if (!ctx || !p || !table || !d_n_ra || (n_positions && (!d_tid || !d_pos0)) || (ra_capacity && (!d_ra || !d_qhist)))
    return fail(ctx, BSQ_ERR_INVALID, "null argument");
  SampleDev* s = find_sample(ctx, sid);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  if (!p->deletion_propagation_cutoff) return fail(ctx, BSQ_ERR_INVALID, "missing deletion cutoffs");
  const uint32_t R = p->n_read_files, Q = p->n_quality;
  if (R == 0 || Q == 0 || R > 255 || Q > 256) return fail(ctx, BSQ_ERR_INVALID, "error table dimensions out of range");
  if ((uint64_t)R * 25 * Q > kNoAllocMaxTable)
    return fail(ctx, BSQ_ERR_SIZE, "error table larger than the no-allocation limit (R x 25 x Q <= 32768)");
  const uint64_t K = (uint64_t)s->mapq_values.size() * R * 2 * Q * 5;
  if (K > kNoAllocMaxClasses)
    return fail(ctx, BSQ_ERR_SIZE, "more likelihood classes than the no-allocation limit (32768)");
  const uint32_t per_warp = std::max<uint32_t>(32, s->max_tile_reads);
  const uint64_t fit = kNoAllocGatherEntries / cand_warp_stride(per_warp);
  if (fit == 0) return fail(ctx, BSQ_ERR_SIZE, "a column is covered by more reads than the no-allocation scratch holds");
  if (s->n_targets > kNoAllocMaxTargets)
    return fail(ctx, BSQ_ERR_SIZE, "more targets than the no-allocation limit (32768)");
  NoAllocJob J;
  {
    const int rc = dp_mask(ctx, *p, J.dp_rg);
    if (rc != BSQ_OK) return rc;
  }
  CK(cudaSetDevice(ctx->device));
  void* scratch = nullptr;
  CK(noalloc_scratch_setup(ctx->device, &scratch));
  cudaStream_t st = ctx->stream;
  J.log10_table = table; J.R = R; J.Q = Q;
  J.mapq_values = s->mapq_values.data(); J.n_mapq = (uint32_t)s->mapq_values.size();
  J.tid = d_tid; J.pos0 = d_pos0; J.n_positions = n_positions;
  J.prop_cutoff = p->deletion_propagation_cutoff; J.n_targets = s->n_targets;
  J.ra = d_ra; J.ra_cap = ra_capacity; J.n_ra = d_n_ra; J.qhist = d_qhist;
  J.base_quality_cutoff = p->base_quality_cutoff; J.log10_ref_len = p->log10_ref_length;
  J.mutation_cutoff = p->mutation_cutoff; J.poly_cutoff = p->polymorphism_cutoff;
  J.precision_decimal = p->polymorphism_precision_decimal;
  J.per_warp = per_warp;
  J.n_warps = (uint32_t)std::min<uint64_t>((uint64_t)ctx->sms * 16, fit);
  uint32_t err = 0;
  CK(launch_noalloc_positions(scratch, make_dev_sample(*s), J, st, &err));
  err &= ~kErrRaOverflow;
  if (err) return fail(ctx, BSQ_ERR_DATA, "score_positions_noalloc: " + err_text(err));
  uint32_t n_ra = 0;
  CK(cudaMemcpy(&n_ra, d_n_ra, sizeof n_ra, cudaMemcpyDeviceToHost));
  if (n_ra > ra_capacity) return fail(ctx, BSQ_ERR_SIZE, "more passing RA items than ra_capacity");
  return BSQ_OK;
}

int bsq_timer_start(bsq_ctx* ctx) {
  if (!ctx) return BSQ_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaEventRecord(ctx->evt0, ctx->stream));
  return BSQ_OK;
}

int bsq_timer_stop(bsq_ctx* ctx, double* ms) {
  if (!ctx || !ms) return BSQ_ERR_INVALID;
  CK(cudaSetDevice(ctx->device));
  CK(cudaEventRecord(ctx->evt1, ctx->stream));
  CK(cudaEventSynchronize(ctx->evt1));
  float f = 0;
  CK(cudaEventElapsedTime(&f, ctx->evt0, ctx->evt1));
  *ms = f;
  return BSQ_OK;
}

int bsq_host_register(void* ptr, uint64_t bytes) {
  if (!ptr || !bytes) return BSQ_ERR_INVALID;
  return cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess ? BSQ_OK : BSQ_ERR_CUDA;
}

int bsq_host_unregister(void* ptr) {
  if (!ptr) return BSQ_ERR_INVALID;
  return cudaHostUnregister(ptr) == cudaSuccess ? BSQ_OK : BSQ_ERR_CUDA;
}


// ============================================================================ BAM input
// The BGZF block table comes from the block headers on the host (each gives its compressed size, so
// no inflating is needed to find them; SAM/BAM specification §4.1); the device does the rest.
}  // extern "C"

struct bsq_bam {
  bsq_ctx* ctx = nullptr;
  DevMem file, stream, blocks, scratch;
  std::vector<BgzfBlock> hblocks;
  uint64_t stream_len = 0, records_begin = 0;
  std::string text;
  std::vector<std::string> names;
  std::vector<const char*> name_ptrs;
  std::vector<uint32_t> lengths;
  std::unique_ptr<RecordsDev> rec;   // the decoded records until they move into a sample
  bool decoded = false;
};

static bool parse_bgzf(const uint8_t* d, uint64_t size, std::vector<BgzfBlock>& out, uint64_t& stream_len, std::string& why) {
  out.clear();
  uint64_t pos = 0, opos = 0;
  auto u16 = [&](uint64_t o) { return (uint32_t)d[o] | ((uint32_t)d[o + 1] << 8); };
  auto u32 = [&](uint64_t o) { return u16(o) | (u16(o + 2) << 16); };
  while (pos < size) {
    if (size - pos < 18) { why = "truncated BGZF block header"; return false; }
    if (d[pos] != 31 || d[pos + 1] != 139 || d[pos + 2] != 8 || !(d[pos + 3] & 4)) { why = "not a BGZF block"; return false; }
    const uint32_t xlen = u16(pos + 10);
    if (size - pos < 12ull + xlen) { why = "truncated BGZF extra field"; return false; }
    uint32_t bsize = 0;
    bool found = false;
    for (uint64_t x = pos + 12; x + 4 <= pos + 12 + xlen;) {
      const uint32_t slen = u16(x + 2);
      if (d[x] == 66 && d[x + 1] == 67 && slen == 2 && x + 6 <= pos + 12 + xlen) { bsize = u16(x + 4); found = true; }
      x += 4 + slen;
    }
    if (!found) { why = "BGZF block without a BC field"; return false; }
    const uint64_t total = (uint64_t)bsize + 1;
    if (total < 12ull + xlen + 8 || total > size - pos) { why = "BGZF block size out of range"; return false; }
    BgzfBlock b;
    b.in_off = pos + 12 + xlen;
    b.in_len = (uint32_t)(total - 12 - xlen - 8);
    b.crc = u32(pos + total - 8);
    b.isize = u32(pos + total - 4);
    b.out_off = opos;
    b.pad = 0;
    if (b.isize > 65536) { why = "BGZF block larger than 64 KiB"; return false; }
    out.push_back(b);
    opos += b.isize;
    pos += total;
  }
  stream_len = opos;
  return true;
}

// The BAM header from the start of the inflated stream: magic, text, reference names and lengths.
// Returns 0 when complete, 1 when more of the stream is needed, -1 when malformed.
static int parse_bam_header(const uint8_t* h, uint64_t n, bsq_bam& B) {
  auto i32 = [&](uint64_t o) { return (int32_t)((uint32_t)h[o] | ((uint32_t)h[o + 1] << 8) | ((uint32_t)h[o + 2] << 16) | ((uint32_t)h[o + 3] << 24)); };
  if (n < 8) return 1;
  if (memcmp(h, "BAM\1", 4) != 0) return -1;
  const int32_t l_text = i32(4);
  if (l_text < 0) return -1;
  uint64_t o = 8 + (uint64_t)l_text;
  if (n < o + 4) return 1;
  const int32_t n_ref = i32(o);
  if (n_ref < 0) return -1;
  o += 4;
  std::vector<std::string> names;
  std::vector<uint32_t> lens;
  for (int32_t r = 0; r < n_ref; r++) {
    if (n < o + 4) return 1;
    const int32_t l_name = i32(o);
    if (l_name < 1) return -1;
    if (n < o + 4 + (uint64_t)l_name + 4) return 1;
    names.emplace_back(reinterpret_cast<const char*>(h + o + 4), strnlen(reinterpret_cast<const char*>(h + o + 4), (size_t)l_name));
    const int32_t l_ref = i32(o + 4 + (uint64_t)l_name);
    if (l_ref < 0) return -1;
    lens.push_back((uint32_t)l_ref);
    o += 4 + (uint64_t)l_name + 4;
  }
  B.text.assign(reinterpret_cast<const char*>(h + 8), (size_t)l_text);
  B.names = std::move(names);
  B.lengths = std::move(lens);
  B.name_ptrs.clear();
  for (auto& x : B.names) B.name_ptrs.push_back(x.c_str());
  B.records_begin = o;
  return 0;
}

static std::string bam_err_text(uint32_t e) {
  std::string s;
  if (e & kBamInflate) s += "BGZF block does not inflate; ";
  if (e & kBamCrc) s += "BGZF block CRC-32 mismatch; ";
  if (e & kBamSpan) s += "a record's size is invalid; ";
  if (e & kBamRecord) s += "record fields out of range; ";
  if (e & kBamAux) s += "malformed aux field; ";
  if (e & kBamOrder) s += "unplaced records before placed ones; ";
  if (e & kBamLongCigar) s += "a CIGAR of more than 65535 operations kept in the CG tag (not supported); ";
  return s;
}

extern "C" {

int bsq_bam_open(bsq_ctx* ctx, const uint8_t* data, uint64_t size, bsq_bam** out) {
  if (!ctx || !data || !out) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  std::unique_ptr<bsq_bam> B(new bsq_bam());
  B->ctx = ctx;
  std::string why;
  if (!parse_bgzf(data, size, B->hblocks, B->stream_len, why)) return fail(ctx, BSQ_ERR_INVALID, why);
  cudaStream_t st = ctx->stream;
  const uint32_t nb = (uint32_t)B->hblocks.size();
  CK(B->file.alloc(size + 16, st));
  CK(cudaMemcpyAsync(B->file.p, data, size, cudaMemcpyHostToDevice, st));
  CK(upload(B->blocks, B->hblocks.data(), nb, st));
  CK(B->stream.alloc(B->stream_len + 64, st));
  CK(B->scratch.alloc(64, st));
  uint32_t* w = B->scratch.as<uint32_t>();
  CK(cudaMemsetAsync(w, 0, 4, st));
  CK(cudaMemsetAsync(w + 1, 0xFF, 4, st));
  // token room for up to 16384 blocks at a time (4 GiB), freed once the stream is inflated
  const uint32_t tok_blocks = std::max<uint32_t>(1, std::min<uint32_t>(nb, 16384));
  DevMem tok;
  CK(tok.alloc(bam_token_bytes(tok_blocks), st));
  uint32_t* tokp = tok.as<uint32_t>();
  CK(record(ctx->ev0, st));
  CK(bam_inflate(B->file.as<uint8_t>(), B->blocks.as<BgzfBlock>(), nb, B->stream.as<uint8_t>(), tokp,
                 tokp + (size_t)tok_blocks * 65536, tok_blocks, w, w + 1, ctx->sms, st));
  CK(record(ctx->ev1, st));
  uint32_t h[2];
  CK(cudaMemcpyAsync(h, w, 8, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_ms = ctx->main_ms = elapsed(ctx->ev0, ctx->ev1);
  ctx->launches = nb ? 1 : 0;
  ctx->last_h2d = size;
  if (h[0]) return fail(ctx, BSQ_ERR_DATA, bam_err_text(h[0]) + "first failing block " + std::to_string(h[1]));
  // the header: fetch a growing prefix of the stream until it parses
  std::vector<uint8_t> pre;
  for (uint64_t want = std::min<uint64_t>(B->stream_len, 1 << 16);; want = std::min<uint64_t>(B->stream_len, want * 4)) {
    pre.resize(want);
    CK(cudaMemcpy(pre.data(), B->stream.p, want, cudaMemcpyDeviceToHost));
    const int r = parse_bam_header(pre.data(), want, *B);
    if (r == 0) break;
    if (r < 0 || want == B->stream_len) return fail(ctx, BSQ_ERR_INVALID, "malformed BAM header");
  }
  *out = B.release();
  return BSQ_OK;
}

void bsq_bam_close(bsq_bam* bam) {
  if (!bam) return;
  cudaSetDevice(bam->ctx->device);
  cudaStreamSynchronize(bam->ctx->stream);
  delete bam;
}

int bsq_bam_header(const bsq_bam* bam, const char** text, uint64_t* text_len, uint32_t* n_ref,
                   const char* const** ref_names, const uint32_t** ref_lengths) {
  if (!bam) return BSQ_ERR_INVALID;
  if (text) *text = bam->text.c_str();
  if (text_len) *text_len = bam->text.size();
  if (n_ref) *n_ref = (uint32_t)bam->names.size();
  if (ref_names) *ref_names = bam->name_ptrs.data();
  if (ref_lengths) *ref_lengths = bam->lengths.data();
  return BSQ_OK;
}

int bsq_bam_decode(bsq_ctx* ctx, bsq_bam* bam, const bsq_bam_groups* groups, uint64_t* n_records,
                   uint64_t* n_cigar_total, uint64_t* n_bases_total) {
  if (!ctx || !bam || bam->ctx != ctx) return fail(ctx, BSQ_ERR_INVALID, "null argument or another context's BAM");
  CK(cudaSetDevice(ctx->device));
  BamGroups G;
  memset(&G, 0, sizeof G);
  std::string ids;
  if (groups && groups->n_groups) {
    if (groups->n_groups > (uint32_t)kBamMaxGroups || !groups->ids)
      return fail(ctx, BSQ_ERR_INVALID, "more than 64 read groups, or no IDs");
    G.n = groups->n_groups;
    for (uint32_t g = 0; g < G.n; g++) {
      G.id_off[g] = (uint32_t)ids.size();
      ids += groups->ids[g];
      G.file_base[g] = groups->file_base ? groups->file_base[g] : 0;
      G.file_count[g] = (groups->file_base && groups->file_count) ? groups->file_count[g] : 0;
    }
    G.id_off[G.n] = (uint32_t)ids.size();
  }
  cudaStream_t st = ctx->stream;
  cudaGetLastError();
  const uint32_t nb = (uint32_t)bam->hblocks.size();
  uint32_t* w = bam->scratch.as<uint32_t>();
  CK(record(ctx->ev0, st));
  CK(cudaMemsetAsync(w, 0, 16, st));
  CK(cudaMemsetAsync(w + 1, 0xFF, 4, st));
  // records per block, then their offsets
  DevMem counts, base;
  CK(counts.alloc((uint64_t)nb * 4 + 16, st));
  CK(bam_walk(bam->stream.as<uint8_t>(), bam->blocks.as<BgzfBlock>(), nb, bam->records_begin, counts.as<uint32_t>(),
              nullptr, nullptr, w, ctx->sms, st));
  std::vector<uint32_t> hc(nb);
  uint32_t herr = 0;
  if (nb) CK(cudaMemcpyAsync(hc.data(), counts.p, (uint64_t)nb * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&herr, w, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  DevMem offsets;
  uint64_t n = 0;
  if (herr == kBamSpan) {
    // a record spans BGZF blocks (htslib's writer never does this, other writers do): the record
    // offsets come from one walk over the whole inflated stream on the host
    std::vector<uint8_t> hs(bam->stream_len);
    CK(cudaMemcpy(hs.data(), bam->stream.p, bam->stream_len, cudaMemcpyDeviceToHost));
    std::vector<uint64_t> ho;
    for (uint64_t p = bam->records_begin; p < bam->stream_len;) {
      if (p + 4 > bam->stream_len) return fail(ctx, BSQ_ERR_INVALID, "a record is cut off at the end of the stream");
      const int32_t bs = (int32_t)(hs[p] | ((uint32_t)hs[p + 1] << 8) | ((uint32_t)hs[p + 2] << 16) |
                                   ((uint32_t)hs[p + 3] << 24));
      if (bs < 32 || p + 4 + (uint64_t)bs > bam->stream_len) return fail(ctx, BSQ_ERR_INVALID, "a record's size is invalid");
      ho.push_back(p);
      p += 4 + (uint64_t)bs;
    }
    n = ho.size();
    if (n >= 0xFFFFFFFFull) return fail(ctx, BSQ_ERR_INVALID, "more than 2^32 - 1 records");
    CK(offsets.alloc(n * 8 + 16, st));
    if (n) CK(cudaMemcpyAsync(offsets.p, ho.data(), n * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w, 0, 4, st));
    CK(cudaStreamSynchronize(st));
  } else {
    if (herr) return fail(ctx, BSQ_ERR_INVALID, bam_err_text(herr));
    std::vector<uint64_t> hb(nb);
    for (uint32_t b = 0; b < nb; b++) { hb[b] = n; n += hc[b]; }
    if (n >= 0xFFFFFFFFull) return fail(ctx, BSQ_ERR_INVALID, "more than 2^32 - 1 records");
    CK(upload(base, hb.data(), nb, st));
    CK(offsets.alloc(n * 8 + 16, st));
    CK(bam_walk(bam->stream.as<uint8_t>(), bam->blocks.as<BgzfBlock>(), nb, bam->records_begin, nullptr,
                base.as<uint64_t>(), offsets.as<uint64_t>(), w, ctx->sms, st));
  }
  // fixed fields and tags
  bam->rec.reset(new RecordsDev());
  bam->decoded = false;
  RecordsDev& R = *bam->rec;
  CK(R.tid.alloc(n * 4 + 16, st)); CK(R.pos.alloc(n * 4 + 16, st)); CK(R.flag.alloc(n * 2 + 16, st));
  CK(R.mapq.alloc(n + 16, st)); CK(R.x1.alloc(n * 4 + 16, st)); CK(R.xl.alloc(n * 4 + 16, st));
  CK(R.xr.alloc(n * 4 + 16, st)); CK(R.rfile.alloc(n + 16, st)); CK(R.rg.alloc(n * 2 + 16, st));
  CK(R.lq.alloc(n * 4 + 16, st)); CK(R.soff.alloc(n * 8 + 16, st)); CK(R.coff.alloc(n * 8 + 16, st));
  CK(R.nc.alloc(n * 2 + 16, st)); CK(R.xj.alloc(n + 16, st));
  CK(R.isize.alloc(n * 4 + 16, st)); CK(R.xp.alloc(n + 16, st)); CK(R.qoff.alloc(n * 8 + 24, st));
  CK(R.mtid.alloc(n * 4 + 16, st)); CK(R.mpos.alloc(n * 4 + 16, st));
  DevMem ncig32, nib, nlen, tmp, ids_dev;
  CK(ncig32.alloc(n * 4 + 16, st));
  CK(nib.alloc(n * 4 + 16, st));
  CK(nlen.alloc(n * 4 + 16, st));
  CK(tmp.alloc((n / 1024 + 4) * 8 + 64, st));
  CK(upload(ids_dev, ids.data(), ids.size() + 1, st));
  BamRecordsDev D;
  D.tid = R.tid.as<int32_t>(); D.pos = R.pos.as<int32_t>(); D.flag = R.flag.as<uint16_t>(); D.mapq = R.mapq.as<uint8_t>();
  D.x1 = R.x1.as<uint32_t>(); D.xl = R.xl.as<int32_t>(); D.xr = R.xr.as<int32_t>(); D.read_file = R.rfile.as<uint8_t>();
  D.read_group = R.rg.as<uint16_t>(); D.l_qseq = R.lq.as<uint32_t>(); D.seq_off = R.soff.as<uint64_t>();
  D.cigar_off = R.coff.as<uint64_t>(); D.n_cigar = R.nc.as<uint16_t>(); D.xj = R.xj.as<uint8_t>();
  D.isize = R.isize.as<int32_t>(); D.xp = R.xp.as<uint8_t>(); D.qoff = R.qoff.as<uint64_t>();
  D.mtid = R.mtid.as<int32_t>(); D.mpos = R.mpos.as<int32_t>();
  D.cigar = nullptr; D.seq = nullptr; D.qual = nullptr; D.qname = nullptr;
  CK(bam_fields(bam->stream.as<uint8_t>(), offsets.as<uint64_t>(), n, (uint32_t)bam->names.size(), G,
                ids_dev.as<char>(), D, ncig32.as<uint32_t>(), nib.as<uint32_t>(), nlen.as<uint32_t>(), w, ctx->sms, st));
  // CIGAR, base and read-name offsets
  uint64_t* tot = reinterpret_cast<uint64_t*>(w + 4);   // [0] CIGAR ops, [1] nibbles, [2] name bytes
  CK(scan_u32(ncig32.as<uint32_t>(), D.cigar_off, n, tmp.as<uint64_t>(), tot, st));
  CK(scan_u32(nib.as<uint32_t>(), D.seq_off, n, tmp.as<uint64_t>(), tot + 1, st));
  CK(scan_u32(nlen.as<uint32_t>(), D.qoff, n, tmp.as<uint64_t>(), tot + 2, st));
  CK(cudaMemcpyAsync(D.qoff + n, tot + 2, 8, cudaMemcpyDeviceToDevice, st));
  uint32_t hw[12];
  CK(cudaMemcpyAsync(hw, w, 48, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (hw[0]) return fail(ctx, BSQ_ERR_INVALID, bam_err_text(hw[0]));
  uint64_t totals[3];
  memcpy(totals, hw + 4, 24);
  // unplaced records: all after the placed ones; they are dropped
  uint64_t used = n;
  if (hw[1] != 0xFFFFFFFFu) {
    if (hw[2] > hw[1]) return fail(ctx, BSQ_ERR_INVALID, bam_err_text(kBamOrder));
    used = hw[1];
  }
  CK(R.cigar.alloc(totals[0] * 4 + 16, st));
  CK(R.seq.alloc(totals[1] / 2 + 16, st));
  CK(R.qual.alloc(totals[1] + 16, st));
  CK(R.qname.alloc(totals[2] + 16, st));
  D.cigar = R.cigar.as<uint32_t>(); D.seq = R.seq.as<uint8_t>(); D.qual = R.qual.as<uint8_t>();
  D.qname = R.qname.as<char>();
  CK(bam_copy(bam->stream.as<uint8_t>(), offsets.as<uint64_t>(), n, D, ctx->sms, st));
  CK(record(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_ms = ctx->main_ms = elapsed(ctx->ev0, ctx->ev1);
  ctx->launches = 12;
  // the dropped unplaced records are the last ones: their CIGARs and bases are at the arrays' ends
  R.n = used;
  if (used < n) {
    uint64_t off[2];
    CK(cudaMemcpy(&off[0], D.cigar_off + used, 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&off[1], D.seq_off + used, 8, cudaMemcpyDeviceToHost));
    R.n_cigar_total = off[0];
    R.n_bases_total = off[1];
  } else {
    R.n_cigar_total = totals[0];
    R.n_bases_total = totals[1];
  }
  R.has_xj = true;
  R.has_pairs = true;
  R.has_mates = true;
  bam->decoded = true;
  if (n_records) *n_records = R.n;
  if (n_cigar_total) *n_cigar_total = R.n_cigar_total;
  if (n_bases_total) *n_bases_total = R.n_bases_total;
  return BSQ_OK;
}

int bsq_bam_copy_records(bsq_ctx* ctx, const bsq_bam* bam, const bsq_read_arrays* out) {
  if (!ctx || !bam || !out) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (!bam->decoded) return fail(ctx, BSQ_ERR_INVALID, "BAM not decoded");
  CK(cudaSetDevice(ctx->device));
  const RecordsDev& R = *bam->rec;
  const uint64_t n = R.n;
  struct Item { void* dst; const DevMem* src; uint64_t bytes; };
  const Item items[] = {
      {out->tid, &R.tid, n * 4}, {out->pos, &R.pos, n * 4}, {out->flag, &R.flag, n * 2}, {out->mapq, &R.mapq, n},
      {out->x1, &R.x1, n * 4}, {out->xl, &R.xl, n * 4}, {out->xr, &R.xr, n * 4}, {out->read_file, &R.rfile, n},
      {out->read_group, &R.rg, n * 2}, {out->l_qseq, &R.lq, n * 4}, {out->seq_off, &R.soff, n * 8},
      {out->cigar_off, &R.coff, n * 8}, {out->n_cigar, &R.nc, n * 2}, {out->xj, &R.xj, n},
      {out->cigar, &R.cigar, R.n_cigar_total * 4}, {out->seq, &R.seq, R.n_bases_total / 2},
      {out->qual, &R.qual, R.n_bases_total}, {out->isize, &R.isize, n * 4}, {out->xp, &R.xp, n},
      {out->qname_off, &R.qoff, (n + 1) * 8}, {out->mtid, &R.mtid, n * 4}, {out->mpos, &R.mpos, n * 4}};
  for (const Item& it : items)
    if (it.dst && it.bytes) CK(cudaMemcpyAsync(it.dst, it.src->p, it.bytes, cudaMemcpyDeviceToHost, ctx->stream));
  if (out->qname) {
    uint64_t nb = 0;
    CK(cudaMemcpyAsync(&nb, R.qoff.as<uint64_t>() + n, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (nb) CK(cudaMemcpyAsync(out->qname, R.qname.p, nb, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return BSQ_OK;
}

int bsq_bam_name_bytes(bsq_ctx* ctx, const bsq_bam* bam, uint64_t* bytes) {
  if (!ctx || !bam || !bytes) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (!bam->decoded) return fail(ctx, BSQ_ERR_INVALID, "BAM not decoded");
  CK(cudaSetDevice(ctx->device));
  CK(cudaMemcpy(bytes, bam->rec->qoff.as<uint64_t>() + bam->rec->n, 8, cudaMemcpyDeviceToHost));
  return BSQ_OK;
}

int bsq_bam_load(bsq_ctx* ctx, bsq_bam* bam, const bsq_reference* ref, int32_t* sample_id) {
  if (!ctx || !bam || !ref || !sample_id || bam->ctx != ctx) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  if (!bam->decoded) return fail(ctx, BSQ_ERR_INVALID, "BAM not decoded");
  CK(cudaSetDevice(ctx->device));
  if (ref->n_targets != bam->names.size()) return fail(ctx, BSQ_ERR_INVALID, "reference and BAM header differ in targets");
  for (uint32_t t = 0; t < ref->n_targets; t++)
    if (ref->target_offset[t + 1] - ref->target_offset[t] != bam->lengths[t])
      return fail(ctx, BSQ_ERR_INVALID, "reference and BAM header differ in target length");
  cudaStream_t st = ctx->stream;
  std::unique_ptr<SampleDev> s;
  int rc = new_sample(ctx, ref, bam->rec->n, s, st);
  if (rc != BSQ_OK) return rc;
  rc = pack_sample(ctx, s, *bam->rec, st, sample_id);
  bam->rec.reset();
  bam->decoded = false;
  return rc;
}

}  // extern "C"
