// C ABI of libbsq_gb300.so (include/breseq_gb300.h): sample residency, the two passes, and the
// host-side steps that follow the kernels (RA assembly with Fisher / K-S, MC and UN intervals).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/breseq_gb300.h"
#include "bsq_common.h"
#include "bsq_host.h"
#include "bsq_kernels.h"
#include "bsq_noalloc.h"

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
  DevMem ref, reads, x1, rg, qb, cigar, seq, qual, tile_range, d_tpoff, tgt_group, tgt_called, tgt_failed, rstart, mapq;
  uint32_t n_targets = 0, n_cols = 0, n_tiles = 0, n_reads = 0, maxspan = 1, max_tile_reads = 0;
  uint32_t n_groups = 0;
  std::vector<uint64_t> toff;       // caller's target offsets
  std::vector<uint32_t> tpoff;      // padded offsets
  std::vector<uint32_t> order;      // pileup order
  std::vector<uint32_t> group;
  std::vector<uint8_t> mapq_values; // distinct MAPQ values, index = mapq_idx
};

}  // namespace

struct bsq_ctx {
  int device = 0;
  int sms = 1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm0 = nullptr, evm1 = nullptr, evt0 = nullptr, evt1 = nullptr;
  std::string err;
  std::map<int32_t, std::unique_ptr<SampleDev>> samples;
  int32_t next_id = 1;
  // working memory reused across calls
  DevMem cov, call, blk, total, cand, next, ra, n_ra, qhist, scratch, errw, lp64, r64, lpmax64, lp32, stats;
  DevMem keep, kcol, kcov, kcall, d_prop, d_seed;
  DevMem counts, hist, found, diff_u, diff_r, qs_flag, blk_u, blk_r;
  std::vector<bsq_ra_record> res_ra;
  std::vector<bsq_mc_record> res_mc;
  std::vector<bsq_un_record> res_un;
  double last_ms = 0, main_ms = 0;
  uint32_t launches = 0;
  uint64_t last_candidates = 0;
};

static int fail(bsq_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
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
  S.reads = s.reads.as<DevRead>();
  S.x1 = s.x1.as<uint32_t>();
  S.rg = s.rg.as<uint16_t>();
  S.qb = s.qb.as<QBounds>();
  S.cigar = s.cigar.as<uint32_t>();
  S.seq = s.seq.as<uint8_t>();
  S.qual = s.qual.as<uint8_t>();
  S.tile_range = s.tile_range.as<uint2>();
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
  auto it = ctx->samples.find(id);
  return it == ctx->samples.end() ? nullptr : it->second.get();
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
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return BSQ_ERR_CUDA;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;   // keep freed blocks in this process's pool for the next sample
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
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
  ctx->samples.clear();
  // pool blocks are returned on the context's stream, so before it goes
  for (DevMem* m : {&ctx->cov, &ctx->call, &ctx->blk, &ctx->total, &ctx->cand, &ctx->next, &ctx->ra, &ctx->n_ra,
                    &ctx->qhist, &ctx->scratch, &ctx->errw, &ctx->lp64, &ctx->r64, &ctx->lpmax64, &ctx->lp32,
                    &ctx->stats, &ctx->counts, &ctx->hist, &ctx->found, &ctx->diff_u, &ctx->diff_r, &ctx->qs_flag,
                    &ctx->blk_u, &ctx->blk_r, &ctx->keep, &ctx->kcol, &ctx->kcov,
                    &ctx->kcall, &ctx->d_prop, &ctx->d_seed})
    m->release();
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaEventDestroy(ctx->ev0); cudaEventDestroy(ctx->ev1); cudaEventDestroy(ctx->evm0); cudaEventDestroy(ctx->evm1);
  cudaEventDestroy(ctx->evt0); cudaEventDestroy(ctx->evt1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* bsq_last_error(const bsq_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

uint64_t bsq_sample_footprint(const bsq_reference* ref, const bsq_read_soa* rd) {
  if (!ref || !rd) return 0;
  const uint64_t cols = ref->target_offset[ref->n_targets] + ref->n_targets;
  const uint64_t tiles = (cols + 31) / 32;
  const uint64_t per_read = sizeof(DevRead) + 4 + 2 + sizeof(QBounds) + 4 + 1;
  const uint64_t upload_tmp = rd->n_reads * 48;  // raw arrays, freed after packing
  return cols + 64 + rd->n_reads * per_read + rd->n_cigar_total * 4 + rd->n_bases_total / 2 + 16 +
         rd->n_bases_total + tiles * 8 + upload_tmp;
}

int bsq_load_sample(bsq_ctx* ctx, const bsq_reference* ref, const bsq_read_soa* rd, int32_t* sample_id) {
  if (!ctx || !ref || !rd || !sample_id) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  CK(cudaSetDevice(ctx->device));
  const uint32_t T = ref->n_targets;
  if (T == 0 || !ref->target_offset || !ref->seq || !ref->coverage_group || !ref->target_order)
    return fail(ctx, BSQ_ERR_INVALID, "reference without targets");
  const uint64_t total = ref->target_offset[T];
  if (total + T >= 0xFFFFFF00ull) return fail(ctx, BSQ_ERR_INVALID, "reference longer than 2^32 - 256 columns");
  if (rd->n_reads >= 0xFFFFFFFFull) return fail(ctx, BSQ_ERR_INVALID, "more than 2^32 - 1 records in one sample");
  if (rd->n_reads && (!rd->tid || !rd->pos || !rd->flag || !rd->mapq || !rd->x1 || !rd->xl || !rd->xr ||
                      !rd->read_file || !rd->read_group || !rd->l_qseq || !rd->seq_off || !rd->cigar_off ||
                      !rd->n_cigar || !rd->cigar || !rd->seq || !rd->qual))
    return fail(ctx, BSQ_ERR_INVALID, "null record array");
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
  s->n_reads = (uint32_t)rd->n_reads;
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
  for (uint64_t i = 0; i < total; i++) {
    const char ch = ref->seq[i];
    if (ch != 'A' && ch != 'C' && ch != 'G' && ch != 'T' && ch != 'N')
      return fail(ctx, BSQ_ERR_DATA, "reference base outside A/C/G/T/N");
  }
  cudaStream_t st = ctx->stream;
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
  // records: raw arrays -> packed 32-byte records on the device
  const uint64_t n = rd->n_reads;
  DevMem tid, pos, flag, xl, xr, rfile, lq, soff, coff, nc;
  CK(upload(tid, rd->tid, n, st));
  CK(upload(pos, rd->pos, n, st));
  CK(upload(flag, rd->flag, n, st));
  CK(upload(s->mapq, rd->mapq, n, st));
  CK(upload(s->x1, rd->x1, n, st));
  CK(upload(xl, rd->xl, n, st));
  CK(upload(xr, rd->xr, n, st));
  CK(upload(rfile, rd->read_file, n, st));
  CK(upload(s->rg, rd->read_group, n, st));
  CK(upload(lq, rd->l_qseq, n, st));
  CK(upload(soff, rd->seq_off, n, st));
  CK(upload(coff, rd->cigar_off, n, st));
  CK(upload(nc, rd->n_cigar, n, st));
  CK(upload(s->cigar, rd->cigar, rd->n_cigar_total, st));
  CK(upload(s->seq, rd->seq, (rd->n_bases_total + 1) / 2, st));
  CK(upload(s->qual, rd->qual, rd->n_bases_total, st));
  CK(s->reads.alloc(n * sizeof(DevRead) + 64, st));
  CK(s->qb.alloc(n * sizeof(QBounds) + 64, st));
  CK(s->rstart.alloc(n * 4 + 64, st));
  CK(ctx->stats.alloc(64, st));
  CK(cudaMemsetAsync(ctx->stats.p, 0, 64, st));
  uint32_t* stats = ctx->stats.as<uint32_t>();  // [0] err, [1] maxspan, [2..9] mapq mask, [10] max tile reads
  RawSoA in;
  in.tid = tid.as<int32_t>(); in.pos = pos.as<int32_t>(); in.flag = flag.as<uint16_t>(); in.mapq = s->mapq.as<uint8_t>();
  in.x1 = s->x1.as<uint32_t>(); in.xl = xl.as<int32_t>(); in.xr = xr.as<int32_t>(); in.read_file = rfile.as<uint8_t>();
  in.l_qseq = lq.as<uint32_t>(); in.seq_off = soff.as<uint64_t>(); in.cigar_off = coff.as<uint64_t>();
  in.n_cigar = nc.as<uint16_t>(); in.cigar = s->cigar.as<uint32_t>(); in.tpoff = s->d_tpoff.as<uint32_t>(); in.called = s->tgt_called.as<uint8_t>();
  in.n = (uint32_t)n; in.n_targets = T; in.n_bases = rd->n_bases_total; in.n_cigar_total = rd->n_cigar_total;
  PackOut po;
  po.reads = s->reads.as<DevRead>(); po.qb = s->qb.as<QBounds>(); po.rstart = s->rstart.as<uint32_t>();
  po.mapq = s->mapq.as<uint8_t>(); po.err = stats; po.maxspan = stats + 1; po.mapq_mask = stats + 2;
  CK(launch_pack(in, po, st));
  uint32_t h[16];
  CK(cudaMemcpyAsync(h, stats, 16 * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h[0]) return fail(ctx, (h[0] & (kErrOrder | kErrCigar | kErrBounds | kErrX1)) ? BSQ_ERR_INVALID : BSQ_ERR_DATA,
                        "invalid records: " + err_text(h[0]));
  s->maxspan = std::max<uint32_t>(1, h[1]);
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
  CK(cudaMemcpyAsync(h + 10, stats + 10, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  s->max_tile_reads = h[10];
  const int32_t id = ctx->next_id++;
  ctx->samples[id] = std::move(s);
  *sample_id = id;
  return BSQ_OK;
}

int bsq_free_sample(bsq_ctx* ctx, int32_t id) {
  if (!ctx) return BSQ_ERR_INVALID;
  auto it = ctx->samples.find(id);
  if (it == ctx->samples.end()) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->samples.erase(it);
  return BSQ_OK;
}

// ============================================================================ pass 1
int bsq_error_count(bsq_ctx* ctx, int32_t sid, const bsq_ec_params* p, bsq_ec_result* out) {
  if (!ctx || !p || !out) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  SampleDev* s = find_sample(ctx, sid);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  if (p->n_read_files == 0 || p->n_read_files > 255 || p->n_quality == 0 || p->n_quality > 256)
    return fail(ctx, BSQ_ERR_INVALID, "covariate dimensions out of range");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const uint32_t R = p->n_read_files, Q = p->n_quality, G = s->n_groups;
  const size_t nbins = (size_t)R * 25 * Q;
  const uint32_t cap = s->max_tile_reads + 2;
  CK(ctx->counts.alloc(nbins * 8, st));
  CK(ctx->hist.alloc((size_t)G * cap * 8, st));
  CK(ctx->found.alloc((size_t)s->n_targets * 16 + 16, st));
  CK(ctx->errw.alloc(16, st));
  CK(cudaMemsetAsync(ctx->counts.p, 0, nbins * 8, st));
  CK(cudaMemsetAsync(ctx->hist.p, 0, (size_t)G * cap * 8, st));
  CK(cudaMemsetAsync(ctx->found.p, 0, (size_t)s->n_targets * 16 + 16, st));
  CK(cudaMemsetAsync(ctx->errw.p, 0, 16, st));
  const uint32_t ncb = (s->n_cols + 1023) / 1024;
  CK(ctx->diff_u.alloc((size_t)(s->n_cols + 16) * 4, st));
  CK(ctx->diff_r.alloc((size_t)(s->n_cols + 16) * 4, st));
  CK(ctx->qs_flag.alloc((size_t)2 * s->n_cols + 16, st));
  CK(ctx->blk_u.alloc((size_t)(ncb + 16) * 4, st));
  CK(ctx->blk_r.alloc((size_t)(ncb + 16) * 4, st));
  CK(cudaMemsetAsync(ctx->diff_u.p, 0, (size_t)(s->n_cols + 16) * 4, st));
  CK(cudaMemsetAsync(ctx->diff_r.p, 0, (size_t)(s->n_cols + 16) * 4, st));
  if (p->preprocess_stage) CK(cudaMemsetAsync(ctx->qs_flag.p, 0, (size_t)2 * s->n_cols + 16, st));
  DevSample S = make_dev_sample(*s);
  EcArgs A;
  A.diff_u = ctx->diff_u.as<int32_t>(); A.diff_r = ctx->diff_r.as<int32_t>(); A.qs_flag = ctx->qs_flag.as<uint8_t>();
  A.blk_u = ctx->blk_u.as<uint32_t>(); A.blk_r = ctx->blk_r.as<uint32_t>();
  A.counts = ctx->counts.as<unsigned long long>();
  A.cov_hist = ctx->hist.as<unsigned long long>();
  A.found = ctx->found.as<unsigned long long>();
  A.err = ctx->errw.as<uint32_t>();
  A.R = R; A.Q = Q; A.hist_cap = cap;
  A.do_errors = p->do_errors; A.preprocess = p->preprocess_stage;
  A.unmatched_min_len = p->unmatched_end_minimum_read_length;
  A.unmatched_factor = (float)p->unmatched_end_length_factor;
  A.unmatched_factor_d = p->unmatched_end_length_factor;
  const uint64_t per_tile = 64ull * std::max<uint32_t>(1, s->max_tile_reads) * 8;
  A.flush_tiles = (uint32_t)std::max<uint64_t>(1, (1ull << 31) / per_tile);
  CK(cudaEventRecord(ctx->ev0, st));
  CK(launch_ec(S, A, ctx->sms, st, ctx->evm0, ctx->evm1));
  std::vector<unsigned long long> counts(nbins), hist((size_t)G * cap), found((size_t)s->n_targets * 2);
  uint32_t err = 0;
  CK(cudaMemcpyAsync(counts.data(), ctx->counts.p, nbins * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hist.data(), ctx->hist.p, (size_t)G * cap * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(found.data(), ctx->found.p, found.size() * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&err, ctx->errw.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0, mms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&mms, ctx->evm0, ctx->evm1);
  ctx->last_ms = ms; ctx->main_ms = mms; ctx->launches = 5;
  if (err) return fail(ctx, BSQ_ERR_DATA, "error_count: " + err_text(err));
  if (out->counts) for (size_t i = 0; i < nbins; i++) out->counts[i] = p->do_errors ? counts[i] : 0;
  int rc = BSQ_OK;
  for (uint32_t g = 0; g < G; g++) {
    uint32_t size = 0;
    for (uint32_t i = 0; i < cap; i++) if (hist[(size_t)g * cap + i]) size = i + 1;
    if (!p->do_coverage) size = 0;
    if (out->hist_size) out->hist_size[g] = size;
    if (out->coverage_hist) {
      for (uint32_t i = 0; i < out->hist_capacity; i++)
        out->coverage_hist[(size_t)g * out->hist_capacity + i] = (i < size) ? hist[(size_t)g * cap + i] : 0;
      if (size > out->hist_capacity) rc = BSQ_ERR_SIZE;
    }
  }
  if (out->no_pos_hash_pr) {
    for (uint32_t t = 0; t < s->n_targets; t++) out->no_pos_hash_pr[t] = 1.0;
    if (p->preprocess_stage)
      for (uint32_t t : s->order) {
        const double tot = (double)(found[2 * t] + found[2 * t + 1]);
        out->no_pos_hash_pr[t] = (tot != 0) ? (double)found[2 * t] / tot : 1.0;
      }
  }
  if (rc == BSQ_ERR_SIZE) return fail(ctx, rc, "coverage histogram larger than hist_capacity; see hist_size");
  return BSQ_OK;
}

int bsq_counts_to_log10_prob(const uint64_t* counts, uint32_t R, uint32_t Q, double* out) {
  if (!counts || !out || R == 0 || Q == 0) return BSQ_ERR_INVALID;
  host::counts_to_log10_prob(counts, R, Q, out);
  return BSQ_OK;
}

// ============================================================================ pass 2
int bsq_identify_mutations(bsq_ctx* ctx, int32_t sid, const bsq_im_params* p, const double* table,
                           bsq_position_arrays* pos_out) {
  if (!ctx || !p || !table) return fail(ctx, BSQ_ERR_INVALID, "null argument");
  SampleDev* s = find_sample(ctx, sid);
  if (!s) return fail(ctx, BSQ_ERR_NOSAMPLE, "unknown sample id");
  if (!p->deletion_propagation_cutoff || !p->deletion_seed_cutoff) return fail(ctx, BSQ_ERR_INVALID, "missing deletion cutoffs");
  if (p->n_read_files == 0 || p->n_read_files > 255 || p->n_quality == 0 || p->n_quality > 256)
    return fail(ctx, BSQ_ERR_INVALID, "error table dimensions out of range");
  CK(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  ctx->res_ra.clear(); ctx->res_mc.clear(); ctx->res_un.clear();
  // ---- likelihood classes, computed on the host exactly as fill_read_base_likelihoods does
  host::ClassTableHost ct;
  host::build_class_table(table, p->n_read_files, p->n_quality, s->mapq_values, ct);
  CK(upload(ctx->lp64, ct.lp64.data(), ct.lp64.size(), st));
  CK(upload(ctx->r64, ct.r64.data(), ct.r64.size(), st));
  CK(upload(ctx->lpmax64, ct.lpmax64.data(), ct.lpmax64.size(), st));
  CK(upload(ctx->lp32, ct.lp32.data(), ct.lp32.size(), st));
  ClassTable T;
  T.lp64 = ctx->lp64.as<double>(); T.r64 = ctx->r64.as<double>(); T.lpmax64 = ctx->lpmax64.as<double>();
  T.lp32 = ctx->lp32.as<float>(); T.K = ct.K; T.R = p->n_read_files; T.Q = p->n_quality;
  T.n_mapq = (uint32_t)s->mapq_values.size();
  std::vector<uint8_t> failed(s->n_targets);
  for (uint32_t t = 0; t < s->n_targets; t++) failed[t] = p->deletion_propagation_cutoff[t] < 0.0;
  CK(cudaMemcpyAsync(s->tgt_failed.p, failed.data(), s->n_targets, cudaMemcpyHostToDevice, st));
  const uint32_t ncol = s->n_cols;
  CK(ctx->cov.alloc((size_t)ncol * sizeof(ColCov), st));
  CK(ctx->call.alloc((size_t)ncol * sizeof(ColCall), st));
  const uint32_t nblk = (ncol + 255) / 256;
  CK(ctx->blk.alloc((size_t)nblk * 4 + 16, st));
  CK(ctx->total.alloc(16, st));
  CK(ctx->cand.alloc((size_t)ncol * 4 + 16, st));
  CK(ctx->next.alloc(16, st));
  CK(ctx->n_ra.alloc(16, st));
  CK(ctx->errw.alloc(16, st));
  CK(cudaMemsetAsync(ctx->errw.p, 0, 16, st));
  DevSample S = make_dev_sample(*s);
  ImArgs A;
  A.cov = ctx->cov.as<ColCov>(); A.call = ctx->call.as<ColCall>(); A.err = ctx->errw.as<uint32_t>();
  A.base_quality_cutoff = p->base_quality_cutoff;
  A.precision = p->precision;
  A.log10_ref_len = p->log10_ref_length;
  A.mutation_cutoff = p->mutation_cutoff;
  A.poly_cutoff = p->polymorphism_cutoff;
  A.screen_margin = 1.0f;
  A.guard = 2e-6f;
  CK(cudaEventRecord(ctx->ev0, st));
  CK(cudaEventRecord(ctx->evm0, st));
  CK(launch_im_column(S, T, A, ctx->sms, st));
  CK(cudaEventRecord(ctx->evm1, st));
  CK(launch_compact(ctx->call.as<ColCall>(), ncol, ctx->blk.as<uint32_t>(), ctx->total.as<uint32_t>(), ctx->cand.as<uint32_t>(), st));
  uint32_t n_cand = 0;
  CK(cudaMemcpyAsync(&n_cand, ctx->total.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  ctx->last_candidates = n_cand;
  // ---- candidate columns: FP64 EM, presence score, bounds
  const int n_warps = ctx->sms * 16;
  const uint32_t per_warp = std::max<uint32_t>(32, s->max_tile_reads);
  CK(ctx->scratch.alloc((size_t)n_warps * cand_warp_stride(per_warp) * sizeof(uint4), st));
  uint32_t ra_cap = n_cand * 2 + 1024;
  const uint32_t Qh = p->n_quality;
  uint32_t n_ra = 0;
  for (int attempt = 0; attempt < 4; attempt++) {
    CK(ctx->ra.alloc((size_t)ra_cap * sizeof(RaDev), st));
    CK(ctx->qhist.alloc((size_t)ra_cap * 2 * Qh * 4, st));
    CK(cudaMemsetAsync(ctx->next.p, 0, 16, st));
    CK(cudaMemsetAsync(ctx->n_ra.p, 0, 16, st));
    CandArgs C;
    C.cand = ctx->cand.as<uint32_t>(); C.n_cand = n_cand; C.next = ctx->next.as<unsigned int>();
    C.call = ctx->call.as<ColCall>(); C.ra = ctx->ra.as<RaDev>(); C.n_ra = ctx->n_ra.as<unsigned int>(); C.ra_cap = ra_cap;
    C.scratch = ctx->scratch.as<uint4>(); C.scratch_per_warp = per_warp; C.err = ctx->errw.as<uint32_t>();
    C.base_quality_cutoff = p->base_quality_cutoff; C.log10_ref_len = p->log10_ref_length;
    C.mutation_cutoff = p->mutation_cutoff; C.poly_cutoff = p->polymorphism_cutoff;
    C.precision_decimal = p->polymorphism_precision_decimal; C.Qhist = Qh; C.qhist = ctx->qhist.as<uint32_t>();
    if (n_cand) CK(launch_candidates(S, T, C, n_warps, st));
    CK(cudaMemcpyAsync(&n_ra, ctx->n_ra.p, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (n_ra <= ra_cap) break;
    uint32_t e = 0;
    CK(cudaMemcpy(&e, ctx->errw.p, 4, cudaMemcpyDeviceToHost));
    e &= ~kErrRaOverflow;
    CK(cudaMemcpy(ctx->errw.p, &e, 4, cudaMemcpyHostToDevice));
    ra_cap = n_ra + 1024;
  }
  std::vector<RaDev> ra(n_ra);
  std::vector<uint32_t> qh((size_t)n_ra * 2 * Qh);
  uint32_t err = 0;
  if (n_ra) {
    CK(cudaMemcpyAsync(ra.data(), ctx->ra.p, (size_t)n_ra * sizeof(RaDev), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(qh.data(), ctx->qhist.p, qh.size() * 4, cudaMemcpyDeviceToHost, st));
  }
  host::SampleLayout L;
  L.tpoff = &s->tpoff; L.toff = &s->toff; L.order = &s->order;
  std::vector<ColCov> cov;
  std::vector<ColCall> call;
  std::vector<uint32_t> kept;
  if (pos_out) {
    // every column comes back: per-position arrays were asked for
    cov.resize(ncol);
    call.resize(ncol);
    CK(cudaMemcpyAsync(cov.data(), ctx->cov.p, (size_t)ncol * sizeof(ColCov), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(call.data(), ctx->call.p, (size_t)ncol * sizeof(ColCall), cudaMemcpyDeviceToHost, st));
  } else {
    // only the columns where the MC / UN state machines can change state
    CK(upload(ctx->d_prop, p->deletion_propagation_cutoff, s->n_targets, st));
    CK(upload(ctx->d_seed, p->deletion_seed_cutoff, s->n_targets, st));
    CK(ctx->keep.alloc(ncol + 16, st));
    CK(ctx->kcol.alloc((size_t)ncol * 4 + 16, st));
    CK(ctx->kcov.alloc((size_t)ncol * sizeof(ColCov) + 16, st));
    CK(ctx->kcall.alloc((size_t)ncol * sizeof(ColCall) + 16, st));
    CK(launch_intervals(ctx->cov.as<ColCov>(), ctx->call.as<ColCall>(), ncol, s->d_tpoff.as<uint32_t>(), s->n_targets,
                        s->tgt_called.as<uint8_t>(), s->tgt_failed.as<uint8_t>(), ctx->d_prop.as<double>(),
                        ctx->d_seed.as<double>(), ctx->keep.as<uint8_t>(), ctx->blk.as<uint32_t>(),
                        ctx->total.as<uint32_t>(), ctx->kcol.as<uint32_t>(), ctx->kcov.as<ColCov>(),
                        ctx->kcall.as<ColCall>(), st));
    uint32_t nk = 0;
    CK(cudaMemcpyAsync(&nk, ctx->total.p, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    kept.resize(nk);
    cov.resize(nk);
    call.resize(nk);
    if (nk) {
      CK(cudaMemcpyAsync(kept.data(), ctx->kcol.p, (size_t)nk * 4, cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(cov.data(), ctx->kcov.p, (size_t)nk * sizeof(ColCov), cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(call.data(), ctx->kcall.p, (size_t)nk * sizeof(ColCall), cudaMemcpyDeviceToHost, st));
    }
  }
  CK(cudaMemcpyAsync(&err, ctx->errw.p, 4, cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->ev1, st));
  CK(cudaStreamSynchronize(st));
  float ms = 0, mms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&mms, ctx->evm0, ctx->evm1);
  ctx->last_ms = ms; ctx->main_ms = mms; ctx->launches = 4 + (n_cand ? 1 : 0) + (pos_out ? 0 : 4);
  if (err) return fail(ctx, BSQ_ERR_DATA, "identify_mutations: " + err_text(err));
  // ---- host assembly
  host::assemble_ra(ra, qh, Qh, L, ctx->res_ra);
  if (pos_out) {
    host::intervals(cov, call, L, p, ctx->res_mc, ctx->res_un);
    host::fill_positions(cov, call, L, pos_out);
  } else {
    host::intervals_sparse(kept, cov, call, L, p, ctx->res_mc, ctx->res_un);
  }
  return BSQ_OK;
}

int bsq_im_result_counts(const bsq_ctx* ctx, uint64_t* n_ra, uint64_t* n_mc, uint64_t* n_un) {
  if (!ctx) return BSQ_ERR_INVALID;
  if (n_ra) *n_ra = ctx->res_ra.size();
  if (n_mc) *n_mc = ctx->res_mc.size();
  if (n_un) *n_un = ctx->res_un.size();
  return BSQ_OK;
}

int bsq_im_result_copy(const bsq_ctx* ctx, bsq_ra_record* ra, uint64_t ra_cap, bsq_mc_record* mc, uint64_t mc_cap,
                       bsq_un_record* un, uint64_t un_cap) {
  if (!ctx) return BSQ_ERR_INVALID;
  if ((ra && ra_cap < ctx->res_ra.size()) || (mc && mc_cap < ctx->res_mc.size()) || (un && un_cap < ctx->res_un.size()))
    return BSQ_ERR_SIZE;
  if (ra) std::copy(ctx->res_ra.begin(), ctx->res_ra.end(), ra);
  if (mc) std::copy(ctx->res_mc.begin(), ctx->res_mc.end(), mc);
  if (un) std::copy(ctx->res_un.begin(), ctx->res_un.end(), un);
  return BSQ_OK;
}

int bsq_last_pass_stats(const bsq_ctx* ctx, double* device_ms, uint32_t* kernel_launches, double* main_kernel_ms) {
  if (!ctx) return BSQ_ERR_INVALID;
  if (device_ms) *device_ms = ctx->last_ms;
  if (kernel_launches) *kernel_launches = ctx->launches;
  if (main_kernel_ms) *main_kernel_ms = ctx->main_ms;
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
  CK(cudaSetDevice(ctx->device));
  void* scratch = nullptr;
  CK(noalloc_scratch_setup(ctx->device, &scratch));
  cudaStream_t st = ctx->stream;
  for (uint32_t t = 0; t < s->n_targets; t++)
    CK(cudaMemsetAsync(s->tgt_failed.as<uint8_t>() + t, p->deletion_propagation_cutoff[t] < 0.0 ? 1 : 0, 1, st));
  NoAllocJob J;
  J.log10_table = table; J.R = R; J.Q = Q;
  J.mapq_values = s->mapq_values.data(); J.n_mapq = (uint32_t)s->mapq_values.size();
  J.tid = d_tid; J.pos0 = d_pos0; J.n_positions = n_positions; J.failed = s->tgt_failed.as<uint8_t>();
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

}  // extern "C"
