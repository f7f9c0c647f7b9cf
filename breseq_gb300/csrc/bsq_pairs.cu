// Discordant-pair / missing-pair scans: read classification and compaction on the device.
//
// breseq tests each read once, at its start column, inside the identify_mutations pileup
// (src/breseq/identify_mutations.cpp:1395-1493).  The tests depend on the read alone, so here one
// thread per read evaluates them (pair_classify_one) over the whole sample, and a scan-ordered
// scatter compacts the window entries in BAM order with their names.
#include <algorithm>

#include "bsq_pairs.h"

namespace bsq {
namespace {

int grid_of(uint64_t units, int sms) {
  const uint64_t need = (units + 255) / 256;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sms * 8));
}

__global__ void __launch_bounds__(256) pair_classify_kernel(PairArgs a) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    const DevRead r = a.reads[i];
    const uint32_t g = a.rg[i];
    const int32_t gi = g < a.n_rg ? a.rg_map[g] : -1;
    uint8_t code, grp;
    uint32_t sel, mem;
    pair_classify_one(r.flags, a.flag[i], a.xp[i], gi, a.mp != 0, code, grp, sel, mem);
    a.code[i] = code;
    a.group[i] = grp;
    a.sel[i] = sel;
    if (a.mem0) {
      const bool rev = (code & kPairRev) != 0;
      a.mem0[i] = mem && !rev;
      a.mem1[i] = mem && rev;
    }
  }
}

__global__ void __launch_bounds__(256) pair_scatter_kernel(PairArgs a, const uint64_t* ev_off, const uint64_t* off0,
                                                           const uint64_t* off1, PairEvent* ev, char* names,
                                                           uint32_t* start0, uint32_t* start1, uint8_t* group0,
                                                           uint8_t* group1) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    if (a.sel[i]) {
      const DevRead r = a.reads[i];
      const uint64_t e = ev_off[i];
      const uint64_t q0 = a.qoff[i], q1 = a.qoff[i + 1];
      const uint64_t span = q1 - q0;
      const uint32_t len = (uint32_t)(span < (uint64_t)(kPairNameSlot - 2) ? span : (uint64_t)(kPairNameSlot - 2));
      PairEvent x;
      x.rec = i;
      x.start = r.start;
      x.end = r.end;
      x.isize = a.isize[i];
      x.code = a.code[i];
      x.group = a.group[i];
      x.redundant = a.x1[i] > 1 ? 1 : 0;
      x.name_len = (uint8_t)len;
      ev[e] = x;
      char* dst = names + e * kPairNameSlot;
      for (uint32_t k = 0; k < len; k++) dst[k] = a.qname[q0 + k];
    }
    if (a.mem0 && a.mem0[i]) {
      start0[off0[i]] = a.reads[i].start;
      group0[off0[i]] = a.group[i];
    }
    if (a.mem1 && a.mem1[i]) {
      start1[off1[i]] = a.reads[i].start;
      group1[off1[i]] = a.group[i];
    }
  }
}

// ------------------------------------------------------------------ pair distance (PD)
// The reference keeps the covering counts in a ring of difference arrays drained column by column
// (identify_mutations.cpp:2588-2655).  The counts at a position are the integer sums over the pairs
// whose gap covers it, so here every qualifying pair adds its gap to global difference arrays with
// integer atomics (order-free, exact), a prefix scan gives every position's counts, and the
// per-position statistics are evaluated in the same pass.

__device__ __forceinline__ uint32_t target_of(const uint32_t* tpoff, uint32_t n_targets, uint32_t col) {
  uint32_t lo = 0, hi = n_targets;   // last t with tpoff[t] <= col
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (tpoff[mid] <= col) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void add64(long long* p, long long v) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

__global__ void __launch_bounds__(256) pd_interval_kernel(PdArgs a) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    const DevRead r = a.reads[i];
    if (r.flags & kSkip) continue;
    const uint32_t t = target_of(a.tpoff, a.n_targets, r.start);
    if (!a.piled[t]) continue;
    const uint32_t g = a.group[i];
    if (g == 0xFF) continue;
    const uint32_t t0 = a.tpoff[t], len = a.tpoff[t + 1] - t0 - 1;
    PdInterval iv;
    pd_interval_one(r.flags, a.flag[i], (a.code[i] & kPairXpSkip) != 0, (int32_t)g, a.x1[i], (int32_t)t, a.mtid[i],
                    a.isize[i], r.start - t0 + 1, r.end - t0, a.mpos[i], a.cdf + a.cdf_off[g], a.cdf_len[g],
                    a.orient[g], a.max_span, a.lower_tail, iv);
    if (!iv.ok) continue;
    if (iv.bad || iv.lo < 1 || (uint32_t)iv.hi > len) {
      atomicAdd(a.n_above + 1, 1u);
      continue;
    }
    long long* d0 = a.diff + 4ull * (t0 + (uint32_t)iv.lo - 1);   // between-base position b at column t0 + b - 1
    long long* d1 = a.diff + 4ull * (t0 + (uint32_t)iv.hi);
    add64(d0 + 0, 1);
    add64(d1 + 0, -1);
    if (iv.bin >= 0) {
      add64(d0 + 1 + iv.bin, 1);
      add64(d1 + 1 + iv.bin, -1);
    }
    add64(d0 + 3, iv.u);
    add64(d1 + 3, -iv.u);
  }
}

struct Q4 { long long v[4]; };
__device__ __forceinline__ Q4 q4_zero() { Q4 q; q.v[0] = q.v[1] = q.v[2] = q.v[3] = 0; return q; }

// 256 threads x 8 columns: the block's totals
__global__ void __launch_bounds__(256) pd_block_sums_kernel(PdArgs a) {
  __shared__ long long part[8][4];
  const uint64_t c0 = (uint64_t)blockIdx.x * kPdScanCols + threadIdx.x * 8;
  Q4 s = q4_zero();
  for (int k = 0; k < 8; k++) {
    const uint64_t c = c0 + k;
    if (c < a.n_cols) for (int j = 0; j < 4; j++) s.v[j] += a.diff[4 * c + j];
  }
  for (int j = 0; j < 4; j++)
    for (int o = 16; o > 0; o >>= 1) s.v[j] += __shfl_down_sync(0xFFFFFFFFu, s.v[j], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) for (int j = 0; j < 4; j++) part[w][j] = s.v[j];
  __syncthreads();
  if (threadIdx.x < 4) {
    long long t = 0;
    for (int k = 0; k < 8; k++) t += part[k][threadIdx.x];
    a.blk[4ull * blockIdx.x + threadIdx.x] = t;
  }
}

// one block: exclusive scan of the block totals, in place
__global__ void __launch_bounds__(1024) pd_block_scan_kernel(PdArgs a, uint32_t nb) {
  __shared__ long long wsum[32][4];
  __shared__ long long carry[4];
  if (threadIdx.x < 4) carry[threadIdx.x] = 0;
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (uint32_t base = 0; base < nb; base += 1024) {
    const uint32_t b = base + threadIdx.x;
    Q4 v = q4_zero();
    if (b < nb) for (int j = 0; j < 4; j++) v.v[j] = a.blk[4ull * b + j];
    Q4 inc = v;
    for (int o = 1; o < 32; o <<= 1)
      for (int j = 0; j < 4; j++) {
        const long long y = __shfl_up_sync(0xFFFFFFFFu, inc.v[j], o);
        if (lane >= o) inc.v[j] += y;
      }
    if (lane == 31) for (int j = 0; j < 4; j++) wsum[w][j] = inc.v[j];
    __syncthreads();
    if (w == 0) {
      Q4 x = q4_zero();
      for (int j = 0; j < 4; j++) x.v[j] = wsum[lane][j];
      for (int o = 1; o < 32; o <<= 1)
        for (int j = 0; j < 4; j++) {
          const long long y = __shfl_up_sync(0xFFFFFFFFu, x.v[j], o);
          if (lane >= o) x.v[j] += y;
        }
      for (int j = 0; j < 4; j++) wsum[lane][j] = x.v[j];   // inclusive over warps
    }
    __syncthreads();
    if (b < nb)
      for (int j = 0; j < 4; j++)
        a.blk[4ull * b + j] = carry[j] + (w ? wsum[w - 1][j] : 0) + inc.v[j] - v.v[j];
    __syncthreads();
    if (threadIdx.x < 4) carry[threadIdx.x] += wsum[31][threadIdx.x];
    __syncthreads();
  }
}

// Every position's counts (block prefix + in-block scan), its statistics, the z histogram and the
// positions above a seed.
__global__ void __launch_bounds__(256) pd_apply_kernel(PdArgs a) {
  __shared__ unsigned long long hist[kPdHistBins];
  __shared__ long long wsum[8][4];
  for (int k = threadIdx.x; k < kPdHistBins; k += blockDim.x) hist[k] = 0;
  const uint64_t c0 = (uint64_t)blockIdx.x * kPdScanCols + threadIdx.x * 8;
  Q4 tot = q4_zero();
  for (int k = 0; k < 8; k++) {   // the thread's 8 columns; read again below (from L1)
    const uint64_t c = c0 + k;
    if (c < a.n_cols) for (int j = 0; j < 4; j++) tot.v[j] += a.diff[4 * c + j];
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Q4 inc = tot;
  for (int o = 1; o < 32; o <<= 1)
    for (int j = 0; j < 4; j++) {
      const long long y = __shfl_up_sync(0xFFFFFFFFu, inc.v[j], o);
      if (lane >= o) inc.v[j] += y;
    }
  if (lane == 31) for (int j = 0; j < 4; j++) wsum[w][j] = inc.v[j];
  __syncthreads();
  Q4 run;
  for (int j = 0; j < 4; j++) {
    long long x = a.blk[4ull * blockIdx.x + j] + inc.v[j] - tot.v[j];
    for (int k = 0; k < w; k++) x += wsum[k][j];
    run.v[j] = x;
  }
  uint32_t tcache = 0xFFFFFFFFu, t0 = 0, t1 = 0;
  bool piled = false;
  for (int k = 0; k < 8; k++) {
    const uint64_t c = c0 + k;
    if (c >= a.n_cols) break;
    for (int j = 0; j < 4; j++) run.v[j] += a.diff[4 * c + j];
    if (tcache == 0xFFFFFFFFu || c < t0 || c >= t1) {
      tcache = target_of(a.tpoff, a.n_targets, (uint32_t)c);
      t0 = a.tpoff[tcache];
      t1 = a.tpoff[tcache + 1];
      piled = a.piled[tcache] != 0;
    }
    uint64_t m = 0;
    if (piled) {
      const uint32_t p = (uint32_t)c - t0 + 1, len = t1 - t0 - 1;
      double z;
      int hb;
      pd_eval_one(run.v[0], run.v[1], run.v[2], run.v[3], p <= len, a.z_seed, a.seed, z, hb, m);
      if (hb >= 0) atomicAdd(&hist[hb], 1ull);
      if (m & 3) {
        const unsigned slot = atomicAdd(a.n_above, 1u);
        if (slot < a.above_cap) {
          PdAbove x;
          x.col = (uint32_t)c;
          x.bits = (uint32_t)(m & 3);
          x.n = (int32_t)run.v[0];
          x.nlong = (int32_t)run.v[1];
          x.nshort = (int32_t)run.v[2];
          x.pad = 0;
          x.z = z;
          a.above[slot] = x;
        }
      }
    }
    a.mask[c] = m;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kPdHistBins; k += blockDim.x)
    if (hist[k]) atomicAdd(a.hist + k, hist[k]);
}

// Ladder counts: each maximal run of a rung's test is one region (it closes at the flush position at
// the latest, which no test passes), counted here at its first position.
__global__ void __launch_bounds__(256) pd_edges_kernel(PdArgs a) {
  __shared__ unsigned long long cnt[2 * kPdLadderSteps];
  for (int k = threadIdx.x; k < 2 * kPdLadderSteps; k += blockDim.x) cnt[k] = 0;
  __syncthreads();
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < a.n_cols; c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t prev = c ? a.mask[c - 1] : 0;
    uint64_t rise = (a.mask[c] & ~prev) >> kPdBitLadder;
    while (rise) {
      const int b = __ffsll((long long)rise) - 1;
      atomicAdd(&cnt[b], 1ull);
      rise &= rise - 1;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 2 * kPdLadderSteps; k += blockDim.x)
    if (cnt[k]) atomicAdd(a.ladder + k, cnt[k]);
}

}  // namespace

cudaError_t pd_launch(const PdArgs& a, int sms, cudaStream_t st) {
  if (a.n) pd_interval_kernel<<<grid_of(a.n, sms), 256, 0, st>>>(a);
  const uint32_t nb = (a.n_cols + kPdScanCols - 1) / kPdScanCols;
  if (nb) {
    pd_block_sums_kernel<<<nb, 256, 0, st>>>(a);
    pd_block_scan_kernel<<<1, 1024, 0, st>>>(a, nb);
    pd_apply_kernel<<<nb, 256, 0, st>>>(a);
    pd_edges_kernel<<<grid_of(a.n_cols, sms), 256, 0, st>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t pair_classify(const PairArgs& a, int sms, cudaStream_t st) {
  if (a.n) pair_classify_kernel<<<grid_of(a.n, sms), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t pair_scatter(const PairArgs& a, const uint64_t* ev_off, const uint64_t* off0, const uint64_t* off1,
                         PairEvent* ev, char* names, uint32_t* start0, uint32_t* start1, uint8_t* group0,
                         uint8_t* group1, int sms, cudaStream_t st) {
  if (a.n)
    pair_scatter_kernel<<<grid_of(a.n, sms), 256, 0, st>>>(a, ev_off, off0, off1, ev, names, start0, start1, group0,
                                                           group1);
  return cudaGetLastError();
}

}  // namespace bsq
