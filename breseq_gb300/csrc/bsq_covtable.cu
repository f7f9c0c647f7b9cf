// BAM2COV coverage columns: coverage_output::pileup_callback (src/breseq/coverage_output.cpp:307-470)
// over the resident records of one region.  The counts are integer sums; the redundant weights are
// summed per column in record order, the order of htslib's pileup, so every output is exact.
#include "bsq_covtable.h"

#include <algorithm>

#include "bsq_device.cuh"

namespace bsq {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kCtSkipFirst = 1u << 24;   // above flags | n_cigar << 8: the record skips its first column

__device__ __forceinline__ void add_block(const CovTabArgs& A, int k, uint32_t a, uint32_t b) {
  // aligned columns [a, b) clipped to the region
  const uint32_t lo = max(a, A.c0), hi = min(b, A.c0 + A.n);
  if (lo >= hi) return;
  atomicAdd(A.diff + (uint64_t)k * A.stride + (lo - A.c0), 1);
  atomicAdd(A.diff + (uint64_t)k * A.stride + (hi - A.c0), -1);
}

// The identify_mutations tallies leave out each entry whose aligned base is N: -1 at that column.
// Query positions q .. q + len - 1 are aligned to columns x .. x + len - 1.
__device__ __forceinline__ void drop_n_bases(const CovTabArgs& A, int k, const DevRead& rd, uint32_t x, uint32_t len,
                                             uint32_t q) {
  const uint32_t lo = max(x, A.c0), hi = min(x + len, A.c0 + A.n);
  for (uint32_t c = lo; c < hi; c++) {
    const uint32_t qp = q + (c - x);
    if (qp < rd.len && nib_at(A.seq, rd.seq_off + qp) == 15) {
      atomicAdd(A.diff + (uint64_t)k * A.stride + (c - A.c0), -1);
      atomicAdd(A.diff + (uint64_t)k * A.stride + (c + 1 - A.c0), 1);
    }
  }
}

__device__ __forceinline__ uint32_t first_start_at(const CovTabArgs& A, uint32_t lo, uint32_t hi, uint32_t key) {
  while (lo < hi) { const uint32_t m = (lo + hi) >> 1; if (__ldg(A.rstart + m) < key) lo = m + 1; else hi = m; }
  return lo;
}

// The records of the target that start before the region ends: [stat[3], stat[4]).
__global__ void ct_range_kernel(const CovTabArgs A) {
  if (threadIdx.x == 0) {
    A.stat[3] = first_start_at(A, 0, A.n_reads, A.t0);
    A.stat[4] = first_start_at(A, 0, A.n_reads, A.c0 + A.n);
  }
}

// One thread per record of the target that starts before the region ends.  The pileup's entries of
// a record are its aligned bases (M/=/X); deletions and N are entries too but this table skips them.
template <uint32_t kMode>
__global__ void __launch_bounds__(256) ct_reads_kernel(const CovTabArgs A) {
  const uint32_t end_col = A.c0 + A.n;
  // block b walks its own contiguous share of the records: neighbouring threads add to
  // neighbouring columns
  const uint32_t r_lo = A.stat[3], r_hi = A.stat[4];
  const uint32_t per = (uint32_t)(((uint64_t)(r_hi - r_lo) + gridDim.x - 1) / gridDim.x);
  const uint32_t b_lo = (uint32_t)min((uint64_t)r_hi, (uint64_t)r_lo + (uint64_t)blockIdx.x * per);
  const uint32_t b_hi = (uint32_t)min((uint64_t)r_hi, (uint64_t)b_lo + per);
  uint32_t last = 0, span = 0;                          // maxima, reduced per warp at the end
  for (uint32_t r = b_lo + threadIdx.x; r < b_hi; r += blockDim.x) {
    const DevRead rd = A.reads[r];
    if (rd.flags & kFiltered) continue;                 // htslib's default pileup mask
    if (rd.end <= A.c0) continue;                       // ends before the region: not fetched
    if (rd.flags & kBadCigar) { atomicOr(A.stat + 2, kErrCigar); continue; }
    if (A.rg_only >= 0 && (int32_t)__ldg(A.rg + r) != A.rg_only) continue;   // another read group's record
    last = max(last, rd.end - A.t0);                    // last column (1-based) of the pileup
    span = max(span, rd.end - rd.start);
    const int rev = (rd.flags & kRev) ? 1 : 0;
    const bool unique = __ldg(A.x1 + r) == 1;
    const int k = (unique ? 0 : 2) + rev;
    // column of the first sequenced base (top strand) or the last (bottom strand) when aligned
    uint32_t first_col = 0xFFFFFFFFu;
    if (rd.flags & kSimple) {
      add_block(A, k, rd.start, rd.end);
      if (kMode != kCtBam2cov) drop_n_bases(A, k, rd, rd.start, rd.end - rd.start, rd.clip);
      if (unique) {
        if (!rev && rd.clip == 0) first_col = rd.start;
        if (rev && (uint32_t)rd.clip + (rd.end - rd.start) == rd.len) first_col = rd.end - 1;
      }
    } else {
      const uint32_t* cg = A.cigar + rd.cigar_off;
      uint32_t x = rd.start, y = 0;                     // reference column, query position
      bool seen_query = false;
      uint32_t last_q_op = 0xFFu, last_q_end = 0;
      // the identify_mutations pileup tally counts a read on every column it spans, deletions too
      if (kMode == kCtImPileup) add_block(A, k, rd.start, rd.end);
      for (uint32_t j = 0; j < rd.n_cigar; j++) {
        const uint32_t op = __ldg(cg + j) & 0xF, len = __ldg(cg + j) >> 4;
        const bool aligned = op == 0 || op == 7 || op == 8;
        if (aligned) {
          if (kMode != kCtImPileup) add_block(A, k, x, x + len);
          if (kMode != kCtBam2cov) drop_n_bases(A, k, rd, x, len, y);
          if (!seen_query && !rev && unique && len > 0) first_col = x;
        }
        if (aligned || op == 1 || op == 4) {            // consumes the query
          if (len > 0) { seen_query = true; last_q_op = op; last_q_end = x + len; }
          y += len;
        }
        if (aligned || op == 2 || op == 3) x += len;    // consumes the reference
      }
      if (rev && unique && (last_q_op == 0 || last_q_op == 7 || last_q_op == 8)) first_col = last_q_end - 1;
    }
    // the discordant-pair enter step ends the per-read loop at the record's first column before its
    // tally: take back what the record added there (a deletion or a base other than N)
    if (kMode == kCtImPileup && (rd.flags & kDpCand) && rd.start >= A.c0 && rd.start < end_col &&
        dp_group_member(A.dp_rg, __ldg(A.rg + r))) {
      Pile e;
      e.del = false;
      e.qpos = (int)rd.clip;
      bool counted = (rd.flags & kSimple) || resolve_cigar(A.cigar + rd.cigar_off, rd.n_cigar, rd.start, rd.start, e);
      if (counted && !e.del) counted = (uint32_t)e.qpos < rd.len && nib_at(A.seq, rd.seq_off + (uint32_t)e.qpos) != 15;
      if (counted) {
        atomicAdd(A.diff + (uint64_t)k * A.stride + (rd.start - A.c0), -1);
        atomicAdd(A.diff + (uint64_t)k * A.stride + (rd.start + 1 - A.c0), 1);
      }
    }
    if (first_col >= A.c0 && first_col < end_col) atomicAdd(A.counts + (uint64_t)(4 + rev) * A.n + (first_col - A.c0), 1u);
  }
  last = __reduce_max_sync(kFull, last);
  span = __reduce_max_sync(kFull, span);
  if ((threadIdx.x & 31) == 0 && last) {
    atomicMax(A.stat, last);
    atomicMax(A.stat + 1, span);
  }
}

// Exclusive block scan of four 64-bit values over 256 threads; `total` gets the block sums.
__device__ __forceinline__ void block_scan4(long long v[4], long long total[4]) {
  __shared__ long long wsum[8][4];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long inc[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    long long x = v[q];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    inc[q] = x;
    if (lane == 31) wsum[w][q] = x;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; q++) {
    long long before = 0, all = 0;
    for (int i = 0; i < 8; i++) { if (i < w) before += wsum[i][q]; all += wsum[i][q]; }
    v[q] = before + inc[q] - v[q];
    total[q] = all;
  }
  __syncthreads();
}

__device__ __forceinline__ void load8(const CovTabArgs& A, uint64_t c0, int d[4][8], long long v[4]) {
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int4* p = reinterpret_cast<const int4*>(A.diff + (uint64_t)q * A.stride + c0);
    const int4 a = p[0], b = p[1];
    d[q][0] = a.x; d[q][1] = a.y; d[q][2] = a.z; d[q][3] = a.w; d[q][4] = b.x; d[q][5] = b.y; d[q][6] = b.z; d[q][7] = b.w;
    v[q] = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) v[q] += d[q][k];
  }
}

__global__ void __launch_bounds__(256) ct_block_sums_kernel(const CovTabArgs A) {
  int d[4][8];
  long long v[4], tot[4];
  load8(A, (uint64_t)blockIdx.x * kCtBlockCols + threadIdx.x * 8, d, v);
  block_scan4(v, tot);
  if (threadIdx.x == 0)
    for (int q = 0; q < 4; q++) A.blk[(uint64_t)q * A.n_blocks + blockIdx.x] = tot[q];
}

// Exclusive scan of the four block-sum arrays together: one block of 1024 threads, chunks of 1024
// blocks, the 32 warp totals of a chunk scanned by warp 0.
__global__ void __launch_bounds__(1024) ct_block_scan_kernel(const CovTabArgs A) {
  __shared__ long long part[4][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long carry[4] = {0, 0, 0, 0};
  for (uint32_t base = 0; base < A.n_blocks; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    long long v[4], x[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      v[q] = i < A.n_blocks ? A.blk[(uint64_t)q * A.n_blocks + i] : 0;
      x[q] = v[q];
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const long long y = __shfl_up_sync(kFull, x[q], o);
        if (lane >= o) x[q] += y;
      }
    }
    if (lane == 31) {
#pragma unroll
      for (int q = 0; q < 4; q++) part[q][w] = x[q];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const long long t = part[q][lane];
        long long s = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const long long y = __shfl_up_sync(kFull, s, o);
          if (lane >= o) s += y;
        }
        part[q][lane] = s - t;
        if (lane == 31) part[q][32] = s;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (i < A.n_blocks) A.blk[(uint64_t)q * A.n_blocks + i] = carry[q] + part[q][w] + x[q] - v[q];
      carry[q] += part[q][32];
    }
    __syncthreads();
  }
}

// The running sums of the difference arrays are the counts.
__global__ void __launch_bounds__(256) ct_apply_kernel(const CovTabArgs A) {
  const uint64_t c0 = (uint64_t)blockIdx.x * kCtBlockCols + threadIdx.x * 8;
  int d[4][8];
  long long v[4], unused[4];
  load8(A, c0, d, v);
  block_scan4(v, unused);
#pragma unroll
  for (int q = 0; q < 4; q++) {
    long long run = A.blk[(uint64_t)q * A.n_blocks + blockIdx.x] + v[q];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      run += d[q][k];
      if (c0 + k < A.n) A.counts[(uint64_t)q * A.n + c0 + k] = (uint32_t)run;
    }
  }
}

// Redundant weights (coverage_output.cpp:418-426): 1/X1 summed over the covering redundant records
// in record order.  One warp per 32-column tile with any redundant coverage, lane k on column k: the
// warp loads the tile's candidate records 32 at a time (one per lane, which also computes the record's
// weight 1.0 / X1), then walks them in record order by shuffle, each lane adding the weight when the
// record covers its column with an aligned base.  Each lane's sum is the reference's sequential sum.
template <uint32_t kMode>
__global__ void __launch_bounds__(256) ct_redundant_kernel(const CovTabArgs A) {
  const int lane = threadIdx.x & 31;
  const uint32_t maxspan = A.stat[1];
  const uint32_t r_lo = A.stat[3], r_hi = A.stat[4];
  const uint32_t n_tiles = (A.n + 31) / 32;
  // consecutive tiles go to different blocks: tiles with redundant coverage come in runs (repeat
  // copies), and a run on one block would queue on one SM
  const uint32_t warp0 = (threadIdx.x >> 5) * gridDim.x + blockIdx.x, n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t tile = warp0; tile < n_tiles; tile += n_warps) {
    const uint32_t i = tile * 32 + lane;
    const bool in = i < A.n;
    const uint32_t raw = in ? A.counts[2ull * A.n + i] + A.counts[3ull * A.n + i] : 0;
    double top = 0.0, bot = 0.0;
    if (__ballot_sync(kFull, raw > 0)) {
      const uint32_t col0 = A.c0 + tile * 32, col = col0 + lane;
      const uint32_t key = col0 + 1 > maxspan ? col0 + 1 - maxspan : 0;   // start > col0 - maxspan
      const uint32_t lo = first_start_at(A, r_lo, r_hi, key);
      const uint32_t hi = first_start_at(A, lo, r_hi, col0 + 32);          // start < tile end
      for (uint32_t base = lo; base < hi; base += 32) {
        const uint32_t r = base + lane;
        uint32_t start = 0, end = 0, coff = 0, fl_nc = kFiltered;   // flags | n_cigar << 8
        uint32_t clip = 0, len = 0;
        uint64_t soff = 0;
        double w = 0.0;
        if (r < hi) {
          const DevRead rd = A.reads[r];
          const uint32_t redundancy = __ldg(A.x1 + r);
          start = rd.start;
          end = rd.end;
          coff = rd.cigar_off;
          fl_nc = rd.flags | ((uint32_t)rd.n_cigar << 8);
          clip = rd.clip;
          len = rd.len;
          soff = rd.seq_off;
          if (redundancy == 1 || (rd.flags & (kFiltered | kBadCigar)) ||
              (A.rg_only >= 0 && (int32_t)__ldg(A.rg + r) != A.rg_only))
            end = 0;   // never covers
          else w = 1.0 / redundancy;
          // left out of its first column (the discordant-pair enter step's `continue`)
          if (kMode == kCtImPileup && (rd.flags & kDpCand) && dp_group_member(A.dp_rg, __ldg(A.rg + r)))
            fl_nc |= kCtSkipFirst;
        }
        const uint32_t cnt = min(32u, hi - base);
        for (uint32_t j = 0; j < cnt; j++) {
          const uint32_t s_start = __shfl_sync(kFull, start, j), s_end = __shfl_sync(kFull, end, j);
          const uint32_t s_fl = __shfl_sync(kFull, fl_nc, j), s_coff = __shfl_sync(kFull, coff, j);
          const double s_w = __shfl_sync(kFull, w, j);
          bool covers = in && s_start <= col && s_end > col && !((s_fl & kCtSkipFirst) && col == s_start);
          if (kMode == kCtBam2cov) {
            if (covers && !(s_fl & kSimple)) {
              Pile e;
              covers = resolve_cigar(A.cigar + s_coff, (int)(s_fl >> 8), s_start, col, e) && !e.del;
            }
          } else {
            const uint32_t s_clip = __shfl_sync(kFull, clip, j), s_len = __shfl_sync(kFull, len, j);
            const uint64_t s_soff = __shfl_sync(kFull, soff, j);
            if (covers) {
              Pile e;
              e.del = false;
              e.qpos = (int)(col - s_start) + (int)s_clip;
              if (!(s_fl & kSimple)) covers = resolve_cigar(A.cigar + s_coff, (int)(s_fl >> 8), s_start, col, e);
              if (covers && e.del) covers = kMode == kCtImPileup;
              else if (covers)
                covers = (uint32_t)e.qpos < s_len && nib_at(A.seq, s_soff + (uint32_t)e.qpos) != 15;
            }
          }
          if (covers) { if (s_fl & kRev) bot += s_w; else top += s_w; }
        }
      }
    }
    if (in) {
      A.red[i] = top;
      A.red[(uint64_t)A.n + i] = bot;
    }
  }
}

// The handled positions first + k * step of the region, k < m, into the compact arrays.
__global__ void __launch_bounds__(256) ct_gather_kernel(const CovTabArgs A, uint32_t first, uint32_t step, uint32_t m,
                                                        uint32_t* counts_out, double* red_out) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const uint64_t src = (uint64_t)first + (uint64_t)k * step;
#pragma unroll
    for (int q = 0; q < 6; q++) counts_out[(uint64_t)q * m + k] = A.counts[(uint64_t)q * A.n + src];
    red_out[k] = A.red[src];
    red_out[(uint64_t)m + k] = A.red[(uint64_t)A.n + src];
  }
}

int grid_for(uint64_t units, uint32_t per_block, int sms, int per_sm) {
  const uint64_t need = (units + per_block - 1) / per_block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sms * per_sm));
}

}  // namespace

cudaError_t ct_launch(const CovTabArgs& A, int sms, cudaStream_t st) {
  ct_range_kernel<<<1, 32, 0, st>>>(A);
  const int g_reads = grid_for(A.n_reads, 256, sms, 8);
  if (A.mode == kCtImPileup) ct_reads_kernel<kCtImPileup><<<g_reads, 256, 0, st>>>(A);
  else if (A.mode == kCtImTabulate) ct_reads_kernel<kCtImTabulate><<<g_reads, 256, 0, st>>>(A);
  else ct_reads_kernel<kCtBam2cov><<<g_reads, 256, 0, st>>>(A);
  ct_block_sums_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  ct_block_scan_kernel<<<1, 1024, 0, st>>>(A);
  ct_apply_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  const int g_red = grid_for(((uint64_t)A.n + 31) / 32 * 32, 256, sms, 8);
  if (A.mode == kCtImPileup) ct_redundant_kernel<kCtImPileup><<<g_red, 256, 0, st>>>(A);
  else if (A.mode == kCtImTabulate) ct_redundant_kernel<kCtImTabulate><<<g_red, 256, 0, st>>>(A);
  else ct_redundant_kernel<kCtBam2cov><<<g_red, 256, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t ct_launch_gather(const CovTabArgs& A, uint32_t first, uint32_t step, uint32_t m, uint32_t* counts_out,
                             double* red_out, int sms, cudaStream_t st) {
  if (m) ct_gather_kernel<<<grid_for(m, 256, sms, 8), 256, 0, st>>>(A, first, step, m, counts_out, red_out);
  return cudaGetLastError();
}

}  // namespace bsq
