// BAM2COV coverage columns: coverage_output::pileup_callback (src/breseq/coverage_output.cpp:307-470)
// over the resident records of one region.  The counts are integer sums; the redundant weights are
// summed per column in record order, the order of htslib's pileup, so every output is exact.
#include "bsq_covtable.h"

#include <algorithm>

#include "bsq_device.cuh"

namespace bsq {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ void add_block(const CovTabArgs& A, int k, uint32_t a, uint32_t b) {
  // aligned columns [a, b) clipped to the region
  const uint32_t lo = max(a, A.c0), hi = min(b, A.c0 + A.n);
  if (lo >= hi) return;
  atomicAdd(A.diff + (uint64_t)k * A.stride + (lo - A.c0), 1);
  atomicAdd(A.diff + (uint64_t)k * A.stride + (hi - A.c0), -1);
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
__global__ void __launch_bounds__(256) ct_reads_kernel(const CovTabArgs A) {
  const uint32_t end_col = A.c0 + A.n;
  const uint32_t r_lo = A.stat[3], r_hi = A.stat[4];
  for (uint32_t r = r_lo + blockIdx.x * blockDim.x + threadIdx.x; r < r_hi; r += gridDim.x * blockDim.x) {
    const DevRead rd = A.reads[r];
    if (rd.flags & kFiltered) continue;                 // htslib's default pileup mask
    if (rd.end <= A.c0) continue;                       // ends before the region: not fetched
    if (rd.flags & kBadCigar) { atomicOr(A.stat + 2, kErrCigar); continue; }
    atomicMax(A.stat, rd.end - A.t0);                   // last column (1-based) of the pileup
    atomicMax(A.stat + 1, rd.end - rd.start);
    const int rev = (rd.flags & kRev) ? 1 : 0;
    const bool unique = __ldg(A.x1 + r) == 1;
    const int k = (unique ? 0 : 2) + rev;
    // column of the first sequenced base (top strand) or the last (bottom strand) when aligned
    uint32_t first_col = 0xFFFFFFFFu;
    if (rd.flags & kSimple) {
      add_block(A, k, rd.start, rd.end);
      if (unique) {
        if (!rev && rd.clip == 0) first_col = rd.start;
        if (rev && (uint32_t)rd.clip + (rd.end - rd.start) == rd.len) first_col = rd.end - 1;
      }
    } else {
      const uint32_t* cg = A.cigar + rd.cigar_off;
      uint32_t x = rd.start;
      bool seen_query = false;
      uint32_t last_q_op = 0xFFu, last_q_end = 0;
      for (uint32_t j = 0; j < rd.n_cigar; j++) {
        const uint32_t op = __ldg(cg + j) & 0xF, len = __ldg(cg + j) >> 4;
        const bool aligned = op == 0 || op == 7 || op == 8;
        if (aligned) {
          add_block(A, k, x, x + len);
          if (!seen_query && !rev && unique && len > 0) first_col = x;
        }
        if (aligned || op == 1 || op == 4) {            // consumes the query
          if (len > 0) { seen_query = true; last_q_op = op; last_q_end = x + len; }
        }
        if (aligned || op == 2 || op == 3) x += len;    // consumes the reference
      }
      if (rev && unique && (last_q_op == 0 || last_q_op == 7 || last_q_op == 8)) first_col = last_q_end - 1;
    }
    if (first_col >= A.c0 && first_col < end_col) atomicAdd(A.counts + (uint64_t)(4 + rev) * A.n + (first_col - A.c0), 1u);
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

// Redundant weights: 1/X1 summed over the covering redundant records in record order, at the
// columns that have any (coverage_output.cpp:418-426).
__global__ void __launch_bounds__(256) ct_redundant_kernel(const CovTabArgs A) {
  const uint32_t maxspan = A.stat[1];
  const uint32_t r_lo = A.stat[3], r_hi = A.stat[4];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    double top = 0.0, bot = 0.0;
    if (A.counts[2ull * A.n + i] + A.counts[3ull * A.n + i] > 0) {
      const uint32_t col = A.c0 + i;
      const uint32_t key = col + 1 > maxspan ? col + 1 - maxspan : 0;   // start > col - maxspan
      for (uint32_t r = first_start_at(A, r_lo, r_hi, key); r < r_hi && __ldg(A.rstart + r) <= col; r++) {
        const DevRead rd = A.reads[r];
        if (rd.flags & (kFiltered | kBadCigar)) continue;
        const uint32_t redundancy = __ldg(A.x1 + r);
        if (redundancy == 1 || rd.end <= col) continue;
        if (!(rd.flags & kSimple)) {
          Pile e;
          if (!resolve_cigar(A.cigar + rd.cigar_off, rd.n_cigar, rd.start, col, e) || e.del) continue;
        }
        if (rd.flags & kRev) bot += 1.0 / redundancy; else top += 1.0 / redundancy;
      }
    }
    A.red[i] = top;
    A.red[(uint64_t)A.n + i] = bot;
  }
}

int grid_for(uint64_t units, uint32_t per_block, int sms, int per_sm) {
  const uint64_t need = (units + per_block - 1) / per_block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sms * per_sm));
}

}  // namespace

cudaError_t ct_launch(const CovTabArgs& A, int sms, cudaStream_t st) {
  ct_range_kernel<<<1, 32, 0, st>>>(A);
  ct_reads_kernel<<<grid_for(A.n_reads, 256, sms, 8), 256, 0, st>>>(A);
  ct_block_sums_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  ct_block_scan_kernel<<<1, 1024, 0, st>>>(A);
  ct_apply_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  ct_redundant_kernel<<<grid_for(A.n, 256, sms, 8), 256, 0, st>>>(A);
  return cudaGetLastError();
}

}  // namespace bsq
