// Soft-clipping tabulation kernels: tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666)
// over the resident records.  All counts are integer sums, so the grid shape changes no result; the
// order of tails inside a row is not fixed, and neither the consensus nor the agreement count
// depends on it.
#include "bsq_softclip.h"

namespace bsq {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned long long kGroupBits = 0x1249249249249249ull;   // bit 0 of each 3-bit column

// base_to_code over BAM 4-bit codes (soft_clipping.cpp:41-50): A, C, G, T = 1, 2, 4, 8 -> 0..3
__device__ __forceinline__ uint32_t sc_code(uint32_t nib) { return __popc(nib) == 1 ? (uint32_t)__ffs(nib) - 1 : 4u; }

__device__ __forceinline__ uint32_t read_nibble(const uint8_t* seq, uint64_t nib) {
  const uint32_t b = __ldg(seq + (nib >> 1));
  return (nib & 1) ? (b & 0xF) : (b >> 4);
}

// sc_position_is_testable (soft_clipping.cpp:162-169); tlen > 0 here
__device__ __forceinline__ bool sc_testable(uint32_t p, uint32_t tlen, uint32_t margin) {
  return p > margin && (uint64_t)p + margin <= tlen;
}

// One pass over the records.  Count: the spanning difference array (soft_clipping.cpp:395-408)
// and one event per clip that qualifies at a testable position (:410-440).  Scatter: the same
// events claim a slot of their row's tail slice and store the packed tail.
template <bool kScatter>
__global__ void __launch_bounds__(256) sc_reads_kernel(const ScArgs A) {
  const uint32_t margin = A.m > 1 ? A.m : 1;
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < A.n_reads; r += gridDim.x * blockDim.x) {
    const DevRead rd = A.reads[r];
    if (rd.flags & (kScSkip | kRedundant)) continue;
    if (rd.flags & kScBad) {
      if (!kScatter) atomicOr(A.err, kErrCigar);
      continue;
    }
    // the record lies inside one target: start .. end - 1 are its columns
    uint32_t lo = 0, hi = A.n_targets;
    while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (__ldg(A.tpoff + mid) <= rd.start) lo = mid; else hi = mid; }
    const uint32_t t0 = __ldg(A.tpoff + lo), tlen = __ldg(A.tpoff + lo + 1) - t0 - 1;
    const uint32_t start1 = rd.start - t0 + 1, end1 = rd.end - t0;   // reference_start_1 / reference_end_1
    uint32_t qs0, qe1;                                               // query_start_1 - 1, query_end_1
    if (rd.flags & kSimple) {
      qs0 = rd.clip;
      qe1 = rd.clip + (rd.end - rd.start);
    } else {
      const QBounds b = A.qb[r];
      qs0 = b.qs0;
      qe1 = (uint32_t)(b.qe0 + 1u) & 0xFFFFu;   // query_end_1 = 0 is stored as qe0 = 0xFFFF
    }
    const uint32_t lead = qs0, trail = (uint32_t)rd.len - qe1;
    if (!kScatter && (uint64_t)end1 >= (uint64_t)start1 + 2ull * A.m) {
      atomicAdd(A.diff + rd.start + A.m, 1);      // position start1 + m
      atomicAdd(A.diff + rd.end - A.m, -1);       // position end1 - m + 1
    }
    if (lead >= A.m && sc_testable(start1, tlen, margin)) {
      uint32_t* c = A.cnt + rd.start;
      if (!kScatter) {
        atomicAdd(c, 1u);
      } else {
        // column 0 is the clipped base next to the wall, then outward (backwards on the read)
        unsigned long long packed = 0;
        for (uint32_t k = 0; k < A.K; k++)
          packed |= (unsigned long long)sc_code(read_nibble(A.seq, rd.seq_off + qs0 - 1 - k)) << (3 * k);
        A.tails[atomicAdd(c, 1u)] = packed;
      }
    }
    if (trail >= A.m && sc_testable(end1, tlen, margin)) {
      uint32_t* c = A.cnt + A.cstride + (rd.end - 1);
      if (!kScatter) {
        atomicAdd(c, 1u);
      } else {
        unsigned long long packed = 0;
        for (uint32_t k = 0; k < A.K; k++)
          packed |= (unsigned long long)sc_code(read_nibble(A.seq, rd.seq_off + qe1 + k)) << (3 * k);
        A.tails[atomicAdd(c, 1u)] = packed;
      }
    }
  }
}

// Exclusive block scan of five 64-bit values over 256 threads; `total` gets the block sums.
__device__ __forceinline__ void block_scan5(long long v[5], long long total[5]) {
  __shared__ long long wsum[8][5];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long inc[5];
#pragma unroll
  for (int q = 0; q < 5; q++) {
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
  for (int q = 0; q < 5; q++) {
    long long before = 0, all = 0;
    for (int i = 0; i < 8; i++) { if (i < w) before += wsum[i][q]; all += wsum[i][q]; }
    v[q] = before + inc[q] - v[q];
    total[q] = all;
  }
  __syncthreads();
}

__device__ __forceinline__ void load4(const ScArgs& A, uint64_t c0, int d[4], uint32_t x[4], uint32_t y[4]) {
  const int4 dv = *reinterpret_cast<const int4*>(A.diff + c0);
  const uint4 xv = *reinterpret_cast<const uint4*>(A.cnt + c0);
  const uint4 yv = *reinterpret_cast<const uint4*>(A.cnt + A.cstride + c0);
  d[0] = dv.x; d[1] = dv.y; d[2] = dv.z; d[3] = dv.w;
  x[0] = xv.x; x[1] = xv.y; x[2] = xv.z; x[3] = xv.w;
  y[0] = yv.x; y[1] = yv.y; y[2] = yv.z; y[3] = yv.w;
}

// Per 1024-column block: sums of the difference array, rows and tails of each direction.
__global__ void __launch_bounds__(256) sc_block_sums_kernel(const ScArgs A) {
  const uint64_t c0 = (uint64_t)blockIdx.x * kScBlockCols + threadIdx.x * 4;
  int d[4];
  uint32_t x[4], y[4];
  load4(A, c0, d, x, y);
  long long v[5] = {0, 0, 0, 0, 0}, tot[5];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[0] += d[k];
    v[1] += x[k] != 0; v[2] += x[k];
    v[3] += y[k] != 0; v[4] += y[k];
  }
  block_scan5(v, tot);
  if (threadIdx.x == 0)
    for (int q = 0; q < 5; q++) A.blk[(uint64_t)q * A.n_blocks + blockIdx.x] = tot[q];
}

// Exclusive scan of the block sums (one block of 1024 threads walking the blocks in chunks).
__global__ void __launch_bounds__(1024) sc_block_scan_kernel(const ScArgs A) {
  __shared__ long long part[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int q = 0; q < 5; q++) {
    long long* a = A.blk + (uint64_t)q * A.n_blocks;
    long long carry = 0;
    for (uint32_t base = 0; base < A.n_blocks; base += 1024) {
      const uint32_t i = base + threadIdx.x;
      const long long v = i < A.n_blocks ? a[i] : 0;
      long long x = v;
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) part[w] = x;
      __syncthreads();
      long long before = carry, all = carry;
      for (int j = 0; j < 32; j++) { if (j < w) before += part[j]; all += part[j]; }
      if (i < A.n_blocks) a[i] = before + x - v;
      __syncthreads();
      carry = all;
    }
    if (threadIdx.x == 0 && q > 0) A.tot[q - 1] = (unsigned long long)carry;
  }
}

// Spanning coverage (soft_clipping.cpp:468-490), rows in (direction, column) order with their tail
// slices, and the event counters turned into tail cursors.
__global__ void __launch_bounds__(256) sc_apply_kernel(const ScArgs A) {
  const uint64_t c0 = (uint64_t)blockIdx.x * kScBlockCols + threadIdx.x * 4;
  int d[4];
  uint32_t x[4], y[4];
  load4(A, c0, d, x, y);
  long long v[5] = {0, 0, 0, 0, 0}, unused[5];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    v[0] += d[k];
    v[1] += x[k] != 0; v[2] += x[k];
    v[3] += y[k] != 0; v[4] += y[k];
  }
  block_scan5(v, unused);
  const uint64_t nb = A.n_blocks;
  long long running = A.blk[blockIdx.x] + v[0];
  uint64_t row_n = (uint64_t)(A.blk[nb + blockIdx.x] + v[1]);
  uint64_t tail_n = (uint64_t)(A.blk[2 * nb + blockIdx.x] + v[2]);
  uint64_t row_p = A.tot[0] + (uint64_t)(A.blk[3 * nb + blockIdx.x] + v[3]);
  uint64_t tail_p = A.tot[1] + (uint64_t)(A.blk[4 * nb + blockIdx.x] + v[4]);
  unsigned long long span = 0, tested = 0;
  if (c0 < A.n_cols) {
    const uint32_t margin = A.m > 1 ? A.m : 1;
    uint32_t lo = 0, hi = A.n_targets;
    while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (__ldg(A.tpoff + mid) <= c0) lo = mid; else hi = mid; }
    uint32_t t = lo;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const uint32_t c = (uint32_t)c0 + k;
      if (c >= A.n_cols) break;
      while (c >= __ldg(A.tpoff + t + 1)) t++;
      running += d[k];
      const uint32_t sp = running > 0 ? (uint32_t)running : 0u;
      const uint32_t tb = __ldg(A.tpoff + t), tlen = __ldg(A.tpoff + t + 1) - tb - 1;
      if (tlen > 0 && sc_testable(c - tb + 1, tlen, margin)) {
        span += 2ull * sp;
        if (sp > 0) tested += 2;
      }
      if (x[k]) {
        A.rows[row_n] = ScRowDev{c, x[k], sp, (uint32_t)tail_n};
        A.cnt[c] = (uint32_t)tail_n;
        row_n++;
        tail_n += x[k];
      }
      if (y[k]) {
        A.rows[row_p] = ScRowDev{c, y[k], sp, (uint32_t)tail_p};
        A.cnt[A.cstride + c] = (uint32_t)tail_p;
        row_p++;
        tail_p += y[k];
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    span += __shfl_xor_sync(kFull, span, o);
    tested += __shfl_xor_sync(kFull, tested, o);
  }
  if ((threadIdx.x & 31) == 0 && (span | tested)) {
    atomicAdd(A.tot + 4, span);
    atomicAdd(A.tot + 5, tested);
  }
}

// compute_clipped_tail_consensus (soft_clipping.cpp:98-147), one warp per row.  Lane k < K keeps the
// four base counts of column k; each round of 32 tails adds one warp-reduced byte-packed tally per
// column.  Agreement: a tail matches a column where its 3-bit code equals the consensus code, so the
// mismatching informative columns are the non-zero groups of (tail ^ consensus) & informative mask.
__global__ void __launch_bounds__(256) sc_consensus_kernel(const ScArgs A, uint32_t n_rows) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = warp0; i < n_rows; i += n_warps) {
    const ScRowDev row = A.rows[i];
    const unsigned long long* T = A.tails + row.tail_off;
    const uint32_t N = row.clipped;
    ScOutDev out{0ull, N, 0u};
    if (A.base_fraction > 0.0) {
      uint32_t c[4] = {0, 0, 0, 0};
      for (uint32_t base = 0; base < N; base += 32) {
        const uint32_t j = base + lane;
        const unsigned long long t = j < N ? T[j] : ~0ull;   // all-ones codes are 7: counted nowhere
        for (uint32_t k = 0; k < A.K; k++) {
          const uint32_t code = (uint32_t)(t >> (3 * k)) & 7u;
          const uint32_t s = __reduce_add_sync(kFull, code < 4 ? 1u << (8 * code) : 0u);
          if ((uint32_t)lane == k) { c[0] += s & 0xFF; c[1] += (s >> 8) & 0xFF; c[2] += (s >> 16) & 0xFF; c[3] += s >> 24; }
        }
      }
      // plurality with strict > keeps the A < C < G < T tie-break
      uint32_t best = 4, best_n = 0;
#pragma unroll
      for (uint32_t b = 0; b < 4; b++) if (c[b] > best_n) { best_n = c[b]; best = b; }
      const bool col = (uint32_t)lane < A.K;
      const unsigned long long mine = col ? (unsigned long long)best << (3 * lane) : 0ull;
      const unsigned long long imask = (col && best < 4) ? 7ull << (3 * lane) : 0ull;
      const unsigned long long cons = (unsigned long long)__reduce_or_sync(kFull, (uint32_t)mine) |
                                      ((unsigned long long)__reduce_or_sync(kFull, (uint32_t)(mine >> 32)) << 32);
      const unsigned long long inf_mask = (unsigned long long)__reduce_or_sync(kFull, (uint32_t)imask) |
                                          ((unsigned long long)__reduce_or_sync(kFull, (uint32_t)(imask >> 32)) << 32);
      const uint32_t informative = __popc(__ballot_sync(kFull, col && best < 4));
      uint32_t agree = 0;
      if (informative > 0) {
        uint32_t required = (uint32_t)floor(A.base_fraction * (double)informative);
        if (required < 1) required = 1;
        for (uint32_t j = lane; j < N; j += 32) {
          const unsigned long long x = (T[j] ^ cons) & inf_mask;
          const uint32_t mismatches = __popcll((x | (x >> 1) | (x >> 2)) & kGroupBits);
          agree += (informative - mismatches) >= required;
        }
        agree = __reduce_add_sync(kFull, agree);
      }
      out.cons = cons;
      out.agree = agree;
      out.informative = informative;
    }
    if (lane == 0) A.outs[i] = out;
  }
}

int grid_for(uint64_t units, uint32_t per_block, int sms, int per_sm) {
  const uint64_t need = (units + per_block - 1) / per_block;
  const uint64_t cap = (uint64_t)sms * per_sm;
  return (int)std::max<uint64_t>(1, std::min(need, cap));
}

}  // namespace

cudaError_t sc_launch_count(const ScArgs& A, int sms, cudaStream_t st) {
  if (A.n_reads) sc_reads_kernel<false><<<grid_for(A.n_reads, 256, sms, 8), 256, 0, st>>>(A);
  sc_block_sums_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  sc_block_scan_kernel<<<1, 1024, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t sc_launch_rows(const ScArgs& A, uint32_t n_rows, int sms, cudaStream_t st) {
  sc_apply_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  if (n_rows) {
    if (A.n_reads) sc_reads_kernel<true><<<grid_for(A.n_reads, 256, sms, 8), 256, 0, st>>>(A);
    sc_consensus_kernel<<<grid_for((uint64_t)n_rows * 32, 256, sms, 8), 256, 0, st>>>(A, n_rows);
  }
  return cudaGetLastError();
}

}  // namespace bsq
