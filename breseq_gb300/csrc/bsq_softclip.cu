// Soft-clipping tabulation kernels: tabulate_soft_clipping_counts (src/breseq/soft_clipping.cpp:285-666)
// over the resident records.  All counts are integer sums, so the grid shape changes no result; the
// order of tails inside a row is not fixed, and neither the consensus nor the agreement count
// depends on it.
#include "bsq_softclip.h"

#include <algorithm>

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

// Per record: whether the tabulation keeps it, its query bounds, and its events.  Bits of the result:
// 1 leading-clip event at reference_start_1, 2 trailing-clip event at reference_end_1, 4 a spanning
// read (min bases aligned on both sides somewhere), 8 a kept record whose CIGAR does not fit.
struct ScRead {
  uint32_t t0, start1, end1, qs0, qe1;
};
__device__ __forceinline__ uint32_t sc_classify(const ScArgs& A, const DevRead& rd, uint32_t r, uint32_t margin,
                                                ScRead& e) {
  if (rd.flags & (kScSkip | kRedundant)) return 0;   // unmapped, X1 > 1, XJ, empty target (:373-393)
  if (rd.flags & kBadCigar) return 8;
  // the record lies inside one target: start .. end - 1 are its columns
  uint32_t lo = 0, hi = A.n_targets;
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (__ldg(A.tpoff + mid) <= rd.start) lo = mid; else hi = mid; }
  e.t0 = __ldg(A.tpoff + lo);
  const uint32_t tlen = __ldg(A.tpoff + lo + 1) - e.t0 - 1;
  e.start1 = rd.start - e.t0 + 1;                    // reference_start_1
  e.end1 = rd.end - e.t0;                            // reference_end_1
  if (rd.flags & kSimple) {                          // query_start_1 - 1, query_end_1
    e.qs0 = rd.clip;
    e.qe1 = rd.clip + (rd.end - rd.start);
  } else {
    const QBounds b = A.qb[r];
    e.qs0 = b.qs0;
    e.qe1 = (uint32_t)(b.qe0 + 1u) & 0xFFFFu;        // query_end_1 = 0 is stored as qe0 = 0xFFFF
  }
  uint32_t bits = 0;
  if ((uint64_t)e.end1 >= (uint64_t)e.start1 + 2ull * A.m) bits |= 4;
  if (e.qs0 >= A.m && sc_testable(e.start1, tlen, margin)) bits |= 1;
  if ((uint32_t)rd.len - e.qe1 >= A.m && sc_testable(e.end1, tlen, margin)) bits |= 2;
  return bits;
}

// Count pass (soft_clipping.cpp:366-453): the spanning difference array (:395-408), one event per clip
// that qualifies at a testable position (:410-440), and the list of reads with events.  Block b walks
// its own contiguous range of reads, kScUnroll records per thread in flight.
constexpr int kScUnroll = 2;
__global__ void __launch_bounds__(256) sc_count_kernel(const ScArgs A) {
  __shared__ unsigned s_n;
  const uint32_t margin = A.m > 1 ? A.m : 1;
  const uint32_t r0 = blockIdx.x * A.ev_per_block;
  const uint32_t r1 = (uint32_t)min((uint64_t)A.n_reads, (uint64_t)r0 + A.ev_per_block);
  if (threadIdx.x == 0) s_n = 0;
  __syncthreads();
  for (uint32_t base = r0 + threadIdx.x; base < r1; base += kScUnroll * blockDim.x) {
    DevRead rd[kScUnroll];
#pragma unroll
    for (int u = 0; u < kScUnroll; u++) {
      const uint32_t r = base + u * blockDim.x;
      if (r < r1) rd[u] = A.reads[r];
    }
#pragma unroll
    for (int u = 0; u < kScUnroll; u++) {
      const uint32_t r = base + u * blockDim.x;
      if (r >= r1) break;
      ScRead e;
      const uint32_t bits = sc_classify(A, rd[u], r, margin, e);
      if (bits & 8) atomicOr(A.err, kErrCigar);
      if (bits & 4) {
        atomicAdd(A.diff + rd[u].start + A.m, 1);      // position start1 + m
        atomicAdd(A.diff + rd[u].end - A.m, -1);       // position end1 - m + 1
      }
      if (bits & 1) atomicAdd(A.cnt + rd[u].start, 1u);
      if (bits & 2) atomicAdd(A.cnt + A.cstride + (rd[u].end - 1), 1u);
      if (bits & 3) A.ev[r0 + atomicAdd(&s_n, 1u)] = r;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) A.ev_n[blockIdx.x] = s_n;
}

// The listed reads claim a slot of their row's tail slice and store the packed tail.
__global__ void __launch_bounds__(256) sc_scatter_kernel(const ScArgs A) {
  const uint32_t margin = A.m > 1 ? A.m : 1;
  const uint32_t n = A.ev_n[blockIdx.x];
  const uint32_t* list = A.ev + (uint64_t)blockIdx.x * A.ev_per_block;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint32_t r = list[i];
    const DevRead rd = A.reads[r];
    ScRead e;
    const uint32_t bits = sc_classify(A, rd, r, margin, e);
    if (bits & 1) {
      // column 0 is the clipped base next to the wall, then outward (backwards on the read)
      unsigned long long packed = 0;
      for (uint32_t k = 0; k < A.K; k++)
        packed |= (unsigned long long)sc_code(read_nibble(A.seq, rd.seq_off + e.qs0 - 1 - k)) << (3 * k);
      A.tails[atomicAdd(A.cnt + rd.start, 1u)] = packed;
    }
    if (bits & 2) {
      unsigned long long packed = 0;
      for (uint32_t k = 0; k < A.K; k++)
        packed |= (unsigned long long)sc_code(read_nibble(A.seq, rd.seq_off + e.qe1 + k)) << (3 * k);
      A.tails[atomicAdd(A.cnt + A.cstride + (rd.end - 1), 1u)] = packed;
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

// The 8 columns of a thread: difference array, leading and trailing event counts.
struct Cols8 { int d[8]; uint32_t x[8], y[8]; };
__device__ __forceinline__ void load8(const ScArgs& A, uint64_t c0, Cols8& c, long long v[5]) {
  const int4* dp = reinterpret_cast<const int4*>(A.diff + c0);
  const uint4* xp = reinterpret_cast<const uint4*>(A.cnt + c0);
  const uint4* yp = reinterpret_cast<const uint4*>(A.cnt + A.cstride + c0);
  const int4 d0 = dp[0], d1 = dp[1];
  const uint4 x0 = xp[0], x1 = xp[1], y0 = yp[0], y1 = yp[1];
  c.d[0] = d0.x; c.d[1] = d0.y; c.d[2] = d0.z; c.d[3] = d0.w; c.d[4] = d1.x; c.d[5] = d1.y; c.d[6] = d1.z; c.d[7] = d1.w;
  c.x[0] = x0.x; c.x[1] = x0.y; c.x[2] = x0.z; c.x[3] = x0.w; c.x[4] = x1.x; c.x[5] = x1.y; c.x[6] = x1.z; c.x[7] = x1.w;
  c.y[0] = y0.x; c.y[1] = y0.y; c.y[2] = y0.z; c.y[3] = y0.w; c.y[4] = y1.x; c.y[5] = y1.y; c.y[6] = y1.z; c.y[7] = y1.w;
#pragma unroll
  for (int q = 0; q < 5; q++) v[q] = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    v[0] += c.d[k];
    v[1] += c.x[k] != 0; v[2] += c.x[k];
    v[3] += c.y[k] != 0; v[4] += c.y[k];
  }
}

// Per block of columns: sums of the difference array, rows and tails of each direction.
__global__ void __launch_bounds__(256) sc_block_sums_kernel(const ScArgs A) {
  const uint64_t c0 = (uint64_t)blockIdx.x * kScBlockCols + threadIdx.x * 8;
  Cols8 c;
  long long v[5], tot[5];
  load8(A, c0, c, v);
  block_scan5(v, tot);
  if (threadIdx.x == 0)
    for (int q = 0; q < 5; q++) A.blk[(uint64_t)q * A.n_blocks + blockIdx.x] = tot[q];
}

// Exclusive scan of the five block-sum arrays together (one block of 1024 threads, chunks of 1024
// blocks; the 32 warp totals of a chunk are scanned by warp 0); tot[0..3] get the row and tail
// totals of each direction.
__global__ void __launch_bounds__(1024) sc_block_scan_kernel(const ScArgs A) {
  __shared__ long long part[5][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long carry[5] = {0, 0, 0, 0, 0};
  for (uint32_t base = 0; base < A.n_blocks; base += 1024) {
    const uint32_t i = base + threadIdx.x;
    long long v[5], x[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      v[q] = i < A.n_blocks ? A.blk[(uint64_t)q * A.n_blocks + i] : 0;
      x[q] = v[q];
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
      for (int q = 0; q < 5; q++) {
        const long long y = __shfl_up_sync(kFull, x[q], o);
        if (lane >= o) x[q] += y;
      }
    }
    if (lane == 31) {
#pragma unroll
      for (int q = 0; q < 5; q++) part[q][w] = x[q];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
      for (int q = 0; q < 5; q++) {
        const long long t = part[q][lane];
        long long s = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const long long y = __shfl_up_sync(kFull, s, o);
          if (lane >= o) s += y;
        }
        part[q][lane] = s - t;               // warps before this one
        if (lane == 31) part[q][32] = s;     // the chunk's total
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 5; q++) {
      if (i < A.n_blocks) A.blk[(uint64_t)q * A.n_blocks + i] = carry[q] + part[q][w] + x[q] - v[q];
      carry[q] += part[q][32];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 1; q < 5; q++) A.tot[q - 1] = (unsigned long long)carry[q];
}

// Spanning coverage (soft_clipping.cpp:468-490), rows in (direction, column) order with their tail
// slices, and the event counters turned into tail cursors.
__global__ void __launch_bounds__(256) sc_apply_kernel(const ScArgs A) {
  const uint64_t c0 = (uint64_t)blockIdx.x * kScBlockCols + threadIdx.x * 8;
  Cols8 c;
  long long v[5], unused[5];
  load8(A, c0, c, v);
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
    uint32_t tb = __ldg(A.tpoff + t), te = __ldg(A.tpoff + t + 1);
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const uint32_t col = (uint32_t)c0 + k;
      if (col >= A.n_cols) break;
      while (col >= te) { t++; tb = te; te = __ldg(A.tpoff + t + 1); }
      running += c.d[k];
      const uint32_t sp = running > 0 ? (uint32_t)running : 0u;
      const uint32_t tlen = te - tb - 1;
      if (tlen > 0 && sc_testable(col - tb + 1, tlen, margin)) {
        span += 2ull * sp;
        if (sp > 0) tested += 2;
      }
      if (c.x[k]) {
        A.rows[row_n] = ScRowDev{col, c.x[k], sp, (uint32_t)tail_n};
        A.cnt[col] = (uint32_t)tail_n;
        row_n++;
        tail_n += c.x[k];
      }
      if (c.y[k]) {
        A.rows[row_p] = ScRowDev{col, c.y[k], sp, (uint32_t)tail_p};
        A.cnt[A.cstride + col] = (uint32_t)tail_p;
        row_p++;
        tail_p += c.y[k];
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

__device__ __forceinline__ uint32_t sc_required(double base_fraction, uint32_t informative) {
  const uint32_t r = (uint32_t)floor(base_fraction * (double)informative);   // rounded down (:130-134)
  return r < 1 ? 1u : r;
}

// compute_clipped_tail_consensus (soft_clipping.cpp:98-147) for a row of at most kScSmallRow tails,
// on one lane.  Agreement: a tail matches a column where its 3-bit code equals the consensus code,
// so the mismatching informative columns are the non-zero groups of (tail ^ consensus) & mask.
__device__ __forceinline__ ScOutDev sc_consensus_small(const ScArgs& A, const ScRowDev& row) {
  const uint32_t N = row.clipped;
  ScOutDev out{0ull, N, 0u};
  if (!(A.base_fraction > 0.0)) return out;
  unsigned long long t[kScSmallRow];
#pragma unroll
  for (uint32_t j = 0; j < kScSmallRow; j++) t[j] = j < N ? A.tails[row.tail_off + j] : ~0ull;   // 7: no base
  unsigned long long cons = 0, mask = 0;
  uint32_t informative = 0;
  for (uint32_t k = 0; k < A.K; k++) {
    uint32_t c[4] = {0, 0, 0, 0};
#pragma unroll
    for (uint32_t j = 0; j < kScSmallRow; j++) {
      const uint32_t code = (uint32_t)(t[j] >> (3 * k)) & 7u;
#pragma unroll
      for (uint32_t b = 0; b < 4; b++) c[b] += code == b;
    }
    uint32_t best = 4, best_n = 0;   // plurality; strict > keeps the A < C < G < T tie-break
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) if (c[b] > best_n) { best_n = c[b]; best = b; }
    cons |= (unsigned long long)best << (3 * k);
    if (best < 4) { mask |= 7ull << (3 * k); informative++; }
  }
  uint32_t agree = 0;
  if (informative > 0) {
    const uint32_t required = sc_required(A.base_fraction, informative);
#pragma unroll
    for (uint32_t j = 0; j < kScSmallRow; j++) {
      const unsigned long long x = (t[j] ^ cons) & mask;
      agree += j < N && (informative - __popcll((x | (x >> 1) | (x >> 2)) & kGroupBits)) >= required;
    }
  }
  return ScOutDev{cons, agree, informative};
}

// The same for a row of any size on a whole warp.  Lane k < K keeps the four base counts of column k;
// each round of 32 tails adds one warp-reduced byte-packed tally per column.
__device__ __forceinline__ void sc_consensus_warp(const ScArgs& A, uint32_t i, int lane) {
  const ScRowDev row = A.rows[i];
  const unsigned long long* T = A.tails + row.tail_off;
  const uint32_t N = row.clipped;
  ScOutDev out{0ull, N, 0u};
  if (A.base_fraction > 0.0) {
    uint32_t c[4] = {0, 0, 0, 0};
    for (uint32_t base = 0; base < N; base += 32) {
      const uint32_t j = base + lane;
      const unsigned long long t = j < N ? T[j] : ~0ull;
      for (uint32_t k = 0; k < A.K; k++) {
        const uint32_t code = (uint32_t)(t >> (3 * k)) & 7u;
        const uint32_t s = __reduce_add_sync(kFull, code < 4 ? 1u << (8 * code) : 0u);
        if ((uint32_t)lane == k) { c[0] += s & 0xFF; c[1] += (s >> 8) & 0xFF; c[2] += (s >> 16) & 0xFF; c[3] += s >> 24; }
      }
    }
    uint32_t best = 4, best_n = 0;
#pragma unroll
    for (uint32_t b = 0; b < 4; b++) if (c[b] > best_n) { best_n = c[b]; best = b; }
    const bool col = (uint32_t)lane < A.K;
    const unsigned long long mine = col ? (unsigned long long)best << (3 * lane) : 0ull;
    const unsigned long long imask = (col && best < 4) ? 7ull << (3 * lane) : 0ull;
    const unsigned long long cons = (unsigned long long)__reduce_or_sync(kFull, (uint32_t)mine) |
                                    ((unsigned long long)__reduce_or_sync(kFull, (uint32_t)(mine >> 32)) << 32);
    const unsigned long long mask = (unsigned long long)__reduce_or_sync(kFull, (uint32_t)imask) |
                                    ((unsigned long long)__reduce_or_sync(kFull, (uint32_t)(imask >> 32)) << 32);
    const uint32_t informative = __popc(__ballot_sync(kFull, col && best < 4));
    uint32_t agree = 0;
    if (informative > 0) {
      const uint32_t required = sc_required(A.base_fraction, informative);
      for (uint32_t j = lane; j < N; j += 32) {
        const unsigned long long x = (T[j] ^ cons) & mask;
        agree += (informative - __popcll((x | (x >> 1) | (x >> 2)) & kGroupBits)) >= required;
      }
      agree = __reduce_add_sync(kFull, agree);
    }
    out = ScOutDev{cons, agree, informative};
  }
  if (lane == 0) A.outs[i] = out;
}

// Rows in chunks of 32 per warp: small rows one lane each, then the chunk's larger rows one at a time
// on the whole warp.
__global__ void __launch_bounds__(256) sc_consensus_kernel(const ScArgs A, uint32_t n_rows) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint64_t c0 = (uint64_t)warp0 * 32; c0 < n_rows; c0 += (uint64_t)n_warps * 32) {
    const uint32_t i = (uint32_t)c0 + lane;
    bool big = false;
    if (i < n_rows) {
      const ScRowDev row = A.rows[i];
      big = row.clipped > kScSmallRow;
      if (!big) A.outs[i] = sc_consensus_small(A, row);
    }
    unsigned todo = __ballot_sync(kFull, big);
    while (todo) {
      const int b = __ffs(todo) - 1;
      todo &= todo - 1;
      sc_consensus_warp(A, (uint32_t)c0 + b, lane);
    }
  }
}

int grid_for(uint64_t units, uint32_t per_block, int sms, int per_sm) {
  const uint64_t need = (units + per_block - 1) / per_block;
  const uint64_t cap = (uint64_t)sms * per_sm;
  return (int)std::max<uint64_t>(1, std::min(need, cap));
}

}  // namespace

void sc_plan(ScArgs& A, int sms) {
  A.n_blocks = (A.n_cols + kScBlockCols - 1) / kScBlockCols;
  A.cstride = (uint64_t)A.n_blocks * kScBlockCols;
  A.ev_blocks = (uint32_t)grid_for(A.n_reads, 256 * kScUnroll, sms, 8);
  A.ev_per_block = (uint32_t)(((uint64_t)A.n_reads + A.ev_blocks - 1) / A.ev_blocks);
}

cudaError_t sc_launch_count(const ScArgs& A, int sms, cudaStream_t st, cudaEvent_t main0, cudaEvent_t main1) {
  (void)sms;
  if (main0) cudaEventRecord(main0, st);
  sc_count_kernel<<<A.ev_blocks, 256, 0, st>>>(A);
  if (main1) cudaEventRecord(main1, st);
  sc_block_sums_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  sc_block_scan_kernel<<<1, 1024, 0, st>>>(A);
  return cudaGetLastError();
}

cudaError_t sc_launch_rows(const ScArgs& A, uint32_t n_rows, int sms, cudaStream_t st) {
  sc_apply_kernel<<<A.n_blocks, 256, 0, st>>>(A);
  if (n_rows) {
    sc_scatter_kernel<<<A.ev_blocks, 256, 0, st>>>(A);
    sc_consensus_kernel<<<grid_for(((uint64_t)n_rows + 31) / 32 * 32, 256, sms, 8), 256, 0, st>>>(A, n_rows);
  }
  return cudaGetLastError();
}

}  // namespace bsq
