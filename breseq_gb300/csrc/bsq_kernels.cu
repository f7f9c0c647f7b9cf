// CUDA kernels of the read-evidence scoring path (sm_103a).
//
// All column work is "tile-gather over start-sorted reads": a warp owns 32 consecutive reference
// columns, walks the reads that can cover them in BAM order (one broadcast 32-byte record load per
// read), and each lane resolves its own column inside the read.  Adjacent lanes therefore read
// adjacent bytes of the same read: base and quality loads coalesce, every column sees its reads in
// BAM order (the order htslib's pileup presents them, so per-column FP64 sums run in the reference's
// order), and there is no global atomic per read base.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "bsq_common.h"
#include "bsq_device.cuh"
#include "bsq_kernels.h"

namespace bsq {

// ============================================================================ pack + validate
// One thread per record: builds the 32-byte DevRead, the query bounds of complex reads, checks the
// record (sortedness, CIGAR, offsets) and gathers the sample statistics the tile kernels need.
// Per-block accumulation of the sample-wide maximum reference span and MAPQ presence bits: one
// global atomic per block instead of one per read (a read-per-thread atomic on a single word
// serialises in L2).
__device__ __forceinline__ void pack_flush(uint32_t span, uint8_t mq, bool has, const PackOut& out) {
  __shared__ uint32_t sh_span, sh_mask[8];
  if (threadIdx.x == 0) sh_span = 0;
  if (threadIdx.x < 8) sh_mask[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t wspan = __reduce_max_sync(0xFFFFFFFFu, has ? span : 0u);
  uint32_t wmask[8];
#pragma unroll
  for (int w = 0; w < 8; w++) wmask[w] = __reduce_or_sync(0xFFFFFFFFu, (has && (mq >> 5) == w) ? (1u << (mq & 31)) : 0u);
  if ((threadIdx.x & 31) == 0) {
    if (wspan) atomicMax(&sh_span, wspan);
#pragma unroll
    for (int w = 0; w < 8; w++) if (wmask[w]) atomicOr(&sh_mask[w], wmask[w]);
  }
  __syncthreads();
  if (threadIdx.x == 0 && sh_span) atomicMax(out.maxspan, sh_span);
  if (threadIdx.x < 8 && sh_mask[threadIdx.x]) atomicOr(out.mapq_mask + threadIdx.x, sh_mask[threadIdx.x]);
}

// Validates and packs record i; returns its reference span and MAPQ when the pileup keeps it.
__device__ __forceinline__ void pack_one(const RawSoA& in, const PackOut& out, uint32_t i, uint32_t& span_out,
                                         uint8_t& mq_out, bool& kept) {
  const int32_t tid = in.tid[i], pos = in.pos[i];
  const uint16_t flag = in.flag[i];
  uint32_t err = 0;
  if (tid < 0 || (uint32_t)tid >= in.n_targets || pos < 0) { atomicOr(out.err, kErrOrder); return; }
  if (i > 0) {
    int32_t pt = in.tid[i - 1], pp = in.pos[i - 1];
    if (pt > tid || (pt == tid && pp > pos)) err |= kErrOrder;
  }
  const uint32_t len = in.l_qseq[i];
  const uint64_t so = in.seq_off[i];
  const uint64_t co = in.cigar_off[i];
  const uint32_t nc = in.n_cigar[i];
  DevRead d;
  d.seq_off = so;
  d.len = (uint16_t)len;
  d.n_cigar = (uint16_t)nc;
  d.cigar_off = (uint32_t)co;
  d.xl = in.xl[i] < 0 ? kNoTag : (uint16_t)in.xl[i];
  d.xr = in.xr[i] < 0 ? kNoTag : (uint16_t)in.xr[i];
  const uint8_t mq = in.mapq[i];
  d.mapq_idx = 0;
  d.rfile = in.read_file[i];
  d.clip = 0;
  uint8_t fl = 0;
  if (flag & 0x10) fl |= kRev;
  const uint32_t x1 = in.x1[i];
  if (x1 == 0) err |= kErrX1;
  if (x1 > 1) fl |= kRedundant;
  // filtered like htslib's pileup does by default, or on a target the pileup never visits
  const bool skip = (flag & 0x704) != 0 || !in.called[tid];
  if (skip) fl |= kSkip;
  if (len > 65535 || (so & 1) || so + len > in.n_bases || co + nc > in.n_cigar_total) err |= kErrBounds;
  if (in.xl[i] >= 65535 || in.xr[i] >= 65535) err |= kErrBounds;
  uint32_t rlen = 0, qlen = 0, nblk = 0;
  int32_t qs1 = 1, qe1 = 0, bs = 1, be = 0;
  bool only_s_m = true;
  uint32_t lead_s = 0;
  if (!(err & kErrBounds)) {
    const uint32_t* cg = in.cigar + co;
    for (uint32_t k = 0; k < nc; k++) {
      uint32_t op = cg[k] & 0xF, l = cg[k] >> 4;
      if (op_ref(op)) rlen += l;
      if (op == 0 || op == 1 || op == 4 || op == 7 || op == 8) qlen += l;
      if (op == 0) nblk++;
      else if (op == 4) { if (k == 0) lead_s = l; else if (k != nc - 1) only_s_m = false; }
      else only_s_m = false;
    }
    for (uint32_t k = 0; k < nc; k++) { if ((cg[k] & 0xF) != 4) break; qs1 += (int32_t)(cg[k] >> 4); }
    qe1 = (int32_t)qlen;
    for (uint32_t k = nc - 1; k > 0 && k < nc; k--) { if ((cg[k] & 0xF) != 4) break; qe1 -= (int32_t)(cg[k] >> 4); }
    be = (int32_t)qlen;
    for (uint32_t k = 0; k < nc; k++) {
      uint32_t op = cg[k] & 0xF;
      if (op != 4 && op != 5 && op != 3) break;
      if (op == 4) bs += (int32_t)(cg[k] >> 4);
    }
    for (uint32_t k = nc - 1; k > 0 && k < nc; k--) {
      uint32_t op = cg[k] & 0xF;
      if (op != 4 && op != 5 && op != 3) break;
      if (op == 4) be -= (int32_t)(cg[k] >> 4);
    }
  }
  const uint32_t tlen = in.tpoff[tid + 1] - in.tpoff[tid] - 1;
  const bool bad_cigar = (err & kErrBounds) || nc == 0 || rlen == 0 || qlen != len || (uint64_t)pos + rlen > tlen;
  if (!skip && !(err & kErrBounds) && bad_cigar) err |= kErrCigar;
  // soft-clipping tabulation: every mapped record on a non-empty target except XJ-tagged ones
  // (soft_clipping.cpp:373-393); X1 > 1 is kRedundant
  if ((flag & 0x4) || (in.xj && in.xj[i]) || tlen == 0) fl |= kScSkip;
  if (bad_cigar) fl |= kBadCigar;
  if (flag & 0x704) fl |= kFiltered;
  // the discordant-pair enter test of identify_mutations.cpp:1400-1415 that ends in `continue`:
  // paired, mapped, not a proper pair, primary, mate mapped, XP absent or not FR / RF / FF
  if ((flag & 0x1) && !(flag & 0x4) && !(flag & 0x2) && !(flag & (0x100 | 0x800 | 0x8)) && (!in.xp || in.xp[i] > 2))
    fl |= kDpCand;
  if (rlen == 0) rlen = 1;
  d.start = in.tpoff[tid] + (uint32_t)pos;
  d.end = d.start + rlen;
  if (only_s_m && nblk == 1 && lead_s < 256) { fl |= kSimple; d.clip = (uint8_t)lead_s; }
  d.flags = fl;
  QBounds qb;
  qb.qs0 = (uint16_t)(qs1 - 1); qb.qe0 = (uint16_t)(qe1 - 1); qb.qbs = (uint16_t)(bs - 1); qb.qbe = (uint16_t)(be - 1);
  out.reads[i] = d;
  out.qb[i] = qb;
  out.rstart[i] = d.start;
  out.mapq[i] = mq;
  if (err) atomicOr(out.err, err);
  span_out = rlen;
  mq_out = mq;
  kept = !skip;
}

__global__ void pack_reads_kernel(RawSoA in, PackOut out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t span = 0;
  uint8_t mq = 0;
  bool kept = false;
  if (i < in.n) pack_one(in, out, i, span, mq, kept);
  pack_flush(span, mq, kept, out);   // every thread of the block, from this one place
}

// apply the host's MAPQ -> class index map
__global__ void mapq_index_kernel(DevRead* reads, const uint8_t* mapq, const uint8_t* map, uint32_t n) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) reads[i].mapq_idx = map[mapq[i]];
}

// tile read ranges: reads with start in (c0 - maxspan, c0 + 32)
__global__ void tile_range_kernel(const uint32_t* rstart, uint32_t n_reads, uint32_t n_tiles, uint32_t maxspan,
                                  uint2* tile_range, uint32_t* max_tile_reads) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tiles) return;
  uint32_t c0 = t * 32;
  uint32_t lo_key = (c0 + 1 > maxspan) ? c0 + 1 - maxspan : 0;   // start >= c0 - maxspan + 1
  uint32_t hi_key = c0 + 32;                                       // start < c0 + 32
  uint32_t a = 0, b = n_reads;
  while (a < b) { uint32_t m = (a + b) >> 1; if (__ldg(rstart + m) < lo_key) a = m + 1; else b = m; }
  uint32_t lo = a;
  b = n_reads;
  while (a < b) { uint32_t m = (a + b) >> 1; if (__ldg(rstart + m) < hi_key) a = m + 1; else b = m; }
  tile_range[t] = make_uint2(lo, a);
  const unsigned act = __activemask();
  const uint32_t wmax = __reduce_max_sync(act, a - lo);   // one atomic per warp
  if ((threadIdx.x & 31) == __ffs(act) - 1) atomicMax(max_tile_reads, wmax);
}

// Tiles whose read range exceeds `thr` reads: listed (any order) and flagged in a bit per tile, so the
// column pass runs them first (see its tile queue).  Lane k of a warp holds tile 32w + k.
__global__ void tile_heavy_kernel(const uint2* tile_range, uint32_t n_tiles, uint32_t thr, uint32_t* heavy,
                                  uint32_t* heavy_bits, uint32_t* n_heavy) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  bool h = false;
  if (t < n_tiles) {
    const uint2 rr = tile_range[t];
    h = rr.y - rr.x > thr;
  }
  const unsigned m = __ballot_sync(0xFFFFFFFFu, h);
  const uint32_t lane = threadIdx.x & 31;
  if (lane == 0 && t < n_tiles) heavy_bits[t >> 5] = m;
  uint32_t base = 0;
  if (lane == 0 && m) base = atomicAdd(n_heavy, (uint32_t)__popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  if (h) heavy[base + __popc(m & ((1u << lane) - 1u))] = t;
}

// ============================================================================ pass 1: error counts
// error_count_pileup::pileup_callback (error_count.cpp:125-199) with count_alignment_position
// (error_count.cpp:854-986), read-parallel: a warp walks one read at a time, lanes over its aligned
// bases (the column a base sits on and its htslib pileup state follow from the CIGAR walk), so every
// (read, column) incidence is one lane-iteration.  Covariate events go to a block-private shared
// histogram with one atomic per distinct bin per warp; the per-column unique / redundant read counts
// the coverage histogram needs are +1/-1 difference arrays over each aligned block, scanned later.

// Both events of one unique read base (error_count.cpp:888-984).
__device__ __forceinline__ void ec_events(const DevSample& S, const EcArgs& A, uint32_t* hist,
                                          bool on, const DevRead& rd, uint32_t r, uint32_t c, int qpos, int indel,
                                          uint32_t& err) {
  const int rev = rd.flags & kRev;
  const uint32_t rs = rd.rfile;
  const uint64_t so = rd.seq_off;
  uint32_t bin1 = 0xFFFFFFFFu, bin2 = 0xFFFFFFFFu;
  if (on) {
    const uint8_t refc = __ldg(S.ref + c);
    // (1) base substitution / match at this column
    const uint8_t ob = nib_at(S.seq, so + qpos);
    if (ob != 15 && refc != 'N') {
      int oi = bam_idx(ob), ri = chr_idx(refc);
      if (oi < 0 || ri < 0 || ri > 3) err |= kErrBase;
      else {
        if (rev) { oi = 3 - oi; ri = 3 - ri; }
        const uint32_t q = __ldg(S.qual + so + qpos);
        if (q >= A.Q || rs >= A.R) err |= kErrCovariate;
        else bin1 = rs + A.R * (ri + 5u * (oi + 5u * q));
      }
    }
    if (indel == 0) {                          // (2a) '..': the next base also aligned
      if (qpos < query_end0(S, rd, r)) {
        const int mq = qpos + 1 - rev;
        const uint8_t ob2 = nib_at(S.seq, so + mq);
        const uint8_t rc2 = rev ? refc : __ldg(S.ref + c + 1);
        if (ob2 != 15 && rc2 != 'N') {
          const uint32_t q = __ldg(S.qual + so + mq);
          if (q >= A.Q || rs >= A.R) err |= kErrCovariate;
          else bin2 = rs + A.R * (4u + 5u * (4u + 5u * q));
        }
      }
    } else if (indel == -1) {                  // (2b) one deleted base follows
      const int mq = qpos + 1 - rev;
      if (mq < 0 || mq >= (int)rd.len) err |= kErrBounds;
      else {
        const uint8_t ob2 = nib_at(S.seq, so + mq);
        const uint8_t rn = __ldg(S.ref + c + 1);
        if (ob2 != 15 && rn != 'N') {
          int ri = chr_idx(rn);
          if (ri < 0 || ri > 3) err |= kErrBase;
          else {
            if (rev) ri = 3 - ri;
            const uint32_t q = __ldg(S.qual + so + mq);
            if (q >= A.Q || rs >= A.R) err |= kErrCovariate;
            else bin2 = rs + A.R * (ri + 5u * (4u + 5u * q));
          }
        }
      }
    } else if (indel == 1) {                   // (2c) one inserted base follows
      const int mq = qpos + 1;
      if (mq >= (int)rd.len) err |= kErrBounds;
      else if (mq <= query_end0(S, rd, r) && mq >= query_start0(S, rd, r)) {
        const uint8_t ob2 = nib_at(S.seq, so + mq);
        if (ob2 != 15) {
          int oi = bam_idx(ob2);
          if (oi < 0) err |= kErrBase;
          else {
            if (rev) oi = 3 - oi;
            const uint32_t q = __ldg(S.qual + so + mq);
            if (q >= A.Q || rs >= A.R) err |= kErrCovariate;
            else bin2 = rs + A.R * (4u + 5u * (oi + 5u * q));
          }
        }
      }
    }
  }
  if (bin1 != 0xFFFFFFFFu) atomicAdd(hist + bin1, 1u);
  if (bin2 != 0xFFFFFFFFu) atomicAdd(hist + bin2, 1u);
}

// required_junction_read_end_min_coordinate test of the preprocess stage (settings.h:345-354)
__device__ __forceinline__ bool read_start_counts(const EcArgs& A, const DevRead& rd, uint32_t bs1, uint32_t be1) {
  const int32_t umax = (int32_t)floor((double)((int32_t)rd.len - (int32_t)A.unmatched_min_len) * A.unmatched_factor_d);
  const uint32_t req = (umax <= 0) ? rd.len : rd.len - (uint32_t)umax;
  const uint32_t send1 = (rd.flags & kRev) ? rd.len - bs1 + 1 : be1;
  return send1 >= req;
}

// Work units are chunks of one job's reads, pulled by whole blocks from a shared counter; the block's
// shared histogram belongs to the chunk's job and is flushed at the chunk's end.
// Packed pairs of FP32 values (element 0 in the low word): Blackwell's two-wide FP32 add / sub.
__device__ __forceinline__ unsigned long long f32x2_add(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f32x2_sub(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ float f32x2_lo(unsigned long long x) { return __uint_as_float((uint32_t)x); }
__device__ __forceinline__ float f32x2_hi(unsigned long long x) { return __uint_as_float((uint32_t)(x >> 32)); }

// count_alignment_position (error_count.cpp:888-944) for a read with one aligned block (soft clips
// allowed), one thread per read: its bases are consecutive query positions on consecutive columns and
// no base has an indel, so base i has event (1) and, when i is not the block's last base, event (2a).
// Event (2a) of base i reads base, quality and reference at i + 1 - rev: for a forward read those of
// base i + 1, for a reverse read its own.  Both events of base j therefore test only base j's own
// values: (1) always, and (2a) on behalf of base j - 1 (forward, j >= 1) or of base j itself (reverse,
// j below the last).
// The thread walks the read in the 16-byte words of the quality array that hold it (a base's quality
// index equals its nibble index in the packed sequence, so each word pairs with one 8-byte sequence
// word), with the reference as 4-bit codes in the same nibble form, shifted into line with the word.
// Most bases match the reference and carry a (2a) event: their two events (rs, b, b, q) and
// (rs, '.', '.', q) are counted with one shared atomic in comb[(q * 4 + b) * R + rs], which the chunk's
// flush adds to both bins.  The rest go through the general per-base test.
__device__ __forceinline__ uint32_t nib_code(uint32_t x) {   // one-hot nibble A/C/G/T -> 0..3
  uint32_t d;
  asm("bfind.u32 %0, %1;" : "=r"(d) : "r"(x));
  return d;
}
// CODES: the words hold class bytes (quality * 5 + base) instead of qualities, and a base equal to the
// reference counts into comb[(strand * 256 + class byte) * R + rs] (one multiply-add for the index;
// the chunk's flush turns it into the two bins); the general test takes an A/C/G/T base's quality
// from its class byte and reads the quality byte only for other codes.
template <bool CODES>
__device__ __forceinline__ void ec_thread_read(const DevSample& S, const EcArgs& A, uint32_t* hist, uint32_t* comb,
                                               const DevRead& rd, uint32_t span, uint32_t& err) {
  const bool rev = rd.flags & kRev;
  const uint32_t rs = rd.rfile, R = A.R, Q = A.Q;
  if (rs >= R) { err |= kErrCovariate; return; }
  const uint32_t flip = rev ? 3u : 0u;                  // 3 - x == x ^ 3 for x in 0..3
  const uint64_t qa = rd.seq_off + rd.clip;             // quality and nibble index of base 0 (seq_off is even)
  const uint64_t w0 = qa >> 4, w1 = (qa + span + 15) >> 4;
  const int off0 = (int)(qa & 15u);                     // slot of base 0 in the first word
  // reference nibble of the column of slot 0 of word w0: column start - off0, stored at nibble + 16
  const uint32_t cb0 = rd.start + 16u - (uint32_t)off0;
  const uint32_t dsh = (cb0 & 15u) * 4u;                // bit offset of that nibble in its word
  const unsigned long long* rw = S.refnib + (cb0 >> 4);
  unsigned long long rlo = __ldg(rw);
  const int lo2 = rev ? 0 : 1, hi2 = rev ? (int)span - 1 : (int)span;   // bases carrying a (2a) event
  const uint32_t qR = 4u * R;
  bool bad_base = false, bad_q = false;
  int ilo = -off0;                                      // base index of slot 0 of the current word
  const uint32_t crow = (rev ? 256u : 0u) * R + rs;     // CODES: the strand's counter rows, read file rs
  for (uint64_t w = w0; w < w1; w++, ilo += 16, rw++) {
    const uint4 qv = __ldg(reinterpret_cast<const uint4*>(CODES ? A.code : S.qual) + w);
    const uint2 sv = __ldg(reinterpret_cast<const uint2*>(S.seq) + w);
    const unsigned long long rhi = __ldg(rw + 1);
    const unsigned long long r64 = dsh ? (rlo >> dsh) | (rhi << (64u - dsh)) : rlo;
    rlo = rhi;
    const uint32_t rr[2] = {(uint32_t)r64, (uint32_t)(r64 >> 32)};
    const uint32_t qq[4] = {qv.x, qv.y, qv.z, qv.w};
    const uint32_t ss[2] = {sv.x, sv.y};
    // slots of the read's bases, and of those with a (2a) event
    const int a = min(max(-ilo, 0), 16), b = min(max((int)span - ilo, 0), 16);
    const int a2 = min(max(lo2 - ilo, 0), 16), b2 = min(max(hi2 - ilo, 0), 16);
    const uint32_t m_in = (0xFFFFu >> (16 - b)) & ~((1u << a) - 1u);
    const uint32_t m_2 = (0xFFFFu >> (16 - b2)) & ~((1u << a2) - 1u);
    // bases equal to the reference and not N, eight to a 32-bit word (same_as_reference8)
    const uint32_t same = same_as_reference8(ss[0], rr[0]) | (same_as_reference8(ss[1], rr[1]) << 8);
    const uint32_t m_comb = same & m_2;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const uint32_t qb = (qq[k >> 2] >> (8 * (k & 3))) & 0xFFu;     // quality, or class byte (CODES)
      if (CODES ? (bool)((m_comb >> k) & 1u) : (((m_comb >> k) & 1u) && qb < Q)) {
        if (CODES) {
          atomicAdd(comb + qb * R + crow, 1u);
        } else {
          const uint32_t rb = (rr[k >> 3] >> (4 * (k & 7))) & 15u;   // A,C,G,T one-hot here
          atomicAdd(comb + qb * qR + (nib_code(rb) ^ flip) * R + rs, 1u);
        }
      } else if ((m_in >> k) & 1u) {
        // CODES: an A/C/G/T base's quality is its class byte / 5; an N's is never used; only another
        // code (254) reads its quality byte
        const uint32_t q = !CODES ? qb : qb < 254u ? qb / 5u : qb == 254u ? (uint32_t)__ldg(S.qual + w * 16 + k) : 0u;
        // BAM packing: the even base of a byte in its high nibble
        const uint32_t ob = (ss[k >> 3] >> (8 * ((k & 7) >> 1) + ((k & 1) ? 0 : 4))) & 15u;
        const uint32_t rb = (rr[k >> 3] >> (4 * (k & 7))) & 15u;   // A,C,G,T one-hot, else 15
        const bool in2 = (m_2 >> k) & 1u;
        const bool valid = ob != 15u && rb != 15u;     // neither the read base nor the reference is N
        const bool base_ok = (0x116u >> ob) & 1u;      // one-hot: A, C, G or T
        const bool q_ok = q < Q;
        bad_base |= valid && !base_ok;
        bad_q |= valid && !q_ok && (base_ok || in2);
        const uint32_t q25 = q * 25u;
        if (valid && base_ok && q_ok)
          atomicAdd(hist + (q25 + (nib_code(ob) ^ flip) * 5u + (nib_code(rb) ^ flip)) * R + rs, 1u);   // (ref, obs, q)
        if (valid && q_ok && in2) atomicAdd(hist + (q25 + 24u) * R + rs, 1u);                          // ('.', '.', q)
      }
    }
  }
  if (bad_base) err |= kErrBase;
  if (bad_q) err |= kErrCovariate;
}

// A read whose CIGAR has more than one aligned block: the CIGAR walk of htslib's pileup
// (resolve_cigar2), M/=/X blocks carrying their read bases, the last base of a block seeing the I / D
// run that follows it as its indel.  Lanes lane, lane + stride, ... of a block's bases; lane 0 adds the
// coverage steps.
__device__ __forceinline__ void ec_complex_read(const DevSample& S, const EcArgs& A, uint32_t* hist, const DevRead& rd,
                                                uint32_t r, uint32_t lane, uint32_t stride, uint32_t& err) {
  const bool red = rd.flags & kRedundant;
  int32_t* diff = red ? A.diff_r : A.diff_u;
  const uint32_t* cg = S.cigar + rd.cigar_off;
  const int nc = rd.n_cigar;
  uint32_t x = rd.start;
  int y = 0;
  const QBounds qb = S.qb[r];
  for (int k = 0; k < nc; k++) {
    const uint32_t w = __ldg(cg + k), op = w & 0xF, len = w >> 4;
    if (op_qm(op)) {
      int ind = 0;
      if (k + 1 < nc) {
        const uint32_t w2 = __ldg(cg + k + 1), op2 = w2 & 0xF;
        if (op2 == 2) {
          ind = -(int)(w2 >> 4);
          for (int j = k + 2; j < nc; j++) { const uint32_t wj = __ldg(cg + j); if ((wj & 0xF) == 2) ind -= (int)(wj >> 4); else break; }
        } else if (op2 == 1) {
          ind = (int)(w2 >> 4);
          for (int j = k + 2; j < nc; j++) {
            const uint32_t wj = __ldg(cg + j), o = wj & 0xF;
            if (o == 1) ind += (int)(wj >> 4); else if (o != 6) break;
          }
        } else if (op2 == 6 && k + 2 < nc) {
          int l3 = 0;
          for (int j = k + 2; j < nc; j++) {
            const uint32_t wj = __ldg(cg + j), o = wj & 0xF;
            if (o == 1) l3 += (int)(wj >> 4); else if (op_ref(o)) break;
          }
          if (l3 > 0) ind = l3;
        }
      }
      if (lane == 0) {
        atomicAdd(diff + x, 1);
        atomicAdd(diff + x + len, -1);
        if (A.preprocess && !red && y == 0 && read_start_counts(A, rd, (uint32_t)qb.qbs + 1u, (uint32_t)qb.qbe + 1u))
          A.qs_flag[(size_t)(rd.flags & kRev) * S.n_cols + x] = 1;
      }
      if (!red && A.do_errors)
        for (uint32_t i = lane; i < len; i += stride)
          ec_events(S, A, hist, true, rd, r, x + i, y + (int)i, (i == len - 1) ? ind : 0, err);
      x += len;
      y += (int)len;
    } else if (op_ref(op)) {
      x += len;                      // D / N columns: deletions, skipped by error counting
    } else if (op == 1 || op == 4) {
      y += (int)len;
    }
  }
}

// Work units are chunks of one job's reads, pulled by whole blocks from a shared counter; the block's
// shared histogram belongs to the chunk's job and is flushed at the chunk's end.  Reads with one
// aligned block are taken one per thread; the others are queued and walked one per warp afterwards
// (one per thread when the queue is full).
constexpr uint32_t kEcQueue = 1024;
__global__ void __launch_bounds__(256, 4) ec_read_kernel(const __grid_constant__ Batch B, const uint4* chunks, uint32_t n_chunks, unsigned int* next) {
  extern __shared__ uint32_t sh_hist[];
  __shared__ uint32_t sh_chunk, sh_nq;
  __shared__ uint32_t sh_queue[kEcQueue];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (;;) {
  if (threadIdx.x == 0) { sh_chunk = atomicAdd(next, 1u); sh_nq = 0; }
  __syncthreads();
  const uint32_t ci = sh_chunk;
  if (ci >= n_chunks) break;
  const uint4 ch = chunks[ci];                 // x = job, y = first read, z = end read
  const DevSample& S = B.jobs[ch.x].S;
  const EcArgs& A = B.jobs[ch.x].E;
  const uint32_t nbins = A.R * 25u * A.Q, ncomb = A.R * 4u * A.Q, nccomb = A.code ? 512u * A.R : 0u;
  uint32_t* sh_comb = sh_hist + nbins;
  uint32_t* sh_ccomb = sh_comb + ncomb;        // class-byte counters (CODES form)
  for (uint32_t i = threadIdx.x; i < nbins + ncomb + nccomb; i += blockDim.x) sh_hist[i] = 0;
  __syncthreads();
  uint32_t err = 0;
  for (uint32_t r = ch.y + threadIdx.x; r < ch.z; r += blockDim.x) {
    const DevRead rd = S.reads[r];
    if (rd.flags & kSkip) continue;      // filtered by flag, or on a target outside the pileup set
    if (!(rd.flags & kSimple)) {
      const uint32_t slot = atomicAdd(&sh_nq, 1u);
      if (slot < kEcQueue) sh_queue[slot] = r;
      else ec_complex_read(S, A, sh_hist, rd, r, 0, 1, err);
      continue;
    }
    const bool red = rd.flags & kRedundant;
    int32_t* diff = red ? A.diff_r : A.diff_u;
    const uint32_t span = rd.end - rd.start;
    atomicAdd(diff + rd.start, 1);
    atomicAdd(diff + rd.end, -1);
    if (A.preprocess && !red && rd.clip == 0 && read_start_counts(A, rd, 1u, span))
      A.qs_flag[(size_t)(rd.flags & kRev) * S.n_cols + rd.start] = 1;
    if (red || !A.do_errors) continue;
    if (A.code) ec_thread_read<true>(S, A, sh_hist, sh_ccomb, rd, span, err);
    else ec_thread_read<false>(S, A, sh_hist, sh_comb, rd, span, err);
  }
  __syncthreads();
  const uint32_t nq = min(sh_nq, kEcQueue);
  for (uint32_t k = warp; k < nq; k += nwarps) {
    const uint32_t r = sh_queue[k];
    ec_complex_read(S, A, sh_hist, S.reads[r], r, lane, 32, err);
  }
  __syncthreads();
  // class-byte counters (strand, quality * 5 + base, rs) of bases equal to the reference: both bins,
  // the base complemented on the reverse strand
  for (uint32_t i = threadIdx.x; i < nccomb; i += blockDim.x) {
    const uint32_t v = sh_ccomb[i];
    if (v) {
      const uint32_t rs = i % A.R, row = i / A.R, code = row & 255u, q = code / 5u;
      const uint32_t b = (code - 5u * q) ^ ((row >> 8) ? 3u : 0u);
      atomicAdd(sh_hist + (q * 25u + b * 6u) * A.R + rs, v);
      atomicAdd(sh_hist + (q * 25u + 24u) * A.R + rs, v);
    }
  }
  // combined counts of (rs, b, b, q) + (rs, '.', '.', q) into both bins
  for (uint32_t i = threadIdx.x; i < ncomb; i += blockDim.x) {
    const uint32_t v = sh_comb[i];
    if (v) {
      const uint32_t rs = i % A.R, qb = i / A.R, b = qb & 3u, q = qb >> 2;
      atomicAdd(sh_hist + (q * 25u + b * 6u) * A.R + rs, v);
      atomicAdd(sh_hist + (q * 25u + 24u) * A.R + rs, v);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nbins; i += blockDim.x) {
    const uint32_t v = sh_hist[i];
    if (v) atomicAdd(A.counts + i, (unsigned long long)v);
  }
  if (err) atomicOr(A.err, err);
  __syncthreads();
  }
}

// Block-wide inclusive scan of (a, b) pairs, 1024 threads.
__device__ __forceinline__ void block_scan2(int& a, int& b, int* sh_a, int* sh_b) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int ya = __shfl_up_sync(0xFFFFFFFFu, a, o), yb = __shfl_up_sync(0xFFFFFFFFu, b, o);
    if (lane >= o) { a += ya; b += yb; }
  }
  if (lane == 31) { sh_a[w] = a; sh_b[w] = b; }
  __syncthreads();
  if (w == 0) {
    int va = sh_a[lane], vb = sh_b[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int ya = __shfl_up_sync(0xFFFFFFFFu, va, o), yb = __shfl_up_sync(0xFFFFFFFFu, vb, o);
      if (lane >= o) { va += ya; vb += yb; }
    }
    sh_a[lane] = va; sh_b[lane] = vb;
  }
  __syncthreads();
  if (w > 0) { a += sh_a[w - 1]; b += sh_b[w - 1]; }
}

__global__ void __launch_bounds__(1024) cov_blocksum_kernel(const __grid_constant__ Batch B) {
  __shared__ int sa[32], sb[32];
  const uint32_t job = job_of(B.cblk_begin, B.n_jobs, blockIdx.x);
  const uint32_t lb = blockIdx.x - B.cblk_begin[job];
  const EcArgs& A = B.jobs[job].E;
  const uint32_t n = B.jobs[job].S.n_cols;
  const uint32_t c = lb * 1024 + threadIdx.x;
  int a = c < n ? A.diff_u[c] : 0, b = c < n ? A.diff_r[c] : 0;
  block_scan2(a, b, sa, sb);
  if (threadIdx.x == 1023) { A.blk_u[lb] = (uint32_t)a; A.blk_r[lb] = (uint32_t)b; }
}

// Unique-only coverage histogram (error_count.cpp:176-191): a column counts when no redundant read
// covers it; preprocess adds the read-start tallies of the same columns.
__global__ void __launch_bounds__(1024) cov_hist_kernel(const __grid_constant__ Batch B) {
  __shared__ int sa[32], sb[32];
  const uint32_t job = job_of(B.cblk_begin, B.n_jobs, blockIdx.x);
  const uint32_t lb = blockIdx.x - B.cblk_begin[job];
  const DevSample& S = B.jobs[job].S;
  const EcArgs& A = B.jobs[job].E;
  const uint32_t c = lb * 1024 + threadIdx.x;
  int a = c < S.n_cols ? A.diff_u[c] : 0, b = c < S.n_cols ? A.diff_r[c] : 0;
  block_scan2(a, b, sa, sb);
  a += (int)A.blk_u[lb];
  b += (int)A.blk_r[lb];
  bool rec = false;
  uint32_t t = 0, key = 0xFFFFFFFFu;
  if (c < S.n_cols && __ldg(S.ref + c) != 0) {
    t = target_of(S, c);
    if (__ldg(S.tgt_called + t) && b == 0) {
      rec = true;
      const uint32_t u = (uint32_t)a;
      if (u >= A.hist_cap) atomicOr(A.err, kErrBounds);
      key = __ldg(S.tgt_group + t) * A.hist_cap + min(u, A.hist_cap - 1);
    }
  }
  const unsigned active = __ballot_sync(0xFFFFFFFFu, rec);
  if (rec) {
    const unsigned peers = __match_any_sync(active, key);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(A.cov_hist + key, (unsigned long long)__popc(peers));
    if (A.preprocess) {
      atomicAdd(A.found + 2 * t + A.qs_flag[c], 1ull);
      atomicAdd(A.found + 2 * t + A.qs_flag[(size_t)S.n_cols + c], 1ull);
    }
  }
}

// ============================================================================ pass 2: column pass
// identify_mutations_pileup::pileup_callback at insert position 0 (identify_mutations.cpp:1359-1686)
// for every column: coverage, the five summed log10 likelihoods, the pure-genotype call, and the
// decision of which columns go on to the EM candidate kernel.  The warp stages the records of each
// 32-read batch in shared memory and walks only those that reach its tile, in BAM order, with the
// base and quality loads of two reads in flight before either is consumed.
constexpr uint32_t kColumnWarps = 8;
constexpr uint32_t kColumnIlp = 4;      // common-path reads whose loads are in flight together

// Per-thread shared-memory accumulators of the column pass, structure of arrays (thread t's values at
// index t of each array: no bank conflicts): the screen bound B[5] and the redundant-read counts and
// 1/X1 weights per strand.
struct ColRare {
  float* b;          // [5][256]
  uint32_t* cnt;     // [2][256]
  double* w;         // [2][256]
  uint32_t t;
  __device__ ColRare(unsigned char* base, uint32_t tid)
      : b(reinterpret_cast<float*>(base)), cnt(reinterpret_cast<uint32_t*>(base + 5 * 256 * 4)),
        w(reinterpret_cast<double*>(base + 7 * 256 * 4)), t(tid) {}
  __device__ void clear() {
#pragma unroll
    for (int i = 0; i < 5; i++) b[i * 256 + t] = 0.0f;
    cnt[t] = cnt[256 + t] = 0;
    w[t] = w[256 + t] = 0.0;
  }
  __device__ float& B(int i) { return b[i * 256 + t]; }
  __device__ void redundant(bool rev, double weight) { cnt[rev * 256 + t] += 1; w[rev * 256 + t] += weight; }
  __device__ uint32_t raw(bool rev) const { return cnt[rev * 256 + t]; }
  __device__ double weight(bool rev) const { return w[rev * 256 + t]; }
};
constexpr size_t kColRareBytes = 256 * (5 * 4 + 2 * 4 + 2 * 8);
// 1/X1 of each staged redundant read, one double per slot (computed once per read and tile by the lane
// that stages it, not by every lane at every column: FP64 division is slow here)
constexpr size_t kColWeightBytes = kColumnWarps * 32 * sizeof(double);

template <bool B> struct BoolC { static constexpr bool value = B; };

// Staged record of a common-path read for one tile: one aligned block (soft clips allowed), unique,
// untrimmed, a known read file, in a tile with no failed-fit column.  What depends on the read alone
// (its likelihood-class base, the addresses of its bases and qualities, its span) is computed once
// per (read, tile) by the lane that stages it, so a lane's work per read base is the coverage test,
// two byte loads, the class lookup and the sums.
struct __align__(16) FastRead {
  uint64_t qual;       // address of qual[seq_off + clip - start]: the quality at column c is at qual + c
                       // (of the class bytes instead, when the sample has them)
  uint64_t seq;        // address of the read's first packed base byte (seq_off is even)
  uint32_t start;      // first column
  uint32_t span_clip;  // reference span (low 16 bits) | leading soft clip << 16
  uint32_t kbase;      // likelihood class of (MAPQ, read file, strand) at quality 0, observed base 0
  uint32_t rev;        // 1 for a reverse-strand read
};
static_assert(sizeof(FastRead) == sizeof(DevRead), "a staging slot holds either form");

template <bool FP64>
__global__ void __launch_bounds__(256, 4) im_column_kernel(const __grid_constant__ Batch Bt) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // one 32-byte slot per read of the staged batch: its FastRead on the common path, else its DevRead
  DevRead* sh_rd = reinterpret_cast<DevRead*>(smem) + warp * 32;
  FastRead* sh_fr = reinterpret_cast<FastRead*>(smem) + warp * 32;
  // with class bytes, a common-path read's slot holds its 16-byte CodeRead (see the staging below)
  uint4* sh_cr = reinterpret_cast<uint4*>(smem) + warp * 64;
  // accumulators only rare reads touch (mismatching or low-likelihood bases, redundant reads): one
  // shared-memory slot per thread, column by column, instead of registers held for the whole tile
  ColRare rare(smem + kColumnWarps * 32 * sizeof(DevRead), threadIdx.x);
  double* sh_w = reinterpret_cast<double*>(smem + kColumnWarps * 32 * sizeof(DevRead) + kColRareBytes) + warp * 32;
  uint32_t local_err = 0;
  // Tiles come from a queue, one per warp at a time: first every job's heavy tiles (a read range more
  // than twice the sample's expected one: repeat copies, coverage peaks), then all tiles in column
  // order, skipping the heavy ones.  A warp holding a heavy tile takes fewer tiles, and the heavy ones
  // start first, so no warp is left running alone at the end.  The next unit is fetched while the
  // current tile runs.  Results do not depend on the order: a tile writes only its own columns.
  const uint32_t n_units = Bt.total_heavy + Bt.total_tiles;
  uint32_t q = 0;
  if (lane == 0) q = atomicAdd(Bt.tile_next, 1u);
  q = __shfl_sync(0xFFFFFFFFu, q, 0);
  while (q < n_units) {
    uint32_t job, tile;
    if (q < Bt.total_heavy) {
      job = job_of(Bt.heavy_begin, Bt.n_jobs, q);
      tile = __ldg(Bt.jobs[job].S.heavy + (q - Bt.heavy_begin[job]));
    } else {
      const uint32_t gt = q - Bt.total_heavy;
      job = job_of(Bt.tile_begin, Bt.n_jobs, gt);
      tile = gt - Bt.tile_begin[job];
    }
    uint32_t q_next = 0;
    if (lane == 0) q_next = atomicAdd(Bt.tile_next, 1u);
    const uint32_t* hb = Bt.jobs[job].S.heavy_bits;
    if (q >= Bt.total_heavy && Bt.total_heavy && hb && ((__ldg(hb + (tile >> 5)) >> (tile & 31)) & 1u)) {
      q = __shfl_sync(0xFFFFFFFFu, q_next, 0);        // run from the heavy list already
      continue;
    }
    const DevSample& S = Bt.jobs[job].S;
    const ClassTable& T = Bt.jobs[job].T;
    const ImArgs& A = Bt.jobs[job].I;
    const uint32_t c0 = tile * 32, c = c0 + lane;
    const bool inr = c < S.n_cols;
    const uint8_t refc = inr ? __ldg(S.ref + c) : 0;
    const uint32_t t = inr ? target_of(S, c) : 0;
    const bool real = inr && refc != 0 && __ldg(S.tgt_called + t);
    const bool failed = real && __ldg(S.tgt_failed + t);
    const int ref_idx = chr_idx(refc) < 0 ? 5 : chr_idx(refc);
    uint32_t utop = 0, ubot = 0, n = 0;
    rare.clear();
    bool uonly = true, slots = false;
    double S64[5] = {0, 0, 0, 0, 0};
    // Kahan sums of hypotheses 0-1 and 2-3 as packed FP32 pairs (one f32x2 instruction per step for
    // two sums, the same IEEE operations per element), hypothesis 4 scalar
    unsigned long long s01 = 0, s23 = 0, k01 = 0, k23 = 0;
    float s4 = 0.0f, k4 = 0.0f;
    const uint2 rr = __ldg(S.tile_range + tile);
    const bool tile_fast = __all_sync(0xFFFFFFFFu, !failed);
    // with the per-base class bytes, a common-path base is one byte: scored when its class byte is at
    // least cut5 and below 254 (code - cut5 < lim, unsigned)
    const uint8_t* const codes = S.code;
    const uint32_t cut5 = A.base_quality_cutoff * 5u;
    const uint32_t lim = cut5 < 254u ? 254u - cut5 : 0u;
    const uint32_t refbit = 1u << ref_idx;
    // Kahan-compensated FP32 sums of one class entry (hypotheses 0-1, 2-3 packed, 4 scalar)
    auto kahan = [&](const ulonglong2& v, float x4) {
      const unsigned long long y01 = f32x2_sub(v.x, k01), y23 = f32x2_sub(v.y, k23);
      const unsigned long long t01 = f32x2_add(s01, y01), t23 = f32x2_add(s23, y23);
      k01 = f32x2_sub(f32x2_sub(t01, s01), y01);
      k23 = f32x2_sub(f32x2_sub(t23, s23), y23);
      s01 = t01; s23 = t23;
      const float y4 = x4 - k4, t4 = s4 + y4;
      k4 = (t4 - s4) - y4;
      s4 = t4;
    };
    // screen bound  B_v = sum_i max(0, lp_i[v] - lp_i[ref]); zero unless the read's own base is not
    // its most likely hypothesis or it differs from the reference
    auto screen = [&](const ulonglong2& v, float x4) {
      const float lp[5] = {f32x2_lo(v.x), f32x2_hi(v.x), f32x2_lo(v.y), f32x2_hi(v.y), x4};
      const float lr = ref_idx == 0 ? lp[0] : ref_idx == 1 ? lp[1] : ref_idx == 2 ? lp[2] : ref_idx == 3 ? lp[3] : lp[4];
#pragma unroll
      for (int b = 0; b < 5; b++) rare.B(b) += fmaxf(0.0f, lp[b] - lr);
    };
    // one scored read base of likelihood class k (identify_mutations.cpp:1640-1658)
    auto accumulate = [&](uint32_t k, int obs) {
      ++n;
      if (FP64) {
        const double* lp = T.lp64 + (size_t)k * 5;
#pragma unroll
        for (int b = 0; b < 5; b++) S64[b] += __ldg(lp + b);
      } else {
        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(T.lp32 + (size_t)k * 8));
        const float2 w = __ldg(reinterpret_cast<const float2*>(T.lp32 + (size_t)k * 8 + 4));
        kahan(v, w.x);
        if (__float_as_uint(w.y) & refbit) screen(v, w.x);
      }
    };
    // One read as this lane sees it in the general case: the pileup state at column c (CIGAR walk,
    // trims, deletions, redundancy) and the base / quality that state selects.
    auto general = [&](const DevRead& rd, uint32_t r, double inv_x1) {
      if (!(real && c >= rd.start && c < rd.end)) return;
      Pile e;
      resolve(S, rd, c, e);
      const bool rev = rd.flags & kRev;
      const bool red = rd.flags & kRedundant;
      int qp = e.qpos;
      if (e.del) qp += 1 - (int)rev;
      uint8_t base = 15, qv = 0;
      if (qp < (int)rd.len) {
        base = nib_at(S.seq, rd.seq_off + qp);            // the base itself, or the one checked for a deletion
        qv = __ldg(S.qual + rd.seq_off + qp);
      }
      if (failed) {
        // tabulate_position_coverage (identify_mutations.cpp:2218-2250)
        if (e.del || base == 15) return;
        if (!red) { if (rev) ++ubot; else ++utop; }
        else rare.redundant(rev, inv_x1);
        return;
      }
      // a discordant-pair candidate without a usable XP tag, at its first column (:1399-1416)
      if ((rd.flags & kDpCand) && c == rd.start && dp_group_member(A.dp_rg, __ldg(S.rg + r))) return;
      if (!e.del && base == 15) return;                       // N read base: not counted at all
      if (red) {
        uonly = false;
        rare.redundant(rev, inv_x1);
        return;
      }
      if (rev) ++ubot; else ++utop;
      if (e.indel > 0 && !e.del) slots = true;
      // trims: a read with XL and XR both absent or 0 is never trimmed except at a deletion column
      if ((e.del || (rd.xl != kNoTag && rd.xl != 0) || (rd.xr != kNoTag && rd.xr != 0)) && is_trimmed(rd, e.qpos, e.del))
        return;
      if (e.del) {
        // the quality comes from the next base; the reference asserts if there is none
        if (e.qpos + 1 - (int)rev >= (int)rd.len || base == 15) return;
      }
      int obs = 4;
      if (!e.del) {
        if (__popc(base) != 1) { local_err |= kErrBase; return; }     // not one of A, C, G, T
        obs = __ffs(base) - 1;
      }
      const uint32_t q = qv;
      const uint32_t rs = rd.rfile;
      if (q >= T.Q || rs >= T.R) { local_err |= kErrCovariate; return; }
      if (q < A.base_quality_cutoff) return;
      const uint32_t k = ((((uint32_t)rd.mapq_idx * T.R + rs) * 2u + (rev ? 1u : 0u)) * T.Q + q) * 5u + (uint32_t)obs;
      accumulate(k, obs);
    };
    // A common-path read at this lane's column, without branches: a lane the read does not cover (or
    // whose base is N) loads nothing and adds zeros, so the warp runs one instruction stream per read.
    // Loads first, so the loads of all the reads in flight are issued before any is consumed.
    struct FastLd { uint32_t q, byte, sh; };
    auto fast_load = [&](const FastRead& f, bool have, FastLd& L) {
      const uint32_t d = c - f.start;
      const bool cov = have && real && d < (f.span_clip & 0xFFFFu);
      const uint32_t qpos = d + (f.span_clip >> 16);
      L.sh = (qpos & 1u) ? 0u : 4u;                                    // high nibble first
      L.q = 0; L.byte = 0xFFu;
      if (cov) {
        L.q = __ldg(reinterpret_cast<const uint8_t*>(f.qual) + c);
        L.byte = __ldg(reinterpret_cast<const uint8_t*>(f.seq) + (qpos >> 1));
      }
    };
    bool bad_base = false, bad_q = false;
    // the same for a sample with class bytes, from its 16-byte CodeRead: one byte per base, its class
    // at kbase + code, the zero entry K when the base is not scored
    auto code_load = [&](const uint4& f, bool have, uint32_t& code) {
      const uint32_t d = c - f.y;
      const bool cov = have && real && d < (f.z & 0xFFFFu);
      code = cov ? (uint32_t)__ldg(codes + (uint32_t)(f.x + c)) : 255u;
    };
    // kRed: the batch holds simple redundant reads (compiled out of the common loop)
    auto code_use = [&](auto red_c, const uint4& f, uint32_t code, uint32_t slot) {
      const bool counted = code != 255u;                              // covered, and not an N read base
      const bool rev = f.z >> 31;
      if constexpr (decltype(red_c)::value) {
        if ((f.z >> 30) & 1u) {
          // a simple redundant read: redundant coverage and its 1/X1 weight, nothing scored (the
          // general path's outcome for such a read); the warp takes this branch together
          if (counted) {
            uonly = false;
            rare.redundant(rev, sh_w[slot]);
          }
          return;
        }
      }
      utop += (counted && !rev) ? 1u : 0u;
      ubot += (counted && rev) ? 1u : 0u;
      bad_base |= code == 254u;                                       // not one of A, C, G, T
      const bool use = code - cut5 < lim;
      if (FP64) {
        if (use) accumulate(f.w + code, 0);
      } else {
        const uint32_t k = use ? f.w + code : T.K;
        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(T.lp32 + (size_t)k * 8));
        const float2 w = __ldg(reinterpret_cast<const float2*>(T.lp32 + (size_t)k * 8 + 4));
        n += use ? 1u : 0u;
        kahan(v, w.x);
        if (__float_as_uint(w.y) & refbit) screen(v, w.x);
      }
    };
    auto fast_use = [&](const FastRead& f, const FastLd& L) {
      const uint32_t base = (L.byte >> L.sh) & 15u;
      const bool counted = base != 15u;                               // covered, and not an N read base
      utop += (counted && !f.rev) ? 1u : 0u;
      ubot += (counted && f.rev) ? 1u : 0u;
      const bool base_ok = (0x116u >> base) & 1u;                     // one-hot: A, C, G or T
      const bool q_ok = L.q < T.Q;
      bad_base |= counted && !base_ok;
      bad_q |= counted && base_ok && !q_ok;
      const bool use = counted && base_ok && q_ok && L.q >= A.base_quality_cutoff;
      const uint32_t obs = 31u - __clz(base);
      if (FP64) {
        if (use) accumulate(f.kbase + L.q * 5u + obs, (int)obs);
      } else {
        // the class entry when the base is scored, zeros otherwise (a Kahan step adding zero)
        ulonglong2 v = make_ulonglong2(0ull, 0ull);
        float2 w = make_float2(0.0f, 0.0f);
        const uint32_t k = f.kbase + L.q * 5u + obs;
        if (use) {
          v = __ldg(reinterpret_cast<const ulonglong2*>(T.lp32 + (size_t)k * 8));
          w = __ldg(reinterpret_cast<const float2*>(T.lp32 + (size_t)k * 8 + 4));
        }
        n += use ? 1u : 0u;
        kahan(v, w.x);
        if (__float_as_uint(w.y) & refbit) screen(v, w.x);     // zeros when not scored
      }
    };
    for (uint32_t b0 = rr.x; b0 < rr.y; b0 += 32) {
      const uint32_t rl = b0 + lane;
      bool rel = false, fast = false;
      DevRead mine;
      if (rl < rr.y) {
        mine = S.reads[rl];
        rel = !(mine.flags & kSkip) && mine.end > c0;
        fast = rel && tile_fast && (mine.flags & (kSimple | kDpCand)) == kSimple &&
               (mine.xl == kNoTag || mine.xl == 0) && (mine.xr == kNoTag || mine.xr == 0) && mine.rfile < T.R;
      }
      // Redundant reads take the common path only with class bytes, and only when every redundant read
      // of the batch does, so that their 1/X1 sums keep BAM order in one loop.
      const bool red = rel && (mine.flags & kRedundant);
      if (__any_sync(0xFFFFFFFFu, red && !(fast && codes))) fast = fast && !red;
      const bool red_batch = __any_sync(0xFFFFFFFFu, fast && red);
      // the batch's common-path reads take slots 0..nf-1 and the others the slots after them, each
      // part in BAM order, so the loops below walk slots by index
      unsigned fmask = __ballot_sync(0xFFFFFFFFu, fast);
      unsigned gmask = __ballot_sync(0xFFFFFFFFu, rel && !fast);
      const uint32_t nf = __popc(fmask);
      const unsigned below = (1u << lane) - 1u;
      if (fast) {
        const uint32_t slot = __popc(fmask & below);
        const uint32_t rev = mine.flags & kRev;
        const uint32_t kbase = (((uint32_t)mine.mapq_idx * T.R + mine.rfile) * 2u + rev) * T.Q * 5u;
        if (codes) {
          // CodeRead: class-byte index of column 0 (mod 2^32), first column, span | redundant << 30 |
          // strand << 31 (a simple read's span is below 2^16), class base
          sh_cr[slot] = make_uint4((uint32_t)(mine.seq_off + mine.clip) - mine.start, mine.start,
                                   (mine.end - mine.start) | ((uint32_t)red << 30) | (rev << 31), kbase);
          if (red) sh_w[slot] = 1.0 / (double)__ldg(S.x1 + rl);
        } else {
          FastRead f;
          f.qual = (uint64_t)(uintptr_t)S.qual + mine.seq_off + mine.clip - mine.start;
          f.seq = (uint64_t)(uintptr_t)S.seq + (mine.seq_off >> 1);
          f.start = mine.start;
          f.span_clip = (mine.end - mine.start) | ((uint32_t)mine.clip << 16);
          f.kbase = kbase;
          f.rev = rev;
          sh_fr[slot] = f;
        }
      } else if (rel) {
        const uint32_t slot = nf + __popc(gmask & below);
        sh_rd[slot] = mine;
        sh_w[slot] = (mine.flags & kRedundant) ? 1.0 / (double)__ldg(S.x1 + rl) : 0.0;
      }
      __syncwarp();
      // common-path reads in BAM order, kColumnIlp at a time
      if (codes) {
        auto code_loop = [&](auto red_c) {
          for (uint32_t j0 = 0; j0 < nf; j0 += kColumnIlp) {
            uint32_t code[kColumnIlp];
#pragma unroll
            for (int u = 0; u < (int)kColumnIlp; u++) code_load(sh_cr[min(j0 + u, 31u)], j0 + u < nf, code[u]);
#pragma unroll
            for (int u = 0; u < (int)kColumnIlp; u++) code_use(red_c, sh_cr[min(j0 + u, 31u)], code[u], min(j0 + u, 31u));
          }
        };
        if (red_batch) code_loop(BoolC<true>());
        else code_loop(BoolC<false>());
      } else {
        for (uint32_t j0 = 0; j0 < nf; j0 += kColumnIlp) {
          FastLd L[kColumnIlp];
#pragma unroll
          for (int u = 0; u < (int)kColumnIlp; u++) fast_load(sh_fr[min(j0 + u, 31u)], j0 + u < nf, L[u]);
#pragma unroll
          for (int u = 0; u < (int)kColumnIlp; u++) fast_use(sh_fr[min(j0 + u, 31u)], L[u]);
        }
      }
      // the other reads of the batch in BAM order (redundant reads keep BAM order among themselves,
      // so the per-column 1/X1 sums run in the reference's order)
      for (uint32_t slot = nf; gmask; slot++) {
        const int j = __ffs(gmask) - 1;
        gmask &= gmask - 1;
        general(sh_rd[slot], b0 + j, sh_w[slot]);
      }
      __syncwarp();
    }
    if (inr) {
      ColCov cv;
      cv.uniq_top = utop; cv.uniq_bot = ubot; cv.rawred_top = rare.raw(false); cv.rawred_bot = rare.raw(true);
      cv.red_top = rare.weight(false); cv.red_bot = rare.weight(true);
      ColCall cl;
      cl.n = n; cl.best = 5; cl.score = __longlong_as_double(0x7ff8000000000000ll); cl.flags = 0;
      cl.pad[0] = cl.pad[1] = 0;
      if (real && !failed) {
        if (uonly) cl.flags |= kUniqueOnly;
        if (slots) cl.flags |= kSlots;
        cl.flags |= kScored;
        if (n > 0) {
          // pure_genotype_call (identify_mutations.cpp:3398-3433) and the Bonferroni shift (:1680)
          int best = 0;
          double score;
          if (FP64) {
            double sb = S64[0];                 // the best sum kept in a register (no indexed array)
#pragma unroll
            for (int b = 1; b < 5; b++) if (S64[b] > sb) { sb = S64[b]; best = b; }
            double off = -DBL_MAX;
#pragma unroll
            for (int b = 0; b < 5; b++) if (b != best) off = fmax(off, S64[b]);
            double te = 0;
#pragma unroll
            for (int b = 0; b < 5; b++) if (b != best) te += exp10(S64[b] - off);
            score = sb - (log10(te) + off) - A.log10_ref_len;
            cl.flags |= kCandidate;            // the plain form runs the EM wherever a base was scored
            if (best != ref_idx && score > 0) cl.flags |= kLikelyRa;
          } else {
            const float s32[5] = {f32x2_lo(s01), f32x2_hi(s01), f32x2_lo(s23), f32x2_hi(s23), s4};
            const float k32[5] = {f32x2_lo(k01), f32x2_hi(k01), f32x2_lo(k23), f32x2_hi(k23), k4};
            double tot[5];
#pragma unroll
            for (int b = 0; b < 5; b++) tot[b] = (double)s32[b] - (double)k32[b];
            double tb = tot[0];
#pragma unroll
            for (int b = 1; b < 5; b++) if (tot[b] > tb) { tb = tot[b]; best = b; }
            double d[5], off = -DBL_MAX;
#pragma unroll
            for (int b = 0; b < 5; b++) { d[b] = tot[b] - tb; if (b != best) off = fmax(off, d[b]); }
            float te = 0.0f;
#pragma unroll
            for (int b = 0; b < 5; b++) if (b != best) te += exp10f((float)(d[b] - off));
            score = -(off + (double)log10f(te)) - A.log10_ref_len;
            // guard band: FP32 sums are within ~n * 6e-7 of FP64; decisions closer than that are
            // recomputed in FP64 by the candidate kernel
            const double g = (double)A.guard * (1.0 + (double)n);
            const bool near = fabs(score - A.mutation_cutoff) < g || (best != ref_idx && fabs(score) < g) || off > -g;
            if (near) cl.flags |= kRecompute;
            if (best != ref_idx && score > 0) cl.flags |= kCandidate | kLikelyRa;
            float bmax = 0.0f;
#pragma unroll
            for (int b = 0; b < 5; b++) if (b != ref_idx) bmax = fmaxf(bmax, rare.B(b));
            if (ref_idx == 5 || (double)bmax - A.log10_ref_len >= A.poly_cutoff - (double)A.screen_margin)
              cl.flags |= kCandidate;
          }
          cl.best = (uint8_t)best;
          cl.score = score;
          if (score >= A.mutation_cutoff) cl.flags |= kBasePredicted;
        }
      }
      A.cov[c] = cv;
      A.call[c] = cl;
    }
    if (bad_base) local_err |= kErrBase;
    if (bad_q) local_err |= kErrCovariate;
    if (local_err) { atomicOr(A.err, local_err); local_err = 0; }
    q = __shfl_sync(0xFFFFFFFFu, q_next, 0);
  }
}

// ============================================================================ candidate compaction
// Deterministic stream compaction of the columns flagged for the candidate kernel, in column order.
// The candidate queue puts the columns likely to emit an RA item (their bounds are the longest
// work) first, the others after them, each part in column order.  `part` 0 / 1 selects which.
__device__ __forceinline__ bool cand_pick(const ColCall& cl, int part) {
  if (!(cl.flags & (kCandidate | kSlots | kRecompute))) return false;
  return ((cl.flags & kLikelyRa) != 0) == (part == 0);
}
__global__ void cand_count_kernel(const ColCall* call, uint32_t n, uint32_t* block_counts, int part) {
  __shared__ uint32_t s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool f = i < n && cand_pick(call[i], part);
  uint32_t b = __popc(__ballot_sync(0xFFFFFFFFu, f));
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, b);
  __syncthreads();
  if (threadIdx.x == 0) block_counts[blockIdx.x] = s;
}

// Exclusive scan of v[0..n) in place by one block of 1024 threads; the sum goes to *total.
__device__ void block_exclusive_scan(uint32_t* v, uint32_t n, uint32_t* total) {
  __shared__ uint32_t carry;
  __shared__ uint32_t warp_sums[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    uint32_t x = i < n ? v[i] : 0;
    uint32_t incl = x;
    for (int o = 1; o < 32; o <<= 1) { uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o); if ((threadIdx.x & 31) >= o) incl += y; }
    if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = incl;
    __syncthreads();
    if (threadIdx.x < 32) {
      uint32_t ws = threadIdx.x < (blockDim.x >> 5) ? warp_sums[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) { uint32_t y = __shfl_up_sync(0xFFFFFFFFu, ws, o); if (threadIdx.x >= o) ws += y; }
      warp_sums[threadIdx.x] = ws;
    }
    __syncthreads();
    uint32_t wpre = (threadIdx.x >> 5) ? warp_sums[(threadIdx.x >> 5) - 1] : 0;
    uint32_t excl = carry + wpre + incl - x;
    if (i < n) v[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + x;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
  __syncthreads();
}

__global__ void scan_kernel(uint32_t* v, uint32_t n, uint32_t* total) { block_exclusive_scan(v, n, total); }

// the coverage block sums of every job, one block per job
__global__ void scan_jobs_kernel(const __grid_constant__ Batch B) {
  const uint32_t job = blockIdx.x;
  const uint32_t nb = B.cblk_begin[job + 1] - B.cblk_begin[job];
  const EcArgs& A = B.jobs[job].E;
  block_exclusive_scan(A.blk_u, nb, A.blk_u + nb);
  block_exclusive_scan(A.blk_r, nb, A.blk_r + nb);
}

__global__ void cand_scatter_kernel(const ColCall* call, uint32_t n, const uint32_t* block_offsets, uint32_t* out,
                                    int part, const uint32_t* base) {
  __shared__ uint32_t warp_base[32];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool f = i < n && cand_pick(call[i], part);
  if (base) out += *base;
  unsigned m = __ballot_sync(0xFFFFFFFFu, f);
  if ((threadIdx.x & 31) == 0) warp_base[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); w++) { uint32_t x = warp_base[w]; warp_base[w] = acc; acc += x; }
  }
  __syncthreads();
  if (f) out[block_offsets[blockIdx.x] + warp_base[threadIdx.x >> 5] + __popc(m & ((1u << (threadIdx.x & 31)) - 1))] = i;
}

// ============================================================================ sparse MC / UN input
// The MC and UN state machines (identify_mutations.cpp:2262-2344, 2972-3007) change state only at a
// column that is not base-predicted, has unique coverage at or below the target's propagation cutoff,
// or total coverage at or below its seed cutoff; the column after such a column closes what it
// opened, and the column before it supplies the left-outside coverage.  Those columns are marked and
// the host replays the state machines over them alone.
__global__ void interval_mark_kernel(const __grid_constant__ Batch B, const ColCov* cov, const ColCall* call, uint8_t* keep) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= B.total_cols) return;
  if (!(call[g].flags & kScored)) return;
  const uint32_t job = job_of(B.col_begin, B.n_jobs, g);
  const uint32_t c = g - B.col_begin[job];
  const DevJob& J = B.jobs[job];
  const uint32_t* tpoff = J.S.tpoff;
  uint32_t lo = 0, hi = J.S.n_targets;
  while (hi - lo > 1) { uint32_t mid = (lo + hi) >> 1; if (tpoff[mid] <= c) lo = mid; else hi = mid; }
  const uint32_t t = lo;
  if (!J.S.tgt_called[t] || J.S.tgt_failed[t]) return;
  const ColCov v = cov[g];
  const double u1 = (double)v.uniq_bot + (double)v.uniq_top;
  const double r1 = v.red_bot + v.red_top;
  const double total = (double)((int)rint(u1) + (int)rint(r1));
  const bool interesting = !(call[g].flags & kBasePredicted) || u1 <= J.prop[t] || total <= J.seed[t];
  if (!interesting) return;
  keep[g] = 1;
  if (c > tpoff[t]) keep[g - 1] = 1;
  if (c + 1 < tpoff[t + 1] - 1) keep[g + 1] = 1;
}

__global__ void flag_count_kernel(const uint8_t* keep, uint32_t n, uint32_t* block_counts) {
  __shared__ uint32_t s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = i < n && keep[i];
  const uint32_t b = __popc(__ballot_sync(0xFFFFFFFFu, f));
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(&s, b);
  __syncthreads();
  if (threadIdx.x == 0) block_counts[blockIdx.x] = s;
}

// scatter the kept columns in column order, with their coverage and call
__global__ void flag_gather_kernel(const uint8_t* keep, uint32_t n, const uint32_t* block_offsets, const ColCov* cov,
                                   const ColCall* call, uint32_t* out_col, ColCov* out_cov, ColCall* out_call) {
  __shared__ uint32_t warp_base[32];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = i < n && keep[i];
  const unsigned m = __ballot_sync(0xFFFFFFFFu, f);
  if ((threadIdx.x & 31) == 0) warp_base[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); w++) { const uint32_t x = warp_base[w]; warp_base[w] = acc; acc += x; }
  }
  __syncthreads();
  if (f) {
    const uint32_t o = block_offsets[blockIdx.x] + warp_base[threadIdx.x >> 5] + __popc(m & ((1u << (threadIdx.x & 31)) - 1));
    out_col[o] = i;
    out_cov[o] = cov[i];
    out_call[o] = call[i];
  }
}

// One warp per candidate column (persistent warps pulling from a work counter); the scoring itself is
// score_candidate_column (bsq_device.cuh).
__global__ void __launch_bounds__(128) im_candidate_kernel(const __grid_constant__ Batch B, CandArgs A, uint32_t hist_cap) {
  extern __shared__ uint32_t sh_hist[];
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint4* ents = A.scratch + (size_t)gw * cand_warp_stride(A.scratch_per_warp);
  const uint32_t n_cand = A.n_cand_dev[0] + A.n_cand_dev[1];
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(A.next, 1u);
    idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
    if (idx >= n_cand) break;
    const uint32_t g = A.cand[idx];
    const uint32_t job = job_of(B.col_begin, B.n_jobs, g);
    const uint32_t col0 = B.col_begin[job];
    const uint32_t c = g - col0;
    const DevJob& J = B.jobs[job];
    const DevSample& S = J.S;
    const ClassTable& T = J.T;
    uint32_t* hist = (T.K <= hist_cap) ? sh_hist + (threadIdx.x >> 5) * hist_cap : nullptr;
    CandOut out;
    out.ra = A.ra; out.n_ra = A.n_ra; out.ra_cap = A.ra_cap; out.qhist = A.qhist; out.Qhist = A.Qhist; out.err = A.err;
    out.base_quality_cutoff = J.I.base_quality_cutoff; out.log10_ref_len = J.I.log10_ref_len;
    out.mutation_cutoff = J.I.mutation_cutoff; out.poly_cutoff = J.I.poly_cutoff;
    out.precision_decimal = J.I.precision_decimal; out.col_offset = col0;
    out.bq = A.bq; out.n_bq = A.n_bq; out.bq_cap = A.bq_cap;
    out.pool = A.pool; out.pool_used = A.pool_used; out.pool_cap = A.pool_cap;
#pragma unroll
    for (int i = 0; i < 8; i++) out.dp_rg[i] = J.I.dp_rg[i];
    const ColCall cl0 = J.I.call[c];
    score_candidate_column(S, T, out, c, (cl0.flags & (kCandidate | kRecompute)) != 0, (cl0.flags & kRecompute) != 0,
                           cl0, J.I.call, ents, A.scratch_per_warp, hist);
    __syncwarp();
  }
}

// ============================================================================ deferred bounds
// One warp per bound job: the lower or upper bisection of one RA item, written into its record.
__global__ void __launch_bounds__(256) im_bounds_kernel(const __grid_constant__ Batch B, CandArgs A, unsigned int* next) {
  const int lane = threadIdx.x & 31;
  const uint32_t n_jobs = min(*A.n_bq, A.bq_cap);
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(next, 1u);
    idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
    if (idx >= n_jobs) break;
    // jobs are written in (lower, upper) pairs; take every lower bisection first, the longer ones
    // for consensus calls (their upper test at f = 1 passes at once)
    const uint32_t half = (n_jobs + 1) / 2;
    const BoundJob J = A.bq[idx < half ? 2 * idx : 2 * (idx - half) + 1];
    const uint32_t job = job_of(B.col_begin, B.n_jobs, J.col);
    const ClassTable& T = B.jobs[job].T;
    EmList L;
    L.e = A.pool + J.pool_off;
    L.m = J.m;
    const double v = J.side == 0 ? ra_lower_bound(L, T, J.full, J.var, J.fh, J.tol, J.target, J.maxsum, J.n)
                                 : ra_upper_bound(L, T, J.full, J.var, J.fh, J.tol, J.target, J.maxsum, J.n);
    if (lane == 0) {
      if (J.side == 0) A.ra[J.slot].lower = v; else A.ra[J.slot].upper = v;
    }
    __syncwarp();
  }
}

// ============================================================================ launch wrappers
static int grid_for(uint32_t work, int per_block, int sms, int min_blocks_per_sm) {
  long g = ((long)work + per_block - 1) / per_block;
  long cap = (long)sms * min_blocks_per_sm;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// Reference characters of the padded column space: every byte of a target is one of A/C/G/T/N and
// the only zero bytes are the one separator after each target.  Counts both kinds for the host and
// writes the 4-bit column codes the pass-1 kernel reads: column c at nibble c + 16 of `refnib` (16
// columns per 64-bit word, the lowest nibble first), A/C/G/T one-hot (1, 2, 4, 8, as BAM codes them),
// anything else 15.  Thread j writes word j.
__global__ void ref_check_kernel(const uint8_t* ref, unsigned long long* refnib, uint32_t n_cols, uint32_t n_words,
                                 uint32_t* bad, uint32_t* zeros) {
  uint32_t nb = 0, nz = 0;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_words; j += gridDim.x * blockDim.x) {
    unsigned long long word = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      const int64_t c = (int64_t)j * 16 + k - 16;
      uint32_t nib = 15;
      if (c >= 0 && c < (int64_t)n_cols) {
        const uint8_t ch = __ldg(ref + c);
        nz += ch == 0;
        nib = ch == 'A' ? 1 : ch == 'C' ? 2 : ch == 'G' ? 4 : ch == 'T' ? 8 : 15;
        nb += !(nib != 15 || ch == 'N' || ch == 0);
      }
      word |= (unsigned long long)nib << (4 * k);
    }
    refnib[j] = word;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nb += __shfl_xor_sync(0xFFFFFFFFu, nb, o);
    nz += __shfl_xor_sync(0xFFFFFFFFu, nz, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nb) atomicAdd(bad, nb);
    if (nz) atomicAdd(zeros, nz);
  }
}
// The per-call parameters a pass stages in page-locked host memory, read straight from it by the SMs
// (the memory is mapped into the device's address space) rather than by a copy engine: a sample upload
// running on another stream keeps the copy engines busy for milliseconds, and a copy queued behind it
// would hold up the pass.  bytes is a multiple of 16 and both pointers are 16-byte aligned.
__global__ void __launch_bounds__(256) host_copy_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, uint64_t n16) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
cudaError_t launch_host_copy(const void* src, void* dst, size_t bytes, int sms, cudaStream_t st) {
  const uint64_t n16 = bytes / 16;
  if (n16 == 0) return cudaSuccess;
  host_copy_kernel<<<grid_for((uint32_t)std::min<uint64_t>(n16, 1u << 30), 256, sms, 4), 256, 0, st>>>(
      static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16);
  return cudaGetLastError();
}

// The class bytes of a sample (class_bytes4, four bases in the bytes of a word).  flags[1] = the
// largest quality of a base that is not N; flags[0] = 1 when it is above kCodeMaxQ (an A/C/G/T byte
// may then not be exact: the passes keep the packed form for the sample).  Sixteen bases a
// thread, read as one 16-byte quality word and one 8-byte word of packed bases (both arrays carry 16
// bytes of slack past their ends, so the last word never leaves them).
__global__ void __launch_bounds__(256) base_code_kernel(const uint8_t* __restrict__ seq, const uint8_t* __restrict__ qual,
                                                        uint64_t n_bases, uint8_t* __restrict__ code, uint32_t* flags) {
  uint32_t mx = 0;                                       // per-byte maximum of the A/C/G/T qualities
  const uint64_t words = (n_bases + 15) / 16;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < words; w += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 q4 = __ldg(reinterpret_cast<const uint4*>(qual) + w);
    const uint2 s2 = __ldg(reinterpret_cast<const uint2*>(seq) + w);
    const uint32_t qw[4] = {q4.x, q4.y, q4.z, q4.w}, sw[2] = {s2.x, s2.y};
    const uint64_t live = n_bases - w * 16;              // bases of this word inside the array (may be > 16)
    uint32_t out[4];
#pragma unroll
    for (int g = 0; g < 4; g++) {
      uint32_t vq;
      out[g] = class_bytes4(qw[g], (sw[g >> 1] >> (16 * (g & 1))) & 0xFFFFu, &vq);
      if (live < 4u * g + 4u) {                          // the array ends inside these four bases
        const uint32_t lv = live > 4u * g ? (uint32_t)(live - 4u * g) : 0u;
        vq &= (1u << (8 * lv)) - 1u;
      }
      mx = bc_max4(mx, vq);
    }
    reinterpret_cast<uint4*>(code)[w] = make_uint4(out[0], out[1], out[2], out[3]);
  }
  uint32_t maxq = max(max(mx & 0xFFu, (mx >> 8) & 0xFFu), max((mx >> 16) & 0xFFu, mx >> 24));
  maxq = __reduce_max_sync(0xFFFFFFFFu, maxq);
  if ((threadIdx.x & 31) == 0 && maxq) {
    atomicMax(flags + 1, maxq);
    if (maxq > kCodeMaxQ) atomicOr(flags, 1u);
  }
}
cudaError_t launch_base_code(const uint8_t* seq, const uint8_t* qual, uint64_t n_bases, uint8_t* code, uint32_t* flags,
                             int sms, cudaStream_t st) {
  const uint64_t words = (n_bases + 15) / 16;
  if (words == 0) return cudaSuccess;
  base_code_kernel<<<grid_for((uint32_t)std::min<uint64_t>(words, 1u << 30), 256, sms, 4), 256, 0, st>>>(
      seq, qual, n_bases, code, flags);
  return cudaGetLastError();
}

cudaError_t launch_ref_check(const uint8_t* ref, unsigned long long* refnib, uint32_t n_cols, uint32_t* bad,
                             uint32_t* zeros, int sms, cudaStream_t st) {
  ref_check_kernel<<<sms * 4, 256, 0, st>>>(ref, refnib, n_cols, refnib_words(n_cols), bad, zeros);
  return cudaGetLastError();
}
cudaError_t launch_pack(const RawSoA& in, const PackOut& out, cudaStream_t st) {
  if (in.n == 0) return cudaSuccess;
  pack_reads_kernel<<<(in.n + 255) / 256, 256, 0, st>>>(in, out);
  return cudaGetLastError();
}
cudaError_t launch_mapq_index(DevRead* reads, const uint8_t* mapq, const uint8_t* map, uint32_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  mapq_index_kernel<<<(n + 255) / 256, 256, 0, st>>>(reads, mapq, map, n);
  return cudaGetLastError();
}
cudaError_t launch_tile_range(const uint32_t* rstart, uint32_t n_reads, uint32_t n_tiles, uint32_t maxspan,
                              uint2* tile_range, uint32_t* max_tile_reads, cudaStream_t st) {
  tile_range_kernel<<<(n_tiles + 255) / 256, 256, 0, st>>>(rstart, n_reads, n_tiles, maxspan, tile_range, max_tile_reads);
  return cudaGetLastError();
}
cudaError_t launch_tile_heavy(const uint2* tile_range, uint32_t n_tiles, uint32_t thr, uint32_t* heavy,
                              uint32_t* heavy_bits, uint32_t* n_heavy, cudaStream_t st) {
  if (n_tiles == 0) return cudaSuccess;
  tile_heavy_kernel<<<(n_tiles + 255) / 256, 256, 0, st>>>(tile_range, n_tiles, thr, heavy, heavy_bits, n_heavy);
  return cudaGetLastError();
}
// An event recorded inside a stream capture becomes an event node only with the external flag.
static cudaError_t record_event(cudaEvent_t ev, cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
    return cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
  return cudaEventRecord(ev, st);
}

int ec_grid(uint32_t n_chunks, int sms, uint32_t blocks_per_sm) {
  return grid_for(n_chunks, 1, sms, (int)std::max<uint32_t>(1, blocks_per_sm));
}
int column_grid(uint32_t total_tiles, int sms, uint32_t blocks_per_sm) {
  return grid_for(total_tiles, kColumnWarps, sms, (int)std::max<uint32_t>(1, blocks_per_sm));
}
// Shared memory of the pass-1 kernel: the R x 25 x Q histogram, the R x 4 x Q combined counts and,
// for jobs with class bytes, 512 x R class-byte counters (max_code_r: the largest such R, else 0).
static size_t ec_smem(uint32_t max_bins, uint32_t max_code_r) {
  return (size_t)(max_bins + max_bins / 25 * 4 + 512u * max_code_r) * sizeof(uint32_t);
}
cudaError_t prepare_ec(uint32_t max_bins, uint32_t max_code_r) {
  const size_t smem = ec_smem(max_bins, max_code_r);
  if (smem <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(ec_read_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
cudaError_t launch_ec(const Batch& B, const uint4* chunks, uint32_t n_chunks, unsigned int* next, uint32_t max_bins,
                      uint32_t max_code_r, int grid, cudaStream_t st, cudaEvent_t main0, cudaEvent_t main1) {
  const size_t smem = ec_smem(max_bins, max_code_r);
  cudaError_t e = cudaMemsetAsync(next, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  if (main0 && (e = record_event(main0, st)) != cudaSuccess) return e;
  ec_read_kernel<<<grid, 256, smem, st>>>(B, chunks, n_chunks, next);
  if (main1 && (e = record_event(main1, st)) != cudaSuccess) return e;
  cov_blocksum_kernel<<<std::max<uint32_t>(1, B.total_cblk), 1024, 0, st>>>(B);
  scan_jobs_kernel<<<B.n_jobs, 1024, 0, st>>>(B);
  cov_hist_kernel<<<std::max<uint32_t>(1, B.total_cblk), 1024, 0, st>>>(B);
  return cudaGetLastError();
}
cudaError_t launch_im_column(const Batch& B, int precision, int grid, cudaStream_t st) {
  const size_t smem = kColumnWarps * 32 * sizeof(DevRead) + kColRareBytes + kColWeightBytes;
  if (precision == 0) im_column_kernel<true><<<grid, 32 * kColumnWarps, smem, st>>>(B);
  else im_column_kernel<false><<<grid, 32 * kColumnWarps, smem, st>>>(B);
  return cudaGetLastError();
}
cudaError_t launch_compact(const ColCall* call, uint32_t n, uint32_t* block_counts, uint32_t* total, uint32_t* out,
                           cudaStream_t st) {
  const uint32_t nb = (n + 255) / 256;
  for (int part = 0; part < 2; part++) {
    cand_count_kernel<<<nb, 256, 0, st>>>(call, n, block_counts, part);
    scan_kernel<<<1, 1024, 0, st>>>(block_counts, nb, total + part);
    cand_scatter_kernel<<<nb, 256, 0, st>>>(call, n, block_counts, out, part, part ? total : nullptr);
  }
  return cudaGetLastError();
}
cudaError_t launch_intervals(const Batch& B, const ColCov* cov, const ColCall* call, uint8_t* keep, uint32_t* block_counts,
                             uint32_t* total, uint32_t* out_col, ColCov* out_cov, ColCall* out_call, cudaStream_t st) {
  const uint32_t n = B.total_cols;
  const uint32_t nb = (n + 255) / 256;
  cudaError_t e = cudaMemsetAsync(keep, 0, n, st);
  if (e != cudaSuccess) return e;
  interval_mark_kernel<<<nb, 256, 0, st>>>(B, cov, call, keep);
  flag_count_kernel<<<nb, 256, 0, st>>>(keep, n, block_counts);
  scan_kernel<<<1, 1024, 0, st>>>(block_counts, nb, total);
  flag_gather_kernel<<<nb, 256, 0, st>>>(keep, n, block_counts, cov, call, out_col, out_cov, out_call);
  return cudaGetLastError();
}

cudaError_t launch_candidates(const Batch& B, const CandArgs& A, uint32_t max_K, int n_warps, cudaStream_t st) {
  // each job compresses by class when its own K fits, so a job's summation order (and its
  // results) do not depend on the other jobs of the batch
  const uint32_t hist_cap = max_K < kEmHistMax ? max_K : kEmHistMax;
  const size_t smem = (size_t)4 * hist_cap * sizeof(uint32_t);
  cudaError_t e = cudaMemsetAsync(A.next, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  im_candidate_kernel<<<(n_warps + 3) / 4, 128, smem, st>>>(B, A, hist_cap);
  return cudaGetLastError();
}
cudaError_t launch_bounds(const Batch& B, const CandArgs& A, unsigned int* next, int sms, uint32_t warps_per_sm,
                          cudaStream_t st) {
  if (A.bq == nullptr) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(next, 0, sizeof(unsigned int), st);
  if (e != cudaSuccess) return e;
  // one block per SM: a few bisections share an SM's FP64 pipe and the SMs pull jobs as they free up
  const uint32_t w = std::min<uint32_t>(8, std::max<uint32_t>(1, warps_per_sm));
  im_bounds_kernel<<<sms, 32 * w, 0, st>>>(B, A, next);
  return cudaGetLastError();
}

}  // namespace bsq
