// BAM input on the device: BGZF inflate (bsq_inflate.cuh) and BAM record decode into the bsq_read_soa
// layout (SAM/BAM specification §4.2), as htslib does it for breseq on the host
// (src/breseq/pileup_base.cpp:61-88, 232-235; tag accessors src/breseq/alignment.cpp:52-80).
// Every read of the inflated stream is checked against the record's and the block's bounds.
#include "bsq_bam.h"

#include <algorithm>

#include "bsq_inflate.cuh"

namespace bsq {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kTokPerBlock = 65536;   // token room per block (a token is at least one byte)

int grid_for(uint64_t units, uint32_t per_block, int sms, int per_sm) {
  const uint64_t need = (units + per_block - 1) / per_block;
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)sms * per_sm));
}

__device__ __forceinline__ uint32_t rd16(const uint8_t* p) { return p[0] | ((uint32_t)p[1] << 8); }
__device__ __forceinline__ uint32_t rd32(const uint8_t* p) {
  return p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// Phase 1 of the two-phase inflate: one thread per block decodes its Huffman symbols into tokens
// (tok_step), with its tables in shared memory.  Every lane runs every iteration of the loop (a lane
// without a block idles in kLaneDone) and the warp reconverges after each step, so the 32 lanes' steps
// run side by side.  A failing block's token count is kTokBad.
constexpr int kLaneThreads = 32;
constexpr uint32_t kTokBad = 0xFFFFFFFFu;
__global__ void __launch_bounds__(kLaneThreads) bgzf_tok_kernel(const uint8_t* file, const BgzfBlock* blocks,
                                                                uint32_t b_lo, uint32_t b_hi, uint32_t* tok,
                                                                uint32_t* ntok, uint32_t* err, uint32_t* first_bad) {
  extern __shared__ __align__(16) unsigned char lane_smem[];
  // the threads' token stages, then their tables
  uint32_t* stage = reinterpret_cast<uint32_t*>(lane_smem) + threadIdx.x * inflate::kTokStage;
  inflate::LaneTables& T =
      reinterpret_cast<inflate::LaneTables*>(lane_smem + kLaneThreads * inflate::kTokStage * 4)[threadIdx.x];
  for (uint32_t b0 = b_lo + blockIdx.x * blockDim.x; b0 < b_hi; b0 += gridDim.x * blockDim.x) {
    const uint32_t b = b0 + threadIdx.x;
    inflate::TokState z;
    if (b < b_hi) {
      const BgzfBlock B = blocks[b];
      inflate::tok_start(z, file + B.in_off, B.in_len, tok + (size_t)(b - b_lo) * kTokPerBlock, stage, B.isize);
    } else {
      z.mode = inflate::kLaneDone;
      z.err = inflate::kOk;
    }
    while (__any_sync(kFull, z.mode != inflate::kLaneDone)) {
      inflate::tok_step(z, T);
      __syncwarp();
    }
    if (b < b_hi) {
      inflate::tok_finish(z);
      ntok[b - b_lo] = z.err ? kTokBad : z.n;
      if (z.err) {
        atomicOr(err, kBamInflate);
        atomicMin(first_bad, b);
      }
    }
  }
}

// Phase 2: one warp per block turns its tokens into bytes.  32 tokens at a time: their lengths are
// scanned into output positions, the literals written at once, then each copy by all 32 lanes in
// order (a source byte is always before the copy's own bytes; an overlapping copy repeats its first
// d bytes), the warp synchronising between writes and the reads that may see them.
__global__ void __launch_bounds__(256) bgzf_resolve_kernel(const BgzfBlock* blocks, uint32_t b_lo, uint32_t b_hi,
                                                           const uint32_t* tok, const uint32_t* ntok, uint8_t* out) {
  const int lane = threadIdx.x & 31;
  for (uint32_t b = b_lo + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); b < b_hi;
       b += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t nt = ntok[b - b_lo];
    if (nt == kTokBad) continue;
    const BgzfBlock B = blocks[b];
    const uint32_t* tk = tok + (size_t)(b - b_lo) * kTokPerBlock;
    uint8_t* o = out + B.out_off;
    uint32_t pos = 0;
    for (uint32_t c = 0; c < nt; c += 32) {
      const bool act = c + lane < nt;
      const uint32_t t = act ? tk[c + lane] : 0u;
      const uint32_t d = t & 0xFFFFu, x = t >> 16;
      const uint32_t len = act ? (d ? x + 3u : 1u) : 0u;
      uint32_t incl = len;
#pragma unroll
      for (int k = 1; k < 32; k <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, k);
        if (lane >= k) incl += y;
      }
      const uint32_t start = pos + incl - len;
      if (act && d == 0) o[start] = (uint8_t)x;
      __syncwarp();
      unsigned m = __ballot_sync(kFull, act && d != 0);
      while (m) {
        const int j = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t dj = __shfl_sync(kFull, d, j), lj = __shfl_sync(kFull, len, j), sj = __shfl_sync(kFull, start, j);
        for (uint32_t i = lane; i < lj; i += 32) o[sj + i] = o[sj - dj + (i < dj ? i : i % dj)];
        __syncwarp();
      }
      pos += __shfl_sync(kFull, incl, 31);
    }
  }
}

// The CRC-32 of every inflated block against its trailer, one warp per block: each lane takes the CRC
// of a 1/32 slice, and the slices are combined in order.
__global__ void __launch_bounds__(256) bgzf_crc_kernel(const uint8_t* out, const BgzfBlock* blocks, uint32_t n,
                                                       uint32_t* err, uint32_t* first_bad) {
  __shared__ uint32_t crc_table[256];
  for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) {
    uint32_t c = i;
    for (int k = 0; k < 8; k++) c = (c & 1) ? inflate::kCrcPoly ^ (c >> 1) : c >> 1;
    crc_table[i] = c;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < n; b += (gridDim.x * blockDim.x) >> 5) {
    const BgzfBlock B = blocks[b];
    const uint8_t* o = out + B.out_off;
    const uint32_t slice = (B.isize + 31) / 32;
    const uint32_t a0 = min(B.isize, lane * slice), a1 = min(B.isize, a0 + slice);
    uint32_t c = 0xFFFFFFFFu;
    for (uint32_t k = a0; k < a1; k++) c = crc_table[(c ^ __ldg(o + k)) & 0xFF] ^ (c >> 8);
    c ^= 0xFFFFFFFFu;
    uint32_t total = __shfl_sync(kFull, c, 0);
    const uint32_t shift_full = inflate::gf2_x8n(slice);
    for (int j = 1; j < 32; j++) {
      const uint32_t cj = __shfl_sync(kFull, c, j);
      const uint32_t bj0 = min(B.isize, (uint32_t)j * slice), bj1 = min(B.isize, bj0 + slice);
      const uint32_t lj = bj1 - bj0;
      if (lj == 0) continue;
      total = inflate::gf2_mulmod(lj == slice ? shift_full : inflate::gf2_x8n(lj), total) ^ cj;
    }
    if (lane == 0 && total != B.crc) {
      atomicOr(err, kBamCrc);
      atomicMin(first_bad, b);
    }
  }
}

// One thread per block: the records of the block, from max(block start, records_begin); each record
// must end inside the block and the last at its end.
__global__ void __launch_bounds__(128) bam_walk_kernel(const uint8_t* stream, const BgzfBlock* blocks, uint32_t n,
                                                       uint64_t records_begin, uint32_t* counts, const uint64_t* base,
                                                       uint64_t* offsets, uint32_t* err) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const uint64_t s = blocks[b].out_off, e = s + blocks[b].isize;
  uint64_t p = s > records_begin ? s : records_begin;
  uint32_t k = 0;
  while (p < e) {
    if (p + 4 > e) { atomicOr(err, kBamSpan); break; }
    const int32_t bs = (int32_t)rd32(stream + p);
    if (bs < 32 || p + 4 + (uint64_t)bs > e) { atomicOr(err, kBamSpan); break; }
    if (offsets) offsets[base[b] + k] = p;
    k++;
    p += 4 + (uint64_t)bs;
  }
  if (!offsets) counts[b] = k;
}

// The fields of a record the decode needs, with its variable parts located.
struct RecordView {
  uint64_t off, end;               // record start (block_size field) and end
  int32_t ref_id, pos, l_seq;
  uint32_t l_read_name, mapq, n_cigar, flag;
  uint64_t cigar, seq, qual, aux;  // stream offsets
  bool ok;
};

__device__ __forceinline__ RecordView view_record(const uint8_t* stream, uint64_t off) {
  RecordView v;
  const uint8_t* p = stream + off;
  v.off = off;
  v.end = off + 4 + (uint64_t)(int32_t)rd32(p);   // block_size >= 32, checked by the walk
  v.ref_id = (int32_t)rd32(p + 4);
  v.pos = (int32_t)rd32(p + 8);
  v.l_read_name = p[12];
  v.mapq = p[13];
  v.n_cigar = rd16(p + 16);
  v.flag = rd16(p + 18);
  v.l_seq = (int32_t)rd32(p + 20);
  v.cigar = off + 36 + v.l_read_name;
  v.seq = v.cigar + 4ull * v.n_cigar;
  const uint64_t ls = v.l_seq < 0 ? 0 : (uint64_t)v.l_seq;
  v.qual = v.seq + (ls + 1) / 2;
  v.aux = v.qual + ls;
  v.ok = v.l_read_name >= 1 && v.l_seq >= 0 && v.aux <= v.end;
  return v;
}

// Integer value of an aux field of type t at p (bam_aux2i: c C s S i I; any other type gives 0).
__device__ __forceinline__ int64_t aux_int(const uint8_t* p, uint8_t t) {
  switch (t) {
    case 'c': return (int8_t)p[0];
    case 'C': return p[0];
    case 's': return (int16_t)rd16(p);
    case 'S': return rd16(p);
    case 'i': return (int32_t)rd32(p);
    case 'I': return rd32(p);
    default: return 0;
  }
}

// Size of an aux value of type t at p within [p, end); -1 when malformed.
__device__ __forceinline__ int64_t aux_size(const uint8_t* p, const uint8_t* end, uint8_t t) {
  switch (t) {
    case 'A': case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    case 'Z': case 'H': {
      for (const uint8_t* q = p; q < end; q++) if (*q == 0) return q - p + 1;
      return -1;
    }
    case 'B': {
      if (end - p < 5) return -1;
      const uint8_t sub = p[0];
      const uint64_t count = rd32(p + 1);
      int es = 0;
      switch (sub) {
        case 'c': case 'C': es = 1; break;
        case 's': case 'S': es = 2; break;
        case 'i': case 'I': case 'f': es = 4; break;
        default: return -1;
      }
      return 5 + (int64_t)(count * es);
    }
    default: return -1;
  }
}

// One thread per record: fixed fields, then the aux fields breseq reads (the first field with each
// tag, as bam_aux_get finds it): X1 (redundancy, 1 when absent), XL / XR (trims, -1 when absent),
// XJ (present or not), RG (read group index: read_group_index_map::index, alignment.h:544-560) and
// the read file of (group, mate) (read_file_partition::index, :580-589).
__global__ void __launch_bounds__(256) bam_fields_kernel(const uint8_t* stream, const uint64_t* offsets, uint64_t n,
                                                         uint32_t n_ref, const __grid_constant__ BamGroups G,
                                                         const char* ids, BamRecordsDev R, uint32_t* ncig32,
                                                         uint32_t* nib, uint32_t* nlen, uint32_t* err) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const RecordView v = view_record(stream, offsets[i]);
    uint32_t e = 0;
    if (!v.ok || v.ref_id < -1 || v.ref_id >= (int32_t)n_ref) e |= kBamRecord;
    int64_t x1 = 1, xl = -1, xr = -1;
    bool has_x1 = false, has_xl = false, has_xr = false, has_xj = false, has_rg = false, has_xp = false;
    uint32_t group = 0, xp = 3;   // BSQ_XP_NONE
    if (v.ok) {
      const uint8_t* q = stream + v.aux;
      const uint8_t* end = stream + v.end;
      while (q < end) {
        if (end - q < 3) { e |= kBamAux; break; }
        const uint8_t t0 = q[0], t1 = q[1], type = q[2];
        q += 3;
        const int64_t sz = aux_size(q, end, type);
        if (sz < 0 || sz > end - q) { e |= kBamAux; break; }
        if (t0 == 'X' && t1 == '1' && !has_x1) { has_x1 = true; x1 = aux_int(q, type); }
        else if (t0 == 'X' && t1 == 'L' && !has_xl) { has_xl = true; xl = aux_int(q, type); }
        else if (t0 == 'X' && t1 == 'R' && !has_xr) { has_xr = true; xr = aux_int(q, type); }
        else if (t0 == 'X' && t1 == 'J') { has_xj = true; }
        else if (t0 == 'C' && t1 == 'G' && type == 'B' && q[0] == 'I') {
          // SAM specification §4.2.2: a CIGAR of more than 65535 operations is kept in CG:B:I, and the
          // record's own CIGAR is the placeholder <l_seq>S<reference length>N, which htslib replaces
          // when it reads the record.  The device record holds 65535 operations at most: refused.
          const uint32_t* cg = reinterpret_cast<const uint32_t*>(stream + v.cigar);
          if (v.n_cigar == 2 && rd32(reinterpret_cast<const uint8_t*>(cg)) == (((uint32_t)v.l_seq << 4) | 4u) &&
              (rd32(reinterpret_cast<const uint8_t*>(cg + 1)) & 0xFu) == 3u)
            e |= kBamLongCigar;
        }
        else if (t0 == 'X' && t1 == 'P' && !has_xp) {
          // the pair orientation breseq writes as XP:Z (FR, RF or FF); read as bam_aux2Z does
          has_xp = true;
          if ((type == 'Z' || type == 'H') && sz == 3 && q[2] == 0) {
            if (q[0] == 'F' && q[1] == 'R') xp = 0;
            else if (q[0] == 'R' && q[1] == 'F') xp = 1;
            else if (q[0] == 'F' && q[1] == 'F') xp = 2;
          }
        }
        else if (t0 == 'R' && t1 == 'G' && !has_rg) {
          has_rg = true;
          // bam_aux2Z: Z and H strings only; one group or none resolves to 0 without a lookup
          if ((type == 'Z' || type == 'H') && G.n > 1) {
            for (uint32_t g = 0; g < G.n; g++) {
              const uint32_t a = G.id_off[g], b = G.id_off[g + 1];
              if ((int64_t)(b - a) + 1 != sz) continue;
              bool same = true;
              for (uint32_t k = 0; k < b - a; k++) if ((uint8_t)ids[a + k] != q[k]) { same = false; break; }
              if (same) { group = g; break; }
            }
          }
        }
        q += sz;
      }
    }
    if (e) atomicOr(err, e);
    // unplaced records (refID -1) must all follow the placed ones: err[1] = first unplaced index,
    // err[2] = one past the last placed index
    const unsigned act = __activemask();
    const uint32_t un = __reduce_min_sync(act, v.ref_id < 0 ? (uint32_t)i : 0xFFFFFFFFu);
    const uint32_t pl = __reduce_max_sync(act, v.ref_id >= 0 ? (uint32_t)i + 1 : 0u);
    if ((threadIdx.x & 31) == __ffs(act) - 1) {
      if (un != 0xFFFFFFFFu) atomicMin(err + 1, un);
      if (pl) atomicMax(err + 2, pl);
    }
    R.tid[i] = v.ref_id;
    R.pos[i] = v.pos;
    R.flag[i] = (uint16_t)v.flag;
    R.mapq[i] = (uint8_t)v.mapq;
    R.x1[i] = (uint32_t)x1;
    R.xl[i] = (int32_t)xl;
    R.xr[i] = (int32_t)xr;
    R.xj[i] = has_xj ? 1 : 0;
    R.xp[i] = (uint8_t)xp;
    R.isize[i] = (int32_t)rd32(stream + offsets[i] + 32);   // TLEN: inside the 32 fixed bytes the walk checked
    R.mtid[i] = (int32_t)rd32(stream + offsets[i] + 24);    // RNEXT
    R.mpos[i] = (int32_t)rd32(stream + offsets[i] + 28);    // PNEXT
    R.read_group[i] = (uint16_t)group;
    uint32_t file = 0;
    if (G.n > 0 && group < G.n && G.file_count[group] > 0)
      file = G.file_base[group] + (((v.flag & 0x80) && G.file_count[group] > 1) ? 1u : 0u);
    R.read_file[i] = (uint8_t)file;
    const uint32_t ls = v.ok ? (uint32_t)v.l_seq : 0;
    R.l_qseq[i] = ls;
    R.n_cigar[i] = (uint16_t)(v.ok ? v.n_cigar : 0);
    ncig32[i] = v.ok ? v.n_cigar : 0;
    nib[i] = ls + (ls & 1);
    nlen[i] = v.ok ? v.l_read_name - 1 : 0;
  }
}

// One warp per record: CIGAR words, packed bases and qualities into the arrays.
__global__ void __launch_bounds__(256) bam_copy_kernel(const uint8_t* stream, const uint64_t* offsets, uint64_t n,
                                                       BamRecordsDev R) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t n_warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t i = warp0; i < n; i += n_warps) {
    const RecordView v = view_record(stream, offsets[i]);
    if (!v.ok) continue;
    uint32_t* cg = R.cigar + R.cigar_off[i];
    for (uint32_t j = lane; j < v.n_cigar; j += 32) cg[j] = rd32(stream + v.cigar + 4ull * j);
    const uint64_t so = R.seq_off[i];
    uint8_t* sq = R.seq + so / 2;
    const uint32_t nb = ((uint32_t)v.l_seq + 1) / 2;
    for (uint32_t j = lane; j < nb; j += 32) sq[j] = stream[v.seq + j];
    uint8_t* ql = R.qual + so;
    for (uint32_t j = lane; j < (uint32_t)v.l_seq; j += 32) ql[j] = stream[v.qual + j];
    if ((v.l_seq & 1) && lane == 0) ql[v.l_seq] = 0;   // the padding position of an odd-length read
    if (R.qname) {
      char* nm = R.qname + R.qoff[i];
      for (uint32_t j = lane; j + 1 < v.l_read_name; j += 32) nm[j] = (char)stream[v.off + 36 + j];
    }
  }
}

// Exclusive scan of 32-bit counts into 64-bit offsets: block sums of 1024 entries, one block scanning
// the sums, then the per-entry offsets.
__global__ void __launch_bounds__(256) scan_sums_kernel(const uint32_t* in, uint64_t n, uint64_t* sums) {
  __shared__ unsigned long long ws[8];
  const uint64_t i0 = (uint64_t)blockIdx.x * 1024 + threadIdx.x * 4;
  unsigned long long v = 0;
  for (int k = 0; k < 4; k++) if (i0 + k < n) v += in[i0 + k];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < 8; w++) t += ws[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) scan_top_kernel(uint64_t* sums, uint64_t nb, uint64_t* total) {
  __shared__ unsigned long long part[33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned long long carry = 0;
  for (uint64_t base = 0; base < nb; base += 1024) {
    const uint64_t i = base + threadIdx.x;
    const unsigned long long v = i < nb ? sums[i] : 0;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) part[w] = x;
    __syncthreads();
    if (w == 0) {
      const unsigned long long t = part[lane];
      unsigned long long s = t;
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(kFull, s, o);
        if (lane >= o) s += y;
      }
      part[lane] = s - t;
      if (lane == 31) part[32] = s;
    }
    __syncthreads();
    if (i < nb) sums[i] = carry + part[w] + x - v;
    carry += part[32];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(256) scan_apply_kernel(const uint32_t* in, uint64_t n, const uint64_t* sums,
                                                         uint64_t* out) {
  __shared__ unsigned long long ws[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t i0 = (uint64_t)blockIdx.x * 1024 + threadIdx.x * 4;
  uint32_t v[4];
  unsigned long long t = 0;
  for (int k = 0; k < 4; k++) { v[k] = i0 + k < n ? in[i0 + k] : 0; t += v[k]; }
  unsigned long long x = t;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  unsigned long long before = sums[blockIdx.x];
  for (int k = 0; k < w; k++) before += ws[k];
  before += x - t;
  for (int k = 0; k < 4; k++) {
    if (i0 + k < n) out[i0 + k] = before;
    before += v[k];
  }
}

}  // namespace

cudaError_t bam_inflate(const uint8_t* file, const BgzfBlock* blocks, uint32_t n_blocks, uint8_t* out, uint32_t* tok,
                        uint32_t* ntok, uint32_t tok_blocks, uint32_t* err, uint32_t* first_bad, int sms,
                        cudaStream_t st) {
  if (!n_blocks) return cudaSuccess;
  // 32 threads' token stages and tables per block of the token kernel: 3 blocks fit an SM's shared memory
  const size_t smem = kLaneThreads * (inflate::kTokStage * 4 + sizeof(inflate::LaneTables));
  cudaError_t e = cudaFuncSetAttribute(bgzf_tok_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // the blocks in groups of tok_blocks, the token room of one group
  for (uint32_t lo = 0; lo < n_blocks; lo += tok_blocks) {
    const uint32_t hi = std::min(n_blocks, lo + tok_blocks);
    bgzf_tok_kernel<<<grid_for(hi - lo, kLaneThreads, sms, 3), kLaneThreads, smem, st>>>(file, blocks, lo, hi, tok, ntok, err,
                                                                                        first_bad);
    bgzf_resolve_kernel<<<grid_for(hi - lo, 8, sms, 8), 256, 0, st>>>(blocks, lo, hi, tok, ntok, out);
  }
  bgzf_crc_kernel<<<grid_for(n_blocks, 8, sms, 8), 256, 0, st>>>(out, blocks, n_blocks, err, first_bad);
  return cudaGetLastError();
}
size_t bam_token_bytes(uint32_t tok_blocks) { return (size_t)tok_blocks * kTokPerBlock * 4 + (size_t)tok_blocks * 4; }

cudaError_t bam_walk(const uint8_t* stream, const BgzfBlock* blocks, uint32_t n_blocks, uint64_t records_begin,
                     uint32_t* counts, const uint64_t* base, uint64_t* offsets, uint32_t* err, int sms, cudaStream_t st) {
  (void)sms;
  if (n_blocks)
    bam_walk_kernel<<<(n_blocks + 127) / 128, 128, 0, st>>>(stream, blocks, n_blocks, records_begin, counts, base, offsets, err);
  return cudaGetLastError();
}

cudaError_t bam_fields(const uint8_t* stream, const uint64_t* offsets, uint64_t n, uint32_t n_ref, const BamGroups& groups,
                       const char* ids, const BamRecordsDev& R, uint32_t* ncig32, uint32_t* nib, uint32_t* nlen,
                       uint32_t* err, int sms, cudaStream_t st) {
  if (n) bam_fields_kernel<<<grid_for(n, 256, sms, 8), 256, 0, st>>>(stream, offsets, n, n_ref, groups, ids, R, ncig32, nib,
                                                                       nlen, err);
  return cudaGetLastError();
}

cudaError_t scan_u32(const uint32_t* in, uint64_t* out, uint64_t n, uint64_t* tmp, uint64_t* total, cudaStream_t st) {
  const uint64_t nb = (n + 1023) / 1024;
  if (nb) scan_sums_kernel<<<(unsigned)nb, 256, 0, st>>>(in, n, tmp);
  scan_top_kernel<<<1, 1024, 0, st>>>(tmp, nb, total);
  if (nb) scan_apply_kernel<<<(unsigned)nb, 256, 0, st>>>(in, n, tmp, out);
  return cudaGetLastError();
}

cudaError_t bam_copy(const uint8_t* stream, const uint64_t* offsets, uint64_t n, const BamRecordsDev& R, int sms,
                     cudaStream_t st) {
  if (n) bam_copy_kernel<<<grid_for(n * 32, 256, sms, 8), 256, 0, st>>>(stream, offsets, n, R);
  return cudaGetLastError();
}

}  // namespace bsq
