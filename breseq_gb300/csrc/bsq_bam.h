// BAM input on the device (bsq_bam.cu), used by bsq_abi.cu.
//
// breseq opens reference.bam through htslib (src/breseq/pileup_base.cpp:61-88, 232-235): BGZF
// blocks are inflated and the BAM records decoded on the host.  Here the file's bytes go to the
// device and:
//   1. every BGZF block is inflated by one warp (bsq_inflate.cuh): one lane decodes through a
//      shared-memory ring that the warp flushes, and the 32 lanes check its CRC-32;
//   2. one thread per block walks the records of its block (htslib's BAM writer starts a new block
//      rather than split a record, so every block after the header starts at a record) and counts
//      them; a second walk writes each record's offset;
//   3. one thread per record decodes the fixed fields and the X1 / XL / XR / XJ / RG tags, scans give
//      each record's CIGAR and base offsets, and one warp per record copies its CIGAR, bases and
//      qualities into the bsq_read_soa layout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bsq {

// One BGZF block: compressed payload [in_off, in_off + in_len) of the file, isize bytes of output at
// out_off of the inflated stream, and the CRC-32 of that output (SAM/BAM specification §4.1).
struct BgzfBlock {
  uint64_t in_off;
  uint64_t out_off;
  uint32_t in_len;
  uint32_t isize;
  uint32_t crc;
  uint32_t pad;
};

// error bits of the BAM path
enum : uint32_t { kBamInflate = 1, kBamCrc = 2, kBamSpan = 4, kBamRecord = 8, kBamAux = 16, kBamOrder = 32,
                  kBamLongCigar = 64 };

constexpr int kBamMaxGroups = 64;

// Read groups as breseq resolves them (src/breseq/alignment.h:533-607): IDs in header order, each
// group's first flat read-file index and file count.
struct BamGroups {
  uint32_t n;
  uint32_t id_off[kBamMaxGroups + 1];   // IDs concatenated in `ids`
  uint32_t file_base[kBamMaxGroups];
  uint32_t file_count[kBamMaxGroups];
};

// Device arrays of the decoded records, in the bsq_read_soa layout.
struct BamRecordsDev {
  int32_t* tid;
  int32_t* pos;
  uint16_t* flag;
  uint8_t* mapq;
  uint32_t* x1;
  int32_t* xl;
  int32_t* xr;
  uint8_t* read_file;
  uint16_t* read_group;
  uint32_t* l_qseq;
  uint64_t* seq_off;     // nibbles, even
  uint64_t* cigar_off;
  uint16_t* n_cigar;
  uint8_t* xj;
  uint32_t* cigar;
  uint8_t* seq;
  uint8_t* qual;
  int32_t* isize;        // TLEN
  uint8_t* xp;           // XP:Z orientation code (BSQ_XP_*)
  uint64_t* qoff;        // [n + 1] read-name offsets
  char* qname;           // names without terminators; null until their total is known
  int32_t* mtid;         // RNEXT
  int32_t* mpos;         // PNEXT
};

// Inflates every BGZF block into out (two phases: Huffman symbols to tokens, one thread per block;
// tokens to bytes, one warp per block; then the CRC-32s), tok_blocks blocks at a time through the
// token buffer tok (bam_token_bytes(tok_blocks) bytes, ntok at its end is the per-block token count).
cudaError_t bam_inflate(const uint8_t* file, const BgzfBlock* blocks, uint32_t n_blocks, uint8_t* out, uint32_t* tok,
                        uint32_t* ntok, uint32_t tok_blocks, uint32_t* err, uint32_t* first_bad, int sms,
                        cudaStream_t st);
size_t bam_token_bytes(uint32_t tok_blocks);
// Records per block (walk from max(block start, records_begin)); with offsets != null, a second walk
// writes each record's stream offset at offsets[base[b] + k].
cudaError_t bam_walk(const uint8_t* stream, const BgzfBlock* blocks, uint32_t n_blocks, uint64_t records_begin,
                     uint32_t* counts, const uint64_t* base, uint64_t* offsets, uint32_t* err, int sms, cudaStream_t st);
// Fixed fields and tags of each record, and the per-record counts the scans turn into offsets: CIGAR
// ops, nibbles (l_seq rounded up to even) and read-name bytes.  n_ref: references in the header.
// err[0] gets error bits, err[1] the first unplaced record (initialise to 0xFFFFFFFF), err[2] one past
// the last placed record (initialise to 0).
cudaError_t bam_fields(const uint8_t* stream, const uint64_t* offsets, uint64_t n, uint32_t n_ref, const BamGroups& groups,
                       const char* ids, const BamRecordsDev& R, uint32_t* ncig32, uint32_t* nib, uint32_t* nlen,
                       uint32_t* err, int sms, cudaStream_t st);
// Exclusive scan of n 32-bit counts into 64-bit offsets; total[0] gets the sum.  tmp holds
// 8 * (n / 1024 + 2) bytes.
cudaError_t scan_u32(const uint32_t* in, uint64_t* out, uint64_t n, uint64_t* tmp, uint64_t* total, cudaStream_t st);
// CIGAR words, bases, qualities and read names of every record into the arrays.
cudaError_t bam_copy(const uint8_t* stream, const uint64_t* offsets, uint64_t n, const BamRecordsDev& R, int sms,
                     cudaStream_t st);

}  // namespace bsq
