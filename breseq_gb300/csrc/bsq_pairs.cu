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
    if (a.mem) a.mem[i] = mem;
  }
}

__global__ void __launch_bounds__(256) pair_scatter_kernel(PairArgs a, const uint64_t* ev_off, const uint64_t* mem_off,
                                                           PairEvent* ev, char* names, uint32_t* mem_start,
                                                           uint16_t* mem_key) {
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
    if (a.mem && a.mem[i]) {
      const uint64_t m = mem_off[i];
      mem_start[m] = a.reads[i].start;
      mem_key[m] = (uint16_t)(a.group[i] * 2 + ((a.code[i] & kPairRev) ? 1 : 0));
    }
  }
}

}  // namespace

cudaError_t pair_classify(const PairArgs& a, int sms, cudaStream_t st) {
  if (a.n) pair_classify_kernel<<<grid_of(a.n, sms), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t pair_scatter(const PairArgs& a, const uint64_t* ev_off, const uint64_t* mem_off, PairEvent* ev, char* names,
                         uint32_t* mem_start, uint16_t* mem_key, int sms, cudaStream_t st) {
  if (a.n) pair_scatter_kernel<<<grid_of(a.n, sms), 256, 0, st>>>(a, ev_off, mem_off, ev, names, mem_start, mem_key);
  return cudaGetLastError();
}

}  // namespace bsq
