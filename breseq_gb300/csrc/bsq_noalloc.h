// Launch interface of the no-allocation scoring variant (bsq_noalloc.cu), used by bsq_abi.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/breseq_gb300.h"
#include "bsq_common.h"

namespace bsq {

constexpr uint32_t kNoAllocMaxClasses = 32768;       // likelihood classes (MAPQ values x R x 2 x Q x 5)
constexpr uint32_t kNoAllocMaxTable = 32768;         // R * 25 * Q error-table entries
constexpr uint64_t kNoAllocGatherEntries = (16u << 20) / 16;   // uint4 gather entries shared by all warps
constexpr uint32_t kNoAllocMaxTargets = 32768;       // deletion propagation cutoffs kept in the scratch

struct NoAllocJob {
  const double* log10_table;    // host
  uint32_t R, Q;
  const uint8_t* mapq_values;   // host, n_mapq distinct values of the sample
  uint32_t n_mapq;
  const uint32_t* tid;          // device, caller's
  const uint32_t* pos0;         // device, caller's
  uint32_t n_positions;
  const double* prop_cutoff;    // host, caller's: per target deletion propagation cutoff (< 0: fit failed)
  uint32_t n_targets;
  uint32_t dp_rg[8];            // discordant-pair read groups (ImArgs::dp_rg)
  bsq_ra_raw* ra;               // device, caller's
  uint32_t ra_cap;
  unsigned int* n_ra;           // device, caller's
  uint32_t* qhist;              // device, caller's [ra_cap][2][Q]
  uint32_t base_quality_cutoff;
  double log10_ref_len, mutation_cutoff, poly_cutoff, precision_decimal;
  uint32_t per_warp, n_warps;
};

// Device address of the fixed scratch array on `device` (which must be current); fetched with
// cudaGetSymbolAddress on the first call for that device.
cudaError_t noalloc_scratch_setup(int device, void** addr);
// Class table + scoring of the requested positions; synchronizes `st` and returns the error word.
cudaError_t launch_noalloc_positions(void* scratch, const DevSample& S, const NoAllocJob& J, cudaStream_t st,
                                     uint32_t* err_host);

}  // namespace bsq
