// No-allocation variant of the candidate-column scoring kernel (bsq_score_positions_noalloc).
//
// Some callers cannot call cudaMalloc while they run: a serving loop with jobs in flight on other
// streams (cudaMalloc / cudaFree may synchronize the whole device and stall them), or a host program
// that hands every byte of HBM to one pre-sized memory arena.  For them this file keeps the scratch
// the scoring kernel needs in one fixed, file-scope device array instead of cudaMalloc'd buffers:
//
//   g_noalloc_scratch, 20 MiB, held by every GPU that loads the library until the process exits:
//     [0, 16 MiB)            per-warp gather lists of covering reads (uint4 each)
//     [16 MiB, +2.75 MiB)    likelihood class table (lp[5], r[5], max per class; up to 32768 classes)
//     [.., +256 KiB)         log10 error table (up to 32768 entries)
//     [.., +256 KiB)         the caller's deletion propagation cutoffs (up to 32768 targets)
//     [.., +256 B)           work counter and error word
//
// Host code must not take the array's name as a device address: the address is fetched with
// cudaGetSymbolAddress once per device, with that device current, the first time the entry point runs
// on it.  Every call shares the array and finds the previous call's contents there; the counters are
// cleared at the start of each call, and calls that overlap on the GPU (two streams, two threads)
// race on it.
//
// The likelihood-class table is computed here on the device (CUDA's pow / log10, each within 2 ulp),
// while bsq_identify_mutations computes it on the host with the C library's: the scores of the two
// agree to ~1e-12, not bit for bit.
#include <cuda_runtime.h>

#include <atomic>

#include "bsq_common.h"
#include "bsq_device.cuh"
#include "bsq_noalloc.h"

namespace bsq {

static_assert(sizeof(bsq_ra_raw) == sizeof(RaDev), "bsq_ra_raw must mirror RaDev");

namespace {

constexpr size_t kGatherBytes = 16u << 20;
constexpr size_t kClassBytes = (size_t)kNoAllocMaxClasses * 11 * sizeof(double);
constexpr size_t kTableBytes = (size_t)kNoAllocMaxTable * sizeof(double);
constexpr size_t kCutOff = kGatherBytes + kClassBytes + kTableBytes;
constexpr size_t kCutBytes = (size_t)kNoAllocMaxTargets * sizeof(double);
constexpr size_t kCounterOff = kCutOff + kCutBytes;
constexpr size_t kNoAllocBytes = 20u << 20;
static_assert(kCounterOff + 256 <= kNoAllocBytes, "no-allocation scratch layout overflows its array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
// device address of g_noalloc_scratch, per device; several host threads may look it up at once
std::atomic<void*> g_scratch_addr[kMaxDevices];

struct NoAllocArgs {
  const uint32_t* tid;
  const uint32_t* pos0;
  uint32_t n;
  unsigned int* next;
  const double* prop_cutoff;  // per target deletion propagation cutoff: < 0, the coverage fit failed and
                              // no RA is scored there (identify_mutations.cpp:1317-1333)
  uint4* gather;
  uint32_t per_warp;
  uint32_t n_warps;           // warps that own a gather list; the launch may round up past it
};

struct ClassArgs {
  const double* log10_table;
  double* lp64;
  double* r64;
  double* lpmax64;
  uint32_t R, Q, M, K;
  uint8_t mapq[256];
};

// fill_read_base_likelihoods (identify_mutations.cpp:3359-3384) for one likelihood class
__global__ void noalloc_class_kernel(ClassArgs A) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.K) return;
  uint32_t t = k;
  const uint32_t obs = t % 5; t /= 5;
  const uint32_t q = t % A.Q; t /= A.Q;
  const uint32_t sb = t % 2; t /= 2;
  const uint32_t rs = t % A.R; t /= A.R;
  const uint32_t m = t;
  const double inc = pow(10.0, -(double)A.mapq[m] / 10.0);
  const double cor = 1.0 - inc;
  const bool top = sb == 0;
  const uint32_t oc = top ? obs : (obs < 4 ? 3 - obs : 4);
  double lp[5], mx = -DBL_MAX;
  for (uint32_t b = 0; b < 5; b++) {
    const uint32_t rb = top ? b : (b < 4 ? 3 - b : 4);
    double pr = cor * pow(10.0, A.log10_table[rs + A.R * (rb + 5 * (oc + 5 * q))]) + inc * 0.2;
    if (pr < 0.0) pr = 0.0;
    lp[b] = log10(pr);
    mx = fmax(mx, lp[b]);
  }
  for (uint32_t b = 0; b < 5; b++) {
    A.lp64[(size_t)k * 5 + b] = lp[b];
    A.r64[(size_t)k * 5 + b] = pow(10.0, lp[b] - mx);
  }
  A.lpmax64[k] = mx;
}

// One warp per requested position, persistent warps over the shared work counter.
__global__ void __launch_bounds__(128) noalloc_positions_kernel(DevSample S, ClassTable T, CandOut out, NoAllocArgs A) {
  extern __shared__ uint32_t sh_hist[];
  const int lane = threadIdx.x & 31;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gw >= A.n_warps) return;
  uint4* ents = A.gather + (size_t)gw * cand_warp_stride(A.per_warp);
  uint32_t* hist = (T.K <= kEmHistMax) ? sh_hist + (threadIdx.x >> 5) * T.K : nullptr;
  ColCall none;
  none.score = 0; none.n = 0; none.best = 5; none.flags = 0; none.pad[0] = none.pad[1] = 0;
  for (;;) {
    uint32_t idx = 0;
    if (lane == 0) idx = atomicAdd(A.next, 1u);
    idx = __shfl_sync(0xFFFFFFFFu, idx, 0);
    if (idx >= A.n) break;
    const uint32_t t = A.tid[idx], p0 = A.pos0[idx];
    if (t >= S.n_targets || p0 >= S.tpoff[t + 1] - S.tpoff[t] - 1) {
      if (lane == 0) atomicOr(out.err, kErrBounds);
      continue;
    }
    if (A.prop_cutoff[t] < 0.0) continue;
    score_candidate_column(S, T, out, S.tpoff[t] + p0, true, false, none, nullptr, ents, A.per_warp, hist);
    __syncwarp();
  }
}

}  // namespace

cudaError_t noalloc_scratch_setup(int device, void** addr) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  void* p = g_scratch_addr[device].load(std::memory_order_acquire);
  if (!p) {
    // two threads may both look it up; they store the same address
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device].store(p, std::memory_order_release);
  }
  *addr = p;
  return cudaSuccess;
}

cudaError_t launch_noalloc_positions(void* scratch, const DevSample& S, const NoAllocJob& J, cudaStream_t st,
                                     uint32_t* err_host) {
  unsigned char* base = static_cast<unsigned char*>(scratch);
  double* lp64 = reinterpret_cast<double*>(base + kGatherBytes);
  double* r64 = lp64 + (size_t)kNoAllocMaxClasses * 5;
  double* lpmax64 = r64 + (size_t)kNoAllocMaxClasses * 5;
  double* table = reinterpret_cast<double*>(base + kGatherBytes + kClassBytes);
  unsigned int* counters = reinterpret_cast<unsigned int*>(base + kCounterOff);   // [0] next, [1] err
  const size_t ntab = (size_t)J.R * 25 * J.Q;
  double* cut = reinterpret_cast<double*>(base + kCutOff);
  cudaError_t e = cudaMemcpyAsync(table, J.log10_table, ntab * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(cut, J.prop_cutoff, (size_t)J.n_targets * sizeof(double), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if ((e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned int), st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(J.n_ra, 0, sizeof(unsigned int), st)) != cudaSuccess) return e;
  ClassArgs CA;
  CA.log10_table = table; CA.lp64 = lp64; CA.r64 = r64; CA.lpmax64 = lpmax64;
  CA.R = J.R; CA.Q = J.Q; CA.M = J.n_mapq; CA.K = J.n_mapq * J.R * 2 * J.Q * 5;
  for (int i = 0; i < 256; i++) CA.mapq[i] = i < (int)J.n_mapq ? J.mapq_values[i] : 0;
  noalloc_class_kernel<<<(CA.K + 127) / 128, 128, 0, st>>>(CA);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  ClassTable T;
  T.lp64 = lp64; T.r64 = r64; T.lpmax64 = lpmax64; T.lp32 = nullptr; T.K = CA.K; T.R = J.R; T.Q = J.Q; T.n_mapq = J.n_mapq;
  CandOut out;
  out.ra = reinterpret_cast<RaDev*>(J.ra); out.n_ra = J.n_ra; out.ra_cap = J.ra_cap; out.qhist = J.qhist; out.Qhist = J.Q;
  out.err = counters + 1; out.base_quality_cutoff = J.base_quality_cutoff; out.log10_ref_len = J.log10_ref_len;
  out.mutation_cutoff = J.mutation_cutoff; out.poly_cutoff = J.poly_cutoff; out.precision_decimal = J.precision_decimal;
  out.col_offset = 0;
  out.bq = nullptr; out.n_bq = nullptr; out.bq_cap = 0;     // bounds inline: no extra device memory
  out.pool = nullptr; out.pool_used = nullptr; out.pool_cap = 0;
  for (int i = 0; i < 8; i++) out.dp_rg[i] = J.dp_rg[i];
  NoAllocArgs A;
  A.tid = J.tid; A.pos0 = J.pos0; A.n = J.n_positions; A.next = counters; A.prop_cutoff = cut;
  A.gather = reinterpret_cast<uint4*>(base); A.per_warp = J.per_warp; A.n_warps = J.n_warps;
  const uint32_t warps = J.n_warps;
  if (J.n_positions) {
    const size_t smem = (T.K <= kEmHistMax) ? (size_t)4 * T.K * sizeof(uint32_t) : 0;
    noalloc_positions_kernel<<<(warps + 3) / 4, 128, smem, st>>>(S, T, out, A);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if ((e = cudaMemcpyAsync(err_host, counters + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

}  // namespace bsq
