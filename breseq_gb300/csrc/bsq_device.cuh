// Device code shared by the scoring kernels (bsq_kernels.cu) and the no-allocation variant
// (bsq_noalloc.cu): pileup state of a read at a column, encodings, warp reductions, the FP64 EM of
// fit_allele_frequencies / profile_log10_likelihood, and the per-column candidate scoring.
#pragma once
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "bsq_common.h"

namespace bsq {
namespace {

__device__ __forceinline__ uint8_t nib_at(const uint8_t* seq, uint64_t nib) {
  uint8_t b = __ldg(seq + (nib >> 1));
  return (nib & 1) ? (b & 0xF) : (b >> 4);
}
// 4-bit BAM base -> index A,C,G,T = 0..3; N/others -> -1 (src/breseq/common.h:253-265)
__device__ __forceinline__ int bam_idx(uint8_t b) {
  return b == 1 ? 0 : b == 2 ? 1 : b == 4 ? 2 : b == 8 ? 3 : -1;
}
// reference char -> index, 'N' -> 5, other -> -1 (common.h:267-279)
__device__ __forceinline__ int chr_idx(uint8_t c) {
  return c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : c == 'T' ? 3 : c == 'N' ? 5 : -1;
}
__device__ __forceinline__ bool op_ref(uint32_t op) { return op == 0 || op == 2 || op == 3 || op == 7 || op == 8; }
__device__ __forceinline__ bool op_qm(uint32_t op) { return op == 0 || op == 7 || op == 8; }

struct Pile { int qpos; int indel; bool del; };

// htslib's per-column read state (bam_plp_auto / resolve_cigar2 semantics) for a CIGAR with more
// than a single aligned block; c must lie in [start, end).
__device__ bool resolve_cigar(const uint32_t* cig, int n, uint32_t start, uint32_t c, Pile& e) {
  uint32_t x = start;
  int y = 0;
  for (int k = 0; k < n; k++) {
    uint32_t w = __ldg(cig + k), op = w & 0xF, len = w >> 4;
    if (op_ref(op)) {
      if (c < x + len) {
        if (op_qm(op)) { e.qpos = y + (int)(c - x); e.del = false; }
        else { e.qpos = y; e.del = true; }
        e.indel = 0;
        if (c == x + len - 1 && k + 1 < n) {
          uint32_t w2 = __ldg(cig + k + 1), op2 = w2 & 0xF;
          if (op2 == 2 && op != 2) {
            int d = -(int)(w2 >> 4);
            for (int j = k + 2; j < n; j++) { uint32_t wj = __ldg(cig + j); if ((wj & 0xF) == 2) d -= (int)(wj >> 4); else break; }
            e.indel = d;
          } else if (op2 == 1) {
            int d = (int)(w2 >> 4);
            for (int j = k + 2; j < n; j++) {
              uint32_t wj = __ldg(cig + j), o = wj & 0xF;
              if (o == 1) d += (int)(wj >> 4); else if (o != 6) break;
            }
            e.indel = d;
          } else if (op2 == 6 && k + 2 < n) {
            int l3 = 0;
            for (int j = k + 2; j < n; j++) {
              uint32_t wj = __ldg(cig + j), o = wj & 0xF;
              if (o == 1) l3 += (int)(wj >> 4); else if (op_ref(o)) break;
            }
            if (l3 > 0) e.indel = l3;
          }
        }
        return true;
      }
      x += len;
      if (op_qm(op)) y += (int)len;
    } else if (op == 1 || op == 4) {
      y += (int)len;
    }
  }
  return false;
}

__device__ __forceinline__ void resolve(const DevSample& S, const DevRead& rd, uint32_t c, Pile& e) {
  if (rd.flags & kSimple) { e.qpos = (int)(c - rd.start) + rd.clip; e.indel = 0; e.del = false; }
  else if (!resolve_cigar(S.cigar + rd.cigar_off, rd.n_cigar, rd.start, c, e)) { e.qpos = 0; e.indel = 0; e.del = true; }
}

// pileup_wrapper::is_trimmed (src/breseq/alignment.h:389-411), unsigned arithmetic as there
__device__ __forceinline__ bool is_trimmed(const DevRead& rd, int qpos, bool past_base) {
  uint32_t qp1 = (uint32_t)(qpos + 1);
  if (rd.xl != kNoTag && qp1 <= rd.xl) return true;
  if (rd.xr != kNoTag) {
    uint32_t len = rd.len;
    if (len - qp1 + 1u <= rd.xr) return true;
    if (past_base && (len - qp1 == rd.xr)) return true;
  }
  return false;
}

__device__ __forceinline__ int query_end0(const DevSample& S, const DevRead& rd, uint32_t r) {
  return (rd.flags & kSimple) ? (int)rd.clip + (int)(rd.end - rd.start) - 1 : (int)S.qb[r].qe0;
}
__device__ __forceinline__ int query_start0(const DevSample& S, const DevRead& rd, uint32_t r) {
  return (rd.flags & kSimple) ? (int)rd.clip : (int)S.qb[r].qs0;
}
__device__ __forceinline__ int bounds_end0(const DevSample& S, const DevRead& rd, uint32_t r) {
  return (rd.flags & kSimple) ? (int)rd.clip + (int)(rd.end - rd.start) - 1 : (int)S.qb[r].qbe;
}

// Index j with prefix[j] <= g < prefix[j + 1] (prefix ascending, n + 1 entries).
// prefix lives in kernel-parameter space: plain loads, no __ldg
__device__ __forceinline__ uint32_t job_of(const uint32_t* prefix, uint32_t n, uint32_t g) {
  uint32_t lo = 0, hi = n;
  while (hi - lo > 1) { const uint32_t mid = (lo + hi) >> 1; if (prefix[mid] <= g) lo = mid; else hi = mid; }
  return lo;
}

__device__ __forceinline__ uint32_t target_of(const DevSample& S, uint32_t c) {
  uint32_t lo = 0, hi = S.n_targets;  // largest t with tpoff[t] <= c
  while (hi - lo > 1) { uint32_t mid = (lo + hi) >> 1; if (__ldg(S.tpoff + mid) <= c) lo = mid; else hi = mid; }
  return lo;
}

// ============================================================================ candidate scoring
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}
// Sums of five values over the warp, returned to every lane, with 8 FP64 adds per lane instead of
// the 25 of five butterflies: each exchange step halves the values a lane keeps (xor 16: 3 of 5,
// xor 8: 2 or 1, xor 4: 1), the last two steps add single values, and five shuffles broadcast the
// sums.  FP64 issue is the scarce resource of the EM on this part.
__device__ __forceinline__ void warp_sum5(const double in[5], double out[5]) {
  const int lane = threadIdx.x & 31;
  const bool hi = lane & 16, b3 = lane & 8, b2 = lane & 4;
  // xor 16: the low half keeps sums 0,1,2 and the high half 3,4
  const double k0 = (hi ? in[3] : in[0]) + __shfl_xor_sync(0xFFFFFFFFu, hi ? in[0] : in[3], 16);
  const double k1 = (hi ? in[4] : in[1]) + __shfl_xor_sync(0xFFFFFFFFu, hi ? in[1] : in[4], 16);
  const double k2 = (hi ? 0.0 : in[2]) + __shfl_xor_sync(0xFFFFFFFFu, hi ? in[2] : 0.0, 16);
  // xor 8: low/low keeps 0,1; low/high keeps 2; high/low keeps 3; high/high keeps 4
  const double m0 = (hi ? (b3 ? k1 : k0) : (b3 ? k2 : k0)) +
                    __shfl_xor_sync(0xFFFFFFFFu, hi ? (b3 ? k0 : k1) : (b3 ? k0 : k2), 8);
  const double m1 = ((!hi && !b3) ? k1 : 0.0) + __shfl_xor_sync(0xFFFFFFFFu, (!hi && b3) ? k1 : 0.0, 8);
  // xor 4: the lanes holding 0,1 split them; every other lane keeps its one value
  const bool pair = !hi && !b3;
  double u = (pair ? (b2 ? m1 : m0) : m0) + __shfl_xor_sync(0xFFFFFFFFu, pair ? (b2 ? m0 : m1) : m0, 4);
  u += __shfl_xor_sync(0xFFFFFFFFu, u, 2);
  u += __shfl_xor_sync(0xFFFFFFFFu, u, 1);
  out[0] = __shfl_sync(0xFFFFFFFFu, u, 0);
  out[1] = __shfl_sync(0xFFFFFFFFu, u, 4);
  out[2] = __shfl_sync(0xFFFFFFFFu, u, 8);
  out[3] = __shfl_sync(0xFFFFFFFFu, u, 16);
  out[4] = __shfl_sync(0xFFFFFFFFu, u, 24);
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  return v;
}
__device__ __forceinline__ uint32_t warp_sum_u(uint32_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Entries of the per-warp gather list (uint4): x = read index, y = qpos | (on_base_indel + 1) << 16,
// z = likelihood class for the current slot (0xFFFFFFFF = not scored), w = obs | q << 8 | strand << 16.
constexpr uint32_t kNoClass = 0xFFFFFFFFu;
// Likelihood classes up to this many get a per-warp shared-memory histogram, so the EM runs over
// distinct classes instead of reads.
constexpr uint32_t kEmHistMax = 2048;

// The slot's scored read bases as (likelihood class, multiplicity) pairs.  Reads of one class add
// identical terms to every sum of fit_allele_frequencies / profile_log10_likelihood
// (identify_mutations.cpp:3241-3318, 3094-3143), so each sum runs over distinct classes with weights.
struct EmList { const uint2* e; uint32_t m; };

// One E-step sweep: g[b] = sum_i r_i(b) / s_i (the gradient of ln L in f[b]) over allowed alleles;
// the E-step sums are sum_w[b] = f[b] g[b].  With `ll` the sweep also returns an FP32 estimate of
// sum_i log10 s_i (error well below 1e-3 for a few thousand reads).
__device__ __forceinline__ void em_class(const EmList& L, const ClassTable& T, const double f[5], uint32_t i,
                                         double a[5], float& lls, float& las, bool want_ll) {
  const uint2 e = L.e[i];
  const double cnt = (double)e.y;
  const double* r = T.r64 + (size_t)e.x * 5;
  double rv[5];
#pragma unroll
  for (int b = 0; b < 5; b++) rv[b] = __ldg(r + b);
  // f[b] is exactly 0 for an allele outside the allowed set, so the unmasked sum equals the masked one
  const double s = (f[0] * rv[0] + f[1] * rv[1]) + (f[2] * rv[2] + f[3] * rv[3]) + f[4] * rv[4];
  if (s > 0.0) {
    const double w = cnt / s;
#pragma unroll
    for (int b = 0; b < 5; b++) a[b] += rv[b] * w;
    if (want_ll) {
      const float lg = log10f((float)s);
      lls += (float)e.y * lg;
      las += (float)e.y * fabsf(lg);
    }
  } else {
    // the reference's fallback keeps sum_w = n exact: each read adds f[b] to sum_w[b], i.e. 1 to g[b]
#pragma unroll
    for (int b = 0; b < 5; b++) a[b] += cnt;
  }
}

__device__ void em_sweep(const EmList& L, const ClassTable& T, const double f[5], unsigned allowed, double g[5],
                         float* ll, float* la = nullptr) {
  // two classes per lane in flight: the FP64 chains of a class are short and latency-bound
  double a0[5] = {0, 0, 0, 0, 0}, a1[5] = {0, 0, 0, 0, 0};
  float l0 = 0.0f, l1 = 0.0f, m0 = 0.0f, m1 = 0.0f;
  const bool want = ll != nullptr;
  uint32_t i = threadIdx.x & 31;
  for (; i + 32 < L.m; i += 64) {
    em_class(L, T, f, i, a0, l0, m0, want);
    em_class(L, T, f, i + 32, a1, l1, m1, want);
  }
  if (i < L.m) em_class(L, T, f, i, a0, l0, m0, want);
  double a[5];
#pragma unroll
  for (int b = 0; b < 5; b++) a[b] = ((allowed >> b) & 1) ? a0[b] + a1[b] : 0.0;
  warp_sum5(a, g);
  if (ll) {
    float lls = l0 + l1, las = m0 + m1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lls += __shfl_xor_sync(0xFFFFFFFFu, lls, o);
      las += __shfl_xor_sync(0xFFFFFFFFu, las, o);
    }
    *ll = lls;
    if (la) *la = las;
  }
}

// A bound on |FP32 estimate - exact FP64 value| of sum_i cnt_i log10 s_i from one sweep: s_i rounded to
// float (2^-24 relative: 2.6e-8 absolute in log10), log10f (at most 2 ulp), the product with cnt_i
// (2^-24 relative) and the FP32 accumulation, a chain of at most m/64 + 1 adds per lane accumulator
// plus one join and five shuffle levels, each adding 2^-24 of the running magnitude, which never
// exceeds A = sum_i cnt_i |log10 s_i|.  Doubled, plus 1e-9 for the difference between this EM's FP64
// trajectory and the reference's.
__device__ __forceinline__ double ll_margin(uint32_t n, uint32_t m, float A) {
  const double chain = (double)(m / 64 + 8);
  return 2.0 * (3.0e-8 * (double)n + (2.5e-7 + chain * 6.0e-8) * (double)A) + 1e-9;
}

// sum_i (log10 s_i + max_i) in FP64 at frequencies f, as the reference accumulates its likelihood
__device__ double em_loglik(const EmList& L, const ClassTable& T, const double f[5], unsigned allowed) {
  double ll = 0;
  for (uint32_t i = threadIdx.x & 31; i < L.m; i += 32) {
    const uint2 e = L.e[i];
    const double* r = T.r64 + (size_t)e.x * 5;
    double s = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) if ((allowed >> b) & 1) s += f[b] * __ldg(r + b);
    if (s > 0.0) ll += (double)e.y * (log10(s) + __ldg(T.lpmax64 + e.x));
  }
  return warp_sum(ll);
}

__device__ double em_maxsum(const EmList& L, const ClassTable& T) {   // sum_i max_i, constant over iterations
  double v = 0;
  for (uint32_t i = threadIdx.x & 31; i < L.m; i += 32) v += (double)L.e[i].y * __ldg(T.lpmax64 + L.e[i].x);
  return warp_sum(v);
}

struct Fit { double f[5]; double ll; };

// fit_allele_frequencies (identify_mutations.cpp:3241-3318).  The log-likelihood the reference
// commits is the one evaluated at the frequencies entering the final iteration, so it is computed
// once, after convergence, at those frequencies.
__device__ Fit em_fit(const EmList& L, uint32_t n, const uint32_t obs_count[5], const ClassTable& T,
                      unsigned allowed, double tol) {
  Fit F;
  double f[5] = {0, 0, 0, 0, 0}, fprev[5];
  double tot = 0;
#pragma unroll
  for (int b = 0; b < 5; b++) if ((allowed >> b) & 1) { f[b] = 0.5 + (double)obs_count[b]; }
#pragma unroll
  for (int b = 0; b < 5; b++) tot += f[b];
#pragma unroll
  for (int b = 0; b < 5; b++) f[b] /= tot;
  const double inv_n = 1.0 / (double)n;
  for (int it = 1; it <= 50; it++) {
    double g[5];
    em_sweep(L, T, f, allowed, g, nullptr);
    double md = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) {
      fprev[b] = f[b];
      if (!((allowed >> b) & 1)) continue;
      const double fn = f[b] * g[b] * inv_n;
      md = fmax(md, fabs(fn - f[b]));
      f[b] = fn;
    }
    if (md < tol) break;
  }
  F.ll = em_loglik(L, T, fprev, allowed);
#pragma unroll
  for (int b = 0; b < 5; b++) F.f[b] = f[b];
  return F;
}

// profile_log10_likelihood (identify_mutations.cpp:3094-3143): the EM with f[v] pinned at ff and the
// other alleles renormalized, warm-started from the free fit.
__device__ void em_profile_init(const double full[5], int v, double ff, double f[5]) {
  double other = 0;
#pragma unroll
  for (int b = 0; b < 5; b++) if (b != v) other += full[b];
#pragma unroll
  for (int b = 0; b < 5; b++) f[b] = (b == v) ? ff : ((other > 0.0) ? (1.0 - ff) * full[b] / other : (1.0 - ff) / 4.0);
}

// One profile M-step; returns max |delta f|.
__device__ __forceinline__ double em_profile_step(double f[5], double fprev[5], const double g[5], int v, double ff) {
  double sw[5], others = 0;
#pragma unroll
  for (int b = 0; b < 5; b++) { sw[b] = f[b] * g[b]; if (b != v) others += sw[b]; }
  double md = 0;
  const double scale = (others > 0.0) ? (1.0 - ff) / others : 0.0, even = (1.0 - ff) * 0.25;
#pragma unroll
  for (int b = 0; b < 5; b++) {
    fprev[b] = f[b];
    if (b == v) continue;
    const double fn = (others > 0.0) ? scale * sw[b] : even;
    md = fmax(md, fabs(fn - f[b]));
    f[b] = fn;
  }
  return md;
}

__device__ double em_profile(const EmList& L, const ClassTable& T, const double full[5], int v, double ff, double tol) {
  double f[5], fprev[5];
  em_profile_init(full, v, ff, f);
  for (int it = 0; it < 50; it++) {
    double g[5];
    em_sweep(L, T, f, 31u, g, nullptr);
    if (em_profile_step(f, fprev, g, v, ff) < tol) break;
  }
  return em_loglik(L, T, fprev, 31u);
}

// profile_log10_likelihood(ff) >= target, decided with two early exits that cannot change the answer.
// EM never decreases the likelihood, and the reference's value is the likelihood at the start of its
// last iteration, so once an iterate clears the target the reference's value does too.  The
// log-likelihood is concave in f, so its maximum over the feasible set is at most
//   ln L(f) + (1 - ff) max_{b != v} g_b - sum_{b != v} f_b g_b
// and once that bound falls short of the target the reference's value does too.  Both tests use the
// FP32 estimate with a margin that covers its error; anything closer runs the exact FP64 evaluation.
__device__ bool em_profile_ge(const EmList& L, const ClassTable& T, const double full[5], int v, double ff,
                              double tol, double target, double maxsum, uint32_t n) {
  double f[5], fprev[5];
  em_profile_init(full, v, ff, f);
  for (int it = 0; it < 50; it++) {
    double g[5];
    float llf, la;
    em_sweep(L, T, f, 31u, g, &llf, &la);
    const double margin = ll_margin(n, L.m, la);
    const double ll = maxsum + (double)llf;
    if (ll - margin >= target) return true;
    double gmax = -DBL_MAX, dot = 0;
#pragma unroll
    for (int b = 0; b < 5; b++) if (b != v) { gmax = fmax(gmax, g[b]); dot += f[b] * g[b]; }
    const double upper = ll + ((1.0 - ff) * gmax - dot) * 0.43429448190325176;   // 1 / ln 10
    if (upper + margin < target) return false;
    if (em_profile_step(f, fprev, g, v, ff) < tol) break;
  }
  return em_loglik(L, T, fprev, 31u) >= target;
}

__device__ __forceinline__ int am_major(const double f[5], uint32_t n) {
  if (n == 0) return 5;
  int best = 0;
  for (int b = 1; b < 5; b++) if (f[b] > f[best]) best = b;
  return f[best] > 0.0 ? best : 5;
}
__device__ __forceinline__ int am_next(const double f[5], uint32_t n, int excl) {
  if (n == 0) return 5;
  const double thr = 0.5 / (double)n;
  int best = 5;
  for (int b = 0; b < 5; b++) {
    if (b == excl || f[b] < thr) continue;
    if (best == 5 || f[b] > f[best]) best = b;
  }
  return best;
}

// Where a scored column's RA items go, and the thresholds of the slot decisions.
struct CandOut {
  RaDev* ra;
  unsigned int* n_ra;
  uint32_t ra_cap;
  uint32_t* qhist;
  uint32_t Qhist;
  uint32_t* err;
  uint32_t base_quality_cutoff;
  double log10_ref_len, mutation_cutoff, poly_cutoff, precision_decimal;
  uint32_t col_offset;        // added to the column reported in each RA item
  BoundJob* bq;               // deferred bounds (null: computed inline)
  unsigned int* n_bq;
  uint32_t bq_cap;
  uint2* pool;
  unsigned int* pool_used;
  uint32_t pool_cap;
  uint32_t dp_rg[8];          // discordant-pair read groups (ImArgs::dp_rg)
};

// write_RA_frequency_bounds (identify_mutations.cpp:3175-3217): the reference's bisections, with each
// "profile >= target" test decided by em_profile_ge.  Used inline and by the bounds kernel.
__device__ double ra_lower_bound(const EmList& L, const ClassTable& T, const double full[5], int var, double fh,
                                 double tol, double target, double maxsum, uint32_t n) {
  if (em_profile_ge(L, T, full, var, 0.0, tol, target, maxsum, n)) return 0.0;
  double lo = 0.0, hi = fh;
  for (int i = 0; i < 40 && (hi - lo) > tol; i++) {
    const double mid = 0.5 * (lo + hi);
    if (em_profile_ge(L, T, full, var, mid, tol, target, maxsum, n)) hi = mid; else lo = mid;
  }
  return hi;
}
__device__ double ra_upper_bound(const EmList& L, const ClassTable& T, const double full[5], int var, double fh,
                                 double tol, double target, double maxsum, uint32_t n) {
  if (em_profile_ge(L, T, full, var, 1.0, tol, target, maxsum, n)) return 1.0;
  double lo = fh, hi = 1.0;
  for (int i = 0; i < 40 && (hi - lo) > tol; i++) {
    const double mid = 0.5 * (lo + hi);
    if (em_profile_ge(L, T, full, var, mid, tol, target, maxsum, n)) lo = mid; else hi = mid;
  }
  return lo;
}

// Scores one reference column (called by a whole warp): gathers the reads covering column c in BAM
// order into the warp's list `ents` (capacity `cap`), then for insert slot 0 (when do_slot0) and every
// insert slot that exists, scores the slot in FP64: summed log10 likelihoods and pure-genotype call,
// the five-allele EM, the variant-presence EM, and for emitted RA items the profile-likelihood
// bounds and the strand / quality tallies (identify_mutations.cpp:1359-1910).  When `recompute`,
// the slot-0 consensus call is written back to call[c].
__device__ void score_candidate_column(const DevSample& S, const ClassTable& T, const CandOut& A, uint32_t c,
                                       bool do_slot0, bool recompute, ColCall cl0, ColCall* call, uint4* ents,
                                       uint32_t cap, uint32_t* hist) {
  const int lane = threadIdx.x & 31;
  uint2* list = reinterpret_cast<uint2*>(ents + cap);   // the warp's (class, multiplicity) list
  // ---- gather covering reads in BAM order
  const uint2 rr = __ldg(S.tile_range + (c >> 5));
  uint32_t m = 0;
  bool overflow = false;
  for (uint32_t b0 = rr.x; b0 < rr.y; b0 += 32) {
    const uint32_t r = b0 + lane;
    bool ok = false;
    Pile e;
    DevRead rd;
    if (r < rr.y) {
      rd = S.reads[r];
      ok = !(rd.flags & kSkip) && c >= rd.start && c < rd.end;
      if (ok) resolve(S, rd, c, e);
    }
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, ok);
    const uint32_t slot = m + __popc(bal & ((1u << lane) - 1));
    if (ok && slot < cap) {
      const int obi = e.del ? -1 : max(e.indel, 0);
      ents[slot] = make_uint4(r, (uint32_t)e.qpos | ((uint32_t)(obi + 1) << 16), 0xFFFFFFFFu, 0);
    }
    m += __popc(bal);
  }
  if (m > cap) { overflow = true; m = cap; }
  if (overflow) { if (lane == 0) atomicOr(A.err, kErrScratch); return; }
  __syncwarp();
  int k = do_slot0 ? 0 : 1;
  const uint8_t refc0 = __ldg(S.ref + c);
  for (;; k++) {
    // ---- build the slot's read bases (identify_mutations.cpp:1392-1658)
    uint32_t pc[5][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
    uint32_t n_local = 0;
    bool next_local = false;
    double s64[5] = {0, 0, 0, 0, 0};
    for (uint32_t i = lane; i < m; i += 32) {
      uint4 en = ents[i];
      en.z = 0xFFFFFFFFu;
      const uint32_t r = en.x;
      const DevRead rd = S.reads[r];
      if (k == 0 && (rd.flags & kDpCand) && c == rd.start && dp_group_member(A.dp_rg, __ldg(S.rg + r))) {
        ents[i] = en;                 // left out of its first column at insert position 0
        continue;
      }
      const int qpos = (int)(en.y & 0xFFFF);
      const int obi = (int)(en.y >> 16) - 1;
      const bool rev = rd.flags & kRev;
      uint8_t base = '.';
      bool past = true;
      if (obi >= k) { base = nib_at(S.seq, rd.seq_off + qpos + k); past = false; }
      if (base != 15) {
        const bool red = rd.flags & kRedundant;
        if (!red && obi > k) next_local = true;
        if (!red && !is_trimmed(rd, qpos, past)) {
          int qp = qpos;
          bool ok = true;
          if (obi == -1) {
            qp += 1 - (int)rev;
            if (qp >= (int)rd.len || nib_at(S.seq, rd.seq_off + qp) == 15) ok = false;
          } else if (k > 0) {
            int mo = k < obi ? k : obi;
            qp += mo + 1 - (int)rev;
            if (qp > bounds_end0(S, rd, r) || nib_at(S.seq, rd.seq_off + qp) == 15) ok = false;
          }
          if (ok) {
            const int obs = (base == '.') ? 4 : bam_idx(base);
            const uint32_t q = __ldg(S.qual + rd.seq_off + qp);
            const uint32_t rs = rd.rfile;
            if (obs < 0 || q >= T.Q || rs >= T.R) ok = false;
            else if (q >= A.base_quality_cutoff) {
              const uint32_t cls = ((((uint32_t)rd.mapq_idx * T.R + rs) * 2u + (rev ? 1u : 0u)) * T.Q + q) * 5u + (uint32_t)obs;
              en.z = cls;
              en.w = (uint32_t)obs | (q << 8) | ((rev ? 1u : 0u) << 16);
              pc[obs][rev ? 1 : 0]++;
              n_local++;
              const double* lp = T.lp64 + (size_t)cls * 5;
#pragma unroll
              for (int b = 0; b < 5; b++) s64[b] += __ldg(lp + b);
            }
          }
        }
      }
      ents[i] = en;
    }
    __syncwarp();
    const uint32_t n = warp_sum_u(n_local);
    const bool next_exists = __any_sync(0xFFFFFFFFu, next_local);
    uint32_t cnt[5];
    uint32_t pinfo[5][2];
#pragma unroll
    for (int b = 0; b < 5; b++) {
      pinfo[b][0] = warp_sum_u(pc[b][0]);
      pinfo[b][1] = warp_sum_u(pc[b][1]);
      cnt[b] = pinfo[b][0] + pinfo[b][1];
      s64[b] = warp_sum(s64[b]);
    }
    const uint8_t refc = (k == 0) ? refc0 : (uint8_t)'.';
    const int ref_idx = (refc == '.') ? 4 : (chr_idx(refc) < 0 ? 5 : chr_idx(refc));
    // ---- pure genotype call (identify_mutations.cpp:3398-3433)
    int best = 5;
    double cscore = __longlong_as_double(0x7ff8000000000000ll);
    if (n > 0) {
      best = 0;
      for (int b = 1; b < 5; b++) if (s64[b] > s64[best]) best = b;
      double off = -DBL_MAX;
      for (int b = 0; b < 5; b++) if (b != best) off = fmax(off, s64[b]);
      double te = 0;
      for (int b = 0; b < 5; b++) if (b != best) te += exp10(s64[b] - off);
      cscore = s64[best] - (log10(te) + off) - A.log10_ref_len;
    }
    if (k == 0 && recompute && call != nullptr && lane == 0) {
      ColCall cl = cl0;
      cl.best = (uint8_t)best;
      cl.score = cscore;
      cl.flags = (uint8_t)((cl.flags & ~kBasePredicted) | ((cscore >= A.mutation_cutoff) ? kBasePredicted : 0));
      call[c] = cl;
    }
    const bool passed_cons = (best != ref_idx) && !isnan(cscore) && cscore > 0;
    // ---- distinct likelihood classes of the slot, in class order (or read order without a histogram)
    EmList L;
    L.e = list;
    {
      uint32_t outn = 0;
      if (hist != nullptr) {
        for (uint32_t i = lane; i < T.K; i += 32) hist[i] = 0;
        __syncwarp();
        for (uint32_t i = lane; i < m; i += 32) { const uint32_t cls = ents[i].z; if (cls != kNoClass) atomicAdd(hist + cls, 1u); }
        __syncwarp();
        for (uint32_t b0 = 0; b0 < T.K; b0 += 32) {
          const uint32_t i = b0 + lane;
          const uint32_t cnt = i < T.K ? hist[i] : 0u;
          const unsigned bal = __ballot_sync(0xFFFFFFFFu, cnt != 0);
          if (cnt) list[outn + __popc(bal & ((1u << lane) - 1))] = make_uint2(i, cnt);
          outn += __popc(bal);
        }
      } else {
        for (uint32_t b0 = 0; b0 < m; b0 += 32) {
          const uint32_t i = b0 + lane;
          const uint32_t cls = i < m ? ents[i].z : kNoClass;
          const unsigned bal = __ballot_sync(0xFFFFFFFFu, cls != kNoClass);
          if (cls != kNoClass) list[outn + __popc(bal & ((1u << lane) - 1))] = make_uint2(cls, 1u);
          outn += __popc(bal);
        }
      }
      L.m = outn;
      __syncwarp();
    }
    // ---- five-allele fit and variant presence (identify_mutations.cpp:1795-1821)
    Fit full;
    for (int b = 0; b < 5; b++) full.f[b] = 0;
    full.ll = 0;
    int maj = 5, mnr = 5, var = 5;
    double vscore = __longlong_as_double(0x7ff8000000000000ll);
    bool passed_poly = false;
    if (n > 0) {
      full = em_fit(L, n, cnt, T, 31u, A.precision_decimal);
      maj = am_major(full.f, n);
      mnr = am_next(full.f, n, maj);
      var = am_next(full.f, n, ref_idx);
      if (var != 5) {
        Fit nf = em_fit(L, n, cnt, T, 31u & ~(1u << var), A.precision_decimal);
        vscore = (full.ll - nf.ll) - A.log10_ref_len;
        passed_poly = vscore >= A.poly_cutoff;
      }
    }
    if (passed_cons || passed_poly) {
      uint32_t slot = 0;
      if (lane == 0) slot = atomicAdd(A.n_ra, 1u);
      slot = __shfl_sync(0xFFFFFFFFu, slot, 0);
      // ---- frequency bounds (identify_mutations.cpp:3175-3217): deferred to the bounds kernel as two
      // independent bisections when there is room, else computed here
      double lower = 0.0, upper = 1.0;
      if (n > 0 && var < 5) {
        const double D = 0.587566;
        const double fh = full.f[var];
        const double tol = A.precision_decimal;
        const double maxsum = em_maxsum(L, T);
        const double target = em_profile(L, T, full.f, var, fh, tol) - D;
        bool deferred = false;
        if (A.bq != nullptr && slot < A.ra_cap) {
          uint32_t off = 0, jb = 0;
          if (lane == 0) { off = atomicAdd(A.pool_used, L.m); jb = atomicAdd(A.n_bq, 2u); }
          off = __shfl_sync(0xFFFFFFFFu, off, 0);
          jb = __shfl_sync(0xFFFFFFFFu, jb, 0);
          if ((uint64_t)off + L.m <= A.pool_cap && (uint64_t)jb + 2 <= A.bq_cap) {
            for (uint32_t i = lane; i < L.m; i += 32) A.pool[off + i] = L.e[i];
            if (lane < 2) {
              BoundJob b;
              for (int q = 0; q < 5; q++) b.full[q] = full.f[q];
              b.target = target; b.maxsum = maxsum; b.fh = fh; b.tol = tol;
              b.slot = slot; b.pool_off = off; b.m = L.m; b.n = n; b.col = c + A.col_offset;
              b.var = (uint8_t)var; b.side = (uint8_t)lane; b.pad[0] = b.pad[1] = 0;
              A.bq[jb + lane] = b;
            }
            deferred = true;
          }
        }
        if (!deferred) {
          lower = ra_lower_bound(L, T, full.f, var, fh, tol, target, maxsum, n);
          upper = ra_upper_bound(L, T, full.f, var, fh, tol, target, maxsum, n);
        }
      }
      if (slot < A.ra_cap) {
        if (lane == 0) {
          RaDev o;
          o.col = c + A.col_offset; o.insert_position = (uint32_t)k;
          o.score = vscore; o.consensus_score = cscore;
          for (int b = 0; b < 5; b++) { o.f[b] = full.f[b]; o.pos_info[b][0] = pinfo[b][0]; o.pos_info[b][1] = pinfo[b][1]; }
          o.lower = lower; o.upper = upper; o.n = n;
          o.ref_idx = (uint8_t)ref_idx; o.var_idx = (uint8_t)var; o.maj_idx = (uint8_t)maj; o.min_idx = (uint8_t)mnr;
          o.passed_cons = passed_cons; o.passed_poly = passed_poly; o.pad[0] = o.pad[1] = 0;
          A.ra[slot] = o;
        }
        // qualities of the major and minor alleles' reads for the K-S test (:3009-3033)
        uint32_t* qh = A.qhist + (size_t)slot * 2 * A.Qhist;
        for (uint32_t i = lane; i < 2 * A.Qhist; i += 32) qh[i] = 0;
        __syncwarp();
        for (uint32_t i = lane; i < m; i += 32) {
          const uint4 en = ents[i];
          if (en.z == 0xFFFFFFFFu) continue;
          const int obs = (int)(en.w & 0xFF);
          const uint32_t q = (en.w >> 8) & 0xFF;
          if (q >= A.Qhist) continue;
          if (obs == maj) atomicAdd(qh + q, 1u);
          if (obs == mnr) atomicAdd(qh + A.Qhist + q, 1u);
        }
      } else if (lane == 0) {
        atomicOr(A.err, kErrRaOverflow);
      }
    }
    if (!next_exists) break;
    __syncwarp();
  }
}

}  // namespace
}  // namespace bsq
