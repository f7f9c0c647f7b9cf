// Coverage-distribution fit: the censored negative-binomial fit of a unique-only coverage histogram
// and the deletion-propagation cutoff derived from it.  breseq runs it on the host after error_count
// (CoverageDistribution::fit, src/breseq/coverage_distribution.cpp:437-505, over
// fit_censored_negative_binomial :115-319 and fit_coverage_distribution :341-396), reading the
// histogram back from <group>.unique_only_coverage_distribution.tab.
//
// The work is 48 independent Nelder-Mead minimisations (six starting means x eight starting sizes),
// each evaluating a sum over the censored window of negative-binomial probabilities in FP64.  GB300's
// FP64 rate is a small fraction of its FP32 rate, and breseq's result depends on every bit of glibc's
// log / exp / pow inside the special functions, so the fit stays on the host cores: the restarts run
// on threads and the best one is chosen in breseq's order, which leaves the result independent of the
// thread count and identical to the sequential evaluation.
//
// Special functions.  breseq uses two forms of the log-gamma function: ALGLIB's translation of the
// Cephes lgam for the negative-binomial PMF (lngamma, src/breseq/stats.cpp:534-650) and the Cephes lgam
// itself inside the incomplete beta integral (lgam, :407-500).  The negative-binomial CDF is Cephes
// nbdtr = incbet(n, k + 1, p) (:982-990) with incbet / incbcf / incbd / pseries (:1385-1700) and the
// Cephes gamma with Stirling's formula (:277-398).  These are the published Cephes Math Library 2.8
// algorithms (S. L. Moshier); the coefficients and the order of every operation are kept as breseq
// evaluates them, because the fit's restarts follow the objective's exact values.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../../include/breseq_gb300.h"

namespace bsq {
namespace nbfit {
namespace {

// ------------------------------------------------------------------ Cephes constants and tables
constexpr double kMachEp = 1.11022302462515654042E-16;
constexpr double kMaxLog = 7.09782712893383996732E2;
constexpr double kMinLog = -7.451332191019412076235E2;
constexpr double kMaxGam = 171.624376956302725;
constexpr double kBig = 4.503599627370496e15;
constexpr double kBigInv = 2.22044604925031308085e-16;
constexpr double kMaxStir = 143.01608;
constexpr double kSqrtTwoPi = 2.50662827463100050242E0;
constexpr double kLogSqrtTwoPi = 0.91893853320467274178;
constexpr double kMaxLgm = 2.556348e305;

// gamma on [2, 3): P / Q
constexpr double kGammaP[7] = {1.60119522476751861407E-4, 1.19135147006586384913E-3, 1.04213797561761569935E-2,
                               4.76367800457137231464E-2, 2.07448227648435975150E-1, 4.94214826801497100753E-1,
                               9.99999999999999996796E-1};
constexpr double kGammaQ[8] = {-2.31581873324120129819E-5, 5.39605580493303397842E-4, -4.45641913851797240494E-3,
                               1.18139785222060435552E-2, 3.58236398605498653373E-2, -2.34591795718243348568E-1,
                               7.14304917030273074085E-2, 1.00000000000000000320E0};
// Stirling's series for gamma
constexpr double kStir[5] = {7.87311395793093628397E-4, -2.29549961613378126380E-4, -2.68132617805781232825E-3,
                             3.47222221605458667310E-3, 8.33333333333482257126E-2};
// log gamma: Stirling's series (A) and the rational form on [2, 3) (x B / C, C monic)
constexpr double kLgamA[5] = {8.11614167470508450300E-4, -5.95061904284301438324E-4, 7.93650340457716943945E-4,
                              -2.77777777730099687205E-3, 8.33333333333331927722E-2};
constexpr double kLgamB[6] = {-1.37825152569120859100E3, -3.88016315134637840924E4, -3.31612992738871184744E5,
                              -1.16237097492762307383E6, -1.72173700820839662146E6, -8.53555664245765465627E5};
constexpr double kLgamC[6] = {-3.51815701436523470549E2, -1.70642106651881159223E4, -2.20528590553854454839E5,
                              -1.13933444367982507207E6, -2.53252307177582951285E6, -2.01889141433532773231E6};
// ALGLIB writes the Stirling coefficients of its lngamma as products with a power of ten; the folded
// products round differently from the E-notation literals above in the last place.
constexpr double kAlgA[5] = {8.11614167470508450300 * 0.0001, -5.95061904284301438324 * 0.0001,
                             7.93650340457716943945 * 0.0001, -2.77777777730099687205 * 0.001,
                             8.33333333333331927722 * 0.01};
constexpr double kAlgLarge1 = 7.9365079365079365079365 * 0.0001;
constexpr double kAlgLarge2 = 2.7777777777777777777778 * 0.001;

// Horner's rule as Cephes polevl: c[0] x^n + ... + c[n]
inline double poly(double x, const double* c, int n) {
  double r = c[0];
  for (int i = 1; i <= n; i++) r = r * x + c[i];
  return r;
}
// Cephes p1evl: the same with an implied leading coefficient 1 (c holds n coefficients)
inline double poly1(double x, const double* c, int n) {
  double r = x + c[0];
  for (int i = 1; i < n; i++) r = r * x + c[i];
  return r;
}

// log Gamma(x) for x > 0 on [.., 13): shift into [2, 3) keeping the product in z, then the rational
// form.  Both forms share this part.
inline double lgamma_small(double x) {
  double z = 1.0, p = 0.0, u = x;
  while (u >= 3.0) {
    p -= 1.0;
    u = x + p;
    z *= u;
  }
  while (u < 2.0) {
    z /= u;
    p += 1.0;
    u = x + p;
  }
  if (u == 2.0) return log(z);
  p -= 2.0;
  x = x + p;
  return log(z) + x * poly(x, kLgamB, 5) / poly1(x, kLgamC, 6);
}

// ALGLIB lngamma (x > 0): the log-gamma of dnbinom_mu.
double lngamma_alglib(double x) {
  if (!(x > 0.0)) return NAN;            // the fit only takes positive arguments
  if (x < 13.0) return lgamma_small(x);
  double q = (x - 0.5) * log(x) - x + kLogSqrtTwoPi;
  if (x > 100000000.0) return q;
  const double p = 1.0 / (x * x);
  if (x >= 1000.0) return q + ((kAlgLarge1 * p - kAlgLarge2) * p + 0.0833333333333333333333) / x;
  double a = kAlgA[0];
  for (int i = 1; i < 5; i++) a = kAlgA[i] + p * a;
  return q + a / x;
}

// Cephes lgam (x > 0): the log-gamma of the incomplete beta integral.
double lgam(double x) {
  if (!(x > 0.0)) return NAN;
  if (x < 13.0) return lgamma_small(x);
  if (x > kMaxLgm) return INFINITY;
  double q = (x - 0.5) * log(x) - x + kLogSqrtTwoPi;
  if (x > 1.0e8) return q;
  const double p = 1.0 / (x * x);
  if (x >= 1000.0)
    q += ((7.9365079365079365079365e-4 * p - 2.7777777777777777777778e-3) * p + 0.0833333333333333333333) / x;
  else
    q += poly(p, kLgamA, 4) / x;
  return q;
}

// Cephes gamma by Stirling's formula (x > 33)
double stirling(double x) {
  double w = 1.0 / x;
  w = 1.0 + w * poly(w, kStir, 4);
  double y = exp(x);
  if (x > kMaxStir) {
    const double v = pow(x, 0.5 * x - 0.25);
    y = v * (v / y);
  } else {
    y = pow(x, x - 0.5) / y;
  }
  return kSqrtTwoPi * y * w;
}

// Cephes gamma (x > 0)
double gamma_fn(double x) {
  if (!(x > 0.0)) return NAN;
  if (x > 33.0) return stirling(x);
  double z = 1.0;
  while (x >= 3.0) {
    x -= 1.0;
    z *= x;
  }
  while (x < 2.0) {
    if (x < 1.e-9) return x == 0.0 ? INFINITY : z / ((1.0 + 0.5772156649015329 * x) * x);
    z /= x;
    x += 1.0;
  }
  if (x == 2.0) return z;
  x -= 2.0;
  const double p = poly(x, kGammaP, 6);
  const double q = poly(x, kGammaQ, 7);
  return z * p / q;
}

// Continued fractions of the incomplete beta integral (Cephes incbcf / incbd).  `second` selects
// incbd's form, whose ratio runs in z = x / (1 - x).
double beta_fraction(double a, double b, double x, bool second) {
  double k1 = a, k2 = second ? b - 1.0 : a + b, k3 = a, k4 = a + 1.0;
  double k5 = 1.0, k6 = second ? a + b : b - 1.0, k7 = a + 1.0, k8 = a + 2.0;
  const double z = second ? x / (1.0 - x) : x;
  double pkm2 = 0.0, qkm2 = 1.0, pkm1 = 1.0, qkm1 = 1.0, ans = 1.0, r = 1.0, t;
  const double thresh = 3.0 * kMachEp;
  int n = 0;
  do {
    double xk = -(z * k1 * k2) / (k3 * k4);
    double pk = pkm1 + pkm2 * xk;
    double qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    xk = (z * k5 * k6) / (k7 * k8);
    pk = pkm1 + pkm2 * xk;
    qk = qkm1 + qkm2 * xk;
    pkm2 = pkm1; pkm1 = pk; qkm2 = qkm1; qkm1 = qk;
    if (qk != 0) r = pk / qk;
    if (r != 0) {
      t = fabs((ans - r) / r);
      ans = r;
    } else {
      t = 1.0;
    }
    if (t < thresh) break;
    k1 += 1.0;
    if (second) k2 -= 1.0; else k2 += 1.0;
    k3 += 2.0;
    k4 += 2.0;
    k5 += 1.0;
    if (second) k6 += 1.0; else k6 -= 1.0;
    k7 += 2.0;
    k8 += 2.0;
    if ((fabs(qk) + fabs(pk)) > kBig) {
      pkm2 *= kBigInv; pkm1 *= kBigInv; qkm2 *= kBigInv; qkm1 *= kBigInv;
    }
    if ((fabs(qk) < kBigInv) || (fabs(pk) < kBigInv)) {
      pkm2 *= kBig; pkm1 *= kBig; qkm2 *= kBig; qkm1 *= kBig;
    }
  } while (++n < 300);
  return ans;
}

// Power series of the incomplete beta integral, for small b x (Cephes pseries)
double beta_series(double a, double b, double x) {
  const double ai = 1.0 / a;
  double u = (1.0 - b) * x;
  double v = u / (a + 1.0);
  const double t1 = v;
  double t = u, n = 2.0, s = 0.0;
  const double z = kMachEp * ai;
  while (fabs(v) > z) {
    u = (n - b) * x / n;
    t *= u;
    v = t / (a + n);
    s += v;
    n += 1.0;
  }
  s += t1;
  s += ai;
  u = a * log(x);
  if ((a + b) < kMaxGam && fabs(u) < kMaxLog) {
    t = gamma_fn(a + b) / (gamma_fn(a) * gamma_fn(b));
    s = s * t * pow(x, a);
  } else {
    t = lgam(a + b) - lgam(a) - lgam(b) + u + log(s);
    s = t < kMinLog ? 0.0 : exp(t);
  }
  return s;
}

}  // namespace

// Regularised incomplete beta integral I_x(aa, bb) (Cephes incbet); 0 outside its domain.
double incbet(double aa, double bb, double xx) {
  if (aa <= 0.0 || bb <= 0.0) return 0.0;
  if (xx <= 0.0 || xx >= 1.0) return xx == 1.0 ? 1.0 : 0.0;
  if ((bb * xx) <= 1.0 && xx <= 0.95) return beta_series(aa, bb, xx);
  double w = 1.0 - xx;
  double a, b, x, xc, t;
  const bool flip = xx > (aa / (aa + bb));
  if (flip) {
    a = bb; b = aa; xc = xx; x = w;
  } else {
    a = aa; b = bb; xc = w; x = xx;
  }
  if (flip && (b * x) <= 1.0 && x <= 0.95) {
    t = beta_series(a, b, x);
  } else {
    double y = x * (a + b - 2.0) - (a - 1.0);
    w = y < 0.0 ? beta_fraction(a, b, x, false) : beta_fraction(a, b, x, true) / xc;
    y = a * log(x);
    t = b * log(xc);
    if ((a + b) < kMaxGam && fabs(y) < kMaxLog && fabs(t) < kMaxLog) {
      t = pow(xc, b);
      t *= pow(x, a);
      t /= a;
      t *= w;
      t *= gamma_fn(a + b) / (gamma_fn(a) * gamma_fn(b));
    } else {
      y += t + lgam(a + b) - lgam(a) - lgam(b);
      y += log(w / a);
      t = y < kMinLog ? 0.0 : exp(y);
    }
  }
  if (flip) t = t <= kMachEp ? 1.0 - kMachEp : 1.0 - t;
  return t;
}

// Negative binomial CDF P(X <= k), size n, success probability p (Cephes nbdtr).
double nbdtr(double k, double n, double p) { return incbet(n, k + 1.0, p); }

// R's dnbinom(k, size, mu) as breseq evaluates it (dnbinom_mu, src/breseq/stats.h:92-100).
double dnbinom_mu(double k, double size, double mu) {
  const double p = size / (size + mu);
  const double log_pmf = lngamma_alglib(k + size) - lngamma_alglib(size) - lngamma_alglib(k + 1) + size * log(p) +
                         k * log(1.0 - p);
  return exp(log_pmf);
}

// Smallest k with nbdtr(k) >= target (qnbinom_mu, src/breseq/stats.cpp:2047-2072): doubling bracket,
// then bisection.  False if no bracket is found within 2^62 (the reference would not return).
bool qnbinom_mu(double target_pr, double size, double mu, uint64_t* out) {
  const double p = size / (size + mu);
  if (target_pr <= 0.0) {
    *out = 0;
    return true;
  }
  uint64_t hi = 1;
  int doublings = 0;
  while (nbdtr((double)hi, size, p) < target_pr) {
    if (++doublings > 62) return false;
    hi *= 2;
  }
  uint64_t lo = hi / 2;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (nbdtr((double)mid, size, p) < target_pr)
      lo = mid + 1;
    else
      hi = mid;
  }
  *out = lo;
  return true;
}

namespace {

// The censored least-squares objective over the fitting window, with the terms that do not depend on
// the bin hoisted out of the loop (each hoisted value is the one the per-bin expression computes).
struct Objective {
  uint32_t lo, hi;                 // window [lo, hi] of the (coarse-grained) histogram
  std::vector<double> target;      // x[i] / inner_total
  std::vector<double> lg_k1;       // lngamma(i + 1)
  mutable std::vector<double> dist;

  // 1e10 for a non-finite (mu, size) or distribution, as breseq's f_nb; *domain set when mu or size
  // underflows to 0 (dnbinom_mu's assertion in the reference).
  double operator()(const double par[2], bool* domain) const {
    const double mu = exp(par[0]);
    const double size = exp(par[1]);
    if (!std::isfinite(mu) || !std::isfinite(size)) return 1e10;
    if (!(size > 0) || !(mu > 0)) {
      *domain = true;
      return 1e10;
    }
    const double p = size / (size + mu);
    const double lg_size = lngamma_alglib(size);
    const double size_log_p = size * log(p);
    const double log_q = log(1.0 - p);
    double total = 0;
    for (uint32_t i = lo; i <= hi; i++) {
      const double k = (double)i;
      const double log_pmf = lngamma_alglib(k + size) - lg_size - lg_k1[i - lo] + size_log_p + k * log_q;
      dist[i - lo] = exp(log_pmf);
      total += dist[i - lo];
    }
    if (!(total > 0) || !std::isfinite(total)) return 1e10;
    double l = 0;
    for (uint32_t i = lo; i <= hi; i++) {
      const double diff = target[i - lo] - (dist[i - lo] / total);
      l += diff * diff;
    }
    return std::isfinite(l) ? l : 1e10;
  }
};

struct Restart {
  double est[2];
  double value;
  bool converged;
  bool domain;
};

// Nelder-Mead over two parameters as breseq's nelder_mead_minimize (src/breseq/stats.cpp:2289-2381):
// reflection 1, expansion 2, contraction 0.5, shrink 0.5, initial steps 5% of each coordinate,
// stop when the spread of the vertex values is below 1e-8, at most 1000 iterations.  Vertices are
// ordered by a stable sort of their values (libstdc++'s std::sort on three elements is an insertion
// sort), so ties keep their previous order.
Restart nelder_mead(const Objective& f, const double init[2], Objective* scratch_owner) {
  (void)scratch_owner;
  constexpr int n = 2;
  constexpr uint32_t kMaxIter = 1000;
  constexpr double kTol = 1e-8;
  Restart out{};
  double s[n + 1][n], v[n + 1];
  for (int i = 0; i <= n; i++)
    for (int j = 0; j < n; j++) s[i][j] = init[j];
  for (int i = 0; i < n; i++) s[i + 1][i] += (init[i] != 0.0) ? 0.05 * fabs(init[i]) : 0.00025;
  bool domain = false;
  for (int i = 0; i <= n; i++) v[i] = f(s[i], &domain);
  bool converged = false;
  for (uint32_t iter = 0; iter < kMaxIter; iter++) {
    for (int i = 1; i <= n; i++) {          // stable insertion sort by value
      double vi = v[i], si[n];
      for (int j = 0; j < n; j++) si[j] = s[i][j];
      int k = i;
      while (k > 0 && vi < v[k - 1]) {
        v[k] = v[k - 1];
        for (int j = 0; j < n; j++) s[k][j] = s[k - 1][j];
        k--;
      }
      v[k] = vi;
      for (int j = 0; j < n; j++) s[k][j] = si[j];
    }
    if ((v[n] - v[0]) < kTol) {
      converged = true;
      break;
    }
    double c[n] = {0.0, 0.0};
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) c[j] += s[i][j];
    for (int j = 0; j < n; j++) c[j] /= (double)n;
    double r[n];
    for (int j = 0; j < n; j++) r[j] = c[j] + 1.0 * (c[j] - s[n][j]);
    const double fr = f(r, &domain);
    if (fr < v[0]) {
      double e[n];
      for (int j = 0; j < n; j++) e[j] = c[j] + 2.0 * (r[j] - c[j]);
      const double fe = f(e, &domain);
      if (fe < fr) {
        for (int j = 0; j < n; j++) s[n][j] = e[j];
        v[n] = fe;
      } else {
        for (int j = 0; j < n; j++) s[n][j] = r[j];
        v[n] = fr;
      }
    } else if (fr < v[n - 1]) {
      for (int j = 0; j < n; j++) s[n][j] = r[j];
      v[n] = fr;
    } else {
      double k[n];
      for (int j = 0; j < n; j++) k[j] = c[j] + 0.5 * (s[n][j] - c[j]);
      const double fk = f(k, &domain);
      if (fk < v[n]) {
        for (int j = 0; j < n; j++) s[n][j] = k[j];
        v[n] = fk;
      } else {
        for (int i = 1; i <= n; i++) {
          for (int j = 0; j < n; j++) s[i][j] = s[0][j] + 0.5 * (s[i][j] - s[0][j]);
          v[i] = f(s[i], &domain);
        }
      }
    }
  }
  int best = 0;
  for (int i = 1; i <= n; i++)
    if (v[i] < v[best]) best = i;
  out.est[0] = s[best][0];
  out.est[1] = s[best][1];
  out.value = v[best];
  out.converged = converged && std::isfinite(v[best]);
  out.domain = domain;
  return out;
}

struct FitResult {
  double size = 0, mu = 0, average = 0, variance = 0, relative_variance = 0, scale = 0;
  uint32_t censor_start = 0, censor_end = 0, converged = 0;
  bool domain = false;
};

// fit_censored_negative_binomial (src/breseq/coverage_distribution.cpp:115-319) over n[0..N].
FitResult fit_censored(const double* n, uint32_t N, int n_threads) {
  FitResult res;
  double total_positions = 0;
  for (uint32_t i = 1; i <= N; i++) total_positions += n[i];
  if (total_positions == 0) return res;
  double m = 0;
  for (uint32_t i = 1; i <= N; i++) m += i * n[i];
  m /= total_positions;
  double v = 0;
  if (total_positions > 1) {
    for (uint32_t i = 1; i <= N; i++) v += n[i] * (i - m) * (i - m);
    v /= (total_positions - 1);
  }
  res.average = m;
  res.variance = v;
  res.relative_variance = (m > 0) ? v / m : 0.0;

  // peak of the 5-point centred moving average (R's filter(), undefined within 2 of either end)
  uint32_t min_i = std::max((uint32_t)(m / 4.0), (uint32_t)1);
  double max_n = 0;
  uint32_t max_i = 0;
  for (uint32_t i = min_i; i <= N; i++) {
    double ma;
    if (N >= 5) {
      if (i < 3 || i > N - 2) continue;
      ma = (n[i - 2] + n[i - 1] + n[i] + n[i + 1] + n[i + 2]) / 5.0;
    } else {
      ma = n[i];
    }
    if (ma > max_n) {
      max_n = ma;
      max_i = i;
    }
  }
  const uint32_t start_i = std::max((uint32_t)floor(max_i * 0.5), (uint32_t)1);
  const uint32_t end_i = std::min((uint32_t)ceil(max_i * 1.5), N);
  if (start_i == end_i) return res;
  res.censor_start = start_i;
  res.censor_end = end_i;

  // coarse-grain to 1000-2000 bins (uint32 arithmetic as the reference's)
  uint32_t per_bin = (end_i - start_i) / 1000;
  uint32_t lo, hi;
  std::vector<double> x;
  if (per_bin > 1) {
    lo = start_i / per_bin;
    hi = (uint32_t)ceil((double)end_i / per_bin);
    x.assign((size_t)hi + 1, 0.0);
    for (uint32_t i = lo; i <= hi; i++)
      for (uint32_t j = 1; j <= per_bin; j++) {
        const uint32_t idx = i * per_bin + j;
        if (idx <= N) x[i] += n[idx];
      }
  } else {
    per_bin = 1;
    lo = start_i;
    hi = end_i;
    x.assign((size_t)hi + 1, 0.0);
    for (uint32_t i = 1; i <= hi; i++) x[i] = n[i];
  }
  double inner_total = 0;
  for (uint32_t i = lo; i <= hi; i++) inner_total += x[i];
  double mean_num = 0, mean_den = 0;
  for (uint32_t i = 1; i <= hi; i++) {
    mean_num += i * x[i];
    mean_den += x[i];
  }
  const double mean_estimate = mean_num / mean_den;

  Objective f;
  f.lo = lo;
  f.hi = hi;
  f.target.resize((size_t)hi - lo + 1);
  f.lg_k1.resize((size_t)hi - lo + 1);
  f.dist.resize((size_t)hi - lo + 1);
  for (uint32_t i = lo; i <= hi; i++) {
    f.target[i - lo] = x[i] / inner_total;
    f.lg_k1[i - lo] = lngamma_alglib((double)i + 1);
  }

  const double means[6] = {mean_estimate,
                           (double)hi,
                           (double)lo,
                           1.0 * (hi + lo) / 4.0,
                           2.0 * (hi + lo) / 4.0,
                           3.0 * (hi + lo) / 4.0};
  double sizes[8];
  double try_size = 100000;
  for (int k = 0; k < 8; k++) {
    try_size /= 10.0;
    sizes[k] = try_size;
  }
  constexpr int kRestarts = 48;
  std::vector<Restart> runs(kRestarts);
  std::atomic<int> next{0};
  auto worker = [&]() {
    Objective g = f;                     // private scratch
    for (int r; (r = next.fetch_add(1)) < kRestarts;) {
      const double init[2] = {log(means[r / 8]), log(sizes[r % 8])};
      runs[r] = nelder_mead(g, init, nullptr);
      if (runs[r].converged) {
        bool d = false;
        runs[r].value = g(runs[r].est, &d);   // breseq re-evaluates the objective at the estimate
        runs[r].domain |= d;
      }
    }
  };
  const int threads = std::max(1, std::min(n_threads, kRestarts));
  if (threads == 1) {
    worker();
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
  }

  double mu = 0, size = 0, best = HUGE_VAL;
  for (int r = 0; r < kRestarts; r++) {
    res.domain |= runs[r].domain;
    if (!runs[r].converged) continue;
    res.converged++;
    if (runs[r].value < best) {
      best = runs[r].value;
      mu = exp(runs[r].est[0]);
      size = exp(runs[r].est[1]);
    }
  }
  if (!(best < HUGE_VAL)) mu = size = 0;

  double included = 0;
  if (mu > 0) {
    const double p = size / (size + mu);
    included = nbdtr((double)hi, size, p) - nbdtr((double)lo, size, p);
    if (included >= 0.01 && per_bin > 1) mu = mu * per_bin;
  }
  if (included < 0.01) mu = size = 0;
  res.mu = mu;
  res.size = size;
  if (mu > 0) res.scale = inner_total / included;
  return res;
}

int default_threads() {
  const unsigned h = std::thread::hardware_concurrency();
  return h ? (int)std::min(h, 48u) : 1;
}

}  // namespace
}  // namespace nbfit
}  // namespace bsq

using namespace bsq::nbfit;

extern "C" int bsq_fit_coverage_distribution(const uint64_t* hist, uint32_t hist_size,
                                             double deletion_propagation_pr_cutoff, int n_threads,
                                             bsq_coverage_fit* out) {
  if (!out || (hist_size && !hist) || !(deletion_propagation_pr_cutoff >= 0.0) || deletion_propagation_pr_cutoff > 1.0)
    return BSQ_ERR_INVALID;
  memset(out, 0, sizeof(*out));
  // the histogram as read back from the .tab file: rows 1..size-1, max_coverage = size - 1
  const uint32_t N = hist_size ? hist_size - 1 : 0;
  std::vector<double> n((size_t)N + 1, 0.0);
  for (uint32_t i = 1; i <= N; i++) n[i] = (double)hist[i];
  const FitResult f = fit_censored(n.data(), N, n_threads > 0 ? n_threads : default_threads());
  if (f.domain) return BSQ_ERR_DATA;

  // fit_coverage_distribution (src/breseq/coverage_distribution.cpp:341-396)
  const double m = f.average, v = f.variance;
  double cutoff;
  uint64_t q;
  if (f.mu > 0) {
    if (!qnbinom_mu(deletion_propagation_pr_cutoff, f.size, f.mu, &q)) return BSQ_ERR_DATA;
    cutoff = (double)(uint32_t)q;
  } else {
    const double size_estimate = (1.0 / (v - m)) * m * m;
    if ((size_estimate > 0) && std::isfinite(size_estimate)) {
      if (!qnbinom_mu(deletion_propagation_pr_cutoff, size_estimate, m, &q)) return BSQ_ERR_DATA;
      cutoff = (double)(uint32_t)q;
    } else {
      cutoff = -1;
    }
    if (!(cutoff >= 1)) cutoff = m * 0.1;
  }
  if (cutoff < 1) cutoff = 1;
  if ((f.mu <= 3) && (m <= 3)) cutoff = -1;

  out->nbinom_size = f.size;
  out->nbinom_mean = f.mu;
  if (f.mu != 0) {   // the summary's derived parameters (coverage_distribution.cpp:570-581)
    out->nbinom_prob = f.size / (f.mu + f.size);
    out->nbinom_variance = f.mu + pow(f.mu, 2) / f.size;
    out->nbinom_relative_variance = out->nbinom_variance / f.mu;
  }
  out->average = f.average;
  out->variance = f.variance;
  out->relative_variance = f.relative_variance;
  out->deletion_coverage_propagation_cutoff = cutoff;
  out->nbinom_scale = f.scale;
  out->censor_start = f.censor_start;
  out->censor_end = f.censor_end;
  out->restarts_converged = f.converged;
  return BSQ_OK;
}

extern "C" int bsq_fit_negative_binomial(const double* n, uint32_t max_index, int n_threads, double* size, double* mu) {
  if (!n || !size || !mu) return BSQ_ERR_INVALID;
  const FitResult f = fit_censored(n, max_index, n_threads > 0 ? n_threads : default_threads());
  if (f.domain) return BSQ_ERR_DATA;
  *size = f.size;
  *mu = f.mu;
  return (f.size > 0.0 && f.mu > 0.0) ? 1 : 0;
}

extern "C" double bsq_nbinom_pmf(double k, double size, double mu) {
  if (!(size > 0) || !(mu > 0)) return NAN;
  return dnbinom_mu(k, size, mu);
}

extern "C" double bsq_nbinom_cdf(double k, double size, double p) {
  if (!(p >= 0.0 && p <= 1.0) || !(k >= 0)) return NAN;
  return nbdtr(k, size, p);
}

extern "C" int bsq_nbinom_quantile(double target_pr, double size, double mu, uint64_t* k) {
  if (!k || !(target_pr >= 0.0 && target_pr <= 1.0) || !(size > 0) || !(mu > 0)) return BSQ_ERR_INVALID;
  return qnbinom_mu(target_pr, size, mu, k) ? BSQ_OK : BSQ_ERR_DATA;
}
