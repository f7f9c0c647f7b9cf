"""Coverage-distribution fit (bsq_fit_coverage_distribution, host code) against the oracle's
restatement, bit for bit, and the negative-binomial special functions against scipy's (Cephes /
R-equivalent) implementations.  No GPU needed."""
import ctypes as C
import math

import numpy as np
import pytest

from breseq_gb300 import _lib, abi
from breseq_gb300.api import fit_coverage_distribution
from oracle import pyoracle as po


def nb_hist(seed, mu, size, n_pos, deleted_fraction=0.0, repeat_fraction=0.0):
    """A unique-only coverage histogram: negative-binomial depths, optionally a deleted stretch (depth 0)
    and a high-depth shoulder."""
    rng = np.random.default_rng(seed)
    cov = rng.negative_binomial(size, size / (size + mu), n_pos)
    cov[: int(n_pos * deleted_fraction)] = 0
    k = int(n_pos * repeat_fraction)
    if k:
        cov[-k:] = rng.negative_binomial(size, size / (size + 2 * mu), k) * 2
    return np.bincount(cov).astype(np.uint64)


def same(a: dict, b: dict):
    for k in a:
        x, y = a[k], b[k]
        assert (x == y) or (x != x and y != y), f"{k}: {x!r} != {y!r}"


CASES = [
    # (seed, mu, size, positions, deleted, repeat)
    (1, 30, 20, 48502, 0.01, 0.0),          # lambda-sized genome
    (2, 125, 15, 200_000, 0.0, 0.02),
    (3, 1000, 30, 300_000, 0.005, 0.0),     # 1000x window: [~500, ~1500], one bin per depth
    (4, 3000, 25, 200_000, 0.0, 0.0),       # window wider than 2000: coarse-grained, mean rescaled
    (5, 8, 5, 50_000, 0.0, 0.0),
    (6, 4, 0.8, 20_000, 0.0, 0.0),          # over-dispersed, low depth
    (7, 60, 2, 100_000, 0.1, 0.0),
    (8, 2.5, 50, 10_000, 0.0, 0.0),         # mean below 3
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"mu{c[1]}-size{c[2]}")
def test_fit_matches_oracle(built_lib, oracle_lib, case):
    seed, mu, size, n_pos, dele, rep = case
    h = nb_hist(seed, mu, size, n_pos, dele, rep)
    pr = 0.05 / math.sqrt(n_pos)
    got = fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr)
    exp = po.fit_coverage_distribution(h, pr)
    same(got, exp)
    if got["nbinom_mean"] > 0:
        assert got["restarts_converged"] > 0
        assert got["nbinom_prob"] == got["nbinom_size"] / (got["nbinom_mean"] + got["nbinom_size"])
    if mu >= 30:     # well-sampled unimodal histograms: the fit recovers the generating mean
        assert got["nbinom_mean"] == pytest.approx(mu, rel=0.05)


def test_fit_thread_count_invariant(built_lib):
    h = nb_hist(11, 200, 12, 150_000)
    pr = 0.05 / math.sqrt(150_000)
    base = fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr, n_threads=1)
    for t in (2, 7, 48):
        same(fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr, n_threads=t), base)


def test_fit_sequence_length_cutoff(built_lib):
    h = nb_hist(12, 90, 20, 80_000)
    a = fit_coverage_distribution(h, sequence_length=4_790_000)
    b = fit_coverage_distribution(h, deletion_propagation_pr_cutoff=0.05 / math.sqrt(4_790_000))
    same(a, b)


@pytest.mark.parametrize("hist", [
    [],                      # no histogram (no covered position)
    [5],                     # only depth 0
    [0, 10],                 # one depth: no window (start == end)
    [0, 0, 0, 7],
    [3, 1, 0, 0, 0, 0, 0],   # a single covered position
    [0, 4, 9, 3, 1],         # fewer than five depths: no smoothing
    [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 5],
], ids=lambda h: "h" + "-".join(map(str, h)) if h else "empty")
def test_fit_degenerate(built_lib, oracle_lib, hist):
    h = np.array(hist, dtype=np.uint64)
    got = fit_coverage_distribution(h, deletion_propagation_pr_cutoff=1e-3)
    same(got, po.fit_coverage_distribution(h, 1e-3))
    assert got["deletion_coverage_propagation_cutoff"] == -1 or got["deletion_coverage_propagation_cutoff"] >= 1


def test_fit_known_answers(built_lib):
    # no covered position: all zero, the sequences count as deleted (coverage_distribution.cpp:389-391)
    f = fit_coverage_distribution(np.zeros(0, dtype=np.uint64), deletion_propagation_pr_cutoff=1e-3)
    assert f["average"] == 0 and f["nbinom_mean"] == 0 and f["deletion_coverage_propagation_cutoff"] == -1
    # ten positions at depth 1: mean 1, variance 0, no window; the moment fallback fails (size < 0), the
    # 10%-of-mean fallback gives 0.1, raised to 1, then -1 because mean <= 3
    f = fit_coverage_distribution(np.array([0, 10], dtype=np.uint64), deletion_propagation_pr_cutoff=1e-3)
    assert (f["average"], f["variance"], f["censor_start"], f["censor_end"]) == (1.0, 0.0, 0, 0)
    assert f["deletion_coverage_propagation_cutoff"] == -1
    # the window is [floor(peak / 2), ceil(1.5 peak)] around the peak of the 5-point moving average
    h = nb_hist(21, 50, 40, 100_000)
    f = fit_coverage_distribution(h, deletion_propagation_pr_cutoff=1e-4)
    ma = np.convolve(h.astype(np.float64), np.ones(5) / 5, mode="same")
    peak = 3 + int(np.argmax(ma[3:len(h) - 2]))
    assert (f["censor_start"], f["censor_end"]) == (peak // 2, math.ceil(1.5 * peak))
    assert 1 <= f["deletion_coverage_propagation_cutoff"] < 50


def test_fit_random_histograms(built_lib, oracle_lib):
    rng = np.random.default_rng(5)
    for _ in range(12):
        n = int(rng.integers(2, 400))
        h = rng.integers(0, 50, n).astype(np.uint64) * (rng.random(n) < 0.6)
        pr = float(10 ** rng.uniform(-6, -1))
        same(fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr), po.fit_coverage_distribution(h, pr))


# ------------------------------------------------------------------ special functions

def _lib_fn():
    return _lib.load()


def test_special_functions_match_oracle(built_lib, oracle_lib):
    L = _lib_fn()
    rng = np.random.default_rng(7)
    for _ in range(400):
        size = float(10 ** rng.uniform(-2, 5))
        mu = float(10 ** rng.uniform(-1, 4))
        k = float(rng.integers(0, 5000))
        assert L.bsq_nbinom_pmf(k, size, mu) == po.special("nbinom_pmf", k, size, mu)
        p = size / (size + mu)
        assert L.bsq_nbinom_cdf(k, size, p) == po.special("nbinom_cdf", k, size, p)


def test_special_functions_vs_scipy(oracle_lib):
    sp = pytest.importorskip("scipy.special")
    st = pytest.importorskip("scipy.stats")
    xs = np.concatenate([np.linspace(0.05, 13, 120), np.geomspace(13, 1e9, 120)])
    for x in xs:
        ref = float(sp.gammaln(x))
        for name in ("lgam", "lngamma"):
            assert po.special(name, x) == pytest.approx(ref, rel=1e-13, abs=1e-14), (name, x)
    for x in np.linspace(0.1, 170, 200):
        assert po.special("gamma", x) == pytest.approx(float(sp.gamma(x)), rel=1e-12)
    rng = np.random.default_rng(3)
    for _ in range(300):
        size = float(10 ** rng.uniform(-1, 4))
        mu = float(10 ** rng.uniform(0, 3.5))
        p = size / (size + mu)
        k = float(rng.integers(0, int(3 * mu) + 5))
        assert po.special("nbinom_pmf", k, size, mu) == pytest.approx(float(st.nbinom.pmf(k, size, p)), rel=1e-9,
                                                                      abs=1e-300)
        # P(X <= k) = I_p(size, k + 1), the regularised incomplete beta integral
        assert po.special("nbinom_cdf", k, size, p) == pytest.approx(float(sp.betainc(size, k + 1, p)), rel=1e-9,
                                                                      abs=1e-300)


def test_quantile_vs_scipy(built_lib):
    st = pytest.importorskip("scipy.stats")
    L = _lib_fn()
    rng = np.random.default_rng(9)
    for _ in range(150):
        size = float(10 ** rng.uniform(-0.5, 3))
        mu = float(10 ** rng.uniform(0, 3))
        q = float(10 ** rng.uniform(-7, -0.1))
        k = C.c_uint64()
        assert L.bsq_nbinom_quantile(q, size, mu, C.byref(k)) == 0
        # R's qnbinom: the smallest k with P(X <= k) >= q
        p = size / (size + mu)
        exp = int(st.nbinom.ppf(q, size, p))
        cdf_k = float(st.nbinom.cdf(k.value, size, p))
        if exp != k.value:   # only a CDF value within rounding of q may place the step differently
            assert abs(cdf_k - q) < 1e-9 * q or abs(float(st.nbinom.cdf(exp, size, p)) - q) < 1e-9 * q
    assert L.bsq_nbinom_quantile(0.0, 5.0, 10.0, C.byref(k)) == 0 and k.value == 0
    assert L.bsq_nbinom_quantile(1.5, 5.0, 10.0, C.byref(k)) == -1
    assert L.bsq_nbinom_quantile(0.5, 0.0, 10.0, C.byref(k)) == -1


def test_fit_negative_binomial_wrapper(built_lib):
    L = _lib_fn()
    h = nb_hist(31, 300, 18, 120_000).astype(np.float64)
    size, mu = C.c_double(), C.c_double()
    rc = L.bsq_fit_negative_binomial(abi.ptr(h, C.c_double), h.size - 1, 0, C.byref(size), C.byref(mu))
    assert rc == 1 and mu.value == pytest.approx(300, rel=0.05)
    f = fit_coverage_distribution(h.astype(np.uint64), deletion_propagation_pr_cutoff=1e-4)
    assert (size.value, mu.value) == (f["nbinom_size"], f["nbinom_mean"])
