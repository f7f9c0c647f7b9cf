"""Measured error of each output of pass 2, for both precision forms, against the FP64 oracle.

The chosen form (BSQ_PRECISION_FP32C) sums the per-position consensus likelihoods in Kahan-compensated
FP32 and recomputes every decision near a threshold in FP64; everything an RA item reports is
rescored in FP64.  This test prints the largest difference of every output over five samples --
the three parity samples and the two samples with the shapes of the E. coli clonal and 1000x
population workloads (0.24 and 0.26 G read-bases) -- and asserts each against its bound:

  output                                      bound (fp32c)   bound (fp64)
  per-position consensus score (log10)        2e-4            1e-9
  best base per position, call set, MC / UN   identical       identical
  counts and coverage                         identical       identical
  RA score, RA consensus score                1e-9            1e-9
  frequencies (f, major, frequency)           1e-12           1e-12
  frequency bounds                            1e-9            1e-9
  Fisher / KS p-values (relative)             1e-9            1e-9

Run with `-s` to see the table."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from tests import compare, samples

pytestmark = pytest.mark.gpu

CASES = {"clonal_small": False, "ecoli_small": False, "population_small": True, "ecoli_quarter": False,
         "population_deep": True}
BOUNDS = {
    1: dict(position_score=2e-4, ra_score=1e-9, frequency=1e-12, bounds=1e-9, p_rel=1e-9),
    0: dict(position_score=1e-9, ra_score=1e-9, frequency=1e-12, bounds=1e-9, p_rel=1e-9),
}


def _maxabs(pairs):
    m = 0.0
    for a, b in pairs:
        if a is None or b is None or (isinstance(a, float) and math.isnan(a)) or \
                (isinstance(b, float) and math.isnan(b)):
            assert (a is None) == (b is None) and (a is None or math.isnan(a) == math.isnan(b))
            continue
        m = max(m, abs(a - b))
    return m


def errors(g, o):
    """Largest differences of every output of one run against the oracle's."""
    gp, op = g["positions"], o["positions"]
    both = ~np.isnan(op["consensus_score"])
    assert np.array_equal(np.isnan(gp["consensus_score"]), ~both)
    d = np.abs(gp["consensus_score"][both] - op["consensus_score"][both])
    ra = list(zip(g["ra"], o["ra"]))
    rel = 0.0
    for a, b in ra:
        for k in ("fisher_strand_p", "ks_quality_p"):
            x, y = a[k], b[k]
            if math.isnan(x) or math.isnan(y):
                assert math.isnan(x) and math.isnan(y)
                continue
            rel = max(rel, abs(x - y) / max(abs(y), 1e-300))
    return dict(
        position_score=float(d.max()) if d.size else 0.0,
        ra_score=max(_maxabs((a["score"], b["score"]) for a, b in ra),
                     _maxabs((a["consensus_score"], b["consensus_score"]) for a, b in ra)),
        frequency=max([_maxabs((a[k], b[k]) for a, b in ra) for k in ("frequency", "major_frequency")] +
                      [_maxabs((a["f"][i], b["f"][i]) for a, b in ra) for i in range(5)]),
        bounds=max(_maxabs((a[k], b[k]) for a, b in ra) for k in ("frequency_lower", "frequency_upper")),
        p_rel=rel)


@pytest.fixture(scope="module")
def table(built_lib, oracle_lib):
    from breseq_gb300.api import ImSettings, Scorer
    rows = {}
    with Scorer(0) as sc:
        for name, poly in CASES.items():
            s = getattr(samples, name)()
            ec = po.error_count(s)
            tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
            o = po.identify(s, tab, po.default_im_params(s, polymorphism_mode=poly))
            sid = sc.load_sample(s)
            g_ec = sc.error_count(sid, hist_capacity=ec["hist"].shape[1])
            assert np.array_equal(g_ec["counts"], ec["counts"]) and np.array_equal(g_ec["hist"], ec["hist"])
            for precision in (0, 1):
                g = sc.identify_mutations(sid, tab, ImSettings(polymorphism_prediction=poly), precision=precision,
                                          positions=True)
                exact = [compare.call_key(r) for r in g["ra"]] == [compare.call_key(r) for r in o["ra"]]
                exact = exact and not compare.compare_intervals(g, o)
                gp, op = g["positions"], o["positions"]
                exact = exact and np.array_equal(gp["best_base"], op["best_base"])
                for k in ("unique_top", "unique_bot", "raw_redundant_top", "raw_redundant_bot", "n_scored"):
                    exact = exact and np.array_equal(gp[k], op[k])
                exact = exact and np.array_equal(gp["redundant_top"], op["redundant_top"]) and \
                    np.array_equal(gp["redundant_bot"], op["redundant_bot"])
                rows[(name, precision)] = dict(identical=exact, ra_items=len(o["ra"]), **errors(g, o))
            sc.free_sample(sid)
    print("\nsample            form   RA  identical  pos.score  RA score   freq       bounds     p (rel)")
    for (name, precision), r in rows.items():
        print(f"{name:17s} {'fp32c' if precision else 'fp64 ':5s} {r['ra_items']:5d} {str(r['identical']):9s}  "
              f"{r['position_score']:.2e}   {r['ra_score']:.2e}   {r['frequency']:.2e}   {r['bounds']:.2e}   "
              f"{r['p_rel']:.2e}")
    return rows


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
@pytest.mark.parametrize("name", list(CASES))
def test_max_error_within_bounds(table, name, precision):
    r = table[(name, precision)]
    assert r["identical"], f"{name}: call set, intervals, best bases or coverage differ from the oracle"
    assert r["ra_items"] > 0
    for k, bound in BOUNDS[precision].items():
        assert r[k] <= bound, f"{name} {'fp32c' if precision else 'fp64'}: {k} error {r[k]:.3e} above {bound:.0e}"
