"""Generates stats_golden.json: two-sided Fisher 2x2 and one-sided two-sample K-S p-values from scipy.

breseq documents fisher_exact_test_2x2 as R's fisher.test(two.sided) and ks_test_two_sample_less as
R's ks.test(alternative = "less") with R's exact lattice method when m*n < 10000
(src/breseq/stats.cpp:2130-2143, 2206-2219).  scipy implements the same tests, so its values pin the
oracle's restatement of those two functions.  Run: python tests/golden/make_stats_golden.py
"""
import json
import os

import numpy as np
from scipy import stats

rng = np.random.default_rng(2024)
fisher = []
for a, b, c, d in [(0, 0, 0, 0), (3, 1, 1, 3), (10, 0, 0, 10), (1, 9, 11, 3), (0, 5, 50, 47), (25, 2, 40, 38),
                   (2, 0, 60, 58), (100, 90, 95, 110), (7, 12, 0, 1), (3, 3, 3, 3)]:
    p = stats.fisher_exact([[a, b], [c, d]], alternative="two-sided").pvalue
    fisher.append({"a": a, "b": b, "c": c, "d": d, "p": float(min(1.0, p))})
for _ in range(20):
    a, b, c, d = (int(x) for x in rng.integers(0, 60, size=4))
    p = stats.fisher_exact([[a, b], [c, d]], alternative="two-sided").pvalue
    fisher.append({"a": a, "b": b, "c": c, "d": d, "p": float(min(1.0, p))})
ks = []
for _ in range(20):
    nx, ny = int(rng.integers(1, 40)), int(rng.integers(1, 60))
    x = rng.normal(0.0, 1.0, nx) + float(rng.normal(0, 0.7))
    y = rng.normal(0.0, 1.0, ny)
    p = stats.ks_2samp(x, y, alternative="less", method="exact").pvalue
    ks.append({"x": x.tolist(), "y": y.tolist(), "p": float(p)})
out = {"source": "scipy " + __import__("scipy").__version__, "fisher": fisher, "ks_less": ks}
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "stats_golden.json"), "w") as f:
    json.dump(out, f, indent=1)
print("wrote", len(fisher), "fisher and", len(ks), "ks cases")
