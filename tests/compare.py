"""Comparison of CUDA-path results with the oracle's, at the tolerances of the scoring path:
integer counts, coverage and call sets bit-exact; log10 E-values (scores) within 1e-3 absolute;
frequencies and bounds within 1e-4 absolute; strand / quality-bias p-values within 1e-6 relative."""
import math

import numpy as np

SCORE_TOL = 1e-3
FREQ_TOL = 1e-4


def _close(a, b, tol):
    if a is None or b is None:
        return a == b
    if math.isnan(a) or math.isnan(b):
        return math.isnan(a) and math.isnan(b)
    return abs(a - b) <= tol


def call_key(r):
    return (r["tid"], r["position"], r["insert_position"], r["ref_base"], r["new_base"], r["major_base"],
            r["minor_base"], bool(r["passed_consensus"]), bool(r["passed_polymorphism"]))


def compare_ra(gpu, ref, score_tol=SCORE_TOL, freq_tol=FREQ_TOL):
    """Returns a list of human-readable mismatches (empty when identical within tolerance)."""
    out = []
    gk = [call_key(r) for r in gpu]
    rk = [call_key(r) for r in ref]
    if gk != rk:
        gs, rs = set(gk), set(rk)
        out.append(f"call set differs: only GPU {sorted(gs - rs)[:5]} only oracle {sorted(rs - gs)[:5]}")
        return out
    for g, r in zip(gpu, ref):
        where = f"{r['tid']}:{r['position']}+{r['insert_position']}"
        for k in ("score", "consensus_score"):
            if not _close(g[k], r[k], score_tol):
                out.append(f"{where} {k} {g[k]} vs {r[k]}")
        for k in ("frequency", "major_frequency", "frequency_lower", "frequency_upper"):
            if not _close(g[k], r[k], freq_tol):
                out.append(f"{where} {k} {g[k]} vs {r[k]}")
        for b in range(5):
            if not _close(g["f"][b], r["f"][b], freq_tol):
                out.append(f"{where} f[{b}] {g['f'][b]} vs {r['f'][b]}")
        for k in ("ref_cov", "new_cov", "major_cov", "minor_cov", "total_cov", "n"):
            if g[k] != r[k]:
                out.append(f"{where} {k} {g[k]} vs {r[k]}")
        for k in ("fisher_strand_p", "ks_quality_p"):
            if not _close(g[k], r[k], 1e-6 * max(1e-300, abs(r[k])) + 1e-15):
                out.append(f"{where} {k} {g[k]} vs {r[k]}")
    return out


def compare_intervals(g, r):
    out = []
    if [(m["tid"], m["start"], m["end"], m["start_range"], m["end_range"]) for m in g["mc"]] != \
       [(m["tid"], m["start"], m["end"], m["start_range"], m["end_range"]) for m in r["mc"]]:
        out.append(f"MC differ: {g['mc'][:3]} vs {r['mc'][:3]}")
    else:
        for a, b in zip(g["mc"], r["mc"]):
            for k in ("left_outside_cov", "left_inside_cov", "right_inside_cov", "right_outside_cov"):
                if not _close(a[k], b[k], 0.0):
                    out.append(f"MC {k} {a[k]} vs {b[k]}")
    if g["un"] != r["un"]:
        out.append(f"UN differ: {len(g['un'])} vs {len(r['un'])}: {g['un'][:3]} vs {r['un'][:3]}")
    return out


def compare_positions(g, r, exact_scores=False):
    out = []
    for k in ("unique_top", "unique_bot", "raw_redundant_top", "raw_redundant_bot", "n_scored"):
        if not np.array_equal(g[k], r[k]):
            bad = np.nonzero(g[k] != r[k])[0]
            out.append(f"{k} differs at {len(bad)} positions, first {bad[:5]}")
    for k in ("redundant_top", "redundant_bot"):
        if not np.array_equal(g[k], r[k]):
            out.append(f"{k} not bit-identical (max diff {np.nanmax(np.abs(g[k] - r[k]))})")
    gs, rs = g["consensus_score"], r["consensus_score"]
    both = ~np.isnan(rs)
    if not np.array_equal(np.isnan(gs), np.isnan(rs)):
        out.append("consensus score NaN pattern differs")
    else:
        d = np.abs(gs[both] - rs[both])
        if d.size and d.max() > SCORE_TOL:
            out.append(f"consensus score max abs diff {d.max()} at {np.nonzero(both)[0][np.argmax(d)]}")
    if not np.array_equal(g["best_base"], r["best_base"]):
        bad = np.nonzero(g["best_base"] != r["best_base"])[0]
        out.append(f"best base differs at {len(bad)} positions, first {bad[:5]}")
    return out


def _same(a, b):
    if isinstance(a, float) and isinstance(b, float):
        return a == b or (math.isnan(a) and math.isnan(b))
    if isinstance(a, (list, tuple)) and isinstance(b, (list, tuple)):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    if isinstance(a, dict) and isinstance(b, dict):
        return a.keys() == b.keys() and all(_same(a[k], b[k]) for k in a)
    return a == b


def identical(a, b):
    """Exact equality of record lists (bit-identical floats, NaN equal to NaN)."""
    return _same(a, b)
