"""The oracle against breseq's own output files.

tests/golden/ref/<case>.json holds what breseq's error_count() and identify_mutations() -- the
reference's unmodified sources, compiled by oracle/ref_build.py with the clean-room htslib subset --
wrote for a seeded sample (tests/golden/make_ref_golden.py): error_rates.tab, base_qual_error_prob.*.tab,
the unique-only coverage distributions and their negative-binomial fits, the stage-08 ra_mc_evidence.gd,
the same after test_RA_evidence, the coverage tables and the discordant-pair candidate regions, and on
one case the soft-clipping counts and BAM2COV tables.  The oracle's own
writers must reproduce every one of them byte for byte (files over 16 KB are compared by SHA-256).
Where the reference tree is present, the fixtures are also checked to be current."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import ra_output as ro
from tests import samples

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref")
SMALL = ["clonal_small", "ecoli_small", "ecoli_small_failed_fit", "population_small", "dp_groups",
         "ecoli_quarter", "population_deep", "softclip_bam2cov", "dp_two_groups"]
DP_HEADER = "seq_id,start,end,strand,orientation,length,max_discordant_count,redundant,discordant_pairs\n"


def load(case):
    with open(os.path.join(GOLDEN, f"{case}.json")) as f:
        return json.load(f)


def same(want, text):
    if "text" in want:
        return want["text"] == text
    return want["sha256"] == hashlib.sha256(text.encode()).hexdigest()


def dp_setup(st, nfiles):
    """DP groups as identify_mutations_pileup's constructor builds them (identify_mutations.cpp:883-911):
    per read-file set, a group when it is paired with a paired-mapping-distance fit of median > 0."""
    fits = {g: (med, mad) for g, med, mad in st.get("pmdd", [])}
    dp, widths, r1, r2, flat = [], [], [], [], 0
    for g in range(len(nfiles)):
        f = fits.get(g)
        if nfiles[g] == 2 and f and f[0] > 0:
            dp.append(len(widths))
            widths.append(f[0] + 2.42 * f[1])
            r1.append(flat + 1)
            r2.append(flat + 2)
        else:
            dp.append(-1)
        flat += nfiles[g]
    return dp, widths, r1, r2


def sc_summary_text(sm):
    """The harness's soft_clipping_summary.txt for a bsq_sc_summary dict (the Summary::soft_clipping fields)."""
    def g(x):
        return "%.17g" % x
    return (f"total_spanning_read_bases {sm['total_spanning_read_bases']}\n"
            f"total_clipped_read_ends {sm['total_clipped_read_ends']}\n"
            f"total_agreeing_clipped_read_ends {sm['total_agreeing_clipped_read_ends']}\n"
            f"soft_clipping_rate {g(sm['soft_clipping_rate'])}\nsoft_clipping_null_rate {g(sm['null_rate'])}\n"
            f"soft_clipping_dispersion {g(sm['dispersion'])}\nsoft_clipping_pearson_phi {g(sm['pearson_phi'])}\n"
            f"soft_clipping_tested_positions {sm['tested_positions']}\n"
            f"soft_clipping_trimmed_positions {sm['trimmed_positions']}\n"
            f"soft_clipping_mean_tested_reads {g(sm['mean_tested_reads'])}\n")


def sc_counts_text(s, result, tmp_path):
    """soft_clipping_counts.tab from a tabulation result, written by the library's host writer."""
    import ctypes as C

    from breseq_gb300 import _lib, abi
    L = _lib.load()
    p = abi.ScParams()
    assert L.bsq_default_sc_params(C.byref(p)) == 0
    sm = abi.ScSummary(**result["summary"])
    rows = (abi.ScPosition * max(1, len(result["rows"])))()
    for i, x in enumerate(result["rows"]):
        rows[i] = abi.ScPosition(*[x[k] for k in abi.SC_ROW_DTYPE.names])
    names = (C.c_char_p * len(s.target_names))(*[n.encode() for n in s.target_names])
    path = str(tmp_path / "soft_clipping_counts.tab")
    assert L.bsq_write_soft_clipping_counts(path.encode(), names, C.byref(p), C.byref(sm), rows, len(result["rows"])) == 0
    return open(path).read()


def coverage_fit_text(r):
    """The harness's coverage_fit.<g>.txt for a bsq_coverage_fit dict (fit_coverage_distribution's result)."""
    def g(x):
        return "%.17g" % x
    return (f"nbinom_size {g(r['nbinom_size'])}\nnbinom_mean {g(r['nbinom_mean'])}\naverage {g(r['average'])}\n"
            f"variance {g(r['variance'])}\nrelative_variance {g(r['relative_variance'])}\n"
            f"deletion_coverage_propagation_cutoff {g(r['deletion_coverage_propagation_cutoff'])}\n"
            f"censor_start {r['censor_start']}\ncensor_end {r['censor_end']}\nnbinom_scale {g(r['nbinom_scale'])}\n")


def coverage_fit_inputs(s, ec):
    """Per coverage group: the unique-only histogram error_count wrote and breseq's cutoff probability,
    0.05 / sqrt(the group's total length) (coverage_distribution.cpp:545)."""
    out = []
    for g in range(s.n_coverage_groups):
        length = sum(int(s.target_offset[t + 1] - s.target_offset[t]) for t in range(len(s.target_names))
                     if int(s.coverage_group[t]) == g)
        out.append((ec["hist"][g][: int(ec["hist_size"][g])], length, 0.05 / np.sqrt(float(length))))
    return out


def bam2cov_region(s, region):
    seq, rng = region.split(":")
    a, b = (int(x) for x in rng.split("-"))
    return s.target_names.index(seq), a, b


def oracle_files(fx, tmp_path):
    """The files the reference wrote, as the oracle's restatement writes them."""
    from breseq_gb300 import synth
    st = fx["settings"]
    s = getattr(samples, st["sample"])()
    assert samples.sample_digest(s) == fx["sample_digest"], "the seeded sample differs from the fixture's"
    poly = st.get("polymorphism", False)
    T = len(s.target_names)
    prop = np.ascontiguousarray(np.broadcast_to(np.asarray(st.get("prop_cutoff", 5.0), dtype=np.float64), (T,)))
    R, Q = s.n_read_files, s.n_quality
    ec = po.error_count(s)
    counts = np.ascontiguousarray(ec["counts"], dtype=np.uint64)
    tab = po.counts_to_log10_prob(counts, R, Q)
    out = {"error_rates.tab": ro.error_rates_text(counts, R, Q, tab)}
    _, _, nfiles = synth.bam_groups(s)
    names = [f"rg{g}_{f + 1}" for g in range(len(nfiles)) for f in range(nfiles[g])]
    for name, text in zip(names, ro.base_qual_texts(counts, R, Q)):
        out[f"base_qual_error_prob.{name}.tab"] = text
    for g in range(s.n_coverage_groups):
        h = np.ascontiguousarray(ec["hist"][g], dtype=np.uint64)
        out[f"{g}.unique_only_coverage_distribution.tab"] = ro.coverage_distribution_text(h, int(ec["hist_size"][g]))
    for g, (h, _, cut) in enumerate(coverage_fit_inputs(s, ec)):
        out[f"coverage_fit.{g}.txt"] = coverage_fit_text(po.fit_coverage_distribution(h, cut))
    dp, widths, r1, r2 = dp_setup(st, nfiles)
    p = po.default_im_params(s, polymorphism_mode=poly, prop_cutoff=prop, dp_group=tuple(dp) if widths else ())
    im = po.identify(s, tab, p)
    places = 8 if poly else 3
    out["ra_mc_evidence.gd"] = ro.gd_text(s, prop, places, im["ra"], None, im["mc"], im["un"])
    calls = ro.classify_all(im["ra"], s, ro.settings(poly))
    out["ra_mc_evidence.classified.gd"] = ro.gd_text(s, prop, places, im["ra"], calls, im["mc"], im["un"])
    for t in s.target_order:
        path = str(tmp_path / f"{s.target_names[t]}.coverage.tsv")
        po.write_coverage_table(s, path, int(t), im["positions"], n_read_groups=len(nfiles),
                                coverage_fit_failed=bool(prop[t] < 0), dp_group=dp if widths else ())
        out[f"08_mutation_identification/{s.target_names[t]}.coverage.tsv"] = open(path).read()
    dp_file = "08_mutation_identification/DP_candidate_regions.csv"
    if s.xp is not None:
        from breseq_gb300.api import PairSettings
        ps = PairSettings(dp_group=tuple(dp), window_width=tuple(widths), r1_prefix=tuple(r1), r2_prefix=tuple(r2))
        dpath, mpath = str(tmp_path / "dp.csv"), str(tmp_path / "mp.csv")
        po.pair_candidates(s, ps, dpath, mpath, deletion_propagation_cutoff=prop)
        out[dp_file] = open(dpath).read()
    else:   # no DP group: the header line alone
        out[dp_file] = DP_HEADER
    if st.get("softclip"):
        r = po.soft_clipping(s)
        out["soft_clipping_counts.tab"] = sc_counts_text(s, r, tmp_path)
        out["soft_clipping_summary.txt"] = sc_summary_text(r["summary"])
    for name, region, res, fmt, tot, prg in st.get("bam2cov", []):
        tid, a, b = bam2cov_region(s, region)
        path = str(tmp_path / name)
        po.write_coverage_region(s, path, tid, a, b, resolution=res, total_only=bool(tot), csv=fmt == "csv",
                                 per_read_group=bool(prg))
        out["bam2cov/" + name] = open(path).read()
    return out


@pytest.mark.parametrize("case", SMALL)
def test_oracle_matches_reference_files(oracle_lib, built_lib, tmp_path, case):
    fx = load(case)
    got = oracle_files(fx, tmp_path)
    assert sorted(got) == sorted(fx["files"])
    for name, want in fx["files"].items():
        assert same(want, got[name]), f"{case}: {name} differs from breseq's own output"


@pytest.mark.parametrize("case", SMALL)
def test_library_coverage_fit_matches_reference(oracle_lib, built_lib, case):
    """bsq_fit_coverage_distribution (host code, all host threads) against breseq's own fit of the same
    histograms."""
    from breseq_gb300 import api
    fx = load(case)
    s = getattr(samples, fx["settings"]["sample"])()
    ec = po.error_count(s)
    for g, (h, length, _) in enumerate(coverage_fit_inputs(s, ec)):
        assert same(fx["files"][f"coverage_fit.{g}.txt"], coverage_fit_text(api.fit_coverage_distribution(h, length)))


def test_fixtures_are_current():
    """Reruns breseq's own code on one small case where the reference tree is available."""
    from oracle import ref_build, ref_run
    if ref_build.ref_src() is None:
        pytest.skip("reference sources not available")
    fx = load("ecoli_small")
    st = fx["settings"]
    s = getattr(samples, st["sample"])()
    out = ref_run.run(s, polymorphism=st.get("polymorphism", False), copy_number=True, classify=True, covfit=True)
    out["ra_mc_evidence.classified.gd"] = "".join(
        l for l in out["ra_mc_evidence.classified.gd"].splitlines(True) if not l.startswith("#=TITLE"))
    assert sorted(out) == sorted(fx["files"])
    for name, want in fx["files"].items():
        assert same(want, out[name]), name
