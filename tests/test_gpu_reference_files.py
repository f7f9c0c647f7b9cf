"""The drop-in error_count() / identify_mutations() (include/breseq_gb300_dropin.h), run on the GPU,
against the files breseq's own code wrote for the same BAM (tests/golden/ref/, made by
tests/golden/make_ref_golden.py from the reference's unmodified sources).

tests/native/dropin_main.cpp reads the same config file as the reference's harness, so both write the
same files: error_rates.tab, base_qual_error_prob.*.tab, the unique-only coverage distributions, the
stage-08 ra_mc_evidence.gd (FP32-compensated sums, FP64 at the candidate columns), the coverage tables
and the discordant-pair candidate regions.  Every file must be byte-identical (files over 16 KB by
SHA-256).  The cases include the E. coli workload's shape at 0.25x genome length with its full 2 x 100x
coverage and the 1000x population shape at 0.05x genome length.  The test_RA_evidence classification
of the GPU's RA items, written by the library, is checked against the reference's classified file too."""
import ctypes as C
import glob
import json
import os
import subprocess

import numpy as np
import pytest

from tests import samples

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CASES = sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(HERE, "golden", "ref", "*.json")))


@pytest.fixture(scope="module")
def dropin_exe(built_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_main")
    lib_dir = os.path.dirname(built_lib)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-o", out, os.path.join(HERE, "native", "dropin_main.cpp"),
                           "-L" + lib_dir, "-lbsq_gb300", "-Wl,-rpath," + lib_dir])
    return out


@pytest.mark.parametrize("case", CASES)
def test_dropin_writes_the_reference_files(dropin_exe, tmp_path, case):
    import hashlib
    from oracle import ref_run
    with open(os.path.join(HERE, "golden", "ref", f"{case}.json")) as f:
        fx = json.load(f)
    st = fx["settings"]
    s = getattr(samples, st["sample"])()
    assert samples.sample_digest(s) == fx["sample_digest"], "the seeded sample differs from the fixture's"
    cfg, out = ref_run.write_inputs(s, str(tmp_path), polymorphism=st.get("polymorphism", False),
                                    prop_cutoff=st.get("prop_cutoff"), copy_number=True,
                                    pmdd=[tuple(x) for x in st.get("pmdd", [])], fast_bam=True)
    r = subprocess.run([dropin_exe, cfg], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr[-3000:]
    got = ref_run.read_outputs(out)
    # the drop-in covers the two passes; the classified GenomeDiff, the soft-clipping and BAM2COV files are
    # checked by the tests below, the coverage fits (host code) by tests/test_ref_golden.py
    want = {k: v for k, v in fx["files"].items()
            if k != "ra_mc_evidence.classified.gd" and not k.startswith(("soft_clipping", "bam2cov/", "coverage_fit."))}
    assert sorted(got) == sorted(want)
    bad = []
    for name, w in want.items():
        text = got[name]
        ok = w["text"] == text if "text" in w else w["sha256"] == hashlib.sha256(text.encode()).hexdigest()
        if not ok:
            bad.append(name)
    assert not bad, f"{case}: differ from breseq's own output: {bad}"


@pytest.mark.parametrize("case", [c for c in CASES if c in ("clonal_small", "ecoli_small", "population_small",
                                                             "dp_groups", "ecoli_quarter")])
def test_classified_genome_diff_matches_reference(built_lib, tmp_path, case):
    """RA items scored on the GPU, classified by bsq_test_ra_evidence and written by bsq_write_gd, against
    the reference's test_RA_evidence output."""
    from breseq_gb300 import _lib, abi, synth
    from breseq_gb300.api import ImSettings, Scorer
    with open(os.path.join(HERE, "golden", "ref", f"{case}.json")) as f:
        fx = json.load(f)
    st = fx["settings"]
    s = getattr(samples, st["sample"])()
    poly = st.get("polymorphism", False)
    T = len(s.target_names)
    prop = np.ascontiguousarray(np.broadcast_to(np.asarray(st.get("prop_cutoff", 5.0), dtype=np.float64), (T,)))
    _, _, nfiles = synth.bam_groups(s)
    from tests.test_ref_golden import dp_setup
    dp, widths, _, _ = dp_setup(st, nfiles)
    L = _lib.load()
    with Scorer(0) as sc:
        sid = sc.load_sample(s)
        ec = sc.error_count(sid)
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im = sc.identify_mutations(sid, tab, ImSettings(polymorphism_prediction=poly, dp_group=tuple(dp) if widths else ()),
                                   deletion_propagation_cutoff=prop, precision=1)
    rs = abi.RaSettings()
    assert L.bsq_default_ra_settings(int(poly), C.byref(rs)) == 0
    view = abi.SampleView(s)
    names = (C.c_char_p * T)(*[n.encode() for n in s.target_names])
    ra = abi.ra_from_dicts(im["ra"])
    calls = (abi.RaCall * max(1, len(im["ra"])))()
    assert L.bsq_test_ra_evidence(C.cast(ra, C.c_void_p), len(im["ra"]), C.byref(rs), C.byref(view.ref), names,
                                  C.cast(calls, C.c_void_p)) == 0
    mc, un = abi.mc_from_dicts(im["mc"]), abi.un_from_dicts(im["un"])
    path = str(tmp_path / "classified.gd")
    assert L.bsq_write_gd(path.encode(), C.byref(view.ref), names, abi.ptr(prop, C.c_double), rs.polymorphism_precision_places,
                          C.cast(ra, C.c_void_p), len(im["ra"]), C.cast(calls, C.c_void_p), C.cast(mc, C.c_void_p),
                          len(im["mc"]), C.cast(un, C.c_void_p), len(im["un"])) == 0
    import hashlib
    want, text = fx["files"]["ra_mc_evidence.classified.gd"], open(path).read()
    assert want["text"] == text if "text" in want else want["sha256"] == hashlib.sha256(text.encode()).hexdigest()


@pytest.mark.parametrize("case", [c for c in CASES if c == "softclip_bam2cov"])
def test_soft_clipping_and_bam2cov_match_reference(built_lib, tmp_path, case):
    """tabulate_soft_clipping_counts and `breseq BAM2COV` tables computed on the GPU (bsq_soft_clipping,
    bsq_write_coverage_region_rg) against breseq's own files."""
    import hashlib
    from breseq_gb300.api import Scorer
    from tests.test_ref_golden import bam2cov_region, sc_counts_text, sc_summary_text
    with open(os.path.join(HERE, "golden", "ref", f"{case}.json")) as f:
        fx = json.load(f)
    st = fx["settings"]
    s = getattr(samples, st["sample"])()
    assert samples.sample_digest(s) == fx["sample_digest"]

    def same(name, text):
        w = fx["files"][name]
        return w["text"] == text if "text" in w else w["sha256"] == hashlib.sha256(text.encode()).hexdigest()

    with Scorer(0) as sc:
        sid = sc.load_sample(s)
        r = sc.soft_clipping(sid)
        assert same("soft_clipping_counts.tab", sc_counts_text(s, r, tmp_path))
        assert same("soft_clipping_summary.txt", sc_summary_text(r["summary"]))
        for name, region, res, fmt, tot, prg in st["bam2cov"]:
            tid, a, b = bam2cov_region(s, region)
            path = str(tmp_path / name)
            sc.write_coverage_region(sid, path, tid, a, b, resolution=res, total_only=bool(tot), csv=fmt == "csv",
                                     per_read_group=bool(prg))
            assert same("bam2cov/" + name, open(path).read()), name
