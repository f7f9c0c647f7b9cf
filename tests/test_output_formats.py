"""The library's output side (host code, no GPU needed) against the oracle restatement: RA
classification of test_RA_evidence, error_rates.tab, base_qual_error_prob, the unique-only coverage
distribution and the GenomeDiff file, byte for byte, on the oracle's results for the test samples."""
import ctypes as C
import functools
import os

import numpy as np
import pytest

from breseq_gb300 import _lib, abi
from oracle import pyoracle as po
from oracle import ra_output as ro
from tests import samples

POLY = {"population_small"}


@functools.lru_cache(maxsize=None)
def oracle_run(name, prop=None):
    s = samples.ALL[name]()
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    p = po.default_im_params(s, polymorphism_mode=name in POLY, prop_cutoff=prop)
    im = po.identify(s, tab, p, positions=False)
    return s, ec, tab, p, im


def lib_settings(L, poly, **over):
    st = abi.RaSettings()
    assert L.bsq_default_ra_settings(int(poly), C.byref(st)) == 0
    for k, v in over.items():
        setattr(st, k, v)
    return st


def lib_classify(L, s, ra, st):
    view = abi.SampleView(s)
    names = (C.c_char_p * len(s.target_names))(*[n.encode() for n in s.target_names])
    arr = abi.ra_from_dicts(ra)
    calls = (abi.RaCall * max(1, len(ra)))()
    assert L.bsq_test_ra_evidence(C.cast(arr, C.c_void_p), len(ra), C.byref(st), C.byref(view.ref), names,
                                  C.cast(calls, C.c_void_p)) == 0
    return [dict(deleted=bool(c.deleted), prediction=c.prediction.decode(), reject=c.reject.decode(),
                 consensus_reject=c.consensus_reject.decode(), polymorphism_reject=c.polymorphism_reject.decode())
            for c in calls[:len(ra)]], calls


FILTERS = [
    {},
    dict(consensus_reject_indel_homopolymer_length=2, polymorphism_reject_surrounding_homopolymer_length=3,
         polymorphism_ks_quality_p_value_cutoff=0.05),
    dict(consensus_minimum_variant_coverage_each_strand=30, consensus_minimum_total_coverage=120,
         polymorphism_minimum_total_coverage_each_strand=40, polymorphism_minimum_variant_coverage=3,
         polymorphism_no_indels=1, mutation_log10_e_value_cutoff=300.0),
]


@pytest.mark.parametrize("extra", range(len(FILTERS)))
@pytest.mark.parametrize("name", list(samples.ALL))
def test_ra_classification_matches_oracle(built_lib, oracle_lib, name, extra):
    L = _lib.load()
    s, _, _, _, im = oracle_run(name)
    poly = name in POLY
    for mode in (poly, not poly):
        over = FILTERS[extra]
        got, _ = lib_classify(L, s, im["ra"], lib_settings(L, mode, **over))
        want = ro.classify_all(im["ra"], s, ro.settings(mode, **over))
        assert got == want


def test_error_tables_and_coverage_distribution(built_lib, oracle_lib, tmp_path):
    L = _lib.load()
    s, ec, tab, _, _ = oracle_run("ecoli_small")
    R, Q = s.n_read_files, s.n_quality
    counts = np.ascontiguousarray(ec["counts"], dtype=np.uint64)
    path = str(tmp_path / "error_rates.tab")
    assert L.bsq_write_error_rates(path.encode(), abi.ptr(counts, C.c_uint64), R, Q) == 0
    assert open(path).read() == ro.error_rates_text(counts, R, Q, tab)
    names = (C.c_char_p * R)(*[f"reads_{i}".encode() for i in range(R)])
    pattern = str(tmp_path / "base_qual_error_prob.#.tab")
    assert L.bsq_write_base_qual_error_prob(pattern.encode(), names, abi.ptr(counts, C.c_uint64), R, Q) == 0
    for i, text in enumerate(ro.base_qual_texts(counts, R, Q)):
        assert open(pattern.replace("#", f"reads_{i}")).read() == text
    for g in range(s.n_coverage_groups):
        h = np.ascontiguousarray(ec["hist"][g], dtype=np.uint64)
        size = int(ec["hist_size"][g])
        p = str(tmp_path / f"{g}.unique_only_coverage_distribution.tab")
        assert L.bsq_write_coverage_distribution(p.encode(), abi.ptr(h, C.c_uint64), size) == 0
        assert open(p).read() == ro.coverage_distribution_text(h, size)


@pytest.mark.parametrize("name,prop", [("clonal_small", None), ("ecoli_small", (5.0, -1.0, 5.0)), ("population_small", None)])
def test_genome_diff_file_matches_oracle(built_lib, oracle_lib, tmp_path, name, prop):
    L = _lib.load()
    s, _, _, p, im = oracle_run(name, prop)
    poly = name in POLY
    st = lib_settings(L, poly)
    calls_d, calls = lib_classify(L, s, im["ra"], st)
    view = abi.SampleView(s)
    names = (C.c_char_p * len(s.target_names))(*[n.encode() for n in s.target_names])
    ra = abi.ra_from_dicts(im["ra"])
    mc = abi.mc_from_dicts(im["mc"])
    un = abi.un_from_dicts(im["un"])
    prop_arr = np.ascontiguousarray(p["deletion_propagation_cutoff"], dtype=np.float64)
    path = str(tmp_path / "ra_mc_evidence.gd")
    assert L.bsq_write_gd(path.encode(), C.byref(view.ref), names, abi.ptr(prop_arr, C.c_double), st.polymorphism_precision_places,
                          C.cast(ra, C.c_void_p), len(im["ra"]), C.cast(calls, C.c_void_p), C.cast(mc, C.c_void_p),
                          len(im["mc"]), C.cast(un, C.c_void_p), len(im["un"])) == 0
    want = ro.gd_text(s, prop_arr, st.polymorphism_precision_places, im["ra"], calls_d, im["mc"], im["un"])
    got = open(path).read()
    assert got == want
    lines = got.splitlines()
    assert lines[0] == "#=GENOME_DIFF\t1.0"
    ids = sorted(int(x.split("\t")[1]) for x in lines[1:])
    assert ids == list(range(1, len(lines)))
