"""BAM2COV coverage table on the GPU (bsq_coverage_columns, bsq_write_coverage_region) against the
CPU oracle: columns identical (counts exact, the 1/X1 weights bit-identical, summed in record order
on both sides) and the written tables byte-identical."""
import dataclasses

import numpy as np
import pytest

from breseq_gb300 import _lib
from oracle import pyoracle as po
from tests import samples

pytestmark = pytest.mark.gpu

COLS = ("unique_top", "unique_bot", "redundant_top", "redundant_bot", "raw_redundant_top", "raw_redundant_bot",
        "unique_top_begin", "unique_bot_begin")


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def target_len(s, t):
    return int(s.target_offset[t + 1] - s.target_offset[t])


def check_columns(sc, sid, s, t, a, b):
    g = sc.coverage_columns(sid, t, a, b)
    o = po.coverage_columns(s, t, a, b)
    assert g["last"] == o["last"]
    for k in COLS:
        assert np.array_equal(g[k], o[k]), k
    return g


def regions(s):
    out = []
    for t in range(len(s.target_names)):
        L = target_len(s, t)
        out += [(t, 1, L), (t, 1, min(L, 700)), (t, max(1, L - 500), L), (t, L // 3, L // 3 + 1234 if L // 3 + 1234 <= L else L)]
    return out


@pytest.mark.parametrize("name", ["clonal_small", "ecoli_small", "population_small"])
def test_columns(scorer, name):
    s = samples.ALL[name]()
    sid = scorer.load_sample(s)
    try:
        for t, a, b in regions(s):
            g = check_columns(scorer, sid, s, t, a, b)
        if name == "ecoli_small":   # repeats: redundant weights present
            g = check_columns(scorer, sid, s, 0, 1, target_len(s, 0))
            assert g["raw_redundant_top"].any() and g["unique_bot_begin"].any()
    finally:
        scorer.free_sample(sid)


def test_columns_flags_and_targets_outside_the_pileup_set(scorer):
    # secondary / QC-failed / unmapped records are filtered; a target left out of the scoring
    # pileup's set is still tabulated
    s = samples.with_flags(samples.softclip_sample())
    s = dataclasses.replace(s, target_order=np.array([0], dtype=np.uint32))
    sid = scorer.load_sample(s)
    try:
        for t in range(3):
            check_columns(scorer, sid, s, t, 1, target_len(s, t))
    finally:
        scorer.free_sample(sid)


TABLES = [dict(resolution=600), dict(resolution=0), dict(resolution=7), dict(resolution=10**7),
          dict(resolution=600, total_only=True), dict(resolution=50, csv=True, reference_average=31.5)]


@pytest.mark.parametrize("kw", TABLES, ids=[",".join(f"{k}={v}" for k, v in d.items()) for d in TABLES])
def test_tables_identical(scorer, tmp_path, kw):
    s = samples.ecoli_small()
    sid = scorer.load_sample(s)
    try:
        for i, (t, a, b) in enumerate(regions(s)):
            pg, po_ = str(tmp_path / f"g{i}.tsv"), str(tmp_path / f"o{i}.tsv")
            scorer.write_coverage_region(sid, pg, t, a, b, **kw)
            po.write_coverage_region(s, po_, t, a, b, **kw)
            assert open(pg).read() == open(po_).read(), (t, a, b)
    finally:
        scorer.free_sample(sid)


def test_known_records_and_driver_rows(scorer, tmp_path):
    s, _ = samples.softclip_known()
    sid = scorer.load_sample(s)
    try:
        check_columns(scorer, sid, s, 0, 1, 60)
        check_columns(scorer, sid, s, 1, 1, 40)
        for t, a, b, res in [(0, 1, 60, 7), (1, 1, 40, 4), (1, 35, 40, 0), (1, 31, 40, 3), (0, 21, 21, 0)]:
            pg, po_ = str(tmp_path / "g.tsv"), str(tmp_path / "o.tsv")
            scorer.write_coverage_region(sid, pg, t, a, b, resolution=res)
            po.write_coverage_region(s, po_, t, a, b, resolution=res)
            assert open(pg).read() == open(po_).read(), (t, a, b, res)
    finally:
        scorer.free_sample(sid)


def test_region_errors(scorer):
    s, _ = samples.softclip_known()
    sid = scorer.load_sample(s)
    try:
        for t, a, b in [(2, 1, 10), (0, 0, 10), (0, 10, 9), (0, 1, 61)]:
            with pytest.raises(_lib.BsqError):
                scorer.coverage_columns(sid, t, a, b)
    finally:
        scorer.free_sample(sid)


def two_read_groups():
    from breseq_gb300 import synth
    cfg = synth.SimConfig(seed=13, target_lengths=(20_000, 3_000), target_names=("chrA", "chrB"), n_snps=5,
                          n_indels=2, max_indel=2, repeat_copies=3, repeat_length=400,
                          read_sets=(synth.ReadFileSet(coverage=30, read_length=101, paired=True),
                                     synth.ReadFileSet(coverage=20, read_length=150)))
    return synth.simulate(cfg)


RG_TABLES = [dict(resolution=0), dict(resolution=600, total_only=True), dict(resolution=7, csv=True),
             dict(resolution=0, n_read_groups=4)]


@pytest.mark.parametrize("kw", RG_TABLES, ids=[",".join(f"{k}={v}" for k, v in d.items()) for d in RG_TABLES])
def test_per_read_group_tables(scorer, tmp_path, kw):
    # --per-read-group: each read group's columns and averages after the aggregate ones; a header with
    # more groups than the records use prints zero columns for the others
    s = two_read_groups()
    sid = scorer.load_sample(s)
    try:
        for i, (t, a, b) in enumerate([(0, 1, 20_000), (0, 5_000, 9_000), (1, 1, 3_000)]):
            pg, po_ = str(tmp_path / f"g{i}.tsv"), str(tmp_path / f"o{i}.tsv")
            scorer.write_coverage_region(sid, pg, t, a, b, per_read_group=True, **kw)
            po.write_coverage_region(s, po_, t, a, b, per_read_group=True, **kw)
            assert open(pg).read() == open(po_).read(), (t, a, b)
    finally:
        scorer.free_sample(sid)


def test_per_read_group_columns(scorer):
    s = two_read_groups()
    sid = scorer.load_sample(s)
    try:
        for g in (0, 1):
            got = scorer.coverage_columns(sid, 0, 1, 20_000, read_group=g)
            keep = (s.read_group == g) | (s.tid != 0)
            import dataclasses
            o = po.coverage_columns(dataclasses.replace(s, flag=np.where(keep, s.flag, s.flag | 0x400).astype(np.uint16)),
                                    0, 1, 20_000)
            for k in COLS:
                assert np.array_equal(got[k], o[k]), (g, k)
    finally:
        scorer.free_sample(sid)
