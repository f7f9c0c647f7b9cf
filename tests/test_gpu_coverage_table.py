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
