"""Soft-clipping tabulation on the GPU (bsq_soft_clipping) against the CPU oracle: rows and summary
identical (integer counts and tails bit-exact, the fit's doubles bit-exact since both sides run the
same arithmetic in the same row order)."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from breseq_gb300 import _lib, abi
from breseq_gb300.api import ScSettings
from oracle import pyoracle as po
from tests import samples

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def check(scorer, s, **kw):
    sid = scorer.load_sample(s)
    try:
        g = scorer.soft_clipping(sid, ScSettings(**kw))
    finally:
        scorer.free_sample(sid)
    o = po.soft_clipping(s, **kw)
    assert g["summary"] == o["summary"]
    assert g["rows"].shape == o["rows"].shape
    assert np.array_equal(g["rows"], o["rows"])
    return g


def test_known_answers(scorer):
    s, expected = samples.softclip_known()
    g = check(scorer, s, minimum_clipped_bases=4)
    got = [(s.target_names[r["target"]], int(r["position"]), int(r["direction"]), int(r["clipped_count"]),
            int(r["total_count"]), int(r["agree_count"]), r["clipped_sequence"].decode()) for r in g["rows"]]
    assert got == expected


SETTINGS = [
    {},
    dict(minimum_clipped_bases=0),
    dict(minimum_clipped_bases=1),
    dict(minimum_clipped_bases=5),
    dict(minimum_clipped_bases=30),
    dict(minimum_clipped_bases=400),
    dict(consensus_base_fraction=0.0),
    dict(consensus_base_fraction=1.0),
    dict(dispersion_trim_frequency=0.0, maximum_dispersion=0.0),
    dict(maximum_dispersion=0.5, minimum_rate=0.0),
    dict(minimum_rate=0.5),
]


@pytest.mark.parametrize("kw", SETTINGS, ids=[",".join(f"{k}={v}" for k, v in d.items()) or "defaults" for d in SETTINGS])
def test_breakpoints_sample(scorer, kw):
    g = check(scorer, samples.softclip_sample(), **kw)
    if not kw:
        assert g["summary"]["n_positions"] > 100 and g["summary"]["trimmed_positions"] > 5


def test_unmapped_secondary_qcfail(scorer):
    check(scorer, samples.with_flags(samples.softclip_sample()))


@pytest.mark.parametrize("name", ["clonal_small", "ecoli_small", "population_small"])
def test_scoring_samples(scorer, name):
    check(scorer, samples.ALL[name](), minimum_clipped_bases=3)


def test_many_targets(scorer):
    check(scorer, samples.many_targets(), minimum_clipped_bases=0)


def test_empty_and_filtered(scorer):
    s = samples.softclip_sample()
    g = check(scorer, samples.empty_reads(s))
    assert g["summary"]["n_positions"] == 0 and g["summary"]["total_spanning_read_bases"] == 0
    # duplicates: the pileup keeps none, the tabulation keeps all of them
    g = check(scorer, samples.all_filtered(s))
    assert g["summary"]["n_positions"] > 100


def test_repeat_calls_and_other_passes_between(scorer):
    s = samples.softclip_sample()
    sid = scorer.load_sample(s)
    try:
        a = scorer.soft_clipping(sid)
        scorer.error_count(sid)
        b = scorer.soft_clipping(sid)
        c = scorer.soft_clipping(sid, ScSettings(minimum_clipped_bases=2))
        d = scorer.soft_clipping(sid)
    finally:
        scorer.free_sample(sid)
    assert a["summary"] == b["summary"] == d["summary"]
    assert np.array_equal(a["rows"], b["rows"]) and np.array_equal(a["rows"], d["rows"])
    assert c["summary"]["n_positions"] != a["summary"]["n_positions"]


def test_kept_record_past_target_is_an_error(scorer):
    s, _ = samples.softclip_known()
    pos, flag = s.pos.copy(), s.flag.copy()
    i = int(np.nonzero(s.tid == 0)[0][-1])
    pos[i] = 58
    flag[i] |= 0x100
    bad = dataclasses.replace(s, pos=pos, flag=flag)
    sid = scorer.load_sample(bad)          # the pileup skips a secondary record: the load accepts it
    try:
        with pytest.raises(_lib.BsqError) as e:
            scorer.soft_clipping(sid, ScSettings(minimum_clipped_bases=4))
        assert e.value.code == -1
    finally:
        scorer.free_sample(sid)
    with pytest.raises(po.OracleError):
        po.soft_clipping(bad, minimum_clipped_bases=4)


def test_argument_errors(scorer):
    s, _ = samples.softclip_known()
    sid = scorer.load_sample(s)
    L = _lib.load()
    try:
        p = abi.ScParams()
        L.bsq_default_sc_params(C.byref(p))
        out = abi.ScSummary()
        order = np.array([0, 0], dtype=np.uint32)
        p.target_name_order = abi.ptr(order, C.c_uint32)
        assert L.bsq_soft_clipping(scorer.ctx, sid, C.byref(p), C.byref(out)) == -1
        p.target_name_order = None
        p.consensus_base_fraction = 1.5
        assert L.bsq_soft_clipping(scorer.ctx, sid, C.byref(p), C.byref(out)) == -1
        p.consensus_base_fraction = 0.95
        assert L.bsq_soft_clipping(scorer.ctx, 987654, C.byref(p), C.byref(out)) == -6
        assert L.bsq_soft_clipping(scorer.ctx, sid, C.byref(p), C.byref(out)) == 0
        rows = (abi.ScPosition * 1)()
        if out.n_positions > 1:
            assert L.bsq_sc_result_copy(scorer.ctx, rows, 1) == -5
    finally:
        scorer.free_sample(sid)
