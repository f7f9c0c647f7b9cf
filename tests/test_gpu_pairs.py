"""Discordant-pair / missing-pair candidate regions on the GPU (bsq_pair_candidates): the written
CSV files identical to the oracle's position-by-position walk, for samples loaded from arrays and
from BAM bytes."""
import os

import numpy as np
import pytest

from breseq_gb300 import _lib, synth
from breseq_gb300.api import PairSettings
from oracle import pyoracle as po
from tests.test_pairs import ecoli_pairs, pd_settings, two_groups

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def gpu_files(sc, sid, s, st, tmp_path, cutoff=None):
    r = sc.pair_candidates(sid, st, cutoff)
    f = [str(tmp_path / x) for x in ("dp.csv", "mp.csv", "pd.csv")]
    pd = st.predict_pair_distance
    sc.write_pair_candidates(r, f[0], f[1], s.target_names, f[2] if pd else None)
    return [open(x).read() for x in (f if pd else f[:2])], r


def oracle_files(s, st, tmp_path, cutoff=None):
    f = [str(tmp_path / x) for x in ("odp.csv", "omp.csv", "opd.csv")]
    pd = st.predict_pair_distance
    po.pair_candidates(s, st, f[0], f[1], cutoff, f[2] if pd else None)
    return [open(x).read() for x in (f if pd else f[:2])]


def test_pairs_ecoli(scorer, tmp_path):
    s = ecoli_pairs()
    st = PairSettings(dp_group=(0,), window_width=(462.75,), predict_missing_pairs=True)
    sid = scorer.load_sample(s)
    got, r = gpu_files(scorer, sid, s, st, tmp_path)
    stats = scorer.last_pass_stats()
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path)
    assert len(r["dp"]) > 5 and len(r["mp"]) > 3 and stats["kernel_launches"] > 0


@pytest.mark.parametrize("dp_group,widths,seeds", [((0, 1), (300.5, 520.0), (3, 3, 0.25)),
                                                   ((-1, 0), (37.25,), (1, 2, 0.0)),
                                                   ((1, 0), (0.5, 2000.0), (0, 0, 0.5)),
                                                   ((0, 0), (1.0,), (6, 4, 1.0))])
def test_pairs_groups(scorer, tmp_path, dp_group, widths, seeds):
    s = two_groups()
    G = len(widths)
    st = PairSettings(dp_group=dp_group, window_width=widths, r1_prefix=tuple(1 + 2 * g for g in range(G)),
                      r2_prefix=tuple(2 + 2 * g for g in range(G)), discordant_pair_seed=seeds[0],
                      predict_missing_pairs=True, missing_pair_seed=seeds[1], missing_pair_seed_fraction=seeds[2])
    sid = scorer.load_sample(s)
    got, _ = gpu_files(scorer, sid, s, st, tmp_path)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path)


def test_pairs_targets_and_skips(scorer, tmp_path):
    import dataclasses
    s = dataclasses.replace(two_groups(seed=4), target_order=np.array([0, 2], dtype=np.uint32))
    st = PairSettings(dp_group=(0, 1), window_width=(350.0, 600.0), r1_prefix=(1, 3), r2_prefix=(2, 4),
                      predict_missing_pairs=True)
    cut = np.array([5.0, 5.0, -1.0])
    sid = scorer.load_sample(s)
    got, _ = gpu_files(scorer, sid, s, st, tmp_path, cut)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path, cut)


def test_pairs_from_bam(scorer, tmp_path):
    # the names, TLEN and XP tags decoded on the device give the same regions
    s = two_groups(seed=7)
    st = PairSettings(dp_group=(0, 1), window_width=(330.0, 480.5), r1_prefix=(1, 3), r2_prefix=(2, 4),
                      predict_missing_pairs=True, missing_pair_seed=2)
    sid = scorer.load_bam(synth.bam_bytes(s), s, synth.bam_groups(s))
    got, _ = gpu_files(scorer, sid, s, st, tmp_path)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path)


def test_pairs_need_annotations(scorer):
    s = synth.simulate(synth.config_ecoli(seed=5, scale=0.01))
    sid = scorer.load_sample(s)
    with pytest.raises(_lib.BsqError):
        scorer.pair_candidates(sid, PairSettings())
    scorer.free_sample(sid)
    bad = synth.with_pairs(s, seed=1)
    bad = bad.__class__(**{**bad.__dict__, "qname_off": bad.qname_off[::-1].copy()})
    with pytest.raises(_lib.BsqError):
        scorer.load_sample(bad)


def test_pd_ecoli(scorer, tmp_path):
    s = ecoli_pairs(seed=9, distance_sites=25)
    st = pd_settings(s)
    sid = scorer.load_sample(s)
    got, r = gpu_files(scorer, sid, s, st, tmp_path)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path)
    assert len(r["pd"]) > 2


@pytest.mark.parametrize("kw", [dict(pd_z_seed=1.0, pair_distance_seed=1), dict(pd_z_seed=2.6),
                                dict(pd_orientation=("",)), dict(pd_cdf=(None,))])
def test_pd_settings(scorer, tmp_path, kw):
    s = ecoli_pairs(scale=0.02, seed=10, distance_sites=10)
    st = pd_settings(s, **kw)
    sid = scorer.load_sample(s)
    got, _ = gpu_files(scorer, sid, s, st, tmp_path)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path)


def test_pd_from_bam_two_groups(scorer, tmp_path):
    import dataclasses
    s = two_groups(seed=11)
    s = dataclasses.replace(s, target_order=np.array([0, 2], dtype=np.uint32))
    s = synth.with_pairs(s, seed=11, distance_sites=6, no_xp_fraction=0.2, background_discordant=0.02)
    st = pd_settings(s, pd_cdf=(synth.pd_null(s), None), window_width=(300.5, 520.0), pd_z_seed=1.5)
    cut = np.array([5.0, 5.0, -1.0])
    sid = scorer.load_bam(synth.bam_bytes(s), s, synth.bam_groups(s))
    got, _ = gpu_files(scorer, sid, s, st, tmp_path, cut)
    scorer.free_sample(sid)
    assert got == oracle_files(s, st, tmp_path, cut)
