"""Discordant-pair / missing-pair candidate regions on the GPU (bsq_pair_candidates): the written
CSV files identical to the oracle's position-by-position walk, for samples loaded from arrays and
from BAM bytes."""
import os

import numpy as np
import pytest

from breseq_gb300 import _lib, synth
from breseq_gb300.api import PairSettings
from oracle import pyoracle as po
from tests.test_pairs import ecoli_pairs, two_groups

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def gpu_files(sc, sid, s, st, tmp_path, cutoff=None):
    r = sc.pair_candidates(sid, st, cutoff)
    dp, mp = str(tmp_path / "dp.csv"), str(tmp_path / "mp.csv")
    sc.write_pair_candidates(r, dp, mp, s.target_names)
    return [open(dp).read(), open(mp).read()], r


def oracle_files(s, st, tmp_path, cutoff=None):
    dp, mp = str(tmp_path / "odp.csv"), str(tmp_path / "omp.csv")
    po.pair_candidates(s, st, dp, mp, cutoff)
    return [open(dp).read(), open(mp).read()]


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
