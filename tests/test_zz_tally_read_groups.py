"""identify_mutations' coverage tally per read group on the GPU (bsq_im_coverage_columns_rg,
bsq_write_coverage_table_rg) against the CPU oracle: columns identical (counts exact, the 1/X1 weights
summed in record order on both sides) and the written <seq_id>.coverage.tsv byte-identical."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.test_coverage_table import IM_INT, IM_RED, im_read_groups

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


@pytest.mark.parametrize("failed", [False, True], ids=["pileup", "failed_fit"])
def test_im_tally_columns(scorer, failed):
    s = im_read_groups()
    sid = scorer.load_sample(s)
    try:
        for t in range(len(s.target_offset) - 1):
            n = int(s.target_offset[t + 1] - s.target_offset[t])
            for g, (a, b) in [(-1, (1, n)), (0, (1, n)), (1, (1, n)), (2, (1, n)), (1, (n // 3, n // 2))]:
                got = scorer.im_coverage_columns(sid, t, a, b, read_group=g, coverage_fit_failed=failed)
                o = po.im_coverage_columns(s, t, a, b, read_group=g, coverage_fit_failed=failed)
                for k in IM_INT + IM_RED:
                    assert np.array_equal(got[k], o[k]), (t, g, a, b, k)
    finally:
        scorer.free_sample(sid)


def test_im_coverage_tables(scorer, tmp_path):
    # the aggregate columns from pass 2's arrays (the same arrays on both sides), each group's from the
    # device tally; one read group writes the aggregate columns alone
    s = im_read_groups()
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    p = po.default_im_params(s)
    p["deletion_propagation_cutoff"][1] = -1.0
    pos = po.identify(s, tab, p)["positions"]
    sid = scorer.load_sample(s)
    try:
        for t in range(len(s.target_offset) - 1):
            for n_rg in (3, 1):
                pg, po_ = str(tmp_path / f"g{t}_{n_rg}.tsv"), str(tmp_path / f"o{t}_{n_rg}.tsv")
                scorer.write_coverage_table(sid, pg, t, pos, n_read_groups=n_rg, coverage_fit_failed=t == 1)
                po.write_coverage_table(s, po_, t, pos, n_read_groups=n_rg, coverage_fit_failed=t == 1)
                assert open(pg).read() == open(po_).read(), (t, n_rg)
    finally:
        scorer.free_sample(sid)


def test_im_tally_discordant_pair_skip(scorer):
    # two paired read groups with a discordant-pair group on the first: that group's records without a
    # usable XP tag leave their first column's tally, the other group's do not
    from tests import samples
    s = samples.dp_two_groups()
    sid = scorer.load_sample(s)
    try:
        differs = False
        for t in range(len(s.target_offset) - 1):
            n = int(s.target_offset[t + 1] - s.target_offset[t])
            for g in (-1, 0, 1):
                got = scorer.im_coverage_columns(sid, t, 1, n, read_group=g, dp_group=(0, -1))
                o = po.im_coverage_columns(s, t, 1, n, read_group=g, dp_group=(0, -1))
                plain = po.im_coverage_columns(s, t, 1, n, read_group=g)
                for k in IM_INT + IM_RED:
                    assert np.array_equal(got[k], o[k]), (t, g, k)
                differs |= any(not np.array_equal(o[k], plain[k]) for k in IM_INT)
        assert differs
    finally:
        scorer.free_sample(sid)


def test_im_coverage_table_in_chunks(scorer, tmp_path):
    # a chromosome of 1.16 Mb is written in two chunks of positions per read group
    import dataclasses
    from breseq_gb300.api import ImSettings
    from tests import samples
    s = samples.ecoli_quarter()
    g = np.where(np.random.default_rng(7).random(len(s.read_group)) < 0.3, 1, 0).astype(np.uint16)
    s = dataclasses.replace(s, read_group=g)
    assert int(s.target_offset[1] - s.target_offset[0]) > 1 << 20
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    sid = scorer.load_sample(s)
    try:
        pos = scorer.identify_mutations(sid, tab, ImSettings(), positions=True)["positions"]
        pg, po_ = str(tmp_path / "g.tsv"), str(tmp_path / "o.tsv")
        scorer.write_coverage_table(sid, pg, 0, pos, n_read_groups=2)
        po.write_coverage_table(s, po_, 0, pos, n_read_groups=2)
        assert open(pg).read() == open(po_).read()
    finally:
        scorer.free_sample(sid)
