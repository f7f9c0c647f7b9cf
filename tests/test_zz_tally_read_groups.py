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
