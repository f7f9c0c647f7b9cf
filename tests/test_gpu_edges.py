"""Edge cases of the scoring path against the oracle: no records, every record filtered, many small
targets (every contig end an edge, many coverage groups)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests import compare, samples

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def _both(scorer, s, poly=False, precision=1):
    from breseq_gb300.api import ImSettings
    ec_o = po.error_count(s)
    tab = po.counts_to_log10_prob(ec_o["counts"], s.n_read_files, s.n_quality)
    im_o = po.identify(s, tab, po.default_im_params(s, polymorphism_mode=poly))
    sid = scorer.load_sample(s)
    try:
        ec_g = scorer.error_count(sid, hist_capacity=ec_o["hist"].shape[1])
        im_g = scorer.identify_mutations(sid, tab, ImSettings(polymorphism_prediction=poly), precision=precision,
                                         positions=True)
    finally:
        scorer.free_sample(sid)
    return ec_o, ec_g, im_o, im_g


def _check(ec_o, ec_g, im_o, im_g):
    assert np.array_equal(ec_g["counts"], ec_o["counts"])
    assert np.array_equal(ec_g["hist_size"], ec_o["hist_size"])
    assert np.array_equal(ec_g["hist"], ec_o["hist"])
    problems = compare.compare_ra(im_g["ra"], im_o["ra"]) + compare.compare_intervals(im_g, im_o)
    problems += compare.compare_positions(im_g["positions"], im_o["positions"])
    assert not problems, "\n".join(problems[:20])


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_no_records(scorer, oracle_lib, precision):
    """A reference with no reads: zero counts, no RA, and the state machines' view of zero coverage."""
    s = samples.empty_reads(samples.clonal_small())
    ec_o, ec_g, im_o, im_g = _both(scorer, s, precision=precision)
    _check(ec_o, ec_g, im_o, im_g)
    assert ec_g["counts"].sum() == 0 and len(im_g["ra"]) == 0


def test_every_record_filtered(scorer, oracle_lib):
    """Duplicates are dropped by the pileup's default filter: the same as no records."""
    s = samples.all_filtered(samples.clonal_small())
    ec_o, ec_g, im_o, im_g = _both(scorer, s)
    _check(ec_o, ec_g, im_o, im_g)
    assert ec_g["counts"].sum() == 0


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_many_small_targets(scorer, oracle_lib, precision):
    s = samples.many_targets()
    ec_o, ec_g, im_o, im_g = _both(scorer, s, precision=precision)
    _check(ec_o, ec_g, im_o, im_g)
    assert len(im_g["ra"]) > 0
