"""CUDA path vs the CPU oracle on seeded samples, through the C ABI (breseq_gb300.api.Scorer)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests import compare, samples

pytestmark = pytest.mark.gpu

POLY = {"population_small"}


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


@pytest.fixture(scope="module")
def loaded(scorer):
    ids = {}
    for name, f in samples.ALL.items():
        ids[name] = scorer.load_sample(f())
    return ids


@pytest.fixture(scope="module")
def oracle_results(oracle_lib):
    res = {}
    for name, f in samples.ALL.items():
        s = f()
        ec = po.error_count(s)
        tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im = po.identify(s, tab, po.default_im_params(s, polymorphism_mode=name in POLY))
        res[name] = (ec, tab, im)
    return res


@pytest.mark.parametrize("name", list(samples.ALL))
def test_error_count_bit_exact(scorer, loaded, oracle_results, name):
    ec_o = oracle_results[name][0]
    ec_g = scorer.error_count(loaded[name], hist_capacity=ec_o["hist"].shape[1])
    assert np.array_equal(ec_g["counts"], ec_o["counts"])
    assert np.array_equal(ec_g["hist_size"], ec_o["hist_size"])
    assert np.array_equal(ec_g["hist"], ec_o["hist"])


@pytest.mark.parametrize("name", list(samples.ALL))
def test_log10_table_round_trip(scorer, oracle_results, name):
    s = samples.ALL[name]()
    ec_o, tab_o, _ = oracle_results[name]
    tab_g = scorer.counts_to_log10_prob(ec_o["counts"], s.n_read_files, s.n_quality)
    assert np.array_equal(tab_g, tab_o)


@pytest.mark.parametrize("positions", [True, False], ids=["dense", "sparse"])
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
@pytest.mark.parametrize("name", list(samples.ALL))
def test_identify_mutations_parity(scorer, loaded, oracle_results, name, precision, positions):
    """RA items, MC/UN intervals and (dense) per-position arrays against the oracle.  The sparse run
    returns no per-position arrays, and its MC/UN come from the marked columns only."""
    from breseq_gb300.api import ImSettings
    _, tab, im_o = oracle_results[name]
    im_g = scorer.identify_mutations(loaded[name], tab, ImSettings(polymorphism_prediction=name in POLY),
                                     precision=precision, positions=positions)
    problems = compare.compare_ra(im_g["ra"], im_o["ra"])
    problems += compare.compare_intervals(im_g, im_o)
    if positions:
        problems += compare.compare_positions(im_g["positions"], im_o["positions"])
    assert not problems, "\n".join(problems[:20])
    assert len(im_o["ra"]) > 0


def test_preprocess_stage(scorer, loaded, oracle_lib):
    s = samples.clonal_small()
    o = po.error_count(s, do_errors=False, preprocess=True)
    g = scorer.error_count(loaded["clonal_small"], do_errors=False, preprocess=True)
    assert np.array_equal(g["hist"][:, :o["hist"].shape[1]], o["hist"][:, :g["hist"].shape[1]])
    assert np.allclose(g["no_pos_hash_pr"], o["no_pos_hash_pr"], rtol=0, atol=0)


def test_failed_coverage_fit_target(scorer, loaded, oracle_results):
    """A target whose coverage fit failed (propagation cutoff < 0) gets coverage only and one MC."""
    from breseq_gb300.api import ImSettings
    s = samples.ecoli_small()
    _, tab, _ = oracle_results["ecoli_small"]
    prop = np.array([5.0, -1.0, 5.0])
    p = po.default_im_params(s, prop_cutoff=prop)
    im_o = po.identify(s, tab, p)
    for positions in (True, False):
        im_g = scorer.identify_mutations(loaded["ecoli_small"], tab, ImSettings(), deletion_propagation_cutoff=prop,
                                         precision=1, positions=positions)
        problems = compare.compare_ra(im_g["ra"], im_o["ra"]) + compare.compare_intervals(im_g, im_o)
        if positions:
            problems += compare.compare_positions(im_g["positions"], im_o["positions"])
        assert not problems, "\n".join(problems[:20])
        assert any(m["tid"] == 1 and m["start"] == 1 for m in im_g["mc"])


@pytest.mark.parametrize("prop_cutoff,seed_cutoff", [(12.0, 2.0), (25.0, 8.0)])
def test_intervals_with_deletion_cutoffs(scorer, loaded, oracle_results, prop_cutoff, seed_cutoff):
    """Higher deletion cutoffs open many MC candidates (30x sample), exercising the MC state machine
    (redundant-coverage ranges, seed reached or not) on both interval paths."""
    from breseq_gb300.api import ImSettings
    s = samples.ecoli_small()
    _, tab, _ = oracle_results["ecoli_small"]
    im_o = po.identify(s, tab, po.default_im_params(s, prop_cutoff=prop_cutoff, seed_cutoff=seed_cutoff))
    assert len(im_o["mc"]) > 5
    for positions in (True, False):
        im_g = scorer.identify_mutations(loaded["ecoli_small"], tab, ImSettings(), deletion_propagation_cutoff=prop_cutoff,
                                         deletion_seed_cutoff=seed_cutoff, precision=1, positions=positions)
        problems = compare.compare_intervals(im_g, im_o) + compare.compare_ra(im_g["ra"], im_o["ra"])
        assert not problems, "\n".join(problems[:20])
