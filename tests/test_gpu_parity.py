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


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_batch_equals_single_calls(scorer, loaded, oracle_results, precision):
    """Every sample scored in one batch (one launch per kernel over all samples' tiles) gets the
    results it gets alone, in both passes, and the oracle's."""
    from breseq_gb300.api import ImSettings
    names = list(samples.ALL) + ["clonal_small"]          # a sample may appear twice in one batch
    sids = [loaded[n] for n in names]
    cap = max(oracle_results[n][0]["hist"].shape[1] for n in names)
    ecs = scorer.error_count_batch(sids, hist_capacity=cap)
    for n, ec in zip(names, ecs):
        alone = scorer.error_count(loaded[n], hist_capacity=cap)
        for k in ("counts", "hist", "hist_size"):
            assert np.array_equal(ec[k], alone[k]), (n, k)
        assert np.array_equal(ec["counts"], oracle_results[n][0]["counts"])
    tabs = [oracle_results[n][1] for n in names]
    sets = [ImSettings(polymorphism_prediction=n in POLY) for n in names]
    ims = scorer.identify_mutations_batch(sids, tabs, sets, precision=precision, positions=False)
    for n, im, tab, st in zip(names, ims, tabs, sets):
        alone = scorer.identify_mutations(loaded[n], tab, st, precision=precision, positions=False)
        assert all(compare.identical(im[k], alone[k]) for k in ("ra", "mc", "un")), n
        problems = compare.compare_ra(im["ra"], oracle_results[n][2]["ra"]) + compare.compare_intervals(im, oracle_results[n][2])
        assert not problems, "\n".join(problems[:20])
    dense = scorer.identify_mutations_batch(sids[:2], tabs[:2], sets[:2], precision=precision, positions=True)
    for n, im in zip(names[:2], dense):
        assert not compare.compare_positions(im["positions"], oracle_results[n][2]["positions"])


def test_batch_larger_than_one_launch_group(scorer, loaded, oracle_results):
    """More samples than one launch carries (64 jobs per kernel parameter block) run as consecutive
    groups; every job still gets the single-call result."""
    from breseq_gb300.api import ImSettings
    names = ["clonal_small", "population_small"] * 35
    sids = [loaded[n] for n in names]
    ecs = scorer.error_count_batch(sids)
    tabs = [oracle_results[n][1] for n in names]
    sets = [ImSettings(polymorphism_prediction=n in POLY) for n in names]
    ims = scorer.identify_mutations_batch(sids, tabs, sets, precision=1)
    for n in set(names):
        alone_ec = scorer.error_count(loaded[n])
        alone = scorer.identify_mutations(loaded[n], oracle_results[n][1], ImSettings(polymorphism_prediction=n in POLY),
                                          precision=1)
        for i in [i for i, m in enumerate(names) if m == n]:
            assert np.array_equal(ecs[i]["counts"], alone_ec["counts"]), i
            assert np.array_equal(ecs[i]["hist"], alone_ec["hist"]), i
            assert all(compare.identical(ims[i][k], alone[k]) for k in ("ra", "mc", "un")), i


def test_graphs_and_launch_shapes_do_not_change_results(scorer, loaded, oracle_results):
    """Graph capture on/off, several launch shapes and the autotuner's pick give bit-identical
    results (integer counts; every column and candidate is scored by one warp whatever the grid)."""
    from breseq_gb300.api import ImSettings
    names = list(samples.ALL)
    sids = [loaded[n] for n in names]
    tabs = [oracle_results[n][1] for n in names]
    sets = [ImSettings(polymorphism_prediction=n in POLY) for n in names]
    default = scorer.tuning()

    def run():
        ecs = scorer.error_count_batch(sids)
        ims = scorer.identify_mutations_batch(sids, tabs, sets, precision=1)
        return ecs, ims

    base_ec, base_im = run()
    shapes = [dict(use_graphs=0), dict(use_graphs=1),
              dict(ec_read_chunk=256, ec_blocks_per_sm=2, col_blocks_per_sm=3, cand_warps_per_sm=4, bound_warps_per_sm=1),
              dict(ec_read_chunk=4096, ec_blocks_per_sm=12, col_blocks_per_sm=12, cand_warps_per_sm=32,
                   bound_warps_per_sm=8, use_graphs=0)]
    try:
        for sh in shapes:
            scorer.set_tuning(**sh)
            for _ in range(2):           # the second call updates the kept graph in place
                ecs, ims = run()
                for a, b in zip(ecs, base_ec):
                    assert np.array_equal(a["counts"], b["counts"]) and np.array_equal(a["hist"], b["hist"]), sh
                for a, b in zip(ims, base_im):
                    assert all(compare.identical(a[k], b[k]) for k in ("ra", "mc", "un")), sh
        chosen = scorer.autotune(sids, tabs, sets)
        assert chosen == scorer.tuning()
        ecs, ims = run()
        for a, b in zip(ims, base_im):
            assert all(compare.identical(a[k], b[k]) for k in ("ra", "mc", "un"))
    finally:
        scorer.set_tuning(**default)


@pytest.mark.parametrize("bad", [b"X", b"\0", b"a"])
def test_reference_characters_checked_at_load(scorer, bad):
    """A reference byte outside A/C/G/T/N (including a NUL inside a target, or lower case) is a
    data error at load; the sample is not kept."""
    import dataclasses
    from breseq_gb300 import _lib
    s = samples.clonal_small()
    ref = s.ref_seq.copy()
    ref[1000] = bad[0]
    with pytest.raises(_lib.BsqError) as e:
        scorer.load_sample(dataclasses.replace(s, ref_seq=ref))
    assert e.value.code == -3


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32c"])
def test_dp_group_first_column_skip(scorer, oracle_lib, precision):
    """A non-proper paired read without a usable XP tag in a discordant-pair read group is left out of
    its first column at insert position 0 (identify_mutations.cpp:1399-1416): RA items, intervals and
    per-position arrays against the oracle, with DP groups on every read group."""
    from breseq_gb300.api import ImSettings
    s = samples.dp_skip_sample()
    dp = tuple(0 for _ in range(int(s.read_group.max()) + 1))
    assert len(samples.dp_skip_reads(s, dp)) > 20
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    im_o = po.identify(s, tab, po.default_im_params(s, dp_group=dp))
    plain = po.identify(s, tab, po.default_im_params(s))
    assert not np.array_equal(plain["positions"]["unique_top"], im_o["positions"]["unique_top"])
    sid = scorer.load_sample(s)
    try:
        for positions in (True, False):
            im_g = scorer.identify_mutations(sid, tab, ImSettings(dp_group=dp), precision=precision, positions=positions)
            problems = compare.compare_ra(im_g["ra"], im_o["ra"]) + compare.compare_intervals(im_g, im_o)
            if positions:
                problems += compare.compare_positions(im_g["positions"], im_o["positions"])
            assert not problems, "\n".join(problems[:20])
    finally:
        scorer.free_sample(sid)
