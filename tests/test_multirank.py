"""The N>1 host path on CPU: two gloo ranks plan the same jobs without communicating, score
disjoint shares that cover every job, and agree on the slowest rank's time."""
import os
import socket

import pytest

from breseq_gb300 import shard
from tests import compare


def test_plan_covers_and_balances():
    work = [5, 1, 9, 3, 3, 7, 2, 8, 1, 4]
    for world in (1, 2, 3, 4):
        p = shard.plan(work, world)
        flat = sorted(i for r in p for i in r)
        assert flat == list(range(len(work)))
        loads = [sum(work[i] for i in r) for r in p]
        assert max(loads) - min(loads) <= max(work)
    assert shard.plan(work, 2) == shard.plan(list(work), 2)   # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, work, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.plan(work, world)[rank]
    fake_ms = 10.0 * (rank + 1) + sum(work[i] for i in mine) * 1e-3
    slow = shard.slowest(fake_ms)
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{','.join(map(str, mine))};{fake_ms!r};{slow!r}\n")
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    work = [300, 120, 80, 75, 60, 40, 22, 9]
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), work, str(tmp_path)), nprocs=world, join=True)
    shares, times, slows = [], [], []
    for r in range(world):
        a, b, c = open(tmp_path / f"rank{r}.txt").read().strip().split(";")
        shares.append([int(x) for x in a.split(",") if x])
        times.append(float(b))
        slows.append(float(c))
    assert sorted(i for s in shares for i in s) == list(range(len(work)))
    assert not set(shares[0]) & set(shares[1])
    assert slows[0] == slows[1] == max(times)


# ---------------------------------------------------------------------------- one sample by position range
class OracleRanges:
    """score_ranges' backend restated by the CPU oracle (test infrastructure; the product backend is
    shard.RangeScorer over a GPU Scorer)."""

    def counts(self, sample):
        from oracle import pyoracle as po
        return po.error_count(sample)["counts"]

    def coverage(self, sample, tid, start_1, end_1):
        from oracle import pyoracle as po
        return po.coverage_columns(sample, tid, start_1, end_1)

    def identify(self, sample, table, settings, prop, seed):
        from oracle import pyoracle as po
        return po.identify(sample, table, po.default_im_params(sample, prop_cutoff=prop, seed_cutoff=seed))


def _range_sample():
    from tests import samples
    return samples.ecoli_small()


def _range_rank(rank, world, port, out_dir, prop):
    import pickle

    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    res = shard.score_ranges(OracleRanges(), _range_sample(), rank, world, deletion_propagation_cutoff=prop,
                             deletion_seed_cutoff=2.0)
    with open(os.path.join(out_dir, f"range{rank}.pkl"), "wb") as f:
        pickle.dump(res, f)
    dist.destroy_process_group()


def _whole(s, prop):
    from oracle import pyoracle as po
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    return ec, tab, po.identify(s, tab, po.default_im_params(s, prop_cutoff=prop, seed_cutoff=2.0))


def test_plan_ranges_cover_every_column():
    s = _range_sample()
    for world in (1, 2, 3, 5):
        rs = shard.plan_ranges(s, world)
        assert rs[0][0] == 0 and rs[-1][1] == int(s.target_offset[-1])
        assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
    # every record is owned by exactly one range, and the halo holds every record reaching the range
    import numpy as np
    start, end = shard._columns(s)
    rs = shard.plan_ranges(s, 3)
    owned = sum(shard.subsample(s, a, b, owned=True).n_reads for a, b in rs)
    assert owned == s.n_reads
    for a, b in rs:
        assert shard.subsample(s, a, b).n_reads == int(np.count_nonzero((start < b) & (end > a)))


def test_one_rank_stitching_equals_oracle(oracle_lib, built_lib):
    """world 1: the stitched MC / UN (bsq_intervals_from_positions over the per-position arrays) equal the
    oracle's own state machines; counts, histogram and calls equal the oracle's."""
    import numpy as np
    s = _range_sample()
    prop = np.array([12.0, -1.0, 25.0])
    ec, tab, im = _whole(s, prop)
    res = shard.score_ranges(OracleRanges(), s, 0, 1, deletion_propagation_cutoff=prop, deletion_seed_cutoff=2.0)
    assert np.array_equal(res["counts"], ec["counts"])
    assert np.array_equal(res["table"], tab)
    assert len(im["mc"]) > 3
    assert not compare.compare_intervals(res, im)
    assert not compare.compare_ra(res["ra"], im["ra"], score_tol=0.0, freq_tol=0.0)


def test_two_gloo_ranks_by_position_equal_one(oracle_lib, built_lib, tmp_path):
    """Two gloo ranks, each scoring its position range (owned reads for the counts, halo reads for the
    columns), all-reduce the integer counts and histograms and stitch MC / UN: the result equals the whole
    sample scored in one place."""
    import pickle

    import numpy as np
    mp = pytest.importorskip("torch.multiprocessing")
    s = _range_sample()
    prop = np.array([12.0, -1.0, 25.0])
    mp.spawn(_range_rank, args=(2, _free_port(), str(tmp_path), prop), nprocs=2, join=True)
    res = [pickle.load(open(tmp_path / f"range{r}.pkl", "rb")) for r in range(2)]
    ec, tab, im = _whole(s, prop)
    for r in res:
        assert np.array_equal(r["counts"], ec["counts"])
        h = ec["hist"][:, :r["hist"].shape[1]]
        assert np.array_equal(r["hist"], h) and not ec["hist"][:, r["hist"].shape[1]:].any()
        assert list(r["hist_size"]) == list(ec["hist_size"])
        assert np.array_equal(r["table"], tab)
        assert not compare.compare_ra(r["ra"], im["ra"], score_tol=0.0, freq_tol=0.0)
        assert not compare.compare_intervals(r, im)
        for k in ("unique_top", "unique_bot", "raw_redundant_top", "n_scored"):
            assert np.array_equal(r["positions"][k], im["positions"][k])
    assert res[0]["range"][1] == res[1]["range"][0]
