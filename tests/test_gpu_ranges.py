"""One sample split by position range over two ranks (breseq_gb300.shard.score_ranges), each rank
scoring its range on the GPU through its own Scorer, against the whole sample scored on the GPU in one
call.  The two rank processes share this run's one GPU; their kernels never wait on each other (the
ranks exchange only host tensors over gloo).  Counts, histograms and MC / UN must be identical, RA
items identical within the parity tolerances (FP32-compensated column sums may add in another order
where a range's read batches start elsewhere)."""
import os
import pickle
import socket

import numpy as np
import pytest

from breseq_gb300 import shard
from tests import compare, samples

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir, prop):
    import torch.distributed as dist

    from breseq_gb300.api import Scorer
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    with Scorer(0) as sc:
        res = shard.score_ranges(shard.RangeScorer(sc), samples.ecoli_small(), rank, world,
                                 deletion_propagation_cutoff=prop, deletion_seed_cutoff=2.0)
    with open(os.path.join(out_dir, f"r{rank}.pkl"), "wb") as f:
        pickle.dump(res, f)
    dist.destroy_process_group()


def test_two_ranks_by_position_equal_one_gpu_call(built_lib, tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    from breseq_gb300.api import ImSettings, Scorer
    s = samples.ecoli_small()
    prop = np.array([12.0, -1.0, 25.0])
    mp.spawn(_rank, args=(2, _free_port(), str(tmp_path), prop), nprocs=2, join=True)
    with Scorer(0) as sc:
        sid = sc.load_sample(s)
        ec = sc.error_count(sid)
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im = sc.identify_mutations(sid, tab, ImSettings(), deletion_propagation_cutoff=prop, deletion_seed_cutoff=2.0,
                                   positions=True)
    for r in (pickle.load(open(tmp_path / f"r{k}.pkl", "rb")) for k in range(2)):
        assert np.array_equal(r["counts"], ec["counts"])
        w = r["hist"].shape[1]
        assert np.array_equal(r["hist"], ec["hist"][:, :w]) and not ec["hist"][:, w:].any()
        assert np.array_equal(r["table"], tab)
        problems = compare.compare_ra(r["ra"], im["ra"]) + compare.compare_intervals(r, im)
        assert not problems, problems[:5]
        for k in ("unique_top", "unique_bot", "raw_redundant_top", "raw_redundant_bot", "n_scored"):
            assert np.array_equal(r["positions"][k], im["positions"][k])
