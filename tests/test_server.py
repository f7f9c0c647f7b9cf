"""The scoring server (continuous batching with HBM-footprint admission): every job's result is the
same as the single-sample calls give for that sample alone, whatever the mix it ran in."""
import threading
import time

import numpy as np
import pytest

from breseq_gb300 import abi
from tests import compare, samples

POLY = {"population_small"}


def test_server_needs_a_device(built_lib):
    """Without a GPU, creating a server fails with an error code rather than a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from breseq_gb300 import _lib
    from breseq_gb300.api import Server
    with pytest.raises(_lib.BsqError):
        Server(0)


@pytest.fixture(scope="module")
def alone(built_lib):
    """Single-call results (fp32c) per sample, the reference for every mix."""
    from breseq_gb300.api import ImSettings, Scorer
    out = {}
    with Scorer(0) as sc:
        for name, f in samples.ALL.items():
            s = f()
            sid = sc.load_sample(s)
            ec = sc.error_count(sid)
            tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
            im = sc.identify_mutations(sid, tab, ImSettings(polymorphism_prediction=name in POLY), precision=1)
            out[name] = (s, ec, im)
    return out


def _check(res, ref):
    _, ec, im = ref
    assert np.array_equal(res["counts"], ec["counts"])
    assert np.array_equal(res["hist"], ec["hist"])
    assert np.array_equal(res["hist_size"], ec["hist_size"])
    for k in ("ra", "mc", "un"):
        assert compare.identical(res[k], im[k]), k


@pytest.mark.gpu
def test_mixed_jobs_match_alone(alone):
    """Jobs of the parity samples, submitted from two threads in bursts of three with gaps between the
    bursts, overlap on the GPU in rounds of several jobs; each result equals the sample's single-call
    result."""
    from breseq_gb300.api import ImSettings, Server
    names = list(samples.ALL) * 4
    ids = {}
    with Server(0, hbm_budget=8e9) as srv:
        def producer(k):
            rng = np.random.default_rng(k)
            for j, i in enumerate(range(k, len(names), 2)):
                n = names[i]
                ids[i] = srv.submit(alone[n][0], ImSettings(polymorphism_prediction=n in POLY))
                if j % 3 == 2:
                    time.sleep(float(rng.uniform(0, 0.02)))
        th = [threading.Thread(target=producer, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        rounds = []
        for i, n in enumerate(names):
            r = srv.result(ids[i])
            _check(r, alone[n])
            rounds.append(r["info"]["round_jobs"])
            assert r["info"]["read_bases"] == alone[n][0].aligned_bases()
            srv.release(ids[i])
        st = srv.stats()
    assert st["jobs_done"] == len(names)
    assert max(rounds) > 1, "no round ran more than one job"
    assert st["peak_in_use"] <= st["budget"]


@pytest.mark.gpu
def test_budget_limits_resident_jobs(alone, built_lib):
    """A budget that holds one job at a time admits the next only after the previous finished."""
    from breseq_gb300 import _lib
    from breseq_gb300.api import ImSettings, Server
    L = _lib.load()
    s = alone["ecoli_small"][0]
    view = abi.SampleView(s)
    fp = L.bsq_job_footprint(view.ref, view.reads)
    with Server(0, hbm_budget=fp * 1.5) as srv:
        jids = [srv.submit(s, ImSettings()) for _ in range(3)]
        for j in jids:
            _check(srv.result(j), alone["ecoli_small"])
        st = srv.stats()
        assert st["max_resident_jobs"] == 1
        assert st["peak_in_use"] == fp


@pytest.mark.gpu
def test_oversized_and_bad_jobs(alone, built_lib):
    """A job larger than the whole budget is refused at submit; a job with invalid records fails
    alone while the jobs around it succeed."""
    import dataclasses
    from breseq_gb300 import _lib
    from breseq_gb300.api import ImSettings, Server
    small = alone["clonal_small"][0]
    with Server(0, hbm_budget=1 << 20) as srv:
        with pytest.raises(_lib.BsqError) as e:
            srv.submit(alone["ecoli_small"][0], ImSettings())
        assert e.value.code == -4
    bad = dataclasses.replace(small, pos=small.pos[::-1].copy())   # records out of order
    with Server(0, hbm_budget=4e9) as srv:
        j0 = srv.submit(small, ImSettings())
        jb = srv.submit(bad, ImSettings())
        j1 = srv.submit(small, ImSettings())
        _check(srv.result(j0), alone["clonal_small"])
        _check(srv.result(j1), alone["clonal_small"])
        with pytest.raises(_lib.BsqError):
            srv.wait(jb)
