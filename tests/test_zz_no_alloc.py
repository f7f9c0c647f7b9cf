"""bsq_score_positions_noalloc: the scoring entry point for callers that cannot allocate device memory
while they run (a serving loop with work in flight on other streams, where cudaMalloc / cudaFree may
synchronize the device; a program that gives all of HBM to its own arena).  Its scratch is a fixed
device array inside the library; the caller brings device buffers for the positions and the results.

The test calls it twice in a row through the C ABI, with the caller's buffers allocated by torch, and
checks each call's RA items against the ones bsq_identify_mutations reports for the same positions and
against the CPU oracle's, at the tolerances of the parity tests (scores 1e-3, frequencies 1e-4, counts
exact).
"""
import ctypes as C

import numpy as np
import pytest

from breseq_gb300 import abi
from tests import samples

pytestmark = pytest.mark.gpu

CHARS = "ACGT.N"


def _device_call(sc, torch, sid, params, table, positions, n_quality):
    L = sc.L
    tid = torch.tensor([t for t, _ in positions], dtype=torch.int32, device="cuda")
    pos = torch.tensor([p for _, p in positions], dtype=torch.int32, device="cuda")
    cap = 4 * len(positions) + 16
    rec = C.sizeof(abi.RaRaw)
    d_ra = torch.zeros(cap * rec, dtype=torch.uint8, device="cuda")
    d_n = torch.full((1,), 12345, dtype=torch.int32, device="cuda")   # the call must reset it
    d_qh = torch.zeros(cap * 2 * n_quality, dtype=torch.int32, device="cuda")
    tab = np.ascontiguousarray(table, dtype=np.float64)
    torch.cuda.synchronize()
    rc = L.bsq_score_positions_noalloc(sc.ctx, sid, C.byref(params), abi.ptr(tab, C.c_double), tid.data_ptr(),
                                       pos.data_ptr(), len(positions), d_ra.data_ptr(), cap, d_n.data_ptr(),
                                       d_qh.data_ptr())
    assert rc == 0, L.bsq_last_error(sc.ctx).decode()
    torch.cuda.synchronize()
    n = int(d_n.item())
    raw = (abi.RaRaw * max(1, n)).from_buffer_copy(d_ra[: max(1, n) * rec].cpu().numpy().tobytes())
    return [raw[i] for i in range(n)]


def test_noalloc_positions_match_identify_mutations(built_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    from breseq_gb300.api import ImSettings, Scorer

    s = samples.ecoli_small()
    padded = np.asarray(s.target_offset, dtype=np.int64) + np.arange(len(s.target_offset))
    with Scorer(0) as sc:
        sid = sc.load_sample(s)
        ec = sc.error_count(sid)
        table = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        expected = sc.identify_mutations(sid, table, ImSettings(), precision=0)["ra"]
        assert expected, "the sample must carry RA items"
        from oracle import pyoracle as po
        from tests import compare
        oracle_ra = po.identify(s, table, po.default_im_params(s))["ra"]
        assert not compare.compare_ra(expected, oracle_ra)
        T = len(s.target_offset) - 1
        prop = np.full(T, 5.0)
        seed = np.zeros(T)
        params = abi.ImParams(n_read_files=s.n_read_files, n_quality=s.n_quality, base_quality_cutoff=3,
                              mutation_cutoff=10.0, polymorphism_cutoff=10.0, polymorphism_precision_decimal=1e-6,
                              polymorphism_precision_places=3, skip_missing_coverage_prediction=0,
                              log10_ref_length=float(np.log10(float(s.target_offset[-1]))),
                              deletion_propagation_cutoff=abi.ptr(prop, C.c_double),
                              deletion_seed_cutoff=abi.ptr(seed, C.c_double), precision=0)
        ra_positions = sorted({(r["tid"], r["position"] - 1) for r in expected})
        rng = np.random.default_rng(7)
        quiet = [(0, int(p)) for p in rng.integers(0, int(s.target_offset[1]), size=300)]
        calls = [ra_positions + quiet, list(reversed(ra_positions))[: max(1, len(ra_positions) // 2)] + quiet[:50]]
        for positions in calls:               # two calls in a row share the fixed scratch
            got = _device_call(sc, torch, sid, params, table, positions, s.n_quality)
            wanted = set(positions)
            exp = {(r["tid"], r["position"], r["insert_position"]): r for r in expected
                   if (r["tid"], r["position"] - 1) in wanted}
            have = {}
            for g in got:
                t = int(np.searchsorted(padded, g.column, side="right") - 1)
                have[(t, int(g.column - padded[t]) + 1, g.insert_position)] = g
            assert sorted(have) == sorted(exp)
            for key, r in exp.items():
                g = have[key]
                assert CHARS[g.var_idx] == r["new_base"] and CHARS[g.major_idx] == r["major_base"]
                assert CHARS[g.minor_idx] == r["minor_base"] and CHARS[g.ref_idx] == r["ref_base"]
                assert bool(g.passed_consensus) == bool(r["passed_consensus"])
                assert bool(g.passed_polymorphism) == bool(r["passed_polymorphism"])
                assert g.score == pytest.approx(r["score"], abs=1e-3, nan_ok=True)
                assert g.consensus_score == pytest.approx(r["consensus_score"], abs=1e-3)
                for b in range(5):
                    assert g.f[b] == pytest.approx(r["f"][b], abs=1e-4)
                assert g.frequency_lower == pytest.approx(r["frequency_lower"], abs=1e-4)
                assert g.frequency_upper == pytest.approx(r["frequency_upper"], abs=1e-4)
                assert g.n == r["n"]
                tot = (sum(g.pos_info[b][0] for b in range(5)), sum(g.pos_info[b][1] for b in range(5)))
                assert tot == tuple(r["total_cov"])
