"""Discordant-pair / missing-pair candidate regions on the CPU: the library's classification
(pair_classify_one) and sliding-window replay (host::pair_replay), driven on the host by
tests/native/pairs_host.cpp, against the oracle's position-by-position walk of the reference's
windows; the written CSV files must be identical.  The device path is checked against the same
oracle by tests/test_gpu_pairs.py."""
import ctypes as C
import dataclasses
import os
import subprocess

import numpy as np
import pytest

from breseq_gb300 import abi, synth
from breseq_gb300.api import PairSettings, pair_params
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRCS = [os.path.join(ROOT, "tests", "native", "pairs_host.cpp"),
        os.path.join(ROOT, "breseq_gb300", "csrc", "bsq_pairs_host.cpp")]
DEPS = SRCS + [os.path.join(ROOT, "breseq_gb300", "csrc", f) for f in ("bsq_pairs.h", "bsq_host.h", "bsq_common.h")]
OUT = os.path.join(ROOT, "tests", "native", "_build", "libpairs_host.so")


@pytest.fixture(scope="module")
def host():
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(os.path.getmtime(d) for d in DEPS):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-ffp-contract=off",
                               "-I" + cuda_inc]
                              + SRCS + ["-o", OUT])
    L = C.CDLL(OUT)
    L.host_pair_candidates.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.POINTER(abi.PairParams),
                                       C.POINTER(C.c_char_p), C.c_char_p, C.c_char_p, C.c_char_p]
    return L


def run_both(host, s, st, tmp_path, cutoff=None):
    view = abi.SampleView(s)
    p, keep = pair_params(s, st, cutoff)
    names = (C.c_char_p * len(s.target_names))(*[n.encode() for n in s.target_names])
    paths = {k: str(tmp_path / f"{k}.csv") for k in ("dp", "mp", "pd", "odp", "omp", "opd")}
    pd = st.predict_pair_distance
    rc = host.host_pair_candidates(C.byref(view.ref), C.byref(view.reads), C.byref(p), names,
                                   paths["dp"].encode(), paths["mp"].encode(), paths["pd"].encode() if pd else None)
    assert rc == 0
    po.pair_candidates(s, st, paths["odp"], paths["omp"], cutoff, paths["opd"] if pd else None)
    keys = ("dp", "mp", "pd") if pd else ("dp", "mp")
    got = [open(paths[k]).read() for k in keys]
    exp = [open(paths["o" + k]).read() for k in keys]
    return got, exp


def pd_settings(s, **kw):
    """Pair-distance settings over a sample's null (one DP group per read group)."""
    G = int(s.read_group.max()) + 1
    base = dict(dp_group=tuple(range(G)), window_width=(400.0,) * G, r1_prefix=tuple(1 + 2 * g for g in range(G)),
                r2_prefix=tuple(2 + 2 * g for g in range(G)), predict_missing_pairs=True, predict_pair_distance=True,
                pd_cdf=(synth.pd_null(s),) * G, pd_orientation=("FR",) * G, pd_max_span=1500, pd_z_seed=2.5,
                pd_mean_covering_gap=137.5)
    base.update(kw)
    return PairSettings(**base)


def ecoli_pairs(scale=0.03, seed=5, **kw):
    return synth.with_pairs(synth.simulate(synth.config_ecoli(seed=seed, scale=scale)), seed=seed, **kw)


def two_groups(seed=3):
    cfg = synth.SimConfig(seed=seed, target_lengths=(30_000, 6_000, 2_500), target_names=("chrA", "plasmid", "chrB"),
                          n_snps=10, n_indels=3, max_indel=2,
                          read_sets=(synth.ReadFileSet(coverage=40, read_length=101, paired=True, insert_mean=300),
                                     synth.ReadFileSet(coverage=25, read_length=150, paired=True, insert_mean=500)))
    return synth.with_pairs(synth.simulate(cfg), seed=seed, discordant_sites=4, unmapped_sites=4,
                            background_discordant=0.02, background_unmapped=0.03, no_xp_fraction=0.1)


def test_pairs_ecoli_matches_oracle(host, tmp_path):
    s = ecoli_pairs()
    st = PairSettings(dp_group=(0,), window_width=(462.75,), predict_missing_pairs=True)
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp
    assert got[0].count("\n") > 5 and got[1].count("\n") > 3   # regions were found on both scans


def test_pairs_skip_without_orientation(host, tmp_path):
    # DP-eligible reads without a usable XP are skipped at their start column, MP included
    s = ecoli_pairs(scale=0.02, seed=8, no_xp_fraction=0.3, background_discordant=0.01)
    st = PairSettings(dp_group=(0,), window_width=(400.0,), predict_missing_pairs=True, missing_pair_seed=2,
                      missing_pair_seed_fraction=0.1)
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp


@pytest.mark.parametrize("dp_group,widths", [((0, 1), (300.5, 520.0)), ((-1, 0), (37.25,)), ((0, 0), (1.0,)),
                                             ((1, 0), (0.5, 2000.0))])
@pytest.mark.parametrize("seeds", [(3, 3, 0.25), (1, 2, 0.0), (0, 0, 0.5), (6, 4, 1.0)])
def test_pairs_groups_and_seeds(host, tmp_path, dp_group, widths, seeds):
    s = two_groups()
    G = len(widths)
    st = PairSettings(dp_group=dp_group, window_width=widths, r1_prefix=tuple(1 + 2 * g for g in range(G)),
                      r2_prefix=tuple(2 + 2 * g for g in range(G)), discordant_pair_seed=seeds[0],
                      predict_missing_pairs=True, missing_pair_seed=seeds[1], missing_pair_seed_fraction=seeds[2])
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp


def test_pairs_targets_skipped(host, tmp_path):
    # a target below the deletion propagation cutoff is not walked; one outside the pileup set neither
    s = two_groups(seed=4)
    s = dataclasses.replace(s, target_order=np.array([0, 2], dtype=np.uint32))
    st = PairSettings(dp_group=(0, 1), window_width=(350.0, 600.0), r1_prefix=(1, 3), r2_prefix=(2, 4),
                      predict_missing_pairs=True)
    got, exp = run_both(host, s, st, tmp_path, cutoff=np.array([5.0, 5.0, -1.0]))
    assert got == exp
    assert "chrB" not in got[0] + got[1] and "plasmid" not in got[0] + got[1]


def test_pairs_mp_off_and_no_groups(host, tmp_path):
    s = two_groups(seed=6)
    got, exp = run_both(host, s, PairSettings(dp_group=(0, 1), window_width=(400.0, 400.0), r1_prefix=(1, 3),
                                              r2_prefix=(2, 4)), tmp_path)
    assert got == exp and got[1].count("\n") == 1       # MP off: header only
    got, exp = run_both(host, s, PairSettings(dp_group=(-1, -1), window_width=(), r1_prefix=(), r2_prefix=(),
                                              predict_missing_pairs=True), tmp_path)
    assert got == exp and got[0].count("\n") == 1 and got[1].count("\n") == 1


def test_pairs_hand_worked(host, tmp_path):
    """Three discordant FR reads starting at 101, 151, 201 (window 100, seed 2) on one 1000-bp target:
    two are in the window at 151 (101 <= 151 < 201) and at 201 the first leaves (201 - 101 >= 100) as the
    third enters, so the count is 2 from 151 to 250; at 251 the second leaves.  Region 151-250, maximum
    2, all three reads listed (two in the snapshot at 151, one appended at 201)."""
    seq = np.frombuffer(b"ACGT" * 250, dtype=np.uint8).copy()
    n = 3
    pos = np.array([100, 150, 200], dtype=np.int32)
    cig = np.array([(50 << 4) | 0] * n, dtype=np.uint32)
    s = synth.Sample(ref_seq=seq, target_offset=np.array([0, 1000], dtype=np.uint64), target_names=["t"],
                     coverage_group=np.zeros(1, np.uint32), n_coverage_groups=1, target_order=np.zeros(1, np.uint32),
                     tid=np.zeros(n, np.int32), pos=pos, flag=np.array([0x1 | 0x40, 0x1 | 0x80, 0x1 | 0x40], np.uint16),
                     mapq=np.full(n, 40, np.uint8), x1=np.array([1, 2, 1], np.uint32), xl=np.full(n, -1, np.int32),
                     xr=np.full(n, -1, np.int32), read_file=np.zeros(n, np.uint8), read_group=np.zeros(n, np.uint16),
                     l_qseq=np.full(n, 50, np.uint32), seq_off=np.arange(n, dtype=np.uint64) * 50,
                     cigar_off=np.arange(n, dtype=np.uint64), n_cigar=np.ones(n, np.uint16), cigar=cig,
                     seq=np.full(n * 25, 0x12, np.uint8), qual=np.full(n * 50, 30, np.uint8), n_read_files=2,
                     n_quality=42, isize=np.array([900, 800, -700], np.int32), xp=np.zeros(n, np.uint8),
                     qname_off=np.array([0, 3, 6, 9], np.uint64), qname=np.frombuffer(b"1:71:82:9", np.uint8).copy())
    st = PairSettings(dp_group=(0,), window_width=(100.0,), r1_prefix=(5,), r2_prefix=(6,), discordant_pair_seed=2)
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp
    want = ("seq_id,start,end,strand,orientation,length,max_discordant_count,redundant,discordant_pairs\n"
            "t,151,250,F,FR,100,2,0,5:7__6:7__900__101__150;5:8__6:8__-800__151__200;5:9__6:9__-700__201__250\n")
    assert got[0] == want


def test_pd_ecoli_matches_oracle(host, tmp_path):
    s = ecoli_pairs(seed=9, distance_sites=25)
    got, exp = run_both(host, s, pd_settings(s), tmp_path)
    assert got == exp
    lines = got[2].splitlines()
    assert lines[0].startswith("#mean_covering_gap=137.500000") and len(lines) > 14   # regions found


@pytest.mark.parametrize("kw", [dict(pd_z_seed=1.0, pair_distance_seed=1), dict(pd_z_seed=2.6),
                                dict(pd_orientation=("",)), dict(pd_orientation=("RF",), pd_max_span=600),
                                dict(pair_distance_tail_quantile=0.25, pair_distance_seed=5),
                                dict(pd_cdf=(None,)), dict(pd_max_span=0)])
def test_pd_settings(host, tmp_path, kw):
    # a low seed seeds many regions (the ladder and tail fit see hundreds), 2.6 is raised to the next
    # rung, an empty orientation takes any opposite-strand pair, no null or no span disables the scan
    s = ecoli_pairs(scale=0.02, seed=10, distance_sites=10)
    got, exp = run_both(host, s, pd_settings(s, **kw), tmp_path)
    assert got == exp


def test_pd_two_groups_and_skips(host, tmp_path):
    import dataclasses
    s = two_groups(seed=11)
    s = dataclasses.replace(s, target_order=np.array([0, 2], dtype=np.uint32))
    s = synth.with_pairs(s, seed=11, distance_sites=6, no_xp_fraction=0.2, background_discordant=0.02)
    st = pd_settings(s, pd_cdf=(synth.pd_null(s), None), window_width=(300.5, 520.0), pd_z_seed=1.5)
    got, exp = run_both(host, s, st, tmp_path, cutoff=np.array([5.0, 5.0, -1.0]))
    assert got == exp


def test_writers_without_regions_and_bad_arguments(built_lib, tmp_path):
    # the library's writers need no GPU: an empty result gives the header (and for PD the calibration)
    from breseq_gb300 import _lib
    L = _lib.load()
    names = (C.c_char_p * 1)(b"chr")
    dp, mp, pd = (str(tmp_path / f) for f in ("dp.csv", "mp.csv", "pd.csv"))
    assert L.bsq_write_dp_candidate_regions(dp.encode(), names, None, 0, b"") == 0
    assert L.bsq_write_mp_candidate_regions(mp.encode(), names, None, 0, b"") == 0
    assert open(dp).read() == ("seq_id,start,end,strand,orientation,length,max_discordant_count,redundant,"
                               "discordant_pairs\n")
    assert open(mp).read().startswith("seq_id,start,end,strand,length,max_unpaired_count,max_window_total_count")
    summ = abi.PdSummary(seed_z_used=2.5, z_iqr_inflation=1.0, region_tail_sigma=1.0)
    assert L.bsq_write_pd_candidate_regions(pd.encode(), names, None, 0, C.byref(summ)) == 0
    lines = open(pd).read().splitlines()
    assert lines[2] == "#seed_z=2.500000" and lines[9].startswith("#region_ladder=1.00:0;1.25:0")
    assert lines[10].startswith("seq_id,start,end,direction") and len(lines) == 11
    assert L.bsq_write_pd_candidate_regions(pd.encode(), names, None, 0, None) != 0
    regs = (abi.PairRegion * 1)()
    assert L.bsq_write_dp_candidate_regions(dp.encode(), None, regs, 1, b"") != 0


def test_pd_setup_helpers(built_lib):
    # the PD null, span and seed z as the pileup constructor derives them, against the Python
    # restatement bit for bit and ndtri against scipy
    from breseq_gb300 import _lib
    from breseq_gb300.api import pd_null_from_histogram, pd_seed_z
    L = _lib.load()
    ys = np.concatenate([np.geomspace(1e-300, 0.135, 200), np.linspace(0.13, 0.87, 200), 1 - np.geomspace(1e-16, 0.135, 200)])
    for y in ys:
        assert L.bsq_ndtri(float(y)) == po.ndtri(float(y))
    sp = pytest.importorskip("scipy.special")
    for y in ys[(ys > 1e-200) & (ys < 1 - 1e-15)]:
        assert L.bsq_ndtri(float(y)) == pytest.approx(float(sp.ndtri(y)), rel=1e-13, abs=1e-300)
    rng = np.random.default_rng(4)
    for _ in range(20):
        n = int(rng.integers(1, 400))
        d = rng.integers(-5, 1500, n)
        c = rng.choice([0.0, 1.0, 3.0, 17.5, 1000.0], n)
        d[: n // 10] = d[0]                       # repeated distances
        trunc, maxd = int(rng.integers(0, 400)), int(rng.choice([0, 600, 1200]))
        got, gap = pd_null_from_histogram(d, c, trunc, maxd)
        exp, egap = po.pd_build_null(d, c, trunc, maxd)
        assert (got is None) == (exp is None) and gap == egap
        if got is not None:
            assert np.array_equal(got, exp)
    for args in [(0.0, 137.5, 4_790_000), (3.25, 137.5, 4_790_000), (0.0, 0.0, 0), (0.0, 2e6, 1000),
                 (0.0, 400.0, 48_502)]:
        assert pd_seed_z(*args) == po.pd_seed_z(*args)
    assert pd_seed_z(0.0, 137.5, 4_790_000) == 2.5 and pd_seed_z(0.0, 2e6, 1000) == 1.0
    cut = (C.c_double * 2)(300.4, 612.25)
    assert L.bsq_pd_max_span(0, cut, 2) == 1225 and L.bsq_pd_max_span(900, cut, 2) == 900


def test_pd_hand_worked(host, tmp_path):
    """Four concordant FR pairs of 50-bp reads at 100, TLEN 500, mates at 550: each gap covers
    positions 149..549 (the read's end to the mate's start - 1).  The null puts distance 500 at the
    0.9 quantile, inside the long tail (quantile 0.15), so at every covered position n = 4, four tail
    pairs and z = (4 u - 4 S / 2) / S * sqrt(12 / 4) with u = 0.9 S: one L region 149-549 peaking at its
    first position, eight ladder rungs (z >= 1 .. 2.75) with one region each, 401 positions in the z
    histogram (fewer than 1000: no inflation), no tail fit."""
    import math
    n, L = 4, 50
    S = 1048576
    u = int(0.9 * S)
    cdf = np.full(1001, S // 2, dtype=np.int64)
    cdf[500] = u
    seq = np.frombuffer(b"ACGT" * 250, dtype=np.uint8).copy()
    s = synth.Sample(ref_seq=seq, target_offset=np.array([0, 1000], dtype=np.uint64), target_names=["t"],
                     coverage_group=np.zeros(1, np.uint32), n_coverage_groups=1, target_order=np.zeros(1, np.uint32),
                     tid=np.zeros(n, np.int32), pos=np.full(n, 99, np.int32), flag=np.full(n, 0x1 | 0x2 | 0x20 | 0x40, np.uint16),
                     mapq=np.full(n, 40, np.uint8), x1=np.ones(n, np.uint32), xl=np.full(n, -1, np.int32),
                     xr=np.full(n, -1, np.int32), read_file=np.zeros(n, np.uint8), read_group=np.zeros(n, np.uint16),
                     l_qseq=np.full(n, L, np.uint32), seq_off=np.arange(n, dtype=np.uint64) * L,
                     cigar_off=np.arange(n, dtype=np.uint64), n_cigar=np.ones(n, np.uint16),
                     cigar=np.full(n, (L << 4) | 0, np.uint32), seq=np.full(n * L // 2, 0x12, np.uint8),
                     qual=np.full(n * L, 30, np.uint8), n_read_files=2, n_quality=42,
                     isize=np.full(n, 500, np.int32), xp=np.zeros(n, np.uint8),
                     qname_off=np.arange(n + 1, dtype=np.uint64) * 3,
                     qname=np.frombuffer(b"1:01:11:21:3", np.uint8).copy(), mtid=np.zeros(n, np.int32),
                     mpos=np.full(n, 549, np.int32))
    st = PairSettings(dp_group=(0,), window_width=(400.0,), predict_pair_distance=True, pd_cdf=(cdf,),
                      pd_orientation=("FR",), pd_max_span=1000, pd_z_seed=2.5, pair_distance_seed=3,
                      pair_distance_tail_quantile=0.15, pd_mean_covering_gap=250.0)
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp
    z = (float(n * u) - float(n) * float(S) / 2.0) / float(S) * math.sqrt(12.0 / float(n))
    lines = got[2].splitlines()
    assert lines[0] == "#mean_covering_gap=250.000000" and lines[1] == "#n_effective_tests=4.000000"
    assert lines[2] == "#seed_z=2.500000" and lines[3] == "#z_iqr_inflation=1.000000"
    assert lines[4] == "#region_tail_fit_ok=0"
    ladder = ";".join(f"{1 + 0.25 * k:.2f}:{1 if 1 + 0.25 * k <= z else 0}" for k in range(21))
    assert lines[9] == "#region_ladder=" + ladder
    assert lines[11:] == [f"t,149,549,L,401,149,4,4,{z:.4f}"]


def test_mp_hand_worked(host, tmp_path):
    """Forward reads of 50 bases starting at 101, 111, 121 with their mates unmapped, and mapped pairs at
    105 and 300 (window 100, seed 2, fraction 0.5).  At 111 two mate-unmapped reads of three in the
    window: the region opens with 101 and 111; at 121 the count reaches 3 of 4 (the maximum, 121
    appended); at 201 and 205 the first two leave (2 of 3, 2 of 2, still enriched); at 211 only one is
    left and the region closes at 210."""
    seq = np.frombuffer(b"ACGT" * 250, dtype=np.uint8).copy()
    pos = np.array([100, 104, 110, 120, 299], dtype=np.int32)
    n, L = len(pos), 50
    unm = np.array([1, 0, 1, 1, 0], dtype=bool)
    flag = np.where(unm, 0x1 | 0x8 | 0x40, 0x1 | 0x2 | 0x20 | 0x40).astype(np.uint16)
    names = [f"1:{i}".encode() for i in range(n)]
    s = synth.Sample(ref_seq=seq, target_offset=np.array([0, 1000], dtype=np.uint64), target_names=["t"],
                     coverage_group=np.zeros(1, np.uint32), n_coverage_groups=1, target_order=np.zeros(1, np.uint32),
                     tid=np.zeros(n, np.int32), pos=pos, flag=flag, mapq=np.full(n, 40, np.uint8),
                     x1=np.ones(n, np.uint32), xl=np.full(n, -1, np.int32), xr=np.full(n, -1, np.int32),
                     read_file=np.zeros(n, np.uint8), read_group=np.zeros(n, np.uint16), l_qseq=np.full(n, L, np.uint32),
                     seq_off=np.arange(n, dtype=np.uint64) * L, cigar_off=np.arange(n, dtype=np.uint64),
                     n_cigar=np.ones(n, np.uint16), cigar=np.full(n, (L << 4) | 0, np.uint32),
                     seq=np.full(n * L // 2, 0x12, np.uint8), qual=np.full(n * L, 30, np.uint8), n_read_files=2,
                     n_quality=42, isize=np.where(unm, 0, 300).astype(np.int32),
                     xp=np.where(unm, 3, 0).astype(np.uint8),
                     qname_off=np.concatenate([[0], np.cumsum([len(x) for x in names])]).astype(np.uint64),
                     qname=np.frombuffer(b"".join(names), np.uint8).copy())
    st = PairSettings(dp_group=(0,), window_width=(100.0,), predict_missing_pairs=True, missing_pair_seed=2,
                      missing_pair_seed_fraction=0.5)
    got, exp = run_both(host, s, st, tmp_path)
    assert got == exp
    assert got[1].splitlines()[1:] == ["t,111,210,F,100,3,4,0,101__150;111__160;121__170"]
    assert got[0].count("\n") == 1    # no discordant pair
