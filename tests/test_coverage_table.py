"""BAM2COV coverage table (coverage_output.cpp:190-470) restated on the CPU, pinned by hand-worked
values on hand-made records and by the rows the reference's pileup driver produces."""
import numpy as np

from oracle import pyoracle as po
from tests import samples


def test_columns_known_answers():
    s, _ = samples.softclip_known()
    c = po.coverage_columns(s, 0, 1, 60)
    assert c["last"] == 60
    # position 21: R1 R2 R3 R4, the XJ-tagged R7 (the pileup ignores XJ), R9 R10 C1; R8 is secondary
    # and R5 unmapped (filtered), R6 has X1 = 2 (redundant weight 1/2)
    assert c["unique_top"][20] == 8 and c["raw_redundant_top"][20] == 1 and c["redundant_top"][20] == 0.5
    # C1 (10M2I5M3D10M5S at 13) has deleted bases at 28-30: deletion entries are not counted
    assert list(c["unique_top"][26:31]) == [8, 7, 7, 7, 8]
    # first sequenced bases aligned: R9 and R10 at 11, C1 at 13, R12 at 51; R11 starts with a clip
    assert np.nonzero(c["unique_top_begin"])[0].tolist() == [10, 12, 50]
    assert c["unique_top_begin"][10] == 2
    assert not c["unique_bot"].any() and not c["unique_bot_begin"].any()


def _rows(path):
    return [l.split("\t") for l in open(path).read().splitlines() if not l.startswith(("#", "position"))]


def test_driver_rows_with_downsampling(tmp_path):
    s, _ = samples.softclip_known()
    p = str(tmp_path / "a.tsv")
    # 60 positions at resolution 7: downsample floor(60/7) = 8, rows where (position + 1) % 8 == 0;
    # the pileup's last column is 60, so there is no tail
    po.write_coverage_region(s, p, 0, 1, 60, resolution=7)
    assert [int(r[0]) for r in _rows(p)] == [7, 15, 23, 31, 39, 47, 55]
    # s0 (40 bp) has one record, on 11-30; downsample 10 keeps 9, 19, 29, 39.  Past the last column
    # (30) only handled positions move the cursor, so position 39 first prints 31-38 as zero rows
    po.write_coverage_region(s, p, 1, 1, 40, resolution=4)
    rows = _rows(p)
    assert [int(r[0]) for r in rows] == [9, 19, 29] + list(range(31, 40))
    assert rows[0][2] == "0" and rows[1][2] == "1" and all(r[2] == "0" for r in rows[3:])
    assert open(p).read().splitlines()[-1] == "#\tnumber_of_positions\t12"
    # no record overlaps 35-40: the cursor stays at 0 and position 35 prints 1-34 first
    po.write_coverage_region(s, p, 1, 35, 40, resolution=0)
    assert [int(r[0]) for r in _rows(p)] == list(range(1, 41))


def test_total_only_csv_and_average(tmp_path):
    s, _ = samples.softclip_known()
    p = str(tmp_path / "b.csv")
    po.write_coverage_region(s, p, 0, 20, 22, resolution=0, total_only=True, csv=True, reference_average=7.25)
    lines = open(p).read().splitlines()
    assert lines[0] == "position,ref_base,unique_cov,redundant_cov,total_cov"
    assert lines[2].split(",")[2:] == ["8", "0.5", "8.5"]
    assert lines[4] == "#,reference_unique_average_cov,7.25"
    assert lines[-1] == "#,number_of_positions,3"


def test_per_read_group_columns_add_up(tmp_path):
    # the oracle's --per-read-group columns: integer columns of the groups sum to the aggregate, the
    # redundant weights to within rounding; header and average lines per group
    from breseq_gb300 import synth
    cfg = synth.SimConfig(seed=13, target_lengths=(8_000,), n_snps=3, n_indels=1, max_indel=1, repeat_copies=2,
                          repeat_length=300, read_sets=(synth.ReadFileSet(coverage=20, read_length=101, paired=True),
                                                        synth.ReadFileSet(coverage=15, read_length=150)))
    s = synth.simulate(cfg)
    path = str(tmp_path / "rg.tsv")
    po.write_coverage_region(s, path, 0, 1, 8_000, resolution=0, per_read_group=True, n_read_groups=3)
    lines = open(path).read().splitlines()
    head = lines[0].split("\t")
    assert head[2:10] == ["unique_top_cov", "unique_bot_cov", "redundant_top_cov", "redundant_bot_cov",
                          "raw_redundant_top_cov", "raw_redundant_bot_cov", "unique_top_begin", "unique_bot_begin"]
    assert head[10] == "RG-0_unique_top_cov" and head[-1] == "RG-2_unique_bot_begin" and len(head) == 2 + 8 * 4
    rows = [x.split("\t") for x in lines[1:] if not x.startswith("#")]
    for r in rows[::97]:
        v = [float(x) for x in r[2:]]
        agg, per = v[:8], [v[8 + 8 * g: 16 + 8 * g] for g in range(3)]
        for c in (0, 1, 4, 5, 6, 7):
            assert agg[c] == sum(p[c] for p in per)
        for c in (2, 3):
            assert abs(agg[c] - sum(p[c] for p in per)) < 1e-9 * max(1.0, agg[c])
        assert per[2] == [0.0] * 8     # a group no record names
    tail = [x for x in lines if x.startswith("#")]
    assert tail[-9].split("\t")[1] == "RG-0_region_unique_average_cov" and len(tail) == 4 + 9


def im_read_groups():
    """The ecoli_small sample (repeats, indels, N bases, trims) with its records spread over three read
    groups: the read file, and a seeded tenth moved to group 2."""
    import dataclasses
    s = samples.ecoli_small()
    rng = np.random.default_rng(5)
    g = np.where(rng.random(len(s.read_group)) < 0.1, 2, s.read_file).astype(np.uint16)
    return dataclasses.replace(s, read_group=g)


IM_INT = ("unique_top", "unique_bot", "raw_redundant_top", "raw_redundant_bot")
IM_RED = ("redundant_top", "redundant_bot")


def test_im_coverage_tally_equals_pass_2(tmp_path):
    # identify_mutations' coverage tally restated alone (all records) equals the per-position coverage
    # the oracle's pass 2 keeps: deletions counted, N read bases not; with the coverage fit failed on
    # one target, tabulate_position_coverage's (deletions left out too).  The groups' integer columns
    # add up to it and their weights to within rounding.
    s = im_read_groups()
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    T = len(s.target_offset) - 1
    p = po.default_im_params(s)
    p["deletion_propagation_cutoff"][1] = -1.0
    pos = po.identify(s, tab, p)["positions"]
    more = fewer = False
    for t in range(T):
        b, e = int(s.target_offset[t]), int(s.target_offset[t + 1])
        failed = t == 1
        allc = po.im_coverage_columns(s, t, 1, e - b, coverage_fit_failed=failed)
        for k in IM_INT + IM_RED:
            assert np.array_equal(allc[k], pos[k][b:e]), (t, k)
        per = [po.im_coverage_columns(s, t, 1, e - b, read_group=g, coverage_fit_failed=failed) for g in range(3)]
        for k in IM_INT:
            assert np.array_equal(sum(x[k].astype(np.int64) for x in per), allc[k].astype(np.int64)), (t, k)
        for k in IM_RED:
            assert np.allclose(sum(x[k] for x in per), allc[k], rtol=1e-12, atol=0), (t, k)
        assert all(x["unique_top"].any() for x in per)
        # the pass-2 tally differs from BAM2COV's exactly by the deletion entries (counted) and the
        # aligned N bases (not counted)
        if not failed:
            bc = po.coverage_columns(s, t, 1, e - b)
            d = allc["unique_top"].astype(np.int64) + allc["unique_bot"] - bc["unique_top"] - bc["unique_bot"]
            more |= bool((d > 0).any())
            fewer |= bool((d < 0).any())
    assert more and fewer


def test_im_coverage_table_read_group_columns(tmp_path):
    s = im_read_groups()
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    pos = po.identify(s, tab, po.default_im_params(s))["positions"]
    path = str(tmp_path / "cov.tsv")
    po.write_coverage_table(s, path, 2, pos, n_read_groups=3)
    lines = open(path).read().splitlines()
    head = lines[0].split("\t")
    assert head[:5] == ["position", "ref_base", "unique_cov", "redundant_cov", "total_cov"]
    assert head[5] == "RG-0_unique_cov" and head[-1] == "RG-2_total_cov" and len(head) == 5 + 9
    b, e = int(s.target_offset[2]), int(s.target_offset[3])
    assert len(lines) == 1 + (e - b)
    for i in range(0, e - b, 37):
        r = lines[1 + i].split("\t")
        assert int(r[0]) == i + 1
        u = float(pos["unique_top"][b + i]) + float(pos["unique_bot"][b + i])
        assert float(r[2]) == u and sum(float(r[5 + 3 * g]) for g in range(3)) == u
    # one read group: no per-group columns (identify_mutations.cpp:862)
    po.write_coverage_table(s, path, 2, pos, n_read_groups=1)
    assert open(path).readline().rstrip("\n").split("\t") == head[:5]


def test_library_writer_matches_oracle(built_lib, tmp_path):
    # the library's host writer of <seq_id>.coverage.tsv (aggregate columns, no device call) against the
    # oracle's, on every target of a sample with a failed coverage fit on one of them
    import ctypes as C
    from breseq_gb300 import _lib, abi
    s = im_read_groups()
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    p = po.default_im_params(s)
    p["deletion_propagation_cutoff"][1] = -1.0
    pos = po.identify(s, tab, p)["positions"]
    L = _lib.load()
    view = abi.SampleView(s)
    pa, keep = abi.position_arrays_view(pos)
    for t in range(len(s.target_offset) - 1):
        a, b = str(tmp_path / f"l{t}.tsv"), str(tmp_path / f"o{t}.tsv")
        assert L.bsq_write_coverage_table(a.encode(), s.target_names[t].encode(), C.byref(view.ref), t, C.byref(pa)) == 0
        po.write_coverage_table(s, b, t, pos, n_read_groups=1, coverage_fit_failed=t == 1)
        assert open(a).read() == open(b).read(), t
    del keep
