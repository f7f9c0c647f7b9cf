"""BAM input on the CPU: the oracle reader (oracle/bam_reader.py) against the synthetic samples it
was written from, and on hand-made files with the tag and read-group rules breseq applies."""
import numpy as np
import pytest

from breseq_gb300 import synth
from oracle import bam_reader
from tests import bam_cases, samples

FIELDS = ("tid", "pos", "flag", "mapq", "x1", "xl", "xr", "read_file", "read_group", "l_qseq", "n_cigar", "cigar_off",
          "seq_off", "cigar", "seq", "qual")


@pytest.mark.parametrize("name", ["clonal_small", "ecoli_small", "population_small"])
def test_round_trip(name):
    s = samples.ALL[name]()
    r = bam_reader.read_bam(synth.bam_bytes(s, level=1), synth.bam_groups(s))
    for k in FIELDS:
        assert np.array_equal(r["records"][k], np.asarray(getattr(s, k)).astype(r["records"][k].dtype)), k
    assert r["header"]["names"] == list(s.target_names)


def test_softclip_sample_xj_round_trip():
    s = samples.softclip_sample()
    r = bam_reader.read_bam(synth.bam_bytes(s, level=1), synth.bam_groups(s))
    assert np.array_equal(r["records"]["xj"], s.xj)


def test_tag_rules():
    recs, groups = bam_cases.tag_cases()
    r = bam_reader.read_bam(bam_cases.bam(recs), groups)["records"]
    assert len(r["tid"]) == 6                                   # the two unplaced records are dropped
    assert r["x1"].tolist() == [3, 2, 1, 0, 1, 4]               # first X1 wins; a float X1 reads as 0
    assert r["xl"].tolist() == [-1, -1, 2, -1, -1, -1]
    assert r["xr"].tolist() == [-1, -1, 4, -1, 6, -1]
    assert r["xj"].tolist() == [0, 0, 0, 1, 0, 0]
    assert r["read_group"].tolist() == [1, 0, 0, 0, 0, 1]       # unknown ID and a non-string RG give 0
    # read files: group 0 has two files (R2 -> 1), group 1 one file at 2 (R2 stays 2)
    assert r["read_file"].tolist() == [2, 1, 0, 0, 0, 2]


def test_single_group_and_unplaced_order():
    recs, _ = bam_cases.tag_cases()
    r = bam_reader.read_bam(bam_cases.bam(recs, rg_ids=("g0",)), (["g0"], [5], [1]))["records"]
    assert r["read_group"].tolist() == [0] * 6 and r["read_file"].tolist() == [5] * 6
    with pytest.raises(bam_reader.BamError):
        bam_reader.read_bam(bam_cases.bam([recs[6]] + recs[:6]))


def test_pair_annotations_round_trip():
    # names, TLEN, RNEXT / PNEXT and XP (FR / RF / FF; none, or another value, reads as 3)
    s = synth.with_pairs(synth.simulate(synth.config_ecoli(seed=5, scale=0.005)), seed=2, no_xp_fraction=0.3,
                         distance_sites=3)
    r = bam_reader.read_bam(synth.bam_bytes(s, level=1), synth.bam_groups(s))["records"]
    for k in ("isize", "xp", "qname_off", "qname", "mtid", "mpos", "flag"):
        assert np.array_equal(r[k], getattr(s, k)), k
    assert set(np.unique(r["xp"])) <= {0, 1, 2, 3} and (r["xp"] == 3).any() and (r["xp"] < 3).any()


def test_spanning_records_and_cg_cigar():
    # blocks cut regardless of records read the same; a CIGAR kept in the CG tag is refused
    import struct
    s = samples.ecoli_small()
    a = bam_reader.read_bam(synth.bam_bytes(s, block_payload=4096), synth.bam_groups(s))
    b = bam_reader.read_bam(synth.bam_bytes(s, block_payload=4096, split_records=True), synth.bam_groups(s))
    for k in a["records"]:
        assert np.array_equal(a["records"][k], b["records"][k]), k
    recs, groups = bam_cases.tag_cases()
    cg = bam_cases.record(0, 30, [(20, "S"), (20, "N")], "ACGT" * 5,
                          b"CGBI" + struct.pack("<I", 1) + struct.pack("<I", (20 << 4) | 0))
    with pytest.raises(bam_reader.BamError):
        bam_reader.read_bam(bam_cases.bam(recs[:6] + [cg]), groups)
