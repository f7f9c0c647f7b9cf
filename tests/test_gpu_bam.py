"""BAM input on the GPU (bsq_bam_open / decode / load): BGZF inflate and record decode against the
oracle reader, byte for byte, and the scoring passes on a sample loaded from BAM bytes identical to
the same sample loaded from arrays."""
import struct

import numpy as np
import pytest

from breseq_gb300 import _lib, synth
from breseq_gb300.api import ImSettings, ScSettings
from oracle import bam_reader
from tests import bam_cases, compare, samples

pytestmark = pytest.mark.gpu

FIELDS = ("tid", "pos", "flag", "mapq", "x1", "xl", "xr", "read_file", "read_group", "l_qseq", "n_cigar", "cigar_off",
          "seq_off", "cigar", "seq", "qual", "xj", "isize", "xp", "qname_off", "qname", "mtid", "mpos")


@pytest.fixture(scope="module")
def scorer(built_lib):
    from breseq_gb300.api import Scorer
    sc = Scorer(0)
    yield sc
    sc.close()


def gpu_decode(sc, data, groups):
    with sc.open_bam(data) as b:
        hdr = b.header()
        n, nc, nb = b.decode(groups)
        rec = b.records()
    return hdr, (n, nc, nb), rec


def check(sc, data, groups):
    hdr, (n, nc, nb), g = gpu_decode(sc, data, groups)
    o = bam_reader.read_bam(data, groups)
    assert hdr == o["header"]
    size = {"cigar": nc, "seq": nb // 2, "qual": nb, "qname_off": n + 1, "qname": len(o["records"]["qname"])}
    assert n == len(o["records"]["tid"])
    for k in FIELDS:
        assert np.array_equal(g[k][:size.get(k, n)], o["records"][k]), k
    return g, (n, nc, nb)


@pytest.mark.parametrize("name", ["clonal_small", "ecoli_small", "population_small"])
def test_samples(scorer, name):
    s = samples.ALL[name]()
    g, (n, _, _) = check(scorer, synth.bam_bytes(s), synth.bam_groups(s))
    assert n == s.n_reads and np.array_equal(g["cigar"][:len(s.cigar)], s.cigar)


@pytest.mark.parametrize("level,payload", [(0, 0xFF00), (1, 0xFF00), (9, 0xFF00), (6, 4096), (6, 300)])
def test_levels_and_block_sizes(scorer, level, payload):
    s = samples.ecoli_small()
    check(scorer, synth.bam_bytes(s, level=level, block_payload=payload, seed=level), synth.bam_groups(s))


@pytest.mark.parametrize("payload", [0xFF00, 4096, 300])
def test_records_spanning_blocks(scorer, payload):
    # blocks cut at fixed sizes regardless of records (as htsjdk writes them): the record offsets come
    # from a walk over the whole inflated stream
    s = samples.ecoli_small()
    check(scorer, synth.bam_bytes(s, block_payload=payload, split_records=True), synth.bam_groups(s))
    recs, groups = bam_cases.tag_cases()
    check(scorer, bam_cases.bam(recs, split=True), groups)


def test_xj_and_single_group(scorer):
    s = samples.softclip_sample()
    check(scorer, synth.bam_bytes(s, rg_tags=False), synth.bam_groups(s))
    check(scorer, synth.bam_bytes(samples.clonal_small(), rg_tags=False), None)


def test_tag_rules(scorer):
    recs, groups = bam_cases.tag_cases()
    g, (n, _, _) = check(scorer, bam_cases.bam(recs), groups)
    assert n == 6 and g["x1"][:6].tolist() == [3, 2, 1, 0, 1, 4] and g["read_file"][:6].tolist() == [2, 1, 0, 0, 0, 2]
    check(scorer, bam_cases.bam(recs), None)
    check(scorer, bam_cases.bam(recs, rg_ids=("g0",)), (["g0"], [5], [1]))


def test_errors(scorer):
    recs, groups = bam_cases.tag_cases()
    good = bam_cases.bam(recs)
    # a CIGAR kept in the CG tag behind the placeholder <l_seq>S<reference length>N
    cg = bam_cases.record(0, 30, [(20, "S"), (20, "N")], "ACGT" * 5,
                          b"CGBI" + struct.pack("<I", 1) + struct.pack("<I", (20 << 4) | 0) + b"RGZg0\0")
    with pytest.raises(_lib.BsqError) as e:
        gpu_decode(scorer, bam_cases.bam(recs[:6] + [cg]), groups)
    assert e.value.code == -1 and "CG tag" in str(e.value)
    # unplaced records before placed ones
    with pytest.raises(_lib.BsqError):
        gpu_decode(scorer, bam_cases.bam([recs[6]] + recs[:6]), groups)
    # CRC-32 of the second block
    bad = bytearray(good)
    first = int.from_bytes(good[16:18], "little") + 1
    bad[first + int.from_bytes(good[first + 16:first + 18], "little") + 1 - 8] ^= 0xFF
    with pytest.raises(_lib.BsqError) as e:
        scorer.open_bam(bytes(bad))
    assert e.value.code == -3
    # flipped bits in compressed data: an inflate error or a CRC mismatch
    for k in range(20):
        bad = bytearray(good)
        bad[first + 20 + 3 * k] ^= 0x5A
        with pytest.raises(_lib.BsqError):
            scorer.open_bam(bytes(bad))
    # not BGZF, and a truncated file
    for data in (b"BAM\1" + bytes(40), good[: len(good) - 40]):
        with pytest.raises(_lib.BsqError) as e:
            scorer.open_bam(data)
        assert e.value.code == -1


def test_scoring_from_bam(scorer):
    s = samples.ecoli_small()
    a = scorer.load_sample(s)
    b = scorer.load_bam(synth.bam_bytes(s), s, synth.bam_groups(s))
    try:
        ea, eb = scorer.error_count(a), scorer.error_count(b)
        assert np.array_equal(ea["counts"], eb["counts"]) and np.array_equal(ea["hist"], eb["hist"])
        tab = scorer.counts_to_log10_prob(ea["counts"], s.n_read_files, s.n_quality)
        ia = scorer.identify_mutations(a, tab, ImSettings(), precision=1)
        ib = scorer.identify_mutations(b, tab, ImSettings(), precision=1)
        for k in ("ra", "mc", "un"):
            assert compare.identical(ia[k], ib[k]), k
    finally:
        scorer.free_sample(a)
        scorer.free_sample(b)
    s = samples.softclip_sample()
    a = scorer.load_sample(s)
    b = scorer.load_bam(synth.bam_bytes(s), s, synth.bam_groups(s))
    try:
        ra, rb = scorer.soft_clipping(a, ScSettings()), scorer.soft_clipping(b, ScSettings())
        assert ra["summary"] == rb["summary"] and np.array_equal(ra["rows"], rb["rows"])
    finally:
        scorer.free_sample(a)
        scorer.free_sample(b)
