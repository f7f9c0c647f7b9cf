"""Soft-clipping tabulation (src/breseq/soft_clipping.cpp:285-666) on the CPU: the oracle against
hand-worked answers and the rules the reference states, and the counts-file writer of the library."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from breseq_gb300 import _lib, abi
from oracle import pyoracle as po

from tests import samples


def rows_as_tuples(s, rows):
    return [(s.target_names[r["target"]], int(r["position"]), int(r["direction"]), int(r["clipped_count"]),
             int(r["total_count"]), int(r["agree_count"]), r["clipped_sequence"].decode()) for r in rows]


def spanning_by_hand(s, m):
    """Sum over testable positions of 2 x the reads with m aligned bases on both sides, and 2 x the
    testable positions with any such read (soft_clipping.cpp:395-408, 468-490), by direct counting."""
    total, tested = 0, 0
    for t in range(len(s.target_names)):
        tlen = int(s.target_offset[t + 1] - s.target_offset[t])
        cov = np.zeros(tlen + 2, dtype=np.int64)
        for i in np.nonzero(s.tid == t)[0]:
            if s.flag[i] & 4 or s.x1[i] > 1 or (s.xj is not None and s.xj[i]):
                continue
            ops = s.cigar[s.cigar_off[i]: s.cigar_off[i] + s.n_cigar[i]]
            rlen = sum(int(c >> 4) for c in ops if (c & 0xF) in (0, 2, 3, 7, 8))
            start1, end1 = int(s.pos[i]) + 1, int(s.pos[i]) + rlen
            for p in range(start1 + m, end1 - m + 1):
                cov[p] += 1
        margin = max(m, 1)
        for p in range(1, tlen + 2):
            if p > margin and p + margin <= tlen:
                total += 2 * int(cov[p])
                tested += 2 if cov[p] > 0 else 0
    return total, tested


def test_oracle_known_answers():
    s, expected = samples.softclip_known()
    r = po.soft_clipping(s, minimum_clipped_bases=4)
    assert rows_as_tuples(s, r["rows"]) == expected
    sm = r["summary"]
    span, tested = spanning_by_hand(s, 4)
    assert sm["total_spanning_read_bases"] == span
    assert sm["total_clipped_read_ends"] == 8
    assert sm["total_agreeing_clipped_read_ends"] == 5
    # positions with clips and nothing spanning them count once more (s0:11)
    tested += 1
    # the fit by its formula (soft_clipping.cpp:570-623), trimming rows at k/n >= 0.25
    opp = 8 + span
    p0 = 5 / opp
    kept = [(k, n) for (_, _, _, _, n, k, _) in expected if not (k / n >= 0.25)]
    trimmed = [(k, n) for (_, _, _, _, n, k, _) in expected if k / n >= 0.25]
    N = tested - len(trimmed)
    S_n = opp - sum(n for _, n in trimmed)
    chi2 = (sum(k * k / n for k, n in kept) - 2 * p0 * sum(k for k, _ in kept) + p0 * p0 * S_n) / (p0 * (1 - p0))
    phi = chi2 / (N - 1)
    rho = (phi - 1) / (S_n / N - 1)
    assert sm["trimmed_positions"] == len(trimmed) and sm["tested_positions"] == N
    assert math.isclose(sm["null_rate"], p0, rel_tol=1e-15)
    assert math.isclose(sm["pearson_phi"], phi, rel_tol=1e-12)
    assert math.isclose(sm["dispersion_raw"], rho, rel_tol=1e-12)
    assert sm["dispersion"] == (0.0 if rho < 1e-6 else min(rho, 0.005))


def _tail_sample(tails, m=12, lead=True):
    """Reads clipped at one position (t:101) with the given tails (column 0 next to the wall)."""
    rng = np.random.default_rng(2)
    ref = "".join("ACGT"[i] for i in rng.integers(0, 4, 300))
    reads = []
    for tail in tails:
        if lead:
            reads.append(dict(tid=0, pos=100, cigar=f"{len(tail)}S50M", seq=tail[::-1] + ref[100:150]))
        else:
            reads.append(dict(tid=0, pos=50, cigar=f"50M{len(tail)}S", seq=ref[50:100] + tail))
    return samples.from_records([("t", ref)], reads)


def test_oracle_one_mismatch_in_twelve_agrees():
    # "0.95 over 12 compared bases requires 11 matches, i.e. tolerates exactly one mismatched base"
    # (soft_clipping.cpp:130-131)
    base = "ACGTACGTTGCA"
    one = "ACGTACGTTGCC"
    two = "ACGTACGTTGGG"
    for lead in (True, False):
        s = _tail_sample([base, base, one, two], lead=lead)
        r = po.soft_clipping(s)
        assert len(r["rows"]) == 1
        row = r["rows"][0]
        assert row["clipped_count"] == 4 and row["agree_count"] == 3
        assert row["clipped_sequence"].decode() == (base[::-1] if lead else base)


def test_oracle_ties_and_uninformative_columns():
    # ties go to the lowest base code (A < C < G < T); an all-N column is 'N' and left out of the
    # match count on both sides (soft_clipping.cpp:65-78)
    s = _tail_sample(["TNGT", "ANGA"], m=4, lead=False)
    r = po.soft_clipping(s, minimum_clipped_bases=4)
    row = r["rows"][0]
    assert row["clipped_sequence"].decode() == "ANGA"
    # informative columns 0, 2, 3: required floor(0.95 * 3) = 2; TNGT matches G only
    assert row["agree_count"] == 1
    # consensus switched off: every clipped read counts and no sequence is reported
    r0 = po.soft_clipping(s, minimum_clipped_bases=4, consensus_base_fraction=0.0)
    assert r0["rows"][0]["agree_count"] == 2 and r0["rows"][0]["clipped_sequence"] == b""


def test_oracle_consensus_capped_at_21_columns():
    tail = "ACGT" * 8
    s = _tail_sample([tail, tail], m=30, lead=False)
    r = po.soft_clipping(s, minimum_clipped_bases=30)
    assert r["rows"][0]["clipped_sequence"].decode() == tail[:21]


def test_oracle_rejects_kept_record_past_target():
    s, _ = samples.softclip_known()
    import dataclasses
    pos = s.pos.copy()
    flag = s.flag.copy()
    i = int(np.nonzero(s.tid == 0)[0][-1])
    pos[i] = 58                      # 30+ reference bases from 58 run past the 60-bp target
    flag[i] |= 0x100                 # secondary: the pileup would skip it, the tabulation keeps it
    with pytest.raises(po.OracleError):
        po.soft_clipping(dataclasses.replace(s, pos=pos, flag=flag), minimum_clipped_bases=4)


def test_counts_file_format(tmp_path, built_lib):
    s, expected = samples.softclip_known()
    r = po.soft_clipping(s, minimum_clipped_bases=4)
    L = _lib.load()
    p = abi.ScParams()
    assert L.bsq_default_sc_params(C.byref(p)) == 0
    assert (p.minimum_clipped_bases, p.consensus_base_fraction, p.dispersion_trim_frequency,
            p.maximum_dispersion, p.minimum_rate) == (12, 0.95, 0.25, 0.005, 1e-5)
    p.minimum_clipped_bases = 4
    sm = abi.ScSummary(**r["summary"])
    rows = (abi.ScPosition * len(r["rows"]))()
    for i, x in enumerate(r["rows"]):
        rows[i] = abi.ScPosition(*[x[k] for k in abi.SC_ROW_DTYPE.names])
    names = (C.c_char_p * 2)(b"t1", b"s0")
    path = str(tmp_path / "soft_clipping_counts.tab")
    assert L.bsq_write_soft_clipping_counts(path.encode(), names, C.byref(p), C.byref(sm), rows, len(r["rows"])) == 0
    # soft_clipping.cpp:630-646, doubles in default ostream form (%g, 6 significant digits)
    want = [f"#sc_format=2\tsoft_clipping_minimum_bases=4\tconsensus_base_fraction=0.95\t"
            f"null_rate={sm.null_rate:g}\tdispersion={sm.dispersion:g}",
            "seq_id\tposition\tdirection\tclipped_count\ttotal_count\tagree_count\tclipped_sequence"]
    want += ["\t".join([n, str(pos), str(d), str(c), str(t), str(a), seq or "."]) for n, pos, d, c, t, a, seq in expected]
    assert open(path).read() == "\n".join(want) + "\n"
    assert "null_rate=0.0122549\tdispersion=0" in open(path).read()
