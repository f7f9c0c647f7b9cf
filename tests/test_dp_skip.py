"""The discordant-pair enter step of breseq's identify_mutations pileup ends its per-read loop
(`continue`, src/breseq/identify_mutations.cpp:1399-1416) for a paired, mapped, non-proper read with a
mapped mate and no usable XP tag, in a read group that has a discordant-pair (DP) group, at the read's
first column and insert position 0: the read adds nothing there (no coverage, no likelihoods).  The
oracle restates it; this checks its effect on the per-position coverage against a count made here."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests import samples


def test_dp_skip_removes_reads_from_their_first_column(oracle_lib):
    s = samples.dp_skip_sample()
    n_rg = int(s.read_group.max()) + 1
    dp = tuple(0 for _ in range(n_rg))
    skipped = samples.dp_skip_reads(s, dp)
    assert len(skipped) > 20, "the sample must carry discordant reads without an XP tag"
    ec = po.error_count(s)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    base = po.identify(s, tab, po.default_im_params(s))["positions"]
    with_dp = po.identify(s, tab, po.default_im_params(s, dp_group=dp))["positions"]
    # expected change: each skipped unique read whose first read base is not N leaves its first column
    col = (s.target_offset[s.tid[skipped]] + s.pos[skipped]).astype(np.int64)
    rev = (s.flag[skipped] & 0x10) != 0
    unique = s.x1[skipped] == 1
    first_q = s.seq_off[skipped].astype(np.int64) + np.array(
        [(s.cigar[s.cigar_off[r]] >> 4) if (s.cigar[s.cigar_off[r]] & 0xF) == 4 else 0 for r in skipped])
    nib = np.where(first_q % 2 == 0, s.seq[first_q // 2] >> 4, s.seq[first_q // 2] & 15)
    keep = unique & (nib != 15)
    d_top = np.zeros_like(base["unique_top"], dtype=np.int64)
    d_bot = np.zeros_like(d_top)
    np.add.at(d_top, col[keep & ~rev], 1)
    np.add.at(d_bot, col[keep & rev], 1)
    assert np.array_equal(base["unique_top"].astype(np.int64) - with_dp["unique_top"], d_top)
    assert np.array_equal(base["unique_bot"].astype(np.int64) - with_dp["unique_bot"], d_bot)
    # no DP group, or DP groups on other read groups only: nothing changes
    none = po.identify(s, tab, po.default_im_params(s, dp_group=tuple(-1 for _ in range(n_rg))))["positions"]
    assert np.array_equal(none["unique_top"], base["unique_top"])
    assert np.array_equal(none["n_scored"], base["n_scored"])


def test_dp_skip_needs_a_usable_xp_tag(oracle_lib):
    """Reads whose XP tag is FR / RF / FF enter the DP window and stay in the column."""
    import dataclasses
    s = samples.dp_skip_sample()
    n_rg = int(s.read_group.max()) + 1
    dp = tuple(0 for _ in range(n_rg))
    tagged = dataclasses.replace(s, xp=np.where(s.xp > 2, 0, s.xp).astype(np.uint8))
    assert len(samples.dp_skip_reads(tagged, dp)) == 0
    ec = po.error_count(tagged)
    tab = po.counts_to_log10_prob(ec["counts"], tagged.n_read_files, tagged.n_quality)
    a = po.identify(tagged, tab, po.default_im_params(tagged))["positions"]
    b = po.identify(tagged, tab, po.default_im_params(tagged, dp_group=dp))["positions"]
    for k in ("unique_top", "unique_bot", "n_scored"):
        assert np.array_equal(a[k], b[k])
