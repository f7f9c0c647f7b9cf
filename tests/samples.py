"""Seeded sample configurations shared by the parity tests (small enough for the CPU oracle)."""
import dataclasses
import functools

from breseq_gb300 import synth


@functools.lru_cache(maxsize=None)
def clonal_small():
    """48,502-bp reference, 60,000 single-end 101-bp reads, 25 SNPs + 5 indels."""
    return synth.simulate(synth.config_clonal_small(seed=11))


@functools.lru_cache(maxsize=None)
def ecoli_small():
    """Three targets with five repeat copies (X1 = 5 reads), PE150 in two read files, indels up to 3 bp,
    plus trims, soft clips, N bases and mixed MAPQ to exercise the rarer branches."""
    c = synth.config_ecoli(seed=21, scale=0.02, coverage=30.0)
    c = dataclasses.replace(c, trim_fraction=0.05, softclip_fraction=0.02, n_base_rate=0.002, low_mapq_fraction=0.05,
                            large_deletions=2)
    return synth.simulate(c)


@functools.lru_cache(maxsize=None)
def population_small():
    """Polymorphism mode: 400x PE150 with frequency-spread variants, strand-bias and low-quality sites."""
    c = synth.config_population(seed=31, scale=0.01, coverage=200.0)
    return synth.simulate(c)


@functools.lru_cache(maxsize=None)
def ecoli_high_quality():
    """ecoli_small with every quality raised by 20 (up to 61): A/C/G/T qualities above 50 do not fit the
    column pass's one-byte classes, so the load keeps the packed bases and qualities for the pass."""
    import numpy as np
    s = ecoli_small()
    q = np.minimum(np.asarray(s.qual, dtype=np.uint16) + 20, 93).astype(np.uint8)
    return dataclasses.replace(s, qual=q, n_quality=int(q.max()) + 1)


@functools.lru_cache(maxsize=None)
def ecoli_q50():
    """ecoli_small with every quality raised by 9 (up to exactly 50, the largest the one-byte classes
    hold): the passes use class bytes up to 253."""
    import numpy as np
    s = ecoli_small()
    q = (np.asarray(s.qual, dtype=np.uint16) + 9).astype(np.uint8)
    assert int(q.max()) == 50
    return dataclasses.replace(s, qual=q, n_quality=51)


ALL = {"clonal_small": clonal_small, "ecoli_small": ecoli_small, "population_small": population_small,
       "ecoli_high_quality": ecoli_high_quality, "ecoli_q50": ecoli_q50}


@functools.lru_cache(maxsize=None)
def many_targets():
    """120 contigs of 1.5-4 kb (many targets, target ends everywhere, several coverage groups),
    paired-end 101-bp reads at 40x per file, short-read edge effects at every contig end."""
    import numpy as np
    rng = np.random.default_rng(5)
    lens = tuple(int(x) for x in rng.integers(1500, 4000, size=120))
    c = synth.SimConfig(seed=51, target_lengths=lens, target_names=tuple(f"contig_{i:03d}" for i in range(120)),
                        n_snps=40, n_indels=10, max_indel=2,
                        read_sets=(synth.ReadFileSet(coverage=40.0, read_length=101, paired=True),))
    return synth.simulate(c)


def empty_reads(s):
    """The sample's reference with no records at all."""
    import numpy as np
    z = lambda a: a[:0].copy()
    return dataclasses.replace(s, tid=z(s.tid), pos=z(s.pos), flag=z(s.flag), mapq=z(s.mapq), x1=z(s.x1), xl=z(s.xl),
                               xr=z(s.xr), read_file=z(s.read_file), read_group=z(s.read_group), l_qseq=z(s.l_qseq),
                               seq_off=z(s.seq_off), cigar_off=z(s.cigar_off), n_cigar=z(s.n_cigar),
                               cigar=np.zeros(1, dtype=np.uint32), seq=np.zeros(1, dtype=np.uint8),
                               qual=np.zeros(1, dtype=np.uint8))


def all_filtered(s):
    """Every record flagged as a duplicate: the pileup keeps none of them."""
    return dataclasses.replace(s, flag=(s.flag | 0x400).astype(s.flag.dtype))


@functools.lru_cache(maxsize=None)
def softclip_sample():
    """Soft-clip evidence: three targets whose std::string order differs from their index order,
    PE150 at 60x per file with five repeat copies, 40 junction breakpoints (each clips a share of the
    reads crossing it with one donor sequence), 1% of reads clipped by 12-40 random bases, the small
    random clips, N bases, and 2% of records tagged XJ."""
    c = synth.config_ecoli(seed=71, scale=0.03, coverage=60.0)
    c = dataclasses.replace(c, target_names=("zeta_chromosome", "Alpha_plasmid", "beta_plasmid"),
                            softclip_fraction=0.02, n_base_rate=0.002, breakpoints=40, long_clip_fraction=0.01,
                            xj_fraction=0.02)
    return synth.simulate(c)


def with_flags(s, seed=3, unmapped=0.01, secondary=0.02, qcfail=0.01):
    """Some records unmapped (no soft-clip events), secondary or QC-failed (the pileup skips them, the
    soft-clip tabulation keeps them)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    f = s.flag.copy()
    u = rng.random(f.size)
    f[u < unmapped] |= 0x4
    f[(u >= unmapped) & (u < unmapped + secondary)] |= 0x100
    f[(u >= unmapped + secondary) & (u < unmapped + secondary + qcfail)] |= 0x200
    return dataclasses.replace(s, flag=f)


_OPS = {"M": 0, "I": 1, "D": 2, "N": 3, "S": 4, "H": 5, "P": 6, "=": 7, "X": 8}
_NIB = {"=": 0, "A": 1, "C": 2, "G": 4, "T": 8, "N": 15}


def from_records(targets, reads, n_quality=42):
    """A sample built record by record.  targets: [(name, sequence)]; reads: dicts with tid, pos
    (0-based), cigar ("5S30M"), seq (A/C/G/T/N; aligned bases may be "" to copy the reference),
    and optional flag, x1, xj, mapq.  Records are sorted by (tid, pos) as a BAM would be."""
    import re
    import numpy as np
    names = [n for n, _ in targets]
    ref = "".join(s for _, s in targets).encode()
    toff = np.zeros(len(targets) + 1, dtype=np.uint64)
    toff[1:] = np.cumsum([len(s) for _, s in targets])
    reads = sorted(reads, key=lambda r: (r["tid"], r["pos"]))
    cig, seqs, n_cigar = [], [], []
    for r in reads:
        ops = [(int(n), _OPS[o]) for n, o in re.findall(r"(\d+)([MIDNSHP=X])", r["cigar"])]
        cig += [(n << 4) | o for n, o in ops]
        n_cigar.append(len(ops))
        seqs.append(r["seq"])
    L = np.array([len(s) for s in seqs], dtype=np.uint32)
    Lp = L + (L & 1)
    seq_off = np.zeros(len(reads), dtype=np.uint64)
    seq_off[1:] = np.cumsum(Lp[:-1])
    nib = np.zeros(max(2, int(Lp.sum())), dtype=np.uint8)
    for i, s in enumerate(seqs):
        nib[int(seq_off[i]): int(seq_off[i]) + len(s)] = [_NIB[c] for c in s]
    cigar_off = np.zeros(len(reads), dtype=np.uint64)
    cigar_off[1:] = np.cumsum(n_cigar[:-1])
    n = len(reads)
    g = lambda k, d, dt: np.array([r.get(k, d) for r in reads], dtype=dt)
    return synth.Sample(
        ref_seq=np.frombuffer(ref, dtype=np.uint8).copy(), target_offset=toff, target_names=names,
        coverage_group=np.arange(len(targets), dtype=np.uint32), n_coverage_groups=len(targets),
        target_order=np.array(sorted(range(len(names)), key=lambda t: names[t]), dtype=np.uint32),
        tid=g("tid", 0, np.int32), pos=g("pos", 0, np.int32), flag=g("flag", 0, np.uint16), mapq=g("mapq", 42, np.uint8),
        x1=g("x1", 1, np.uint32), xl=np.full(n, -1, dtype=np.int32), xr=np.full(n, -1, dtype=np.int32),
        read_file=np.zeros(n, dtype=np.uint8), read_group=np.zeros(n, dtype=np.uint16), l_qseq=L,
        seq_off=seq_off, cigar_off=cigar_off, n_cigar=np.array(n_cigar, dtype=np.uint16),
        cigar=np.array(cig or [0], dtype=np.uint32), seq=((nib[0::2] << 4) | nib[1::2]).astype(np.uint8),
        qual=np.full(max(2, int(Lp.sum())), 30, dtype=np.uint8), n_read_files=1, n_quality=n_quality,
        xj=g("xj", 0, np.uint8))


def softclip_known():
    """Hand-made records with the soft-clip tabulation worked out by hand (minimum clipped bases 4,
    so four consensus columns and a margin of 4).  Target 0 "t1" (60 bp), target 1 "s0" (40 bp):
    std::string order puts s0 first.

    t1 position 21, direction -1: R1 R2 R3 and the secondary R8 are clipped by >= 4; R4 by 3 (too
    short); R5 unmapped, R6 X1 = 2, R7 XJ are skipped.  Tails outward from the wall: ACGT, ACGT, ACGG,
    CAGT -> consensus ACGT (col 3: T 3 : G 1), 3 of 4 matches required, R8 matches 2 -> agree 3,
    stored reference-forward as TGCA.  Spanning (4 aligned bases both sides): R9, R10, C1 -> total 7.
    t1 position 40, direction +1: R9 (A N G T), R10 (C N G A), C1 (A G G T, complex CIGAR) -> consensus
    col 0 A (2:1), col 1 G (the only base), col 2 G, col 3 T (2:1) = AGGT; R10 matches 1 -> agree 2.
    Spanning: R1 R2 R3 R4 R8 -> total 8.
    s0 position 11, direction -1: one read clipped by NNNNN -> no informative column, agree 0, no
    sequence, nothing spans it.
    R11 clipped at t1 position 1 and R12 at position 60 are not testable (margin)."""
    import numpy as np
    rng = np.random.default_rng(17)
    t1 = "".join("ACGT"[i] for i in rng.integers(0, 4, 60))
    s0 = "".join("ACGT"[i] for i in rng.integers(0, 4, 40))

    def rd(tid, pos, cigar, clip_l="", clip_r="", aligned=None, **kw):
        import re
        ops = re.findall(r"(\d+)([MIDNSHP=X])", cigar)
        ref = t1 if tid == 0 else s0
        body, x = "", pos
        for n_, o in ops:
            n_ = int(n_)
            if o == "M":
                body += ref[x:x + n_]; x += n_
            elif o == "I":
                body += "A" * n_
            elif o == "D":
                x += n_
        return dict(tid=tid, pos=pos, cigar=cigar, seq=clip_l + body + clip_r, **kw)

    reads = [
        rd(0, 20, "5S30M", clip_l="NTGCA"),              # R1 tail ACGT
        rd(0, 20, "6S30M", clip_l="GGTGCA"),             # R2 tail ACGT
        rd(0, 20, "4S30M", clip_l="GGCA"),               # R3 tail ACGG
        rd(0, 20, "3S30M", clip_l="TTT"),                # R4 clip too short
        rd(0, 20, "5S30M", clip_l="NTGCA", flag=0x4),    # R5 unmapped
        rd(0, 20, "5S30M", clip_l="NTGCA", x1=2),        # R6 redundant
        rd(0, 20, "5S30M", clip_l="NTGCA", xj=1),        # R7 junction side
        rd(0, 20, "5S30M", clip_l="NTGAC", flag=0x100),  # R8 secondary, tail CAGT
        rd(0, 10, "30M6S", clip_r="ANGTCC"),             # R9 tail ANGT
        rd(0, 10, "30M4S", clip_r="CNGA"),               # R10 tail CNGA
        rd(0, 0, "3S20M", clip_l="GGG"),                 # R11 at position 1
        rd(0, 50, "10M5S", clip_r="ACGTA"),              # R12 at position 60
        rd(0, 12, "10M2I5M3D10M5S", clip_r="AGGTC"),     # C1 ends at 40, tail AGGT
        rd(1, 10, "5S20M", clip_l="NNNNN"),              # s0 position 11
    ]
    expected = [
        ("s0", 11, -1, 1, 1, 0, ""),
        ("t1", 21, -1, 4, 7, 3, "TGCA"),
        ("t1", 40, 1, 3, 8, 2, "AGGT"),
    ]
    return from_records([("t1", t1), ("s0", s0)], reads), expected


@functools.lru_cache(maxsize=None)
def dp_skip_sample():
    """Paired-end sample with discordant pairs at 10 sites and a 2% background, half of the discordant
    reads without an XP tag: the reads breseq's identify_mutations pileup leaves out of their first
    column when their read group has a discordant-pair group (identify_mutations.cpp:1399-1416)."""
    c = synth.config_ecoli(seed=23, scale=0.01, coverage=30.0)
    return synth.with_pairs(synth.simulate(c), seed=4, discordant_sites=10, background_discordant=0.02,
                            no_xp_fraction=0.5)


@functools.lru_cache(maxsize=None)
def dp_two_groups():
    """dp_skip_sample with a seeded 40% of its fragments (records 2k and 2k + 1) moved to a second
    paired read group (read files 2 and 3): with a discordant-pair group on the first group only, the
    coverage table's per-read-group columns show the first-column skip in one group and not the other."""
    import dataclasses
    import numpy as np
    s = dp_skip_sample()
    frag = np.arange(len(s.read_group)) // 2
    move = np.random.default_rng(9).random(int(frag.max()) + 1 if len(frag) else 0)[frag] < 0.4
    return dataclasses.replace(s, read_group=np.where(move, 1, s.read_group).astype(np.uint16),
                               read_file=np.where(move, s.read_file + 2, s.read_file).astype(np.uint8),
                               n_read_files=4)


def dp_skip_reads(s, dp_group):
    """Indices of the records the discordant-pair enter step ends at their first column."""
    import numpy as np
    f = s.flag.astype(np.int64)
    rg = s.read_group.astype(np.int64)
    member = np.array([g < len(dp_group) and dp_group[g] >= 0 for g in rg], dtype=bool)
    cand = ((f & 0x1) != 0) & ((f & 0x4) == 0) & ((f & 0x2) == 0) & ((f & (0x100 | 0x800 | 0x8)) == 0)
    return np.nonzero(cand & member & (s.xp > 2) & ((f & 0x704) == 0))[0]


@functools.lru_cache(maxsize=None)
def ecoli_quarter():
    """The E. coli-scale clonal workload's shape at 0.25x genome length with its full coverage: 1.16 Mb +
    25 kb + 15 kb targets, five 1.3-kb repeats, 2 x 100x paired-end 150-bp reads (0.24 G read-bases)."""
    return synth.simulate(synth.config_ecoli(seed=61, scale=0.25))


@functools.lru_cache(maxsize=None)
def population_deep():
    """The 1000x population workload's shape at 0.05x genome length: paired-end 150-bp reads at 1000x,
    variants at log-uniform frequencies, strand-biased and low-quality sites (0.26 G read-bases)."""
    return synth.simulate(synth.config_population(seed=62, scale=0.05))


def sample_digest(s):
    """SHA-256 of a sample's reference and records: the golden files were made from exactly this."""
    import hashlib
    import numpy as np
    h = hashlib.sha256()
    for a in (s.ref_seq, s.target_offset, s.tid, s.pos, s.flag, s.mapq, s.x1, s.xl, s.xr, s.read_file, s.read_group,
              s.l_qseq, s.seq_off, s.cigar_off, s.n_cigar, s.cigar, s.seq, s.qual):
        h.update(np.ascontiguousarray(a).tobytes())
    if s.xp is not None:
        h.update(np.ascontiguousarray(s.xp).tobytes())
    return h.hexdigest()
