"""Seeded synthetic genomes and aligned reads in the packed record layout of the library.

There is no aligner and no public data set here, so reads are simulated together with their true
alignment, the way breseq's own SIMULATE-READS command draws them (src/breseq/fastq.cpp:1301-1459)
but with the quality law of the scoring benchmarks: Q_i ~ N(36 - 8 i / L, 4) rounded and clipped to
[2, 41] in sequencing order, and a substitution to a uniformly chosen other base with probability
10^(-Q/10).  Tags follow breseq's reference.bam conventions (src/breseq/alignment.cpp:915-945):
X1 = number of equally good locations (reads inside repeat copies are written at every copy, with
MAPQ 0), XL/XR trims present on every record, and the read group + mate flag giving the read file.

Everything is numpy; generation is chunked so the 4.8 Mb x 200x workload stays within a few GB.
"""
from __future__ import annotations

import concurrent.futures as cf
import dataclasses
import os
from dataclasses import dataclass, field, replace

import numpy as np

BASES = np.frombuffer(b"ACGT", dtype=np.uint8)
# ASCII -> 4-bit BAM code
_ASCII2BAM = np.full(256, 15, dtype=np.uint8)
for _c, _v in zip(b"ACGTN", (1, 2, 4, 8, 15)):
    _ASCII2BAM[_c] = _v
BAM_M, BAM_I, BAM_D, BAM_S = 0, 1, 2, 4
FLAG_PAIRED, FLAG_PROPER, FLAG_REVERSE, FLAG_MREVERSE, FLAG_READ1, FLAG_READ2 = 0x1, 0x2, 0x10, 0x20, 0x40, 0x80


@dataclass
class ReadFileSet:
    """One read group: single-end (one read file) or paired-end (two files, R1 then R2)."""
    coverage: float            # fold coverage contributed by EACH file of the set
    read_length: int
    paired: bool = False
    insert_mean: float = 350.0
    insert_sd: float = 50.0


@dataclass
class SimConfig:
    seed: int = 1
    target_lengths: tuple = (48502,)
    target_names: tuple | None = None
    gc: float = 0.5
    n_snps: int = 25
    n_indels: int = 5
    max_indel: int = 1
    # population mode: variant frequencies log-uniform in [freq_min, 1]; clonal when None
    freq_min: float | None = None
    repeat_copies: int = 0
    repeat_length: int = 1300
    read_sets: tuple = (ReadFileSet(coverage=125.0, read_length=101),)
    strand_bias_sites: int = 0
    low_quality_sites: int = 0
    # rates of features that exercise the rarer branches of the scoring path
    trim_fraction: float = 0.0      # reads with non-zero XL/XR
    softclip_fraction: float = 0.0  # reads with a soft clip at one end
    n_base_rate: float = 0.0        # read bases replaced by N (quality 2)
    low_mapq_fraction: float = 0.0  # unique reads with MAPQ drawn in [20, 41]
    large_deletions: int = 0        # regions of the reference missing from the sample (MC evidence)
    large_deletion_length: int = 800
    # soft-clip evidence: junctions whose crossing reads are clipped at the junction with one donor
    # sequence each, longer clips of random bases, and records tagged XJ
    breakpoints: int = 0
    long_clip_fraction: float = 0.0  # unique reads clipped by 12-40 random bases at one end
    xj_fraction: float = 0.0
    chunk_reads: int = 400_000


@dataclass
class Sample:
    """Reference + coordinate-sorted records, in the bsq_reference / bsq_read_soa layout."""
    ref_seq: np.ndarray            # uint8 ASCII, all targets concatenated
    target_offset: np.ndarray      # uint64 [T+1]
    target_names: list
    coverage_group: np.ndarray     # uint32 [T]
    n_coverage_groups: int
    target_order: np.ndarray       # uint32: lexicographic seq_id order
    tid: np.ndarray
    pos: np.ndarray
    flag: np.ndarray
    mapq: np.ndarray
    x1: np.ndarray
    xl: np.ndarray
    xr: np.ndarray
    read_file: np.ndarray
    read_group: np.ndarray
    l_qseq: np.ndarray
    seq_off: np.ndarray
    cigar_off: np.ndarray
    n_cigar: np.ndarray
    cigar: np.ndarray
    seq: np.ndarray                # packed 4-bit, high nibble first
    qual: np.ndarray
    n_read_files: int
    n_quality: int
    variants: list = field(default_factory=list)
    xj: np.ndarray | None = None   # uint8, XJ tag present; None when no record has one
    # pair annotations (with_pairs): TLEN, XP orientation code (0 FR, 1 RF, 2 FF, 3 none), read names
    isize: np.ndarray | None = None
    xp: np.ndarray | None = None
    qname_off: np.ndarray | None = None
    qname: np.ndarray | None = None
    mtid: np.ndarray | None = None     # mate reference id and 0-based position (RNEXT / PNEXT)
    mpos: np.ndarray | None = None

    @property
    def n_reads(self) -> int:
        return int(self.tid.shape[0])

    def aligned_bases(self) -> int:
        """Aligned read-bases (M/=/X + I lengths) over records the pileup keeps: the unit of work."""
        ops = self.cigar & 0xF
        lens = (self.cigar >> 4).astype(np.int64)
        keep = (self.flag & 0x704) == 0
        per_op = np.where((ops == 0) | (ops == 1) | (ops == 7) | (ops == 8), lens, 0)
        owner = np.repeat(np.arange(self.n_reads), self.n_cigar.astype(np.int64))
        return int(per_op[keep[owner]].sum())

    def total_length(self) -> int:
        return int(self.target_offset[-1])


def _lexicographic_order(names):
    return np.array(sorted(range(len(names)), key=lambda i: names[i]), dtype=np.uint32)


_ERR_LUT = np.power(10.0, -np.arange(256, dtype=np.float64) / 10.0).astype(np.float32)
_CODE2BAM = np.array([1, 2, 4, 8], dtype=np.uint8)


def _quality_table(L):
    """[L, 65536] inverse-CDF tables: quality at read position i for a uniform 16-bit draw, following
    Q_i ~ N(36 - 8 i / L, 4) rounded to the nearest integer and clipped to [2, 41]."""
    from math import erf, sqrt
    qs = np.arange(2, 42)
    u = (np.arange(65536) + 0.5) / 65536.0
    tab = np.empty((L, 65536), dtype=np.uint8)
    for i in range(L):
        mu = 36.0 - 8.0 * i / L
        # P(round(X) <= q) = Phi((q + 0.5 - mu) / 4); clipping moves the tails onto 2 and 41
        cdf = np.array([0.5 * (1 + erf((q + 0.5 - mu) / (4.0 * sqrt(2.0)))) for q in qs])
        cdf[-1] = 1.0
        tab[i] = qs[np.searchsorted(cdf, u, side="right").clip(0, len(qs) - 1)]
    return tab


def simulate(cfg: SimConfig) -> Sample:
    rng = np.random.default_rng(cfg.seed)
    T = len(cfg.target_lengths)
    names = list(cfg.target_names) if cfg.target_names else [f"seq{t + 1}" for t in range(T)]
    lens = np.array(cfg.target_lengths, dtype=np.int64)
    toff = np.zeros(T + 1, dtype=np.uint64)
    toff[1:] = np.cumsum(lens)
    total = int(toff[-1])
    # ---------------------------------------------------------------- reference
    probs = np.array([(1 - cfg.gc) / 2, cfg.gc / 2, cfg.gc / 2, (1 - cfg.gc) / 2])
    ref = BASES[rng.choice(4, size=total, p=probs)]
    repeat_spans = []
    if cfg.repeat_copies > 1:
        L0 = int(lens[0])
        seg = BASES[rng.choice(4, size=cfg.repeat_length, p=probs)]
        slots = np.sort(rng.choice(L0 // (cfg.repeat_length * 3), size=cfg.repeat_copies, replace=False))
        for s in slots:
            p0 = int(s) * cfg.repeat_length * 3 + cfg.repeat_length
            ref[p0:p0 + cfg.repeat_length] = seg
            repeat_spans.append((0, p0, p0 + cfg.repeat_length))
    # ---------------------------------------------------------------- variants
    def _in_repeat(t, p, margin):
        return any(t == rt and rs - margin <= p < re + margin for rt, rs, re in repeat_spans)

    variants = []   # dict(tid, pos, kind, alt/len, freq, artifact)
    taken = set()
    def _pick_site(margin=8):
        for _ in range(10000):
            t = int(rng.choice(T, p=lens / lens.sum()))
            p = int(rng.integers(200, max(201, int(lens[t]) - 400)))
            if _in_repeat(t, p, 200) or any((t, q) in taken for q in range(p - margin, p + margin)):
                continue
            taken.add((t, p))
            return t, p
        raise RuntimeError("no free site")

    def _freq():
        if cfg.freq_min is None:
            return 1.0
        return float(np.exp(rng.uniform(np.log(cfg.freq_min), 0.0)))

    for _ in range(cfg.n_snps):
        t, p = _pick_site()
        r = ref[toff[t] + p]
        alt = BASES[rng.choice([b for b in range(4) if BASES[b] != r])]
        variants.append(dict(tid=t, pos=p, kind="snp", alt=int(alt), freq=_freq()))
    for _ in range(cfg.n_indels):
        t, p = _pick_site(margin=8 + cfg.max_indel)
        k = int(rng.integers(1, cfg.max_indel + 1))
        if rng.random() < 0.5:
            variants.append(dict(tid=t, pos=p, kind="del", length=k, freq=_freq()))
        else:
            ins = BASES[rng.integers(0, 4, size=k)]
            variants.append(dict(tid=t, pos=p, kind="ins", seq=ins, freq=_freq()))
    for _ in range(cfg.strand_bias_sites):
        t, p = _pick_site()
        r = ref[toff[t] + p]
        alt = BASES[rng.choice([b for b in range(4) if BASES[b] != r])]
        variants.append(dict(tid=t, pos=p, kind="strand_bias", alt=int(alt), freq=0.15, strand=int(rng.integers(0, 2))))
    for _ in range(cfg.low_quality_sites):
        t, p = _pick_site()
        r = ref[toff[t] + p]
        alt = BASES[rng.choice([b for b in range(4) if BASES[b] != r])]
        variants.append(dict(tid=t, pos=p, kind="low_quality", alt=int(alt), freq=0.10))

    deleted = []   # (tid, start, end) regions absent from the sample: no read covers them
    for _ in range(cfg.large_deletions):
        t, p = _pick_site(margin=cfg.large_deletion_length + 300)
        deleted.append((t, p, p + cfg.large_deletion_length))
        variants.append(dict(tid=t, pos=p, kind="large_del", length=cfg.large_deletion_length, freq=1.0))
    # ---------------------------------------------------------------- read placement
    recs = {k: [] for k in ("tid", "pos", "flag", "rfile", "rg", "L", "clipL", "clipR", "x1", "group")}
    rfile_base = 0
    max_indel_span = cfg.max_indel + 1
    group_counter = 0
    for gi, rs in enumerate(cfg.read_sets):
        L = rs.read_length
        n_frag = int(round(rs.coverage * total / L))
        tids = rng.choice(T, size=n_frag, p=lens / lens.sum())
        if rs.paired:
            ins = np.clip(np.rint(rng.normal(rs.insert_mean, rs.insert_sd, n_frag)), L, None).astype(np.int64)
        else:
            ins = np.full(n_frag, L, dtype=np.int64)
        hi = lens[tids] - ins - max_indel_span
        start = (rng.random(n_frag) * np.maximum(hi, 1)).astype(np.int64)
        fwd = rng.random(n_frag) < 0.5
        mates = [(start, ~fwd, 0)] if not rs.paired else [(start, ~fwd, 0), (start + ins - L, fwd, 1)]
        for p_arr, rev, mate in mates:
            # in a pair, mate 0 takes the fragment's strand, mate 1 the opposite
            flag = np.where(rev, FLAG_REVERSE, 0).astype(np.uint16)
            if rs.paired:
                flag |= FLAG_PAIRED | FLAG_PROPER | (FLAG_READ1 if mate == 0 else FLAG_READ2)
                flag |= np.where(~rev, FLAG_MREVERSE, 0).astype(np.uint16)
            recs["tid"].append(tids); recs["pos"].append(p_arr); recs["flag"].append(flag)
            recs["rfile"].append(np.full(n_frag, rfile_base + mate, dtype=np.uint8))
            recs["rg"].append(np.full(n_frag, gi, dtype=np.uint16))
            recs["L"].append(np.full(n_frag, L, dtype=np.int64))
            recs["group"].append(np.arange(group_counter, group_counter + n_frag))
            group_counter += n_frag
        rfile_base += 2 if rs.paired else 1
    tid = np.concatenate(recs["tid"]).astype(np.int32)
    pos = np.concatenate(recs["pos"]).astype(np.int64)
    flag = np.concatenate(recs["flag"])
    rfile = np.concatenate(recs["rfile"])
    rg = np.concatenate(recs["rg"])
    L_arr = np.concatenate(recs["L"])
    if deleted:
        keep = np.ones(tid.shape[0], dtype=bool)
        for t, a, b in deleted:
            keep &= ~((tid == t) & (pos < b) & (pos + L_arr + max_indel_span > a))
        tid, pos, flag, rfile, rg, L_arr = tid[keep], pos[keep], flag[keep], rfile[keep], rg[keep], L_arr[keep]
    n = tid.shape[0]
    mapq = np.full(n, 42, dtype=np.uint8)
    if cfg.low_mapq_fraction > 0:
        m = rng.random(n) < cfg.low_mapq_fraction
        mapq[m] = rng.integers(20, 42, size=int(m.sum())).astype(np.uint8)
    x1 = np.ones(n, dtype=np.uint32)
    clip_l = np.zeros(n, dtype=np.int64)
    clip_r = np.zeros(n, dtype=np.int64)
    if cfg.softclip_fraction > 0:
        m = rng.random(n) < cfg.softclip_fraction
        k = rng.integers(1, 11, size=n)
        left = rng.random(n) < 0.5
        clip_l[m & left] = k[m & left]
        clip_r[m & ~left] = k[m & ~left]
    # reads fully inside a repeat copy map equally well to every copy
    src_index = np.arange(n)
    if repeat_spans:
        inside = np.zeros(n, dtype=bool)
        which = np.full(n, -1)
        for ci, (rt, rs0, re0) in enumerate(repeat_spans):
            m = (tid == rt) & (pos >= rs0) & (pos + L_arr <= re0)
            inside |= m
            which[m] = ci
        idx = np.nonzero(inside)[0]
        ncp = len(repeat_spans)
        x1[idx] = ncp
        mapq[idx] = 0
        extra_src = np.repeat(idx, ncp - 1)
        extra_pos = []
        for i0 in idx:
            off = pos[i0] - repeat_spans[which[i0]][1]
            for cj, (rt, rs0, re0) in enumerate(repeat_spans):
                if cj != which[i0]:
                    extra_pos.append(rs0 + off)
        extra_pos = np.array(extra_pos, dtype=np.int64)
        clip_l[idx] = 0
        clip_r[idx] = 0

        def ext(a, v=None):
            return np.concatenate([a, a[extra_src] if v is None else v])
        tid = ext(tid); flag = ext(flag); rfile = ext(rfile); rg = ext(rg); L_arr = ext(L_arr)
        mapq = ext(mapq); x1 = ext(x1); clip_l = ext(clip_l); clip_r = ext(clip_r)
        pos = ext(pos, extra_pos)
        src_index = np.concatenate([src_index, extra_src])
        n = tid.shape[0]
    # junction breakpoints: a share of the unique reads crossing the junction is clipped there, the
    # clipped bases taken from the breakpoint's donor sequence (outward from the junction)
    donor = np.full(n, -1, dtype=np.int64)
    donors = []
    if cfg.breakpoints > 0:
        Lmax = int(L_arr.max())
        for b in range(cfg.breakpoints):
            t, p = _pick_site(margin=Lmax + 50)
            d = -1 if rng.random() < 0.5 else 1
            f = float(np.exp(rng.uniform(np.log(0.02), 0.0)))   # low-frequency ones stay in the null fit
            donors.append(rng.integers(0, 4, size=Lmax).astype(np.uint8))
            variants.append(dict(tid=t, pos=p, kind="breakpoint", direction=d, freq=f))
            cand = np.nonzero((tid == t) & (x1 == 1) & (pos < p) & (pos + L_arr > p) & (donor < 0))[0]
            a = np.where(d > 0, p - pos[cand], pos[cand] + L_arr[cand] - p)   # aligned bases kept
            cand = cand[(a >= 20) & (a <= L_arr[cand] - 1)]
            cand = cand[rng.random(cand.size) < f]
            donor[cand] = b
            if d > 0:
                clip_r[cand] = L_arr[cand] - (p - pos[cand])
                clip_l[cand] = 0
            else:
                clip_l[cand] = p - pos[cand]
                clip_r[cand] = 0
    if cfg.long_clip_fraction > 0:
        m = (rng.random(n) < cfg.long_clip_fraction) & (x1 == 1) & (donor < 0)
        k = np.minimum(rng.integers(12, 41, size=n), L_arr - 20)
        left = rng.random(n) < 0.5
        clip_l[m & left] = k[m & left]
        clip_r[m & left] = 0
        clip_r[m & ~left] = k[m & ~left]
        clip_l[m & ~left] = 0
    # soft clipped reads start later on the reference by the left clip
    pos = pos + clip_l
    order = np.lexsort((pos, tid))
    tid, pos, flag, rfile, rg, L_arr = tid[order], pos[order], flag[order], rfile[order], rg[order], L_arr[order]
    mapq, x1, clip_l, clip_r, src_index = mapq[order], x1[order], clip_l[order], clip_r[order], src_index[order]
    donor = donor[order]
    xl = np.zeros(n, dtype=np.int32)
    xr = np.zeros(n, dtype=np.int32)
    if cfg.trim_fraction > 0:
        m = rng.random(n) < cfg.trim_fraction
        xl[m] = rng.integers(0, 6, size=int(m.sum()))
        xr[m] = rng.integers(0, 6, size=int(m.sum()))
    xl = xl + clip_l.astype(np.int32)
    xr = xr + clip_r.astype(np.int32)

    # ---------------------------------------------------------------- read content
    Lp = L_arr + (L_arr & 1)
    seq_off = np.zeros(n, dtype=np.uint64)
    seq_off[1:] = np.cumsum(Lp[:-1]).astype(np.uint64)
    n_bases = int(Lp.sum())
    qual = np.zeros(n_bases, dtype=np.uint8)
    nib = np.zeros(n_bases, dtype=np.uint8)   # unpacked 4-bit codes
    gpos = toff[tid].astype(np.int64) + pos
    ref_code = np.searchsorted(BASES, ref).astype(np.uint8)          # A,C,G,T -> 0..3
    chunk_seeds = np.random.SeedSequence([cfg.seed, 7]).spawn((n + cfg.chunk_reads - 1) // cfg.chunk_reads + 1)
    qtabs = {}

    def fill(ci):
        c0 = ci * cfg.chunk_reads
        c1 = min(n, c0 + cfg.chunk_reads)
        crng = np.random.default_rng(chunk_seeds[ci])
        for L in np.unique(L_arr[c0:c1]):
            sel = np.nonzero(L_arr[c0:c1] == L)[0] + c0
            m = len(sel)
            L = int(L)
            aligned = L - clip_l[sel] - clip_r[sel]
            col = np.arange(L, dtype=np.int64)[None, :] - clip_l[sel][:, None]
            inref = (col >= 0) & (col < aligned[:, None])
            gidx = np.minimum(gpos[sel][:, None] + np.maximum(col, 0), total - 1)
            code = ref_code[gidx]
            rnd = crng.integers(0, 4, size=(m, L), dtype=np.uint8)
            code = np.where(inref, code, rnd)
            q = qtabs[L][np.arange(L)[None, :], crng.integers(0, 65536, size=(m, L), dtype=np.uint16)]
            rev = (flag[sel] & FLAG_REVERSE) != 0
            q[rev] = q[rev, ::-1]            # sequencing order runs right to left on the reverse strand
            err = crng.random((m, L), dtype=np.float32) < _ERR_LUT[q]
            shift = crng.integers(1, 4, size=(m, L), dtype=np.uint8)
            code = np.where(err, (code + shift) & 3, code)
            codes = _CODE2BAM[code]
            if cfg.n_base_rate > 0:
                nm = crng.random((m, L), dtype=np.float32) < cfg.n_base_rate
                codes[nm] = 15
                q[nm] = 2
            off = seq_off[sel].astype(np.int64)[:, None] + np.arange(L)[None, :]
            qual[off] = q
            nib[off] = codes

    for L in np.unique(L_arr):
        qtabs[int(L)] = _quality_table(int(L))
    n_chunks = (n + cfg.chunk_reads - 1) // cfg.chunk_reads
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(fill, range(n_chunks)))
    for r in np.nonzero(donor >= 0)[0]:
        D = donors[donor[r]]
        o = int(seq_off[r])
        k = int(clip_l[r] or clip_r[r])
        tail = D[:k].copy()
        e = rng.random(k) < 0.01     # sequencing errors in the donor part as well
        tail[e] = (tail[e] + rng.integers(1, 4, size=int(e.sum()))) & 3
        if clip_l[r]:
            nib[o: o + k] = _CODE2BAM[tail[::-1]]
        else:
            L = int(L_arr[r])
            nib[o + L - k: o + L] = _CODE2BAM[tail]
    # ---------------------------------------------------------------- variants in reads
    cigar_list = [None] * n
    starts_sorted = gpos
    reads_end = gpos + L_arr - clip_l - clip_r
    for v in variants:
        gp = int(toff[v["tid"]]) + v["pos"]
        lo = np.searchsorted(starts_sorted, gp - int(L_arr.max()) - 4, side="left")
        hi = np.searchsorted(starts_sorted, gp, side="right")
        cand = np.arange(lo, hi)
        cand = cand[(reads_end[cand] > gp) & (x1[cand] == 1)]
        if cand.size == 0:
            continue
        kind = v["kind"]
        if kind == "breakpoint":
            continue
        if kind in ("snp", "strand_bias", "low_quality"):
            carry = rng.random(cand.size) < v["freq"]
            if kind == "strand_bias":
                carry &= ((flag[cand] & FLAG_REVERSE) != 0) == bool(v["strand"])
            cand = cand[carry]
            qoff = gp - gpos[cand] + clip_l[cand]
            idx = seq_off[cand].astype(np.int64) + qoff
            nib[idx] = _ASCII2BAM[v["alt"]]
            if kind == "low_quality":
                qual[idx] = rng.integers(2, 16, size=cand.size).astype(np.uint8)
            continue
        # indels: rebuild each carrying read with its gapped alignment
        for r in cand:
            if clip_l[r] or clip_r[r] or rng.random() >= v["freq"]:
                continue
            L = int(L_arr[r])
            a = gp - int(gpos[r])
            o = int(seq_off[r])
            if kind == "del":
                k = v["length"]
                if a < 1 or a > L - 1:
                    continue
                tail = ref[gp + k: gp + k + (L - a)]
                nib[o + a: o + L] = _ASCII2BAM[tail]
                cigar_list[r] = [(a << 4) | BAM_M, (k << 4) | BAM_D, ((L - a) << 4) | BAM_M]
            else:
                k = len(v["seq"])
                if a < 1 or a > L - k - 1:
                    continue
                tail = np.concatenate([v["seq"], ref[gp: gp + (L - a - k)]])
                nib[o + a: o + L] = _ASCII2BAM[tail]
                cigar_list[r] = [(a << 4) | BAM_M, (k << 4) | BAM_I, ((L - a - k) << 4) | BAM_M]
    # identical content for every copy of a redundant read
    if repeat_spans:
        first = {}
        for r in np.nonzero(x1 > 1)[0]:
            s = int(src_index[r])
            if s in first:
                f = first[s]
                L = int(L_arr[r])
                nib[int(seq_off[r]): int(seq_off[r]) + L] = nib[int(seq_off[f]): int(seq_off[f]) + L]
                qual[int(seq_off[r]): int(seq_off[r]) + L] = qual[int(seq_off[f]): int(seq_off[f]) + L]
            else:
                first[s] = r
    # ---------------------------------------------------------------- CIGARs
    n_cigar = np.ones(n, dtype=np.uint16)
    n_cigar[(clip_l > 0) | (clip_r > 0)] = 2
    special = [r for r in range(n) if cigar_list[r] is not None]
    for r in special:
        n_cigar[r] = len(cigar_list[r])
    cigar_off = np.zeros(n, dtype=np.uint64)
    cigar_off[1:] = np.cumsum(n_cigar[:-1].astype(np.uint64))
    cigar = np.zeros(int(n_cigar.astype(np.int64).sum()), dtype=np.uint32)
    simple = n_cigar == 1
    cigar[cigar_off[simple].astype(np.int64)] = (L_arr[simple].astype(np.uint32) << 4) | BAM_M
    for side, arr in (("l", clip_l), ("r", clip_r)):
        m = (arr > 0) & (n_cigar == 2)
        o = cigar_off[m].astype(np.int64)
        aligned = (L_arr[m] - arr[m]).astype(np.uint32)
        if side == "l":
            cigar[o] = (arr[m].astype(np.uint32) << 4) | BAM_S
            cigar[o + 1] = (aligned << 4) | BAM_M
        else:
            cigar[o] = (aligned << 4) | BAM_M
            cigar[o + 1] = (arr[m].astype(np.uint32) << 4) | BAM_S
    for r in special:
        o = int(cigar_off[r])
        cigar[o:o + len(cigar_list[r])] = cigar_list[r]
    # ---------------------------------------------------------------- pack nibbles
    seq = ((nib[0::2] << 4) | nib[1::2]).astype(np.uint8)
    n_read_files = sum(2 if rs.paired else 1 for rs in cfg.read_sets)
    return Sample(
        ref_seq=ref, target_offset=toff, target_names=names,
        coverage_group=np.arange(T, dtype=np.uint32), n_coverage_groups=T,
        target_order=_lexicographic_order(names),
        tid=tid, pos=pos.astype(np.int32), flag=flag.astype(np.uint16), mapq=mapq, x1=x1,
        xl=xl, xr=xr, read_file=rfile.astype(np.uint8), read_group=rg.astype(np.uint16),
        l_qseq=L_arr.astype(np.uint32), seq_off=seq_off, cigar_off=cigar_off, n_cigar=n_cigar,
        cigar=cigar, seq=seq, qual=qual, n_read_files=n_read_files, n_quality=42, variants=variants,
        xj=(rng.random(n) < cfg.xj_fraction).astype(np.uint8) if cfg.xj_fraction > 0 else None)


# ------------------------------------------------------------------ benchmark workloads
def config_clonal_small(seed=11) -> SimConfig:
    """48,502-bp reference, 25 SNPs + 5 single-base indels, 60,000 single-end 101-bp reads (~125x)."""
    return SimConfig(seed=seed, target_lengths=(48502,), gc=0.5, n_snps=25, n_indels=5, max_indel=1,
                     read_sets=(ReadFileSet(coverage=60000 * 101 / 48502, read_length=101),))


def config_ecoli(seed=21, scale=1.0, coverage=100.0) -> SimConfig:
    """4.63 Mb chromosome + 100 kb + 60 kb plasmids, 50.8% GC, five 1.3-kb repeat copies, 300 SNPs and
    40 indels of length <= 3, paired-end 150-bp reads (two read files, `coverage` x each)."""
    lens = tuple(max(2000, int(x * scale)) for x in (4_630_000, 100_000, 60_000))
    return SimConfig(seed=seed, target_lengths=lens, target_names=("chromosome", "plasmid1", "plasmid2"),
                     gc=0.508, n_snps=max(3, int(300 * scale)), n_indels=max(2, int(40 * scale)), max_indel=3,
                     repeat_copies=5, repeat_length=1300,
                     read_sets=(ReadFileSet(coverage=coverage, read_length=150, paired=True),))


def config_population(seed=31, scale=1.0, coverage=500.0) -> SimConfig:
    """Same genome in polymorphism mode: 1000x paired-end 150 (500x per file), 400 variants at
    frequencies log-uniform in [0.01, 1], 50 strand-biased and 50 low-quality-skewed sites."""
    c = config_ecoli(seed=seed, scale=scale, coverage=coverage)
    return dataclasses.replace(c, n_snps=max(4, int(360 * scale)), n_indels=max(2, int(40 * scale)),
                               freq_min=0.01, strand_bias_sites=max(1, int(50 * scale)),
                               low_quality_sites=max(1, int(50 * scale)))


def config_batch(seed=41, n_samples=96, scale=1.0):
    """Many samples of uneven shape: genome length log-uniform in [40 kb, 6 Mb], total coverage
    uniform in [20, 500]x, read length from {36, 101, 150}, single- or paired-end, consensus or
    polymorphism mode; each sample uses the clonal (planted SNPs and short indels, repeats on
    genomes of 1 Mb and more) or population (variant frequencies log-uniform in [0.01, 1],
    strand-biased and low-quality sites) variant model.  `scale` multiplies every genome length
    (profiling and quick runs).  Returns [(SimConfig, polymorphism_mode)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_samples):
        g = max(5000, int(np.exp(rng.uniform(np.log(40e3), np.log(6e6))) * scale))
        cov = float(rng.uniform(20.0, 500.0))
        L = int(rng.choice([36, 101, 150]))
        paired = bool(rng.random() < 0.5)
        poly = bool(rng.random() < 0.5)
        mb = g / 1e6
        rs = ReadFileSet(coverage=cov / 2 if paired else cov, read_length=L, paired=paired)
        c = SimConfig(seed=seed * 1000 + i, target_lengths=(g,), target_names=(f"sample{i}_chr",), gc=0.5,
                      n_snps=max(5, int(65 * mb)), n_indels=max(2, int(9 * mb)), max_indel=3,
                      repeat_copies=5 if g >= 1_000_000 else 0, repeat_length=1300, read_sets=(rs,),
                      chunk_reads=16_000)
        if poly:
            c = dataclasses.replace(c, freq_min=0.01, strand_bias_sites=max(1, int(11 * mb)),
                                    low_quality_sites=max(1, int(11 * mb)))
        out.append((c, poly))
    return out


# ------------------------------------------------------------------ BAM bytes of a sample
BGZF_EOF = bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")


def _reg2bin(beg: int, end: int) -> int:
    """BAM bin of a 0-based half-open interval (SAM/BAM specification §5.3)."""
    end -= 1
    for shift, off in ((14, 4681), (17, 585), (20, 73), (23, 9), (26, 1)):
        if beg >> shift == end >> shift:
            return off + (beg >> shift)
    return 0


def _bgzf_block(payload: bytes, level: int) -> bytes:
    import struct
    import zlib
    co = zlib.compressobj(level, zlib.DEFLATED, -15)
    cdata = co.compress(payload) + co.flush()
    bsize = 12 + 6 + len(cdata) + 8 - 1
    head = struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, 66, 67, 2, bsize)
    return head + cdata + struct.pack("<II", zlib.crc32(payload) & 0xFFFFFFFF, len(payload))


def bam_groups(s: Sample):
    """The read groups the BAM of bam_bytes() declares: IDs, and each group's first read-file index
    and file count, from the sample's read files."""
    groups = sorted(set(int(g) for g in np.unique(s.read_group)))
    n = max(groups) + 1 if groups else 1
    ids = [f"rg{g}" for g in range(n)]
    base, count = [], []
    for g in range(n):
        f = s.read_file[s.read_group == g]
        lo = int(f.min()) if f.size else 0
        hi = int(f.max()) if f.size else 0
        base.append(lo)
        count.append(hi - lo + 1)
    return ids, base, count


def with_pairs(s: Sample, seed: int = 0, discordant_sites: int = 6, unmapped_sites: int = 6, site_span: int = 250,
               site_fraction: float = 0.6, background_discordant: float = 0.002, background_unmapped: float = 0.004,
               no_xp_fraction: float = 0.0, supplementary_fraction: float = 0.001, distance_sites: int = 0,
               distance_shift: int = 300) -> Sample:
    """Pair annotations for a sample, as breseq's alignment resolution leaves them
    (src/breseq/resolve_alignments.cpp:1255-1300): read names <read file + 1>:<fragment>, TLEN, and the
    XP orientation of every pair with both mates mapped.  Paired reads are proper pairs with XP FR,
    except near `discordant_sites` breakpoints (and a background rate), where pairs are discordant
    (not proper, XP FR / RF / FF, long TLEN), and near `unmapped_sites` insertions (and a background
    rate), where the mate is unmapped (0x8, no XP, TLEN 0).  no_xp_fraction of the discordant reads
    lose their XP tag.  Mate positions follow TLEN (a positive TLEN puts the mate's end there); near
    `distance_sites` points the pairs starting up to 450 bases before it are `distance_shift` longer.
    The scoring passes read none of these fields (the flag filter is 0x704), so their results do not
    change."""
    rng = np.random.default_rng(seed)
    n = s.n_reads
    flag = s.flag.astype(np.uint16).copy()
    paired = (flag & FLAG_PAIRED) != 0
    col = s.target_offset[s.tid].astype(np.int64) + s.pos.astype(np.int64)
    total = int(s.target_offset[-1])
    near = lambda sites: np.isin(col // site_span, (rng.integers(0, max(1, total), sites) // site_span)) \
        if sites else np.zeros(n, bool)
    disc = paired & ((near(discordant_sites) & (rng.random(n) < site_fraction)) | (rng.random(n) < background_discordant))
    unm = paired & ~disc & ((near(unmapped_sites) & (rng.random(n) < site_fraction)) | (rng.random(n) < background_unmapped))
    flag[disc | unm] &= np.uint16(~FLAG_PROPER & 0xFFFF)
    flag[unm] |= np.uint16(0x8)
    flag[unm] &= np.uint16(~FLAG_MREVERSE & 0xFFFF)
    flag[rng.random(n) < supplementary_fraction] |= np.uint16(0x800)
    xp = np.where(paired, 0, 3).astype(np.uint8)
    xp[disc] = rng.integers(0, 3, int(disc.sum())).astype(np.uint8)
    xp[unm] = 3
    xp[disc & (rng.random(n) < no_xp_fraction)] = 3
    isize = np.zeros(n, dtype=np.int32)
    mag = rng.integers(250, 450, n)
    isize[paired] = np.where(rng.random(int(paired.sum())) < 0.5, 1, -1) * mag[paired]
    isize[disc] = rng.integers(-60000, 60000, int(disc.sum()))
    isize[unm] = 0
    tlen_t = (s.target_offset[s.tid + 1] - s.target_offset[s.tid]).astype(np.int64)
    pos64 = s.pos.astype(np.int64)
    if distance_sites:
        sites = rng.integers(0, max(1, total), distance_sites)
        near_site = np.zeros(n, bool)
        for c in sites:
            near_site |= (col > c - 450) & (col <= c)
        shift = paired & ~disc & ~unm & (isize > 0) & near_site
        isize[shift] += distance_shift
    # mates: a positive TLEN ends the mate there, a negative one starts it |TLEN| before this read's end
    L = s.l_qseq.astype(np.int64)
    mpos = np.where(isize > 0, pos64 + isize - L, pos64 + L + isize)
    mpos = np.clip(mpos, 0, tlen_t - 1)
    mpos[unm] = pos64[unm]
    mpos[~paired] = -1
    mtid = np.where(paired, s.tid, -1).astype(np.int32)
    keep_in = (isize > 0) & (pos64 + isize > tlen_t)
    isize[keep_in] = (tlen_t - pos64)[keep_in].astype(np.int32)   # mates stay on the target
    # names "<read file + 1>:<fragment>", assembled digit by digit
    a = s.read_file.astype(np.int64) + 1
    b = np.arange(n, dtype=np.int64) // 2
    nd_a = np.maximum(1, np.floor(np.log10(np.maximum(a, 1))).astype(np.int64) + 1)
    nd_b = np.maximum(1, np.floor(np.log10(np.maximum(b, 1))).astype(np.int64) + 1)
    ln = nd_a + 1 + nd_b
    qname_off = np.zeros(n + 1, dtype=np.uint64)
    qname_off[1:] = np.cumsum(ln)
    qname = np.zeros(int(qname_off[-1]), dtype=np.uint8)
    o = qname_off[:-1].astype(np.int64)
    for d in range(int(nd_a.max()) if n else 0):
        k = d < nd_a
        qname[o[k] + nd_a[k] - 1 - d] = (a[k] // 10 ** d) % 10 + 48
    qname[o + nd_a] = ord(":")
    for d in range(int(nd_b.max()) if n else 0):
        k = d < nd_b
        qname[o[k] + nd_a[k] + nd_b[k] - d] = (b[k] // 10 ** d) % 10 + 48
    if n and no_xp_fraction > 0:   # a name without ':' takes the fallback key
        i = int(rng.integers(0, n))
        names = [qname[int(qname_off[j]):int(qname_off[j + 1])].tobytes() for j in range(n)]
        names[i] = b"plainname"
        qname_off[1:] = np.cumsum([len(x) for x in names])
        qname = np.frombuffer(b"".join(names), dtype=np.uint8).copy()
    return replace(s, flag=flag, isize=isize, xp=xp, qname_off=qname_off, qname=qname, mtid=mtid,
                   mpos=mpos.astype(np.int32))


def pd_null(s: Sample, max_distance: int = 2000) -> np.ndarray:
    """A pair-distance null for tests: the mid-CDF (G(d-1) + G(d)) / 2 of the positive TLENs of proper
    pairs in 2^20 fixed point, indexed by distance, as identify_mutations' pd_build_cdf scales it.  Each
    distance is weighted by the gap its pairs leave between two reads (d - 2 x read length), the number
    of positions a pair of that distance covers, so the null is that of the covering pairs."""
    d = s.isize[((s.flag & 0x3) == 0x3) & (s.isize > 0)].astype(np.int64)
    trunc = 2 * int(np.median(s.l_qseq)) if s.n_reads else 0
    w = np.bincount(np.clip(d, 0, max_distance), minlength=max_distance + 1).astype(np.float64)
    w *= np.maximum(np.arange(max_distance + 1) - trunc, 0)
    total = w.sum()
    below = np.concatenate([[0.0], np.cumsum(w)[:-1]])
    mid = (below + 0.5 * w) / total
    return np.clip((mid * 1048576 + 0.5).astype(np.int64), 0, 1048576)


def bam_bytes(s: Sample, level: int = 6, block_payload: int = 0xFF00, seed: int = 0, rg_tags: bool = True,
              split_records: bool = False) -> bytes:
    """The sample as a coordinate-sorted BAM (SAM/BAM specification §4.2), compressed in BGZF blocks
    the way htslib writes them: the header in its own blocks, a record never split across blocks
    (a block is closed before a record would overflow block_payload bytes), an EOF block at the end.
    split_records: the record stream cut every block_payload bytes instead, records spanning blocks,
    as other writers (htsjdk's) do.
    Tags: X1 when the redundancy is not 1, XL / XR when present, XJ when set, RG when the sample has
    several read groups (or always, with rg_tags); integer tags in varying BAM integer types."""
    import struct
    rng = np.random.default_rng(seed)
    ids, _, _ = bam_groups(s)
    T = len(s.target_names)
    text = "@HD\tVN:1.6\tSO:coordinate\n"
    for t in range(T):
        text += f"@SQ\tSN:{s.target_names[t]}\tLN:{int(s.target_offset[t + 1] - s.target_offset[t])}\n"
    for g in ids:
        text += f"@RG\tID:{g}\tLB:{g}\tSM:sample\n"
    head = b"BAM\1" + struct.pack("<i", len(text)) + text.encode() + struct.pack("<i", T)
    for t in range(T):
        name = s.target_names[t].encode() + b"\0"
        head += struct.pack("<i", len(name)) + name + struct.pack("<i", int(s.target_offset[t + 1] - s.target_offset[t]))
    out = [_bgzf_block(head[i:i + block_payload], level) for i in range(0, len(head), block_payload)]
    int_types = [("C", "<B", 0, 255), ("S", "<H", 0, 65535), ("i", "<i", -2**31, 2**31 - 1), ("I", "<I", 0, 2**32 - 1),
                 ("c", "<b", -128, 127), ("s", "<h", -32768, 32767)]

    def int_tag(tag, v):
        ok = [t for t in int_types if t[2] <= v <= t[3]]
        code, fmt, _, _ = ok[int(rng.integers(0, len(ok)))]
        return tag.encode() + code.encode() + struct.pack(fmt, v)

    buf = bytearray()
    for i in range(s.n_reads):
        L = int(s.l_qseq[i])
        nc = int(s.n_cigar[i])
        co = int(s.cigar_off[i])
        cig = s.cigar[co:co + nc]
        ops, lens = cig & 0xF, cig >> 4
        rlen = int(lens[(ops == 0) | (ops == 2) | (ops == 3) | (ops == 7) | (ops == 8)].sum())
        pos = int(s.pos[i])
        if s.qname is not None:
            name = s.qname[int(s.qname_off[i]): int(s.qname_off[i + 1])].tobytes() + b"\0"
        else:
            name = f"r{i}".encode() + b"\0"
        so = int(s.seq_off[i])
        seq = s.seq[so // 2: so // 2 + (L + 1) // 2].tobytes()
        if L & 1 and seq:   # the spare low nibble of an odd-length read is zero in BAM
            seq = seq[:-1] + bytes([seq[-1] & 0xF0])
        qual = s.qual[so: so + L].tobytes()
        aux = b""
        if int(s.x1[i]) != 1:
            aux += int_tag("X1", int(s.x1[i]))
        if int(s.xl[i]) >= 0:
            aux += int_tag("XL", int(s.xl[i]))
        if int(s.xr[i]) >= 0:
            aux += int_tag("XR", int(s.xr[i]))
        if rng.random() < 0.3:
            aux += b"NMi" + struct.pack("<i", int(rng.integers(0, 5)))
        if s.xj is not None and s.xj[i]:
            aux += int_tag("XJ", 1)
        if rg_tags or len(ids) > 1:
            aux += b"RGZ" + ids[int(s.read_group[i])].encode() + b"\0"
        if rng.random() < 0.1:
            aux += b"ZBBs" + struct.pack("<I", 3) + struct.pack("<3h", 1, -2, 3)
        if s.xp is not None:
            if s.xp[i] <= 2:
                aux += b"XPZ" + (b"FR", b"RF", b"FF")[int(s.xp[i])] + b"\0"
            elif rng.random() < 0.2:
                aux += b"XPZRR\0"    # an XP value other than FR / RF / FF: no orientation
        tlen = int(s.isize[i]) if s.isize is not None else 0
        mt = int(s.mtid[i]) if s.mtid is not None else -1
        mp = int(s.mpos[i]) if s.mpos is not None else -1
        body = struct.pack("<iiBBHHHiiii", int(s.tid[i]), pos, len(name), int(s.mapq[i]), _reg2bin(pos, pos + max(rlen, 1)),
                           nc, int(s.flag[i]), L, mt, mp, tlen)
        rec = body + name + cig.astype("<u4").tobytes() + seq + qual + aux
        rec = struct.pack("<i", len(rec)) + rec
        if split_records:
            buf += rec
            while len(buf) >= block_payload:
                out.append(_bgzf_block(bytes(buf[:block_payload]), level))
                del buf[:block_payload]
            continue
        if len(buf) + len(rec) > block_payload and buf:
            out.append(_bgzf_block(bytes(buf), level))
            buf = bytearray()
        buf += rec
    if buf:
        out.append(_bgzf_block(bytes(buf), level))
    out.append(BGZF_EOF)
    return b"".join(out)


def bam_bytes_fast(s: Sample, level: int = 6, block_payload: int = 0xFF00, threads: int = 16,
                   chunk: int = 65536) -> bytes:
    """bam_bytes() for large samples: records assembled with numpy gathers, chunk by chunk, and the
    BGZF blocks compressed on host threads.  Read names r0000000000.., tags X1:I when the redundancy
    is not 1, XL:i / XR:i when present, XJ:C when set, RG:Z always."""
    import struct
    n = s.n_reads
    ids, _, _ = bam_groups(s)
    T = len(s.target_names)
    text = "@HD\tVN:1.6\tSO:coordinate\n"
    for t in range(T):
        text += f"@SQ\tSN:{s.target_names[t]}\tLN:{int(s.target_offset[t + 1] - s.target_offset[t])}\n"
    for g in ids:
        text += f"@RG\tID:{g}\tLB:{g}\tSM:sample\n"
    head = b"BAM\1" + struct.pack("<i", len(text)) + text.encode() + struct.pack("<i", T)
    for t in range(T):
        name = s.target_names[t].encode() + b"\0"
        head += struct.pack("<i", len(name)) + name + struct.pack("<i", int(s.target_offset[t + 1] - s.target_offset[t]))
    rg_str = [g.encode() + b"\0" for g in ids]
    rg_bytes = np.frombuffer(b"".join(rg_str), dtype=np.uint8)
    rg_off_tab = np.concatenate([[0], np.cumsum([len(x) for x in rg_str])]).astype(np.int64)
    rg_len_tab = np.array([len(x) for x in rg_str], dtype=np.int64)
    LNAME = 12   # "r" + 10 digits + NUL

    def build(a, b):
        """The records a..b-1 as bytes."""
        m = b - a
        L = s.l_qseq[a:b].astype(np.int64)
        nc = s.n_cigar[a:b].astype(np.int64)
        co = s.cigar_off[a:b].astype(np.int64)
        so = s.seq_off[a:b].astype(np.int64)
        nb = (L + 1) // 2
        has_x1 = s.x1[a:b] != 1
        has_xl = s.xl[a:b] >= 0
        has_xr = s.xr[a:b] >= 0
        has_xj = (s.xj[a:b] != 0) if s.xj is not None else np.zeros(m, bool)
        rg = s.read_group[a:b].astype(np.int64)
        rg_len = rg_len_tab[rg]
        rec_len = 36 + LNAME + 4 * nc + nb + L + has_x1 * 7 + has_xl * 7 + has_xr * 7 + has_xj * 4 + 3 + rg_len
        off = np.zeros(m + 1, dtype=np.int64)
        off[1:] = np.cumsum(rec_len)
        buf = np.zeros(int(off[-1]), dtype=np.uint8)

        def put(dst, src, src_start, length):
            tot = int(length.sum())
            if tot == 0:
                return
            rep = np.repeat(np.arange(m), length)
            k = np.arange(tot) - np.repeat(np.cumsum(length) - length, length)
            buf[dst[rep] + k] = src[src_start[rep] + k]

        def put_rows(dst, rows):
            w = rows.shape[1]
            buf[(dst[:, None] + np.arange(w)[None, :]).ravel()] = rows.ravel()

        # bin (SAM/BAM specification §5.3) from the reference span
        cig = s.cigar[co[0]: co[-1] + nc[-1]] if m else s.cigar[:0]
        ops, lens = cig & 0xF, (cig >> 4).astype(np.int64)
        refc = ((ops == 0) | (ops == 2) | (ops == 3) | (ops == 7) | (ops == 8)) * lens
        starts = co - co[0]
        rlen = np.add.reduceat(refc, starts) if len(refc) else np.zeros(m, np.int64)
        rlen = np.where(nc > 0, rlen, 0)
        pos = s.pos[a:b].astype(np.int64)
        last = pos + np.maximum(rlen, 1) - 1
        binv = np.zeros(m, dtype=np.int64)
        done = np.zeros(m, bool)
        for shift, o in ((14, 4681), (17, 585), (20, 73), (23, 9), (26, 1)):
            hit = ~done & ((pos >> shift) == (last >> shift))
            binv[hit] = o + (pos[hit] >> shift)
            done |= hit
        fixed = np.zeros(m, dtype=[("bs", "<i4"), ("ref", "<i4"), ("pos", "<i4"), ("ln", "u1"), ("mq", "u1"),
                                   ("bin", "<u2"), ("nc", "<u2"), ("flag", "<u2"), ("ls", "<i4"), ("nref", "<i4"),
                                   ("npos", "<i4"), ("tlen", "<i4")])
        fixed["bs"] = rec_len - 4
        fixed["ref"] = s.tid[a:b]
        fixed["pos"] = s.pos[a:b]
        fixed["ln"] = LNAME
        fixed["mq"] = s.mapq[a:b]
        fixed["bin"] = binv
        fixed["nc"] = nc
        fixed["flag"] = s.flag[a:b]
        fixed["ls"] = L
        fixed["nref"] = -1
        fixed["npos"] = -1
        cur = off[:-1].copy()
        put_rows(cur, fixed.view(np.uint8).reshape(m, 36))
        cur += 36
        idx = np.arange(a, b, dtype=np.int64)
        digits = np.zeros((m, LNAME), dtype=np.uint8)
        digits[:, 0] = ord("r")
        for d in range(10):
            digits[:, 10 - d] = (idx // 10 ** d) % 10 + 48
        put_rows(cur, digits)
        cur += LNAME
        put(cur, s.cigar.astype("<u4").view(np.uint8), co * 4, nc * 4)
        cur += 4 * nc
        seq = s.seq[so[0] // 2: (so[-1] + L[-1] + 1) // 2 + 1].copy() if m else s.seq[:0]
        base = so[0] // 2 if m else 0
        odd = np.nonzero((L & 1) == 1)[0]
        seq[so[odd] // 2 + nb[odd] - 1 - base] &= 0xF0
        put(cur, seq, so // 2 - base, nb)
        cur += nb
        put(cur, s.qual, so, L)
        cur += L
        for tag, has, fmt, vals in ((b"X1I", has_x1, "<u4", s.x1[a:b]), (b"XLi", has_xl, "<i4", s.xl[a:b]),
                                    (b"XRi", has_xr, "<i4", s.xr[a:b])):
            w = np.nonzero(has)[0]
            if len(w):
                v = np.zeros(len(w), dtype=[("t", "S3"), ("v", fmt)])
                v["t"] = tag
                v["v"] = vals[w]
                put_rows(cur[w], v.view(np.uint8).reshape(len(w), 7))
            cur += has * 7
        w = np.nonzero(has_xj)[0]
        if len(w):
            put_rows(cur[w], np.tile(np.frombuffer(b"XJC\1", np.uint8), (len(w), 1)))
        cur += has_xj * 4
        put_rows(cur, np.tile(np.frombuffer(b"RGZ", np.uint8), (m, 1)))
        cur += 3
        put(cur, rg_bytes, rg_off_tab[rg], rg_len)
        # record-aligned blocks of at most block_payload bytes
        pieces, first = [], 0
        while first < m:
            j = int(np.searchsorted(off, off[first] + block_payload, side="right")) - 1
            j = max(j, first + 1)
            pieces.append(_bgzf_block(bytes(buf[off[first]:off[j]]), level))
            first = j
        return pieces

    bounds = [(a, min(n, a + chunk)) for a in range(0, n, chunk)]
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        parts = list(ex.map(lambda ab: build(*ab), bounds))
    out = [_bgzf_block(head[i:i + block_payload], level) for i in range(0, len(head), block_payload)]
    for p in parts:
        out += p
    return b"".join(out + [BGZF_EOF])
