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


ALL = {"clonal_small": clonal_small, "ecoli_small": ecoli_small, "population_small": population_small}


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
