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
