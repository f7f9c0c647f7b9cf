"""Writes tests/golden/ref/<case>.json: the output files of breseq's own error_count() and
identify_mutations() (compiled by oracle/ref_build.py from the reference sources) on the seeded samples of
tests/samples.py.  Run in a checkout that has the reference tree:

    python tests/golden/make_ref_golden.py [case ...]

Each fixture holds the sample's digest, the settings of the run, and per file either its text or, for
files over 16 KB, its SHA-256 and size.  Besides the two passes' files, every case holds the coverage
distribution fit of each coverage group (coverage_fit.<g>.txt, the harness's %.17g dump of
fit_coverage_distribution's result).  The classified GenomeDiff is the harness's
test_RA_evidence + cGenomeDiff::write output without the `#=TITLE` line that write adds."""
import hashlib
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_run  # noqa: E402
from tests import samples  # noqa: E402

CASES = {
    "clonal_small": dict(sample="clonal_small"),
    "ecoli_small": dict(sample="ecoli_small"),
    "ecoli_small_failed_fit": dict(sample="ecoli_small", prop_cutoff=[5.0, -1.0, 5.0]),
    "population_small": dict(sample="population_small", polymorphism=True),
    "dp_groups": dict(sample="dp_skip_sample", pmdd=[[0, 300.0, 20.0]]),
    # two paired read groups, a discordant-pair group on the first only: per-read-group coverage columns
    "dp_two_groups": dict(sample="dp_two_groups", pmdd=[[0, 300.0, 20.0]]),
    "ecoli_quarter": dict(sample="ecoli_quarter"),
    "population_deep": dict(sample="population_deep", polymorphism=True),
    # tabulate_soft_clipping_counts and BAM2COV tables (coverage_output::table) on the clipped sample
    "softclip_bam2cov": dict(sample="softclip_sample", softclip=True, bam2cov=[
        ["full.tsv", "zeta_chromosome:1-138900", 0, "tsv", 0, 0],
        ["mid7.csv", "Alpha_plasmid:101-3000", 7, "csv", 0, 0],
        ["tot.tsv", "zeta_chromosome:500-90000", 600, "tsv", 1, 0],
        ["rg.tsv", "beta_plasmid:1-2000", 0, "tsv", 0, 1]]),
}
TEXT_LIMIT = 16 * 1024


def make(case):
    c = CASES[case]
    s = getattr(samples, c["sample"])()
    t0 = time.time()
    out = ref_run.run(s, polymorphism=c.get("polymorphism", False), prop_cutoff=c.get("prop_cutoff"),
                      copy_number=True, classify=True, pmdd=[tuple(x) for x in c.get("pmdd", [])],
                      softclip=c.get("softclip", False), bam2cov=[tuple(x) for x in c.get("bam2cov", [])], covfit=True)
    files = {}
    for name, text in sorted(out.items()):
        if name == "ra_mc_evidence.classified.gd":
            text = "".join(l for l in text.splitlines(True) if not l.startswith("#=TITLE"))
        if len(text) <= TEXT_LIMIT:
            files[name] = {"text": text}
        else:
            files[name] = {"sha256": hashlib.sha256(text.encode()).hexdigest(), "bytes": len(text.encode())}
    fx = dict(case=case, settings=c, sample_digest=samples.sample_digest(s), reference_seconds=round(time.time() - t0, 1),
              files=files)
    with open(os.path.join(ROOT, "tests", "golden", "ref", f"{case}.json"), "w") as f:
        json.dump(fx, f, indent=1, sort_keys=True)
    print(case, fx["reference_seconds"], "s", len(files), "files", flush=True)


if __name__ == "__main__":
    for case in (sys.argv[1:] or list(CASES)):
        make(case)
