"""Runs the reference oracle (breseq's own error_count + identify_mutations, built by ref_build.py) on
a synthetic sample: the sample is written as BAM and FASTA with a config file, the harness reads them,
and the files it writes come back as text.  write_inputs() also serves the drop-in test driver
(tests/native/dropin_main.cpp), which reads the same config.  Test infrastructure."""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from . import ref_build


def write_fasta(s, path):
    """The targets as FASTA (80 bases per line) and its samtools-style .fai index."""
    off, fai = 0, []
    with open(path, "w") as f:
        for t, name in enumerate(s.target_names):
            seq = bytes(s.ref_seq[int(s.target_offset[t]):int(s.target_offset[t + 1])]).decode()
            head = f">{name}\n"
            f.write(head)
            off += len(head)
            fai.append(f"{name}\t{len(seq)}\t{off}\t80\t81\n")
            for i in range(0, len(seq), 80):
                f.write(seq[i:i + 80] + "\n")
                off += len(seq[i:i + 80]) + 1
    with open(path + ".fai", "w") as f:
        f.write("".join(fai))


def write_inputs(s, d, polymorphism=False, prop_cutoff=None, seed_cutoff=None, copy_number=False, classify=False,
                 pmdd=(), fast_bam=False, softclip=False, bam2cov=(), covfit=False) -> tuple:
    """reference.bam, reference.fasta, an empty out/ folder and config.txt in folder d; returns the
    config path and the output folder.  pmdd: (read group, median, mad) of the paired-mapping-distance
    fits that make discordant-pair groups.  fast_bam: the vectorised BAM writer (same records; its read
    names are placeholders, so only for samples without pair annotations)."""
    from breseq_gb300 import synth
    T = len(s.target_names)
    prop = np.broadcast_to(np.asarray(5.0 if prop_cutoff is None else prop_cutoff, dtype=np.float64), (T,))
    seed = np.broadcast_to(np.asarray(0.0 if seed_cutoff is None else seed_cutoff, dtype=np.float64), (T,))
    called = set(int(t) for t in s.target_order)
    _, _, counts = synth.bam_groups(s)
    bam = os.path.join(d, "reference.bam")
    with open(bam, "wb") as f:
        f.write(synth.bam_bytes_fast(s) if fast_bam and s.xp is None else synth.bam_bytes(s, rg_tags=True))
    fasta = os.path.join(d, "reference.fasta")
    write_fasta(s, fasta)
    out = os.path.join(d, "out")
    os.makedirs(out)
    cfg = os.path.join(d, "config.txt")
    with open(cfg, "w") as f:
        f.write(f"bam {bam}\nfasta {fasta}\noutdir {out}\n")
        f.write("groups " + " ".join(str(c) for c in counts) + "\n")
        f.write(f"quality {s.n_quality}\npolymorphism {int(polymorphism)}\n")
        f.write(f"copy_number {int(copy_number)}\nclassify {int(classify)}\n")
        for g, med, mad in pmdd:
            f.write(f"pmdd {int(g)} {float(med)!r} {float(mad)!r}\n")
        f.write(f"softclip {int(softclip)}\ncovfit {int(covfit)}\n")
        for name, region, res, fmt, tot, prg in bam2cov:
            f.write(f"bam2cov {name} {region} {int(res)} {fmt} {int(tot)} {int(prg)}\n")
        for t, name in enumerate(s.target_names):
            f.write(f"target {name} {int(s.coverage_group[t])} {int(t in called)} {float(prop[t])!r} {float(seed[t])!r}\n")
    return cfg, out


def read_outputs(out) -> dict:
    files = {}
    for root, _, names in os.walk(out):
        for n in names:
            p = os.path.join(root, n)
            files[os.path.relpath(p, out)] = open(p, errors="replace").read()
    return files


def run(s, polymorphism=False, prop_cutoff=None, seed_cutoff=None, copy_number=False, classify=False,
        pmdd=(), workdir=None, softclip=False, bam2cov=(), covfit=False) -> dict:
    """Outputs of the reference on sample `s`: {file name: text}.  Raises when the binary is absent."""
    exe = ref_build.build()
    if exe is None:
        raise FileNotFoundError("the reference sources are not available")
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        cfg, out = write_inputs(s, d, polymorphism, prop_cutoff, seed_cutoff, copy_number, classify, pmdd,
                                softclip=softclip, bam2cov=bam2cov, covfit=covfit)
        env = dict(os.environ, BRESEQ_DATA_PATH=ref_build.data_path())
        r = subprocess.run([exe, cfg], capture_output=True, text=True, cwd=d, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness failed ({r.returncode}):\n{r.stderr[-3000:]}\n{r.stdout[-2000:]}")
        return read_outputs(out)
