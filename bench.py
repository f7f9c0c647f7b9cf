#!/usr/bin/env python
"""Benchmark of the read-evidence scoring path: aligned read-bases scored per second.

One step = the full path on one sample: error_count (pass 1), the error-table round trip, and
identify_mutations (pass 2), on the E. coli-scale clonal workload (4.63 Mb chromosome + 100 kb + 60 kb
plasmids, five 1.3-kb repeats, 300 SNPs + 40 indels, 2 x 100x paired-end 150-bp reads; seeded
synthetic data of that shape).  `value` is input aligned read-bases / device time of a step with the
sample resident in HBM; `e2e` runs the same step through the C ABI from pinned host buffers
(upload + both passes + result download + free inside the timed region).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Two more legs on rank 0 report the batched and served forms on a mix of samples of uneven shape
(genome length log-uniform in [40 kb, 6 Mb], 20-500x, reads of 36/101/150 bp, SE/PE, consensus and
polymorphism modes), drawn from a pool of distinct seeded samples:
  "batched": all jobs resident, both passes as one batch call per pass (one launch per kernel per
             64 jobs), against the plain FP64 form run one sample per call;
  "served":  open-loop Poisson arrivals at 0.5/1/2x the batched capacity into the scoring server
             (HBM-footprint admission, continuous batching), with p50/p99 job latency.

A "bam_input" leg runs the same step from the workload's BAM bytes (written by the vectorised
synthetic writer, zlib level 6, htslib's record-aligned blocks): upload of the compressed file, BGZF
inflate and record decode on the device, sample load, both passes; against zlib inflating the same
blocks on all host cores.

A "coverage_table" leg times the BAM2COV coverage columns of the workload's chromosome (every position)
and the table at BAM2COV's default resolution, against the oracle on a 200 kb region.

A "soft_clipping" leg times the soft-clipping tabulation (tabulate_soft_clipping_counts) on a sample
of the same shape with 50 junction breakpoints and 1% of reads clipped by 12-40 random bases, against
the oracle's CPU tabulation of the same sample.

A "coverage_fit" leg times the coverage-distribution fit (host threads) of each coverage group's
histogram from pass 1, against the oracle's sequential restatement.

A "pair_scans" leg times the discordant-pair and missing-pair candidate scans on the workload with
pair annotations (discordant and mate-unmapped pairs planted at 40 sites each and at background
rates), against the oracle's position-by-position walk.

Under torchrun each rank scores its own sample (weak scaling, no collective in the data path); the
timed region is bracketed by barriers and the slowest rank's time is used.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "read-bases/s scored, served vs plain on same GPU (identical calls); p50/p99 ms"
UNIT = "read-bases/s"
WORKLOAD = "ecoli_clonal_4.79Mb_pe150_2x100x"
# DRAM bytes (read + write) per aligned read-base of one launch: ncu's dram__bytes_read.sum +
# dram__bytes_write.sum for one launch of each kernel on the same workload at 0.25x genome length
# (0.2441 G read-bases), scaled linearly with read-bases (both kernels read every base once, and the
# per-read and per-column bytes grow with them at a fixed coverage).  The column kernel reads one
# class byte per base (quality * 5 + base, built when the sample is loaded) where the formula's
# algorithmic bytes count the 1.5 bytes of packed base and quality, so its traffic sits below them.
IM_COLUMN_DRAM_PER_BASE = (323.486464e6 + 51.284736e6) / 0.2441e9
EC_READ_DRAM_PER_BASE = (416.378368e6 + 8.300544e6) / 0.2441e9
# the plain FP64 form: same kernels, FP64 everywhere, one sample per call, launched without graphs
PLAIN_TUNING = dict(ec_read_chunk=1024, ec_blocks_per_sm=8, col_blocks_per_sm=8, cand_warps_per_sm=16,
                    bound_warps_per_sm=4, use_graphs=0)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1])); mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def _barrier(pg):
    if pg is not None:
        pg.barrier()


def _max_over_ranks(pg, v: float) -> float:
    from breseq_gb300 import shard
    return shard.slowest(v) if pg is not None else v


def _workload(seed: int, scale: float = 1.0):
    from breseq_gb300 import synth
    return synth.simulate(synth.config_ecoli(seed=seed, scale=scale))


SC_WORKLOAD = "ecoli_4.79Mb_pe150_2x100x_50breakpoints_1pct_long_clips"
# DRAM bytes (read + write) of one launch of the tabulation's count pass per record, from an ncu
# capture of one launch on the same workload
SC_READS_DRAM_PER_READ = (230.080768e6 + 14.4256e6) / 6416810
# DRAM bytes of the four main coverage-table kernels over their algorithmic bytes, from an ncu capture
# of one call on the same chromosome
COV_TABLE_DRAM_OVER_ALGORITHMIC = 580.482284e6 / (32 * 6206454 + 80 * 4630000)
# DRAM bytes of one pair-classification launch per record, from an ncu capture of the same workload at
# half the genome length
PAIR_CLASSIFY_DRAM_PER_READ = (116.804608e6 + 10.306816e6) / 3223958


COV_COLUMNS = ("unique_top", "unique_bot", "redundant_top", "redundant_bot", "raw_redundant_top",
               "raw_redundant_bot", "unique_top_begin", "unique_bot_begin")


def _cpu_inflate(data: bytes, threads: int):
    """zlib inflating every BGZF block of data on `threads` host threads: seconds, output bytes."""
    import concurrent.futures as cf
    import struct
    import zlib
    blocks, pos = [], 0
    while pos < len(data):
        xlen = struct.unpack_from("<H", data, pos + 10)[0]
        bsize = struct.unpack_from("<H", data, pos + 16)[0]
        blocks.append(data[pos + 12 + xlen: pos + bsize + 1 - 8])
        pos += bsize + 1
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        out = sum(len(x) for x in ex.map(lambda c: zlib.decompress(c, -15), blocks, chunksize=64))
    return time.perf_counter() - t0, out


def run_bam(args, device, s):
    """The step from BAM bytes: open (upload + inflate), decode, load, pass 1, table, pass 2, free."""
    from breseq_gb300 import synth
    from breseq_gb300.api import ImSettings, Scorer
    t0 = time.perf_counter()
    data = synth.bam_bytes_fast(s)
    gen_s = time.perf_counter() - t0
    groups = synth.bam_groups(s)
    arr = np.frombuffer(bytearray(data), dtype=np.uint8)
    bases = s.aligned_bases()
    prec = 1 if args.precision == "fp32c" else 0
    st = ImSettings()
    with Scorer(device) as sc:
        pinned = sc.L.bsq_host_register(arr.ctypes.data, arr.nbytes) == 0
        steps, phases = [], {"open": [], "decode": [], "load": [], "passes": []}
        kern = {"inflate": [], "decode": []}
        for i in range(args.warmup + args.steps):
            sc.timer_start()
            t0 = time.perf_counter()
            bam = sc.open_bam(arr)
            k_inf = sc.last_pass_stats()["main_kernel_ms"]
            t1 = time.perf_counter()
            bam.decode(groups)
            k_dec = sc.last_pass_stats()["device_ms"]
            t2 = time.perf_counter()
            sid = bam.load(s)
            bam.close()
            t3 = time.perf_counter()
            ec = sc.error_count(sid)
            tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
            sc.identify_mutations(sid, tab, st, precision=prec, as_dicts=False)
            sc.free_sample(sid)
            t = sc.timer_stop()
            t4 = time.perf_counter()
            if i >= args.warmup:
                steps.append(t)
                for k, a, b in (("open", t0, t1), ("decode", t1, t2), ("load", t2, t3), ("passes", t3, t4)):
                    phases[k].append(1e3 * (b - a))
                kern["inflate"].append(k_inf)
                kern["decode"].append(k_dec)
        if pinned:
            sc.L.bsq_host_unregister(arr.ctypes.data)
    cpu_s, out_bytes = _cpu_inflate(data, os.cpu_count() or 1)
    ms = statistics.mean(steps)
    inf_ms = statistics.mean(kern["inflate"])
    hbm, peak_kind = _peaks()
    return {"workload": f"{WORKLOAD} as BAM (zlib level 6, {len(data) / 1e6:.0f} MB compressed)",
            "compressed_bytes": len(data), "inflated_bytes": out_bytes, "records": s.n_reads,
            "value": bases / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "e2e": {"value": bases / (ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": len(data),
                    "mode": "sequential: open, decode, load, both passes, free per step"},
            "host_ms_by_phase": {k: statistics.mean(v) for k, v in phases.items()},
            "inflate_kernel_ms": inf_ms, "decode_device_ms": statistics.mean(kern["decode"]),
            # the three inflate kernels together: Huffman symbols to tokens (one thread per block, 32
            # blocks per warp in lockstep), tokens to bytes (one warp per block), CRC-32s
            "roofline": {"bound": "latency and divergence (each thread decodes its block's Huffman stream serially)",
                         "kernel": "bgzf_tok_kernel + bgzf_resolve_kernel + bgzf_crc_kernel",
                         "achieved": (len(data) + out_bytes) / (inf_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": (len(data) + out_bytes) / (inf_ms / 1e3) / 1e9 / hbm, "peak_kind": peak_kind,
                         "algorithmic_bytes": len(data) + out_bytes, "traffic": None},
            "writer_seconds": gen_s,
            "cpu_baseline": {"value": out_bytes / cpu_s, "unit": "inflated bytes/s", "cores": os.cpu_count() or 1,
                             "kind": "port", "sample": f"zlib inflating all {len(data) / 1e6:.0f} MB of blocks ({cpu_s:.2f} s)"}}


def run_coverage(args, sc, sid, s):
    """BAM2COV coverage columns of target 0 (all positions) on the resident sample: device time of
    the kernels, the call, the written table at resolution 600, and the oracle on a bounded region."""
    from oracle import pyoracle as po
    L = int(s.target_offset[1] - s.target_offset[0])
    reads = int(np.count_nonzero(s.tid == 0))
    for _ in range(args.warmup):
        sc.coverage_columns(sid, 0, 1, L)
    dev, main, wall = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        c = sc.coverage_columns(sid, 0, 1, L)
        wall.append(1e3 * (time.perf_counter() - t0))
        st = sc.last_pass_stats()
        dev.append(st["device_ms"]); main.append(st["main_kernel_ms"])
    with tempfile.TemporaryDirectory() as d:
        table = []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            sc.write_coverage_region(sid, os.path.join(d, "c.tsv"), 0, 1, L, resolution=600)
            if i >= args.warmup:
                table.append(1e3 * (time.perf_counter() - t0))
        table_ms = statistics.mean(table)
    n_cpu = min(L, 200_000)
    t0 = time.perf_counter()
    o = po.coverage_columns(s, 0, 1, n_cpu)
    cpu_s = time.perf_counter() - t0
    same = all(np.array_equal(c[k][:n_cpu], o[k]) for k in COV_COLUMNS)
    ms, kms = statistics.mean(dev), statistics.mean(main)
    hbm, peak_kind = _peaks()
    # 32 B per record; per position the difference arrays read twice (32 B), the counts written and
    # re-read (32 B) and the two weights written (16 B)
    kbytes = 32 * reads + 80 * L
    return {"workload": f"{WORKLOAD}: chromosome, {L} positions", "positions": L, "records": reads,
            "device_ms": ms, "kernels_ms": kms, "wall_ms": statistics.mean(wall), "kernel_launches": st["kernel_launches"],
            "value": L / (ms / 1e3), "unit": "positions/s",
            "table_ms_resolution_600": table_ms,
            "roofline": {"bound": "hbm", "kernel": "coverage-table kernels (all six)", "achieved": kbytes / (kms / 1e3) / 1e9,
                         "peak": hbm, "unit": "GB/s", "frac": kbytes / (kms / 1e3) / 1e9 / hbm,
                         "algorithmic_bytes": kbytes, "peak_kind": peak_kind,
                         "traffic": COV_TABLE_DRAM_OVER_ALGORITHMIC * kbytes, "traffic_unit": "bytes per call"},
            "identical_to_oracle": bool(same),
            "cpu_baseline": {"value": n_cpu / cpu_s, "unit": "positions/s", "cores": 1, "kind": "port",
                             "sample": f"positions 1-{n_cpu} of the same chromosome ({cpu_s:.2f} s)"}}


def run_covfit(args, ec, s):
    """The coverage-distribution fit (host threads) of every coverage group's unique-only histogram
    from pass 1, against the oracle's sequential restatement."""
    from breseq_gb300.api import fit_coverage_distribution
    from oracle import pyoracle as po
    groups = []
    for g in range(s.n_coverage_groups):
        h = np.ascontiguousarray(ec["hist"][g, : int(ec["hist_size"][g])])
        length = int(sum(s.target_offset[t + 1] - s.target_offset[t] for t in range(len(s.target_offset) - 1)
                         if s.coverage_group[t] == g))
        groups.append((h, 0.05 / np.sqrt(float(length))))
    for _ in range(args.warmup):
        fits = [fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr) for h, pr in groups]
    wall = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fits = [fit_coverage_distribution(h, deletion_propagation_pr_cutoff=pr) for h, pr in groups]
        wall.append(1e3 * (time.perf_counter() - t0))
    t0 = time.perf_counter()
    ofits = [po.fit_coverage_distribution(h, pr) for h, pr in groups]
    cpu_s = time.perf_counter() - t0
    same = all(a == b for a, b in zip(fits, ofits))
    ms = statistics.mean(wall)
    return {"workload": f"{WORKLOAD}: unique-only coverage histogram of each coverage group from pass 1",
            "groups": len(groups), "host_threads": os.cpu_count(), "wall_ms": ms, "value": len(groups) / (ms / 1e3),
            "unit": "fits/s",
            "fits": [{k: f[k] for k in ("nbinom_mean", "nbinom_size", "deletion_coverage_propagation_cutoff",
                                        "censor_start", "censor_end", "restarts_converged")} for f in fits],
            "identical_to_oracle": bool(same),
            "cpu_baseline": {"value": len(groups) / cpu_s, "unit": "fits/s", "cores": 1, "kind": "port",
                             "sample": f"the same histograms, one sequential run ({cpu_s * 1e3:.0f} ms)"}}


def run_pairs(args, device, s):
    """Discordant-pair, missing-pair and pair-distance candidate scans (bsq_pair_candidates) on the
    headline sample with pair annotations (discordant and mate-unmapped pairs planted near breakpoints
    and at a background rate, longer pairs near 40 deletion-like sites): device time, the
    classification pass over every read, the host replay, and the oracle's position-by-position walk
    on the CPU."""
    from breseq_gb300 import synth
    from breseq_gb300.api import PairSettings, Scorer
    from oracle import pyoracle as po
    sp = synth.with_pairs(s, seed=31, discordant_sites=40, unmapped_sites=40, distance_sites=40)
    st = PairSettings(dp_group=tuple([0] * (int(sp.read_group.max()) + 1)), window_width=(462.75,),
                      predict_missing_pairs=True, predict_pair_distance=True, pd_cdf=(synth.pd_null(sp),),
                      pd_orientation=("FR",), pd_max_span=1500, pd_z_seed=2.5, pd_mean_covering_gap=137.5)
    with Scorer(device) as sc:
        sid = sc.load_sample(sp)
        for _ in range(args.warmup):
            r = sc.pair_candidates(sid, st)
        dev, main, wall = [], [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = sc.pair_candidates(sid, st)
            wall.append(1e3 * (time.perf_counter() - t0))
            ps = sc.last_pass_stats()
            dev.append(ps["device_ms"]); main.append(ps["main_kernel_ms"])
        launches = ps["kernel_launches"]
        with tempfile.TemporaryDirectory() as d:
            dp, mp, pd, odp, omp, opd = (os.path.join(d, f) for f in ("dp", "mp", "pd", "odp", "omp", "opd"))
            sc.write_pair_candidates(r, dp, mp, sp.target_names, pd)
            t0 = time.perf_counter()
            po.pair_candidates(sp, st, odp, omp, None, opd)
            cpu_s = time.perf_counter() - t0
            same = all(open(a).read() == open(b).read() for a, b in ((dp, odp), (mp, omp), (pd, opd)))
        sc.free_sample(sid)
    n = sp.n_reads
    ms, kms = statistics.mean(dev), statistics.mean(main)
    hbm, peak_kind = _peaks()
    kbytes = 47 * n   # per read: 32-byte record, flag, XP, read group read; code, group, two selections written
    return {"workload": f"{WORKLOAD} with pair annotations", "reads": n, "dp_regions": len(r["dp"]),
            "mp_regions": len(r["mp"]), "pd_regions": len(r["pd"]), "device_ms": ms, "wall_ms": statistics.mean(wall),
            "host_replay_ms": statistics.mean(wall) - ms, "kernel_launches": launches,
            "value": n / (statistics.mean(wall) / 1e3), "unit": "records/s",
            "roofline": {"bound": "hbm", "kernel": "pair_classify_kernel", "achieved": kbytes / (kms / 1e3) / 1e9,
                         "peak": hbm, "unit": "GB/s", "frac": kbytes / (kms / 1e3) / 1e9 / hbm, "kernel_ms": kms,
                         "algorithmic_bytes": kbytes, "peak_kind": peak_kind,
                         "traffic": PAIR_CLASSIFY_DRAM_PER_READ * n},
            "identical_to_oracle": bool(same),
            "cpu_baseline": {"value": n / cpu_s, "unit": "records/s", "cores": 1, "kind": "port",
                             "sample": f"the same sample, one position-by-position walk ({cpu_s:.2f} s)"}}


def run_softclip(args, device):
    """tabulate_soft_clipping_counts on a resident sample: device time of the call, its read pass
    (the dominant kernel), the end-to-end call from host buffers, and the oracle on the CPU."""
    import dataclasses
    from breseq_gb300 import abi, synth
    from breseq_gb300.api import Scorer, ScSettings
    from oracle import pyoracle as po
    c = synth.config_ecoli(seed=23, scale=args.scale)
    s = synth.simulate(dataclasses.replace(c, breakpoints=50, long_clip_fraction=0.01, softclip_fraction=0.02))
    n_cols = s.total_length() + len(s.target_offset) - 1
    with Scorer(device) as sc:
        sid = sc.load_sample(s)
        for _ in range(args.warmup):
            g = sc.soft_clipping(sid)
        dev, main, wall = [], [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            g = sc.soft_clipping(sid)
            wall.append(1e3 * (time.perf_counter() - t0))
            st = sc.last_pass_stats()
            dev.append(st["device_ms"]); main.append(st["main_kernel_ms"])
        launches = st["kernel_launches"]
        sc.free_sample(sid)
        # end to end: upload from pinned host buffers, tabulation, rows back, free
        view = abi.SampleView(s)
        pinned = [a for a in view._keep if a.nbytes >= 1 << 16 and sc.L.bsq_host_register(a.ctypes.data, a.nbytes) == 0]
        e2e = []
        for i in range(args.warmup + args.steps):
            sc.timer_start()
            sid2 = sc.load_sample(s)
            sc.soft_clipping(sid2)
            sc.free_sample(sid2)
            t = sc.timer_stop()
            if i >= args.warmup:
                e2e.append(t)
        for a in pinned:
            sc.L.bsq_host_unregister(a.ctypes.data)
    t0 = time.perf_counter()
    o = po.soft_clipping(s)
    cpu_s = time.perf_counter() - t0
    same = g["summary"] == o["summary"] and np.array_equal(g["rows"], o["rows"])
    ms, kms = statistics.mean(dev), statistics.mean(main)
    hbm, peak_kind = _peaks()
    kbytes = 32 * s.n_reads + 4 * n_cols
    out = {"workload": SC_WORKLOAD if args.scale == 1.0 else f"{SC_WORKLOAD} scaled x{args.scale:g}",
           "reads": s.n_reads, "genome_bp": s.total_length(), "rows": int(g["summary"]["n_positions"]),
           "clip_events": int(g["summary"]["total_clipped_read_ends"]),
           "device_ms": ms, "wall_ms": statistics.mean(wall), "kernel_launches": launches,
           "value": s.n_reads / (ms / 1e3), "unit": "records/s",
           "e2e": {"ms": statistics.mean(e2e), "value": s.n_reads / (statistics.mean(e2e) / 1e3), "unit": "records/s",
                   "h2d_bytes": int(sum(a.nbytes for a in view._keep))},
           "roofline": {"bound": "hbm", "kernel": "sc_count_kernel", "achieved": kbytes / (kms / 1e3) / 1e9,
                        "peak": hbm, "unit": "GB/s", "frac": kbytes / (kms / 1e3) / 1e9 / hbm, "kernel_ms": kms,
                        "algorithmic_bytes": kbytes, "peak_kind": peak_kind,
                        "traffic": SC_READS_DRAM_PER_READ * s.n_reads if SC_READS_DRAM_PER_READ else None},
           "identical_to_oracle": bool(same),
           "cpu_baseline": {"value": s.n_reads / cpu_s, "unit": "records/s", "cores": 1, "kind": "port",
                            "sample": f"the same sample, one run ({cpu_s:.2f} s)"}}
    return out


_CPU_SAMPLE = {}


def _cpu_reference(sample_scale: float, threads: int, min_seconds: float = 0.0):
    """The oracle port of the reference algorithm on a bounded sample of the same workload, repeated
    until at least `min_seconds` of CPU work were timed."""
    from oracle import pyoracle as po
    if sample_scale not in _CPU_SAMPLE:
        _CPU_SAMPLE[sample_scale] = _workload(seed=21, scale=sample_scale)
    s = _CPU_SAMPLE[sample_scale]
    bases = s.aligned_bases()
    reps = 0
    t0 = time.perf_counter()
    while True:
        ec = po.error_count(s, n_threads=threads)
        tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        po.identify(s, tab, po.default_im_params(s), n_threads=threads, positions=False)
        reps += 1
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    return reps * bases / dt, reps * bases, dt, s.total_length(), reps


def _oracle_run(s, threads):
    """The oracle port of the reference algorithm (both passes) on sample s: results and seconds."""
    from oracle import pyoracle as po
    t0 = time.perf_counter()
    ec = po.error_count(s, n_threads=threads)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    im = po.identify(s, tab, po.default_im_params(s), n_threads=threads, positions=False)
    return ec, im, time.perf_counter() - t0


def _oracle_check(s, ec_gpu, im_gpu, threads):
    """The headline sample through the oracle as well: covariate counts and coverage histograms
    bit-exact, RA calls identical (scores within 1e-3, frequencies within 1e-4), MC / UN identical."""
    from tests import compare
    ec_o, im_o, dt = _oracle_run(s, threads)
    problems = []
    if not np.array_equal(ec_gpu["counts"], ec_o["counts"]):
        problems.append("covariate counts differ")
    h = min(ec_gpu["hist"].shape[1], ec_o["hist"].shape[1])
    if not np.array_equal(ec_gpu["hist"][:, :h], ec_o["hist"][:, :h]):
        problems.append("coverage histograms differ")
    problems += compare.compare_ra(im_gpu["ra"], im_o["ra"])
    problems += compare.compare_intervals(im_gpu, im_o)
    return {"identical": not problems, "ra_items": len(im_o["ra"]), "mc": len(im_o["mc"]), "un": len(im_o["un"]),
            "problems": problems[:5]}, dt


def _calls(im):
    """The call set of a result (RA records as dicts or as a structured array)."""
    def b(x):
        return x.decode() if isinstance(x, bytes) else str(x)
    return [(int(r["tid"]), int(r["position"]), int(r["insert_position"]), b(r["new_base"]),
             bool(r["passed_consensus"]), bool(r["passed_polymorphism"])) for r in im["ra"]]


def run_reference(args, world, rank, pg):
    """The reference arm: the oracle port of error_count + identify_mutations on the host cores, on the
    same sample the GPU arm scores (one full run per step, all host threads)."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    s = _workload(seed=21, scale=args.scale)
    bases = s.aligned_bases()
    ln = s.total_length()
    times = []
    for i in range(args.warmup + args.steps):
        _, _, dt = _oracle_run(s, threads)
        if i >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.mean(times)
    value = bases / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD if args.scale == 1.0 else f"{WORKLOAD} scaled x{args.scale:g}",
                       "genome_bp": ln, "read_bases_per_step": bases},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "same_config": True,
                             "sample": f"the same sample as the GPU arm ({ln} bp, {bases} read-bases), one run per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, pg):
    from breseq_gb300 import abi
    from breseq_gb300.api import ImSettings, Scorer
    s = _workload(seed=21 + rank, scale=args.scale)
    bases = s.aligned_bases()
    n_cols = s.total_length() + len(s.target_offset) - 1
    sc = Scorer(local)
    sid = sc.load_sample(s)
    prec = 1 if args.precision == "fp32c" else 0
    st = ImSettings()
    kstats = {"ec": [], "im": []}
    launches = [0]

    def step(sample_id, record=False):
        ec = sc.error_count(sample_id)
        if record:
            ps = sc.last_pass_stats(); kstats["ec"].append(ps["main_kernel_ms"]); launches[0] += ps["kernel_launches"]
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im = sc.identify_mutations(sample_id, tab, st, precision=prec, as_dicts=False)
        if record:
            ps = sc.last_pass_stats(); kstats["im"].append(ps["main_kernel_ms"]); launches[0] += ps["kernel_launches"]
        return im

    ec0 = sc.error_count(sid)
    tab0 = sc.counts_to_log10_prob(ec0["counts"], s.n_read_files, s.n_quality)
    tuning = sc.autotune([sid], [tab0], st, precision=prec) if not args.no_tune else sc.tuning()
    clocks = ClockSampler(local)   # sampling from the warm-up on, so the short timed region is covered
    clocks.start()
    for _ in range(args.warmup):
        ref_im = step(sid)
    _barrier(pg)
    sc.timer_start()
    for _ in range(args.steps):
        im = step(sid, record=True)
    ms = sc.timer_stop() / args.steps
    _barrier(pg)
    clk = clocks.stop()
    ms_max = _max_over_ranks(pg, ms)
    value = world * bases / (ms_max / 1000.0)
    # ---- plain FP64 form on the same sample, same calls: default launch shapes, no graphs
    sc.set_tuning(**PLAIN_TUNING)
    t_plain = []
    for i in range(1 + args.plain_steps):
        sc.timer_start()
        ec = sc.error_count(sid)
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im_plain = sc.identify_mutations(sid, tab, st, precision=0, as_dicts=False)
        if i > 0:
            t_plain.append(sc.timer_stop())
        else:
            sc.timer_stop()
    same_calls = _calls(im_plain) == _calls(im)
    plain_ms = statistics.mean(t_plain) if t_plain else None
    sc.set_tuning(**tuning)
    # ---- end to end through the C ABI from pinned host buffers
    view = abi.SampleView(s)
    pinned = []
    for a in view._keep:
        if a.nbytes >= 1 << 16 and sc.L.bsq_host_register(a.ctypes.data, a.nbytes) == 0:
            pinned.append(a)
    h2d = int(sum(a.nbytes for a in view._keep))
    e2e_ms = []
    phases = {"load": [], "pass1": [], "table": [], "pass2": [], "free": []}
    xfer = {"h2d": 0, "d2h": 0}
    for i in range(args.warmup + args.steps):
        sc.timer_start()
        t0 = time.perf_counter()
        sid2 = sc.load_sample(s)
        t1 = time.perf_counter()
        ec2 = sc.error_count(sid2)
        b1 = sc.last_pass_bytes()
        t2 = time.perf_counter()
        tab2 = sc.counts_to_log10_prob(ec2["counts"], s.n_read_files, s.n_quality)
        t3 = time.perf_counter()
        im2 = sc.identify_mutations(sid2, tab2, st, precision=prec, as_dicts=False)
        b2 = sc.last_pass_bytes()
        t4 = time.perf_counter()
        sc.free_sample(sid2)
        t = sc.timer_stop()
        t5 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append(t)
            for k, a, b in (("load", t0, t1), ("pass1", t1, t2), ("table", t2, t3), ("pass2", t3, t4), ("free", t4, t5)):
                phases[k].append(1e3 * (b - a))
            xfer = {"h2d": b1["h2d"] + b2["h2d"], "d2h": b1["d2h"] + b2["d2h"]}
    h2d += xfer["h2d"]
    d2h = xfer["d2h"]
    # ---- end to end as a stream of samples: the next step's upload (its own load stream) runs while
    # this step's passes do; every step's host-to-device copy and result read stay inside the timed
    # region, which starts with the first step's upload and ends after the last step's free
    import concurrent.futures as cf

    def run_stream(k):
        with cf.ThreadPoolExecutor(1) as ex:
            sc.timer_start()
            fut = ex.submit(sc.load_sample, s)
            for i in range(k):
                sid_i = fut.result()
                if i + 1 < k:
                    fut = ex.submit(sc.load_sample, s)
                ec_i = sc.error_count(sid_i)
                tab_i = sc.counts_to_log10_prob(ec_i["counts"], s.n_read_files, s.n_quality)
                sc.identify_mutations(sid_i, tab_i, st, precision=prec, as_dicts=False)
                sc.free_sample(sid_i)
            return sc.timer_stop()

    run_stream(args.warmup)
    stream_ms = run_stream(args.steps) / args.steps
    for a in pinned:
        sc.L.bsq_host_unregister(a.ctypes.data)
    e2e_seq_ms = _max_over_ranks(pg, statistics.mean(e2e_ms))
    e2e_ms_max = _max_over_ranks(pg, stream_ms)
    # ---- roofline of the dominant kernel
    hbm, peak_kind = _peaks()
    ec_ms = statistics.mean(kstats["ec"]); im_ms = statistics.mean(kstats["im"])
    n_reads = s.n_reads
    # algorithmic bytes: 4-bit base + 8-bit quality per aligned read-base, ~20 B record per read,
    # 2-bit reference per column, plus the 48 B per column the column pass writes
    bytes_ec = bases * 1.5 + n_reads * 20 + n_cols * 0.25
    bytes_im = bytes_ec + n_cols * 48
    if im_ms >= ec_ms:
        kname, kms, kbytes, dram_per_base = "im_column_kernel", im_ms, bytes_im, IM_COLUMN_DRAM_PER_BASE
    else:
        kname, kms, kbytes, dram_per_base = "ec_read_kernel", ec_ms, bytes_ec, EC_READ_DRAM_PER_BASE
    achieved = kbytes / (kms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32c+f64" if prec == 1 else "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.scale == 1.0 else f"{WORKLOAD} scaled x{args.scale:g}", "genome_bp": s.total_length(), "reads": n_reads, "read_bases_per_step": bases,
                   "precision": args.precision, "l2": "inputs (%.2f GB) larger than L2" % ((s.qual.nbytes + s.seq.nbytes) / 1e9)},
        "e2e": {"value": world * bases / (e2e_ms_max / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms_max,
                "mode": "stream: step i+1's upload overlaps step i's passes",
                "sequential": {"value": world * bases / (e2e_seq_ms / 1000.0), "ms_per_step": e2e_seq_ms,
                               "host_ms_by_phase": {k: statistics.mean(v) for k, v in phases.items()}}},
        "gpu_launches": launches[0],
        "plain_fp64": {"ms_per_step": plain_ms, "value": (bases / (plain_ms / 1000.0)) if plain_ms else None,
                       "served_over_plain": (plain_ms / ms) if plain_ms else None, "identical_calls": same_calls},
        "passes_ms": {"error_count_kernel": ec_ms, "im_column_kernel": im_ms},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": dram_per_base * bases, "traffic_unit": "bytes per launch",
                     "algorithmic_bytes": kbytes, "peak_kind": peak_kind},
        "clocks": clk,
        "tuning": tuning,
        "ra_items": len(im["ra"]),
    }
    if rank == 0 and not args.no_coverage:
        line["coverage_table"] = run_coverage(args, sc, sid, s)
        line["coverage_fit"] = run_covfit(args, ec0, s)
    if rank == 0 and not args.no_cpu:
        # the oracle on the same sample with every host thread: the agreement of the headline result
        # and the CPU baseline on the same input; and one host core on a bounded sample
        threads = os.cpu_count() or 1
        ec_chk = sc.error_count(sid)
        im_chk = sc.identify_mutations(sid, sc.counts_to_log10_prob(ec_chk["counts"], s.n_read_files, s.n_quality), st,
                                       precision=prec)
        check, dt = _oracle_check(s, ec_chk, im_chk, threads)
        line["identical_to_oracle"] = check
        rate1, cb1, dt1, ln1, reps1 = _cpu_reference(args.cpu_scale, 1, args.cpu_seconds)
        line["cpu_baseline"] = {"value": bases / dt, "unit": UNIT, "cores": threads, "kind": "port", "same_config": True,
                                "sample": f"the same sample ({s.total_length()} bp, {bases} read-bases), one run, {dt:.1f} s",
                                "one_core": {"value": rate1, "unit": UNIT, "cores": 1,
                                             "sample": f"same workload at {args.cpu_scale:g} x genome length ({ln1} bp), "
                                                       f"{reps1} runs, {cb1} read-bases in {dt1:.1f} s"}}
    sc.close()
    # the mixed-shape legs first: the BAM leg leaves gigabytes of freed host and pooled device memory
    if rank == 0 and args.batch_jobs > 0:
        line["batched"], line["served"] = run_mix(args, local)
    if rank == 0 and not args.no_bam:
        line["bam_input"] = run_bam(args, local, s)
    if rank == 0 and not args.no_softclip:
        line["soft_clipping"] = run_softclip(args, local)
    if rank == 0 and not args.no_pairs:
        line["pair_scans"] = run_pairs(args, local, s)
    if rank == 0:
        print(json.dumps(line), flush=True)


def _simulate(cfg):
    from breseq_gb300 import synth
    return synth.simulate(cfg)


def _pool(args):
    """Distinct seeded samples of the mixed-shape distribution; job i uses pool[i % len(pool)].  The
    samples are generated in spawned worker processes (the GPU is already in use by this process)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from breseq_gb300 import synth
    cfgs = synth.config_batch(seed=41, n_samples=max(args.batch_jobs, args.batch_pool), scale=args.batch_scale)
    cfgs = cfgs[:args.batch_pool]
    workers = max(1, min(len(cfgs), (os.cpu_count() or 1)))
    with cf.ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        sims = list(ex.map(_simulate, [c for c, _ in cfgs]))
    return [(sim, poly) for sim, (_, poly) in zip(sims, cfgs)]


def run_mix(args, device):
    from breseq_gb300 import abi
    from breseq_gb300.api import ImSettings, Scorer, Server
    pool = _pool(args)
    P = len(pool)
    views = [abi.SampleView(s) for s, _ in pool]
    sc = Scorer(device)
    pinned = []
    for v in views:                        # page-locked once: every job's upload is a DMA copy
        for a in v._keep:
            if a.nbytes >= 1 << 16 and sc.L.bsq_host_register(a.ctypes.data, a.nbytes) == 0:
                pinned.append(a)
    jobs = [i % P for i in range(args.batch_jobs)]
    sets = [ImSettings(polymorphism_prediction=pool[k][1]) for k in range(P)]
    pool_bases = [s.aligned_bases() for s, _ in pool]
    job_bases = sum(pool_bases[k] for k in jobs)
    cfg = {"workload": "mixed_shapes_genome40k-6Mb_cov20-500_L36/101/150_se/pe_consensus/polymorphism",
           "jobs": len(jobs), "distinct_samples": P, "genome_scale": args.batch_scale,
           "genome_bp": [int(s.total_length()) for s, _ in pool], "read_bases_per_step": job_bases}
    # ---- batched: every job resident, one batch call per pass
    sids = [sc.load_sample(pool[k][0]) for k in jobs]

    def batch_step():
        ecs = sc.error_count_batch(sids)
        tabs = sc.counts_to_log10_prob_batch([ec["counts"] for ec in ecs], [pool[k][0].n_read_files for k in jobs],
                                             [pool[k][0].n_quality for k in jobs])
        return sc.identify_mutations_batch(sids, tabs, [sets[k] for k in jobs], precision=1, as_dicts=False)

    if not args.no_tune:
        ecs = sc.error_count_batch(sids)
        tabs = [sc.counts_to_log10_prob(ec["counts"], pool[k][0].n_read_files, pool[k][0].n_quality)
                for ec, k in zip(ecs, jobs)]
        tuning = sc.autotune(sids, tabs, [sets[k] for k in jobs], precision=1)
    else:
        tuning = sc.tuning()
    for _ in range(max(1, args.warmup)):
        ims = batch_step()
    sc.timer_start()
    for _ in range(args.batch_steps):
        ims = batch_step()
    batch_ms = sc.timer_stop() / args.batch_steps
    for sid in sids:
        sc.free_sample(sid)
    # ---- plain FP64, one sample per call, each distinct sample once, default shapes, no graphs
    sc.set_tuning(**PLAIN_TUNING)
    plain_ms = 0.0
    same = True
    for k, (s, _) in enumerate(pool):
        sid = sc.load_sample(s)
        sc.timer_start()
        ec = sc.error_count(sid)
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im = sc.identify_mutations(sid, tab, sets[k], precision=0, as_dicts=False)
        plain_ms += sc.timer_stop()
        sc.free_sample(sid)
        same &= _calls(im) == _calls(ims[k])
    plain_rate = sum(pool_bases) / (plain_ms / 1000.0)
    batched = {"config": cfg, "ms_per_step": batch_ms, "value": job_bases / (batch_ms / 1000.0), "unit": UNIT,
               "plain_fp64": {"value": plain_rate, "ms_per_pool_pass": plain_ms,
                              "batched_over_plain": job_bases / (batch_ms / 1000.0) / plain_rate},
               "identical_calls": bool(same), "tuning": tuning}
    sc.close()
    # ---- served: the server's own capacity (every job submitted at once, completions per second),
    # then open-loop Poisson arrivals at 0.5 / 1 / 2 x that capacity
    batched_cap = len(jobs) / (batch_ms / 1000.0)     # jobs/s the batched form sustains
    n_sat = args.served_jobs
    with Server(device, hbm_budget=args.budget_gb * 1e9, max_batch_jobs=64) as srv:
        srv.set_tuning(**tuning)
        sat_ids = [(srv.submit(pool[i % P][0], sets[i % P], view=views[i % P]), i % P) for i in range(n_sat)]
        sat_infos = [srv.wait(j) for j, _ in sat_ids]
    sat_span = (max(i["done_ms"] for i in sat_infos) - min(i["submit_ms"] for i in sat_infos)) / 1000.0
    cap = n_sat / sat_span
    sat_value = sum(pool_bases[k] for _, k in sat_ids) / sat_span
    levels = []
    rng = np.random.default_rng(7)
    for rho in (0.5, 1.0, 2.0):
        lam = rho * cap
        n = args.served_jobs
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=n))
        with Server(device, hbm_budget=args.budget_gb * 1e9, max_batch_jobs=64) as srv:
            srv.set_tuning(**tuning)   # the batched leg's autotuned launch shapes
            ids = []
            t0 = time.perf_counter()
            for i in range(n):
                d = arrivals[i] - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                k = i % P
                ids.append((srv.submit(pool[k][0], sets[k], view=views[k]), k))
            infos = [srv.wait(j) for j, _ in ids]
            st = srv.stats()
        lat = np.array([i["done_ms"] - i["submit_ms"] for i in infos])
        stage = {k: float(np.mean([i[b] - i[a] for i in infos])) for k, a, b in
                 (("queue_ms", "submit_ms", "admit_ms"), ("upload_ms", "admit_ms", "ready_ms"),
                  ("wait_gpu_ms", "ready_ms", "start_ms"), ("round_ms", "start_ms", "done_ms"))}
        span = (max(i["done_ms"] for i in infos) - min(i["submit_ms"] for i in infos)) / 1000.0
        bases = sum(pool_bases[k] for _, k in ids)
        levels.append({"load": rho, "arrival_rate_jobs_s": lam, "jobs": n, "p50_ms": float(np.percentile(lat, 50)),
                       "p99_ms": float(np.percentile(lat, 99)), "value": bases / span, "unit": UNIT,
                       "served_over_plain": bases / span / plain_rate, "max_round_jobs": st["max_round_jobs"],
                       "max_resident_jobs": st["max_resident_jobs"], "peak_hbm_gb": st["peak_in_use"] / 1e9,
                       "rounds": st["rounds"], "gpu_busy_frac": st["gpu_busy_ms"] / 1000.0 / span,
                       "round_phase_ms": st["phase_ms"],
                       "mean_stage_ms": stage})
    from breseq_gb300 import _lib
    L = _lib.load()
    for a in pinned:
        L.bsq_host_unregister(a.ctypes.data)
    served = {"capacity_jobs_s": cap, "capacity_value": sat_value, "batched_capacity_jobs_s": batched_cap,
              "budget_gb": args.budget_gb, "levels": levels,
              "p50_ms": levels[1]["p50_ms"], "p99_ms": levels[1]["p99_ms"], "plain_fp64_value": plain_rate}
    return batched, served


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-scale", type=float, default=0.05)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0, help="genome length scale of the workload (profiling cases)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="minimum CPU work timed for cpu_baseline")
    ap.add_argument("--batch-jobs", type=int, default=96, help="jobs of the batched / served legs (0: skip them)")
    ap.add_argument("--batch-pool", type=int, default=96, help="distinct samples the jobs are drawn from")
    ap.add_argument("--batch-scale", type=float, default=0.25, help="genome length scale of the mixed samples")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--served-jobs", type=int, default=288)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--no-softclip", action="store_true", help="skip the soft-clipping leg")
    ap.add_argument("--no-coverage", action="store_true", help="skip the coverage-table leg")
    ap.add_argument("--no-bam", action="store_true", help="skip the BAM-input leg")
    ap.add_argument("--no-pairs", action="store_true", help="skip the discordant / missing-pair leg")
    args = ap.parse_args()
    world, rank, local, pg = _dist()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        from breseq_gb300 import build
        build.build()
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
