#!/usr/bin/env python
"""Benchmark of the read-evidence scoring path: aligned read-bases scored per second.

One step = the full path on one sample: error_count (pass 1), the error-table round trip, and
identify_mutations (pass 2), on the E. coli-scale clonal workload (4.63 Mb chromosome + 100 kb + 60 kb
plasmids, five 1.3-kb repeats, 300 SNPs + 40 indels, 2 x 100x paired-end 150-bp reads; seeded
synthetic data of that shape).  `value` is input aligned read-bases / device time of a step with the
sample resident in HBM; `e2e` runs the same step through the C ABI from pinned host buffers
(upload + both passes + result download + free inside the timed region).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

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
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def _workload(seed: int, scale: float = 1.0):
    from breseq_gb300 import synth
    return synth.simulate(synth.config_ecoli(seed=seed, scale=scale))


def _cpu_reference(sample_scale: float, threads: int):
    """The oracle port of the reference algorithm on a bounded sample of the same workload."""
    from oracle import pyoracle as po
    s = _workload(seed=21, scale=sample_scale)
    bases = s.aligned_bases()
    t0 = time.perf_counter()
    ec = po.error_count(s, n_threads=threads)
    tab = po.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
    po.identify(s, tab, po.default_im_params(s), n_threads=threads, positions=False)
    dt = time.perf_counter() - t0
    return bases / dt, bases, dt, s.total_length()


def run_reference(args, world, rank, pg):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    times = []
    rate = bases = ln = None
    for i in range(args.warmup + args.steps):
        rate, bases, dt, ln = _cpu_reference(args.cpu_scale, threads)
        if i >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.mean(times)
    value = bases / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sample_length_bp": ln, "sample_read_bases": bases},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"same workload at {args.cpu_scale:g} x genome length ({ln} bp, {bases} read-bases)"},
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
        im = sc.identify_mutations(sample_id, tab, st, precision=prec)
        if record:
            ps = sc.last_pass_stats(); kstats["im"].append(ps["main_kernel_ms"]); launches[0] += ps["kernel_launches"]
        return im

    for _ in range(args.warmup):
        ref_im = step(sid)
    clocks = ClockSampler(local)
    clocks.start()
    _barrier(pg)
    sc.timer_start()
    for _ in range(args.steps):
        im = step(sid, record=True)
    ms = sc.timer_stop() / args.steps
    _barrier(pg)
    clk = clocks.stop()
    ms_max = _max_over_ranks(pg, ms)
    value = world * bases / (ms_max / 1000.0)
    # ---- plain FP64 form on the same sample (the spec comparison), same calls
    t_plain = []
    for i in range(1 + args.plain_steps):
        sc.timer_start()
        ec = sc.error_count(sid)
        tab = sc.counts_to_log10_prob(ec["counts"], s.n_read_files, s.n_quality)
        im_plain = sc.identify_mutations(sid, tab, st, precision=0)
        if i > 0:
            t_plain.append(sc.timer_stop())
        else:
            sc.timer_stop()
    same_calls = [(r["tid"], r["position"], r["insert_position"], r["new_base"]) for r in im_plain["ra"]] == \
                 [(r["tid"], r["position"], r["insert_position"], r["new_base"]) for r in im["ra"]]
    plain_ms = statistics.mean(t_plain) if t_plain else None
    # ---- end to end through the C ABI from pinned host buffers
    view = abi.SampleView(s)
    pinned = []
    for a in view._keep:
        if a.nbytes >= 1 << 16 and sc.L.bsq_host_register(a.ctypes.data, a.nbytes) == 0:
            pinned.append(a)
    h2d = int(sum(a.nbytes for a in view._keep))
    e2e_ms = []
    d2h = 0
    for i in range(args.warmup + args.steps):
        sc.timer_start()
        sid2 = sc.load_sample(s)
        im2 = step(sid2)
        sc.free_sample(sid2)
        t = sc.timer_stop()
        if i >= args.warmup:
            e2e_ms.append(t)
    d2h = n_cols * 48 + len(im2["ra"]) * 200 + s.n_read_files * 25 * s.n_quality * 8
    for a in pinned:
        sc.L.bsq_host_unregister(a.ctypes.data)
    e2e_ms_max = _max_over_ranks(pg, statistics.mean(e2e_ms))
    # ---- roofline of the dominant kernel
    hbm, peak_kind = _peaks()
    ec_ms = statistics.mean(kstats["ec"]); im_ms = statistics.mean(kstats["im"])
    n_reads = s.n_reads
    # algorithmic bytes: 4-bit base + 8-bit quality per aligned read-base, ~20 B record per read,
    # 2-bit reference per column, plus the 48 B per column the column pass writes
    bytes_ec = bases * 1.5 + n_reads * 20 + n_cols * 0.25
    bytes_im = bytes_ec + n_cols * 48
    if im_ms >= ec_ms:
        kname, kms, kbytes = "im_column_kernel", im_ms, bytes_im
    else:
        kname, kms, kbytes = "ec_kernel", ec_ms, bytes_ec
    achieved = kbytes / (kms / 1000.0) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32c+f64" if prec == 1 else "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD if args.scale == 1.0 else f"{WORKLOAD} scaled x{args.scale:g}", "genome_bp": s.total_length(), "reads": n_reads, "read_bases_per_step": bases,
                   "precision": args.precision, "l2": "inputs (%.2f GB) larger than L2" % ((s.qual.nbytes + s.seq.nbytes) / 1e9)},
        "e2e": {"value": world * bases / (e2e_ms_max / 1000.0), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches[0],
        "plain_fp64": {"ms_per_step": plain_ms, "value": (bases / (plain_ms / 1000.0)) if plain_ms else None,
                       "served_over_plain": (plain_ms / ms) if plain_ms else None, "identical_calls": same_calls},
        "passes_ms": {"error_count_kernel": ec_ms, "im_column_kernel": im_ms},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind},
        "clocks": clk,
        "ra_items": len(im["ra"]),
    }
    if rank == 0 and not args.no_cpu:
        rate, cb, dt, ln = _cpu_reference(args.cpu_scale, os.cpu_count() or 1)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                "sample": f"same workload at {args.cpu_scale:g} x genome length ({ln} bp, {cb} read-bases), {dt:.1f} s"}
    sc.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


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
