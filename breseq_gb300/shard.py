"""Sharding of scoring jobs across ranks (one process per GPU).

The path shards by sample: samples are independent through both passes, so each rank scores its
own jobs with no collective in the data path (weak scaling).  A job is placed by its work, the
aligned read-bases of its sample, with the longest-processing-time rule: heaviest job first, onto
the rank with the least work so far (ties to the lower rank), which is deterministic on every rank
without communication.  Timing across ranks takes the slowest rank (all_reduce MAX)."""
from __future__ import annotations


def plan(work: list[int] | list[float], world: int) -> list[list[int]]:
    """Job indices per rank; every job on exactly one rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(work)), key=lambda i: (-work[i], i))
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += work[i]
    for r in out:
        r.sort()
    return out


def slowest(value: float, group=None) -> float:
    """Maximum of `value` over the ranks of the default process group (itself without one)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


# ---------------------------------------------------------------------------- one sample, by position
# One sample split across ranks by contiguous position ranges of its concatenated targets.  Columns
# are independent given the reads that cover them, so:
#   pass 1  the covariate counts are per read: a rank counts the reads that START in its range (each
#           read exactly once); the unique-only coverage histogram is per column: a rank tabulates the
#           columns of its range over every read that covers them (its "halo": reads starting before
#           the range but reaching into it).  Both are integer sums, added exactly by one all-reduce
#           before the error table is made (counts_to_log10_prob, error_count.cpp:1005-1026);
#   pass 2  a rank scores its range's columns over its halo reads and keeps the RA items and
#           per-position arrays of its own columns; the MC / UN state machines, which run along each
#           target, are replayed over the ranks' per-position arrays joined in order
#           (bsq_intervals_from_positions).
# The result equals scoring the whole sample in one place.


def _columns(s):
    """Start and end (exclusive) column of every record in the concatenated target space."""
    import numpy as np
    ops = s.cigar & 0xF
    ref = np.where(np.isin(ops, (0, 2, 3, 7, 8)), (s.cigar >> 4).astype(np.int64), 0)
    cs = np.concatenate([[0], np.cumsum(ref)])
    co = s.cigar_off.astype(np.int64)
    span = cs[co + s.n_cigar.astype(np.int64)] - cs[co]
    start = s.target_offset[s.tid].astype(np.int64) + s.pos.astype(np.int64)
    return start, start + np.maximum(span, 1)


def plan_ranges(s, world: int) -> list[tuple[int, int]]:
    """Contiguous ranges [c0, c1) of the concatenated targets, one per rank, holding about equal shares
    of the sample's aligned read-bases (by read start); they cover every column exactly once."""
    import numpy as np
    if world < 1:
        raise ValueError("world must be >= 1")
    total = int(s.target_offset[-1])
    start, end = _columns(s)
    w = np.cumsum((end - start).astype(np.float64))
    cuts = [0]
    for r in range(1, world):
        k = int(np.searchsorted(w, w[-1] * r / world)) if len(w) else 0
        c = int(start[min(k, len(start) - 1)]) if len(start) else total * r // world
        cuts.append(min(max(c, cuts[-1]), total))
    cuts.append(total)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def subsample(s, c0: int, c1: int, owned: bool = False):
    """The records of sample s that cover a column of [c0, c1) (owned=False) or start in it (owned=True),
    in their order, over the same reference and base / quality / CIGAR arrays."""
    import dataclasses
    import numpy as np
    start, end = _columns(s)
    keep = (start >= c0) & (start < c1) if owned else (start < c1) & (end > c0)
    idx = np.nonzero(keep)[0]
    f = {k: getattr(s, k)[idx] for k in ("tid", "pos", "flag", "mapq", "x1", "xl", "xr", "read_file", "read_group",
                                         "l_qseq", "seq_off", "cigar_off", "n_cigar")}
    for k in ("xj", "isize", "xp", "mtid", "mpos"):
        v = getattr(s, k)
        f[k] = None if v is None else v[idx]
    if s.qname_off is not None:
        lo, hi = s.qname_off[idx].astype(np.int64), s.qname_off[idx + 1].astype(np.int64)
        off = np.concatenate([[0], np.cumsum(hi - lo)]).astype(s.qname_off.dtype)
        take = np.concatenate([np.arange(a, b) for a, b in zip(lo, hi)]) if len(idx) else np.zeros(0, np.int64)
        f["qname_off"], f["qname"] = off, s.qname[take]
    return dataclasses.replace(s, **f)


def score_ranges(backend, s, rank: int, world: int, settings=None, deletion_propagation_cutoff=None,
                 deletion_seed_cutoff=None, group=None) -> dict:
    """Both passes of sample s with this rank scoring its position range; every rank returns the whole
    sample's result: covariate counts, coverage histograms, the error table, RA items, MC / UN
    intervals and per-position arrays.  backend: counts(sample) -> covariate counts;
    coverage(sample, tid, start_1, end_1) -> BAM2COV columns; identify(sample, table, settings, prop, seed)
    -> result with per-position arrays (Scorer-backed in RangeScorer below).  group: a torch.distributed
    process group (None: the default one; without one initialised, world must be 1)."""
    import numpy as np
    from . import _lib, abi
    c0, c1 = plan_ranges(s, world)[rank]
    T = len(s.target_offset) - 1
    R, Q = s.n_read_files, s.n_quality
    # ---- pass 1
    counts = np.asarray(backend.counts(subsample(s, c0, c1, owned=True)), dtype=np.int64)
    halo = subsample(s, c0, c1)
    called = set(int(t) for t in s.target_order)
    hist = {}
    for t in range(T):
        a, b = max(c0, int(s.target_offset[t])), min(c1, int(s.target_offset[t + 1]))
        if a >= b or t not in called:
            continue
        cols = backend.coverage(halo, t, a - int(s.target_offset[t]) + 1, b - int(s.target_offset[t]))
        u = (cols["unique_top"].astype(np.int64) + cols["unique_bot"])[
            (cols["raw_redundant_top"].astype(np.int64) + cols["raw_redundant_bot"]) == 0]
        g = int(s.coverage_group[t])
        h = hist.setdefault(g, np.zeros(1, np.int64))
        bc = np.bincount(u, minlength=len(h)) if len(u) else np.zeros(len(h), np.int64)
        if len(bc) > len(h):
            h = np.concatenate([h, np.zeros(len(bc) - len(h), np.int64)])
        h[:len(bc)] += bc
        hist[g] = h
    G = s.n_coverage_groups
    width = max([len(h) for h in hist.values()] + [1])
    hist_arr = np.zeros((G, width), np.int64)
    for g, h in hist.items():
        hist_arr[g, :len(h)] = h
    counts, hist_arr = _sum_over_ranks(counts, hist_arr, world, group)
    hist_size = np.array([int(np.max(np.nonzero(hist_arr[g])[0])) + 1 if hist_arr[g].any() else 0 for g in range(G)])
    L = _lib.load()
    tab = np.zeros(R * 25 * Q, np.float64)
    cu = np.ascontiguousarray(counts, dtype=np.uint64)
    rc = L.bsq_counts_to_log10_prob(abi.ptr(cu, abi.C.c_uint64), R, Q, abi.ptr(tab, abi.C.c_double))
    if rc != 0:
        raise _lib.BsqError(rc, "counts_to_log10_prob")
    # ---- pass 2
    prop = np.ascontiguousarray(np.broadcast_to(np.asarray(5.0 if deletion_propagation_cutoff is None
                                                           else deletion_propagation_cutoff, np.float64), (T,)))
    seed = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if deletion_seed_cutoff is None
                                                           else deletion_seed_cutoff, np.float64), (T,)))
    im = backend.identify(halo, tab, settings, prop, seed)
    toff = s.target_offset.astype(np.int64)
    ra = [r for r in im["ra"] if c0 <= toff[r["tid"]] + r["position"] - 1 < c1]
    pos = {k: v[c0:c1] for k, v in im["positions"].items()}
    parts = _gather_over_ranks((ra, pos), world, group)
    ra_all = [r for p in parts for r in p[0]]
    pos_all = {k: np.concatenate([p[1][k] for p in parts]) for k in pos}
    mc, un = intervals_from_positions(s, pos_all, settings, prop, seed)
    return dict(counts=counts.astype(np.uint64), hist=hist_arr.astype(np.uint64), hist_size=hist_size, table=tab,
                ra=ra_all, mc=mc, un=un, positions=pos_all, range=(c0, c1))


def intervals_from_positions(s, positions, settings, prop, seed):
    """MC / UN of a whole sample from its per-position arrays (bsq_intervals_from_positions)."""
    import ctypes as C
    import numpy as np
    from . import _lib, abi
    from .api import ImSettings, im_params
    L = _lib.load()
    p, keep = im_params(s, settings or ImSettings(), prop, seed)
    view = abi.SampleView(s)
    arrs = {k: np.ascontiguousarray(positions[k]) for k in ("unique_top", "unique_bot", "redundant_top",
                                                             "redundant_bot", "consensus_score")}
    pa = abi.PositionArrays(unique_top=abi.ptr(arrs["unique_top"], C.c_uint32),
                            unique_bot=abi.ptr(arrs["unique_bot"], C.c_uint32),
                            redundant_top=abi.ptr(arrs["redundant_top"], C.c_double),
                            redundant_bot=abi.ptr(arrs["redundant_bot"], C.c_double),
                            consensus_score=abi.ptr(arrs["consensus_score"], C.c_double))
    n_mc, n_un = C.c_uint64(), C.c_uint64()
    rc = L.bsq_intervals_from_positions(C.byref(view.ref), C.byref(pa), C.byref(p), None, 0, C.byref(n_mc), None, 0,
                                        C.byref(n_un))
    mc = (abi.McRecord * max(1, n_mc.value))()
    un = (abi.UnRecord * max(1, n_un.value))()
    rc = L.bsq_intervals_from_positions(C.byref(view.ref), C.byref(pa), C.byref(p), mc, n_mc.value, C.byref(n_mc),
                                        un, n_un.value, C.byref(n_un))
    if rc != 0:
        raise _lib.BsqError(rc, "intervals_from_positions")
    return abi.mc_to_dicts(mc[:n_mc.value]), abi.un_to_dicts(un[:n_un.value])


def _sum_over_ranks(counts, hist, world, group):
    """Exact integer sum of the covariate counts and the coverage histograms over the ranks."""
    import numpy as np
    if world == 1:
        return counts, hist
    import torch
    import torch.distributed as dist
    w = torch.tensor([hist.shape[1]], dtype=torch.int64)
    dist.all_reduce(w, op=dist.ReduceOp.MAX, group=group)
    h = np.zeros((hist.shape[0], int(w.item())), np.int64)
    h[:, :hist.shape[1]] = hist
    flat = torch.from_numpy(np.concatenate([counts.ravel(), h.ravel()]))
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    a = flat.numpy()
    return a[:counts.size].reshape(counts.shape), a[counts.size:].reshape(h.shape)


def _gather_over_ranks(obj, world, group):
    if world == 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, obj, group=group)
    return out


class RangeScorer:
    """The GPU backend of score_ranges: the passes through a breseq_gb300.api.Scorer on this rank's GPU."""

    def __init__(self, scorer):
        self.sc = scorer

    def counts(self, sample):
        sid = self.sc.load_sample(sample)
        try:
            return self.sc.error_count(sid)["counts"]
        finally:
            self.sc.free_sample(sid)

    def coverage(self, sample, tid, start_1, end_1):
        if not hasattr(self, "_cov") or self._cov[0] is not sample:
            if hasattr(self, "_cov"):
                self.sc.free_sample(self._cov[1])
            self._cov = (sample, self.sc.load_sample(sample))
        return self.sc.coverage_columns(self._cov[1], tid, start_1, end_1)

    def identify(self, sample, table, settings, prop, seed):
        from .api import ImSettings
        sid = self._cov[1] if hasattr(self, "_cov") and self._cov[0] is sample else self.sc.load_sample(sample)
        try:
            return self.sc.identify_mutations(sid, table, settings or ImSettings(), deletion_propagation_cutoff=prop,
                                              deletion_seed_cutoff=seed, positions=True)
        finally:
            self.sc.free_sample(sid)
            if hasattr(self, "_cov") and self._cov[1] == sid:
                del self._cov
