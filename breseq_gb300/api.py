"""Host API over the C ABI, mirroring breseq's entry points of the scoring path.

    error_count(...)         <- breseq::error_count          (src/breseq/error_count.h:44-56)
    identify_mutations(...)  <- breseq::identify_mutations   (src/breseq/identify_mutations.h:46-60)
    soft_clipping(...)       <- breseq::tabulate_soft_clipping_counts (src/breseq/soft_clipping.h)

Both take a decoded sample (breseq_gb300.synth.Sample or anything with the same record arrays)
instead of BAM/FASTA file names, and return what breseq writes to its output files: the covariate
count table and unique-only coverage histograms, and the RA / MC / UN evidence with raw values.
Settings defaults are breseq's (src/breseq/settings.cpp:857-950, 1335)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib, abi

PRECISION_FP64 = 0
PRECISION_FP32C = 1


@dataclass
class ScSettings:
    """Soft-clipping settings with breseq's defaults (src/breseq/settings.cpp:1369-1374)."""
    minimum_clipped_bases: int = 12
    consensus_base_fraction: float = 0.95
    dispersion_trim_frequency: float = 0.25
    maximum_dispersion: float = 0.005
    minimum_rate: float = 1e-5


def header_read_groups(sample) -> int:
    """The @RG count of the header of a sample's BAM: `n_header_read_groups` when the sample has it, else
    the groups synth.bam_bytes declares for it (the highest read group + 1)."""
    n = getattr(sample, "n_header_read_groups", None)
    if n is not None:
        return int(n)
    return int(np.max(sample.read_group)) + 1 if len(sample.read_group) else 1


def sc_params(sample, st: ScSettings):
    """bsq_sc_params for a sample; rows follow the std::string order of its target names."""
    names = list(sample.target_names)
    order = np.array(sorted(range(len(names)), key=lambda t: names[t].encode()), dtype=np.uint32)
    p = abi.ScParams(minimum_clipped_bases=st.minimum_clipped_bases, consensus_base_fraction=st.consensus_base_fraction,
                     dispersion_trim_frequency=st.dispersion_trim_frequency, maximum_dispersion=st.maximum_dispersion,
                     minimum_rate=st.minimum_rate, target_name_order=abi.ptr(order, C.c_uint32))
    return p, order


@dataclass
class PairSettings:
    """Discordant / missing-pair scan settings with breseq's defaults (src/breseq/settings.cpp:376-392).
    dp_group: DP group of each read group (-1 none); window_width, r1_prefix, r2_prefix: per DP group."""
    dp_group: tuple = (0,)
    window_width: tuple = (400.0,)
    r1_prefix: tuple = (1,)
    r2_prefix: tuple = (2,)
    discordant_pair_seed: int = 3
    predict_missing_pairs: bool = False
    missing_pair_seed: int = 3
    missing_pair_seed_fraction: float = 0.25
    # pair distance: per DP group the null (pd_build_cdf's mid-CDF in 2^20 fixed point, None: none) and
    # its orientation ("FR", "RF" or "" for any); the span and seed z as the pileup constructor derives them
    predict_pair_distance: bool = False
    pd_cdf: tuple = ()
    pd_orientation: tuple = ()
    pd_max_span: int = 0
    pd_z_seed: float = 2.5
    pair_distance_seed: int = 3
    pair_distance_tail_quantile: float = 0.05
    pd_mean_covering_gap: float = 0.0
    total_reference_length: int = 0


def pd_null_from_histogram(distance, count, trunc: int, max_distance: int):
    """bsq_pd_build_null: a read-file set's PD null (mid-CDF in 2^20 fixed point) and its mean covering
    gap from the rows of its paired-mapping distance histogram; (None, 0.0) when it has no usable weight."""
    d = np.ascontiguousarray(distance, dtype=np.int32)
    n = np.ascontiguousarray(count, dtype=np.float64)
    L = _lib.load()
    cap = int(max(d.max(initial=0), 0)) + 1
    out = np.zeros(cap, dtype=np.int64)
    ln, gap = C.c_uint32(), C.c_double()
    rc = L.bsq_pd_build_null(abi.ptr(d, C.c_int32), abi.ptr(n, C.c_double), len(d), trunc, max_distance,
                             abi.ptr(out, C.c_int64), cap, C.byref(ln), C.byref(gap))
    if rc != 0:
        raise RuntimeError(f"bsq_pd_build_null failed ({rc})")
    return (out[: ln.value].copy() if ln.value else None), gap.value


def pd_seed_z(pair_distance_seed_z: float, mean_covering_gap: float, total_reference_length: int) -> float:
    return _lib.load().bsq_pd_seed_z(float(pair_distance_seed_z), float(mean_covering_gap), int(total_reference_length))


def pair_params(sample, st: PairSettings, deletion_propagation_cutoff=None):
    """bsq_pair_params for a sample; returns (params, arrays they point into)."""
    T = len(sample.target_offset) - 1
    keep = dict(dpg=np.ascontiguousarray(st.dp_group, dtype=np.int32),
                w=np.ascontiguousarray(st.window_width, dtype=np.float64),
                r1=np.ascontiguousarray(st.r1_prefix, dtype=np.uint32),
                r2=np.ascontiguousarray(st.r2_prefix, dtype=np.uint32),
                cut=np.broadcast_to(np.asarray(5.0 if deletion_propagation_cutoff is None else deletion_propagation_cutoff,
                                               dtype=np.float64), (T,)).copy())
    G = len(keep["w"])
    cdfs = [np.ascontiguousarray(st.pd_cdf[g] if g < len(st.pd_cdf) and st.pd_cdf[g] is not None else [], dtype=np.int64)
            for g in range(G)]
    keep["cdfs"] = cdfs
    keep["cdf_ptrs"] = (C.POINTER(C.c_int64) * max(1, G))(*[abi.ptr(c, C.c_int64) for c in cdfs])
    keep["cdf_len"] = np.array([len(c) for c in cdfs] or [0], dtype=np.uint32)
    keep["orient"] = np.array([abi.XP_CODES.get(st.pd_orientation[g], abi.XP_NONE) if g < len(st.pd_orientation)
                               else abi.XP_NONE for g in range(G)] or [3], dtype=np.uint8)
    p = abi.PairParams(n_read_groups=len(keep["dpg"]), dp_group=abi.ptr(keep["dpg"], C.c_int32),
                       n_dp_groups=len(keep["w"]), window_width=abi.ptr(keep["w"], C.c_double),
                       r1_name_prefix=abi.ptr(keep["r1"], C.c_uint32), r2_name_prefix=abi.ptr(keep["r2"], C.c_uint32),
                       discordant_pair_seed=st.discordant_pair_seed, predict_missing_pairs=int(st.predict_missing_pairs),
                       missing_pair_seed=st.missing_pair_seed, missing_pair_seed_fraction=st.missing_pair_seed_fraction,
                       deletion_propagation_cutoff=abi.ptr(keep["cut"], C.c_double),
                       predict_pair_distance=int(st.predict_pair_distance), pd_cdf=keep["cdf_ptrs"],
                       pd_cdf_len=abi.ptr(keep["cdf_len"], C.c_uint32), pd_orientation=abi.ptr(keep["orient"], C.c_uint8),
                       pd_max_span=st.pd_max_span, pd_z_seed=st.pd_z_seed, pair_distance_seed=st.pair_distance_seed,
                       pair_distance_tail_quantile=st.pair_distance_tail_quantile,
                       pd_mean_covering_gap=st.pd_mean_covering_gap,
                       total_reference_length=int(st.total_reference_length or sample.target_offset[-1]))
    return p, keep


@dataclass
class ImSettings:
    """The Settings fields identify_mutations reads, with breseq's defaults."""
    polymorphism_prediction: bool = False
    base_quality_cutoff: int = 3
    mutation_log10_e_value_cutoff: float = 10.0
    polymorphism_log10_e_value_cutoff: float | None = None   # 2 (polymorphism mode) / 10 (consensus mode)
    polymorphism_precision_decimal: float = 1e-6
    polymorphism_precision_places: int | None = None          # 8 / 3
    skip_missing_coverage_prediction: bool = False
    # DP group of each dense read group (-1: none), as identify_mutations_pileup builds it from the
    # paired read-file sets with a paired-mapping-distance fit (identify_mutations.cpp:883-911); empty:
    # no DP group.  A non-proper paired read of a DP group without a usable XP tag is left out of
    # its first column (:1399-1416).
    dp_group: tuple = ()

    def resolved(self):
        poly = self.polymorphism_log10_e_value_cutoff
        if poly is None:
            poly = 2.0 if self.polymorphism_prediction else 10.0
        places = self.polymorphism_precision_places
        if places is None:
            places = 8 if self.polymorphism_prediction else 3
        return poly, places


def im_params(s, st: ImSettings, deletion_propagation_cutoff=None, deletion_seed_cutoff=None, precision=PRECISION_FP32C,
              n_read_files=None, n_quality=None):
    """bsq_im_params for sample `s`; returns (params, arrays the params point into)."""
    poly, places = st.resolved()
    T = len(s.target_offset) - 1
    keep = dict(
        prop=np.broadcast_to(np.asarray(5.0 if deletion_propagation_cutoff is None else deletion_propagation_cutoff,
                                        dtype=np.float64), (T,)).copy(),
        seed=np.broadcast_to(np.asarray(0.0 if deletion_seed_cutoff is None else deletion_seed_cutoff,
                                        dtype=np.float64), (T,)).copy(),
        dpg=np.ascontiguousarray(st.dp_group or [-1], dtype=np.int32))
    p = abi.ImParams(n_read_files=n_read_files or s.n_read_files, n_quality=n_quality or s.n_quality,
                     base_quality_cutoff=st.base_quality_cutoff,
                     mutation_cutoff=st.mutation_log10_e_value_cutoff, polymorphism_cutoff=poly,
                     polymorphism_precision_decimal=st.polymorphism_precision_decimal,
                     polymorphism_precision_places=places,
                     skip_missing_coverage_prediction=int(st.skip_missing_coverage_prediction),
                     log10_ref_length=float(np.log10(float(s.target_offset[-1]))),
                     deletion_propagation_cutoff=abi.ptr(keep["prop"], C.c_double),
                     deletion_seed_cutoff=abi.ptr(keep["seed"], C.c_double), precision=precision,
                     n_read_groups=len(st.dp_group), dp_group=abi.ptr(keep["dpg"], C.c_int32))
    return p, keep


class Scorer:
    """One library context on one GPU; samples stay resident until freed."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        self.ctx = C.c_void_p()
        rc = self.L.bsq_create(C.byref(self.ctx), device)
        if rc != 0:
            raise _lib.BsqError(rc, "bsq_create failed (no CUDA device?)")
        self._views = {}
        self._rg_count = {}    # sample id -> the @RG count of its BAM header (identify_mutations.cpp:862)

    def _check(self, rc):
        if rc != 0:
            raise _lib.BsqError(rc, self.L.bsq_last_error(self.ctx).decode())

    def close(self):
        if self.ctx:
            self.L.bsq_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ samples
    def load_sample(self, sample) -> int:
        view = abi.SampleView(sample)
        sid = C.c_int32()
        self._check(self.L.bsq_load_sample(self.ctx, C.byref(view.ref), C.byref(view.reads), C.byref(sid)))
        self._views[sid.value] = (sample, view)
        self._rg_count[sid.value] = header_read_groups(sample)
        return sid.value

    def free_sample(self, sid: int):
        self._check(self.L.bsq_free_sample(self.ctx, sid))
        self._views.pop(sid, None)
        self._rg_count.pop(sid, None)

    def sample(self, sid):
        return self._views[sid][0]

    # ------------------------------------------------------------------ pass 1
    def _ec_job(self, sid, n_read_files, n_quality, do_coverage, do_errors, preprocess,
                unmatched_end_minimum_read_length, unmatched_end_length_factor, hist_capacity):
        s = self.sample(sid)
        R = n_read_files or s.n_read_files
        Q = n_quality or s.n_quality
        G = s.n_coverage_groups
        res = dict(counts=np.zeros(R * 25 * Q, dtype=np.uint64), hist=np.zeros((G, hist_capacity), dtype=np.uint64),
                   hist_size=np.zeros(G, dtype=np.uint32),
                   no_pos_hash_pr=np.zeros(len(s.target_offset) - 1, dtype=np.float64))
        p = abi.EcParams(n_read_files=R, n_quality=Q, do_coverage=int(do_coverage), do_errors=int(do_errors),
                         preprocess_stage=int(preprocess),
                         unmatched_end_minimum_read_length=unmatched_end_minimum_read_length,
                         unmatched_end_length_factor=unmatched_end_length_factor)
        out = abi.EcResult(counts=abi.ptr(res["counts"], C.c_uint64), coverage_hist=abi.ptr(res["hist"], C.c_uint64),
                           hist_capacity=hist_capacity, hist_size=abi.ptr(res["hist_size"], C.c_uint32),
                           no_pos_hash_pr=abi.ptr(res["no_pos_hash_pr"], C.c_double))
        return p, out, res

    def error_count_batch(self, sids, n_read_files=None, n_quality=None, do_coverage=True, do_errors=True,
                          preprocess=False, unmatched_end_minimum_read_length=50, unmatched_end_length_factor=0.1,
                          hist_capacity=8192):
        """Pass 1 over several resident samples in one launch; one result dict per sample."""
        sids = list(sids)
        n = len(sids)
        jobs = [self._ec_job(sid, n_read_files, n_quality, do_coverage, do_errors, preprocess,
                             unmatched_end_minimum_read_length, unmatched_end_length_factor, hist_capacity)
                for sid in sids]
        ids = (C.c_int32 * n)(*sids)
        ps = (abi.EcParams * n)(*[j[0] for j in jobs])
        outs = (abi.EcResult * n)(*[j[1] for j in jobs])
        self._check(self.L.bsq_error_count_batch(self.ctx, n, ids, ps, outs))
        return [j[2] for j in jobs]

    def error_count(self, sid: int, **kw):
        return self.error_count_batch([sid], **kw)[0]

    def counts_to_log10_prob(self, counts, R, Q):
        out = np.zeros(R * 25 * Q, dtype=np.float64)
        c = np.ascontiguousarray(counts, dtype=np.uint64)
        self._check(self.L.bsq_counts_to_log10_prob(abi.ptr(c, C.c_uint64), R, Q, abi.ptr(out, C.c_double)))
        return out

    def counts_to_log10_prob_batch(self, counts_list, Rs, Qs):
        """Tables of several samples at once (host threads); per-sample R, Q lists."""
        n = len(counts_list)
        cs = [np.ascontiguousarray(c, dtype=np.uint64) for c in counts_list]
        outs = [np.zeros(int(R) * 25 * int(Q), dtype=np.float64) for R, Q in zip(Rs, Qs)]
        self._check(self.L.bsq_counts_to_log10_prob_batch(
            n, (C.POINTER(C.c_uint64) * n)(*[abi.ptr(c, C.c_uint64) for c in cs]), (C.c_uint32 * n)(*Rs),
            (C.c_uint32 * n)(*Qs), (C.POINTER(C.c_double) * n)(*[abi.ptr(o, C.c_double) for o in outs])))
        return outs

    # ------------------------------------------------------------------ pass 2
    def _im_job(self, sid, log10_table, st, deletion_propagation_cutoff, deletion_seed_cutoff, precision, positions,
                n_read_files, n_quality):
        s = self.sample(sid)
        p, keep = im_params(s, st, deletion_propagation_cutoff, deletion_seed_cutoff, precision, n_read_files, n_quality)
        keep["tab"] = np.ascontiguousarray(log10_table, dtype=np.float64)
        arrs = pa = None
        if positions:
            n = int(s.target_offset[-1])
            arrs = dict(unique_top=np.zeros(n, np.uint32), unique_bot=np.zeros(n, np.uint32),
                        redundant_top=np.zeros(n, np.float64), redundant_bot=np.zeros(n, np.float64),
                        raw_redundant_top=np.zeros(n, np.uint32), raw_redundant_bot=np.zeros(n, np.uint32),
                        consensus_score=np.zeros(n, np.float64), best_base=np.zeros(n, np.uint8),
                        n_scored=np.zeros(n, np.uint32))
            cm = dict(unique_top=C.c_uint32, unique_bot=C.c_uint32, redundant_top=C.c_double, redundant_bot=C.c_double,
                      raw_redundant_top=C.c_uint32, raw_redundant_bot=C.c_uint32, consensus_score=C.c_double,
                      best_base=C.c_uint8, n_scored=C.c_uint32)
            pa = abi.PositionArrays(**{k: abi.ptr(v, cm[k]) for k, v in arrs.items()})
        return p, pa, arrs, keep

    def identify_mutations_batch(self, sids, log10_tables, settings: ImSettings | None = None,
                                 deletion_propagation_cutoff=None, deletion_seed_cutoff=None,
                                 precision=PRECISION_FP32C, positions=False, n_read_files=None, n_quality=None,
                                 as_dicts=True):
        """Pass 2 over several resident samples in one launch per kernel.  `log10_tables`, `settings`
        and the deletion cutoffs are per sample (a list) or shared (one value).  With as_dicts=False
        the RA / MC / UN records come back as numpy structured arrays of the C structs."""
        sids = list(sids)
        n = len(sids)

        def per(x, j):
            return x[j] if isinstance(x, (list, tuple)) else x

        jobs = [self._im_job(sid, per(log10_tables, j), per(settings, j) or ImSettings(), per(deletion_propagation_cutoff, j),
                             per(deletion_seed_cutoff, j), precision, positions, n_read_files, n_quality)
                for j, sid in enumerate(sids)]
        ids = (C.c_int32 * n)(*sids)
        ps = (abi.ImParams * n)(*[j[0] for j in jobs])
        tabs = (C.POINTER(C.c_double) * n)(*[abi.ptr(j[3]["tab"], C.c_double) for j in jobs])
        pas = None
        if positions:
            pas = (C.POINTER(abi.PositionArrays) * n)(*[C.pointer(j[1]) for j in jobs])
        self._check(self.L.bsq_identify_mutations_batch(self.ctx, n, ids, ps, tabs, pas))
        outs = []
        for j in range(n):
            n_ra, n_mc, n_un = C.c_uint64(), C.c_uint64(), C.c_uint64()
            self._check(self.L.bsq_im_batch_result_counts(self.ctx, j, C.byref(n_ra), C.byref(n_mc), C.byref(n_un)))
            ra = (abi.RaRecord * max(1, n_ra.value))()
            mc = (abi.McRecord * max(1, n_mc.value))()
            un = (abi.UnRecord * max(1, n_un.value))()
            self._check(self.L.bsq_im_batch_result_copy(self.ctx, j, C.cast(ra, C.c_void_p), n_ra.value,
                                                        C.cast(mc, C.c_void_p), n_mc.value, C.cast(un, C.c_void_p),
                                                        n_un.value))
            if as_dicts:
                out = dict(ra=abi.ra_to_dicts(ra[:n_ra.value]), mc=abi.mc_to_dicts(mc[:n_mc.value]),
                           un=abi.un_to_dicts(un[:n_un.value]))
            else:   # the C records as numpy structured arrays (no per-item Python objects)
                out = dict(ra=np.ctypeslib.as_array(ra)[:n_ra.value], mc=np.ctypeslib.as_array(mc)[:n_mc.value],
                           un=np.ctypeslib.as_array(un)[:n_un.value])
            if jobs[j][2] is not None:
                out["positions"] = jobs[j][2]
            outs.append(out)
        return outs

    def identify_mutations(self, sid: int, log10_table, settings: ImSettings | None = None, **kw):
        return self.identify_mutations_batch([sid], [log10_table], [settings], **kw)[0]

    # ------------------------------------------------------------------ soft clipping
    def soft_clipping(self, sid: int, settings: ScSettings | None = None) -> dict:
        """tabulate_soft_clipping_counts over a resident sample: the summary (Summary::soft_clipping)
        and the rows of soft_clipping_counts.tab as a structured array."""
        p, keep = sc_params(self.sample(sid), settings or ScSettings())
        s = abi.ScSummary()
        self._check(self.L.bsq_soft_clipping(self.ctx, sid, C.byref(p), C.byref(s)))
        rows = (abi.ScPosition * max(1, s.n_positions))()
        self._check(self.L.bsq_sc_result_copy(self.ctx, rows, s.n_positions))
        return dict(summary=abi.sc_summary_dict(s), rows=abi.sc_rows_array(rows, s.n_positions))

    # ------------------------------------------------------------------ BAM input
    def pair_candidates(self, sid: int, settings: PairSettings | None = None, deletion_propagation_cutoff=None) -> dict:
        """Discordant-pair and missing-pair candidate regions (bsq_pair_candidates): the regions as
        structured arrays in detection order and the descriptor text they index."""
        s = self.sample(sid)
        p, keep = pair_params(s, settings or PairSettings(), deletion_propagation_cutoff)
        nd, nm, nt = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.L.bsq_pair_candidates(self.ctx, sid, C.byref(p), C.byref(nd), C.byref(nm), C.byref(nt)))
        dp = (abi.PairRegion * max(1, nd.value))()
        mp = (abi.PairRegion * max(1, nm.value))()
        text = C.create_string_buffer(max(1, nt.value))
        self._check(self.L.bsq_pair_result_copy(self.ctx, dp, nd.value, mp, nm.value, text, nt.value))
        npd = C.c_uint64()
        summ = abi.PdSummary()
        self._check(self.L.bsq_pd_result(self.ctx, C.byref(npd), None, 0, C.byref(summ)))
        pd = (abi.PdRegion * max(1, npd.value))()
        self._check(self.L.bsq_pd_result(self.ctx, C.byref(npd), pd, npd.value, None))
        return dict(dp=list(dp)[: nd.value], mp=list(mp)[: nm.value], text=text.raw[: nt.value],
                    pd=list(pd)[: npd.value], pd_summary=summ)

    def write_pair_candidates(self, result: dict, dp_path: str | None, mp_path: str | None, target_names,
                              pd_path: str | None = None):
        """dp / mp / pd_candidate_regions.csv from a pair_candidates() result."""
        names = (C.c_char_p * len(target_names))(*[n.encode() for n in target_names])
        text = C.create_string_buffer(result["text"], max(1, len(result["text"])))
        for path, key, fn in ((dp_path, "dp", self.L.bsq_write_dp_candidate_regions),
                              (mp_path, "mp", self.L.bsq_write_mp_candidate_regions)):
            if path is None:
                continue
            regs = (abi.PairRegion * max(1, len(result[key])))(*result[key])
            rc = fn(path.encode(), names, regs, len(result[key]), text)
            if rc != 0:
                raise _lib.BsqError(rc, f"cannot write {path}")
        if pd_path is not None:
            regs = (abi.PdRegion * max(1, len(result["pd"])))(*result["pd"])
            rc = self.L.bsq_write_pd_candidate_regions(pd_path.encode(), names, regs, len(result["pd"]),
                                                       C.byref(result["pd_summary"]))
            if rc != 0:
                raise _lib.BsqError(rc, f"cannot write {pd_path}")

    def open_bam(self, data) -> "Bam":
        """Uploads a BAM file's bytes (bytes, or a uint8 numpy array, e.g. page-locked) and inflates
        every BGZF block on the device."""
        h = C.c_void_p()
        if isinstance(data, np.ndarray):
            addr, size = data.ctypes.data, data.nbytes
        else:
            addr, size = C.cast(C.c_char_p(data), C.c_void_p).value, len(data)
        self._check(self.L.bsq_bam_open(self.ctx, addr, size, C.byref(h)))
        return Bam(self, h)

    def load_bam(self, data: bytes, reference_sample, groups=None) -> int:
        """BAM bytes -> resident sample: inflate, decode and pack on the device.  reference_sample
        supplies the reference (any object with the bsq_reference arrays, e.g. a synth.Sample)."""
        with self.open_bam(data) as bam:
            bam.decode(groups)
            return bam.load(reference_sample)

    # ------------------------------------------------------------------ BAM2COV coverage table
    def coverage_columns(self, sid: int, tid: int, start: int, end: int, read_group: int = -1) -> dict:
        """Per-position coverage of positions start..end (1-based) of target tid as `breseq BAM2COV`
        tabulates it (of one read group's records when read_group >= 0), and the pileup's last column
        ("last")."""
        arrs, st = abi.cov_columns(end - start + 1)
        last = C.c_uint32()
        self._check(self.L.bsq_coverage_columns_rg(self.ctx, sid, tid, start, end, read_group, C.byref(st),
                                                   C.byref(last)))
        arrs["last"] = last.value
        return arrs

    def im_coverage_columns(self, sid: int, tid: int, start: int, end: int, read_group: int = -1,
                            coverage_fit_failed: bool = False, dp_group=()) -> dict:
        """identify_mutations' coverage tally at positions start..end (1-based) of target tid, of one read
        group's records when read_group >= 0: deletions count and N read bases do not, or, for a target
        whose coverage fit failed, neither counts.  dp_group: per read group its discordant-pair group or
        -1 (ImSettings.dp_group); pass 2's first-column skip applies to the tally too."""
        arrs, st = abi.cov_columns(end - start + 1)
        dp = np.ascontiguousarray(dp_group, dtype=np.int32)
        self._check(self.L.bsq_im_coverage_columns_rg(self.ctx, sid, tid, start, end, read_group,
                                                      1 if coverage_fit_failed else 0, len(dp),
                                                      abi.ptr(dp, C.c_int32) if len(dp) else None, C.byref(st)))
        return arrs

    def write_coverage_table(self, sid: int, path: str, tid: int, positions: dict, n_read_groups: int | None = None,
                             coverage_fit_failed: bool = False, dp_group=()):
        """<seq_id>.coverage.tsv of identify_mutations into path: the aggregate columns from `positions`
        (identify_mutations(..., positions=True)["positions"]) and, with more than one read group, each
        group's columns tallied on the device.  n_read_groups: the BAM header's @RG count (default: the
        groups the sample's BAM declares).  dp_group: as for im_coverage_columns."""
        s = self.sample(sid)
        if n_read_groups is None:
            n_read_groups = self._rg_count.get(sid, 1)
        dp = np.zeros(n_read_groups, np.int32) - 1
        dp[:min(len(dp_group), n_read_groups)] = np.asarray(dp_group, dtype=np.int32)[:n_read_groups]
        view = self._views[sid][1]
        pa, keep = abi.position_arrays_view(positions)
        self._check(self.L.bsq_write_coverage_table_rg(self.ctx, sid, path.encode(), s.target_names[tid].encode(),
                                                       C.byref(view.ref), tid, C.byref(pa), n_read_groups,
                                                       1 if coverage_fit_failed else 0, abi.ptr(dp, C.c_int32)))
        del keep

    def write_coverage_region(self, sid: int, path: str, tid: int, start: int, end: int, resolution: int = 600,
                              total_only: bool = False, csv: bool = False, reference_average=None,
                              per_read_group: bool = False, n_read_groups: int | None = None):
        """`breseq BAM2COV --format TSV|CSV -r seq:start-end --resolution N [--per-read-group]` into path;
        n_read_groups: the BAM header's @RG count (default: the one the sample was loaded with)."""
        s = self.sample(sid)
        flags = (1 if total_only else 0) | (2 if csv else 0) | (4 if per_read_group else 0)
        avg = C.byref(C.c_double(reference_average)) if reference_average is not None else None
        if n_read_groups is None:
            n_read_groups = self._rg_count.get(sid, 1)
        self._check(self.L.bsq_write_coverage_region_rg(self.ctx, sid, path.encode(), s.target_names[tid].encode(), tid,
                                                        start, end, resolution, flags, avg, n_read_groups))

    # ------------------------------------------------------------------ launch shapes
    def tuning(self) -> dict:
        t = abi.Tuning()
        self._check(self.L.bsq_get_tuning(self.ctx, C.byref(t)))
        return {k: getattr(t, k) for k, _ in abi.Tuning._fields_}

    def set_tuning(self, **kw):
        t = abi.Tuning(**{**self.tuning(), **kw})
        self._check(self.L.bsq_set_tuning(self.ctx, C.byref(t)))

    def autotune(self, sids, log10_tables, settings=None, precision=PRECISION_FP32C) -> dict:
        """Pick the fastest launch shapes for these resident samples (results are unaffected)."""
        sids = list(sids)
        n = len(sids)

        def per(x, j):
            return x[j] if isinstance(x, (list, tuple)) else x

        ec = [self._ec_job(sid, None, None, True, True, False, 50, 0.1, 8)[0] for sid in sids]
        im = [self._im_job(sid, per(log10_tables, j), per(settings, j) or ImSettings(), None, None, precision, False,
                           None, None) for j, sid in enumerate(sids)]
        ids = (C.c_int32 * n)(*sids)
        eps = (abi.EcParams * n)(*ec)
        ips = (abi.ImParams * n)(*[j[0] for j in im])
        tabs = (C.POINTER(C.c_double) * n)(*[abi.ptr(j[3]["tab"], C.c_double) for j in im])
        t = abi.Tuning()
        self._check(self.L.bsq_autotune(self.ctx, n, ids, eps, ips, tabs, C.byref(t)))
        return {k: getattr(t, k) for k, _ in abi.Tuning._fields_}

    def timer_start(self):
        self._check(self.L.bsq_timer_start(self.ctx))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self.L.bsq_timer_stop(self.ctx, C.byref(ms)))
        return ms.value

    def last_pass_bytes(self):
        h, d = C.c_uint64(), C.c_uint64()
        self._check(self.L.bsq_last_pass_bytes(self.ctx, C.byref(h), C.byref(d)))
        return dict(h2d=h.value, d2h=d.value)

    def last_pass_stats(self):
        ms, launches, main = C.c_double(), C.c_uint32(), C.c_double()
        self._check(self.L.bsq_last_pass_stats(self.ctx, C.byref(ms), C.byref(launches), C.byref(main)))
        return dict(device_ms=ms.value, kernel_launches=launches.value, main_kernel_ms=main.value)


def error_count(sample, device=0, **kw):
    """breseq::error_count for one decoded sample: covariate counts + unique-only coverage histograms."""
    with Scorer(device) as sc:
        sid = sc.load_sample(sample)
        return sc.error_count(sid, **kw)


def identify_mutations(sample, log10_table, device=0, **kw):
    """breseq::identify_mutations for one decoded sample: RA / MC / UN evidence with raw values."""
    with Scorer(device) as sc:
        sid = sc.load_sample(sample)
        return sc.identify_mutations(sid, log10_table, **kw)


def fit_coverage_distribution(hist, sequence_length: int | None = None, deletion_propagation_pr_cutoff=None,
                              n_threads: int = 0) -> dict:
    """CoverageDistribution::fit + analyze_unique_coverage_distribution (src/breseq/coverage_distribution.cpp:
    437-505, 519-588) on one coverage group's unique-only histogram, as error_count returns it
    (hist[0 .. hist_size-1]).  The cutoff probability is breseq's 0.05 / sqrt(group length) unless given.
    Host code; needs no GPU."""
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    if deletion_propagation_pr_cutoff is None:
        if not sequence_length:
            raise ValueError("give sequence_length or deletion_propagation_pr_cutoff")
        deletion_propagation_pr_cutoff = 0.05 / np.sqrt(float(sequence_length))
    out = abi.CoverageFit()
    rc = _lib.load().bsq_fit_coverage_distribution(abi.ptr(h, C.c_uint64), h.size, float(deletion_propagation_pr_cutoff),
                                                  int(n_threads), C.byref(out))
    if rc != 0:
        raise RuntimeError(f"bsq_fit_coverage_distribution failed ({rc})")
    return abi.coverage_fit_dict(out)


class Server:
    """Continuous-batching scoring server (bsq_server_*): jobs are admitted by HBM footprint,
    uploaded while earlier jobs run, and every GPU round runs both passes over all resident jobs as
    one batch per pass.  A job is one sample through error_count, the error-table round trip and
    identify_mutations."""

    def __init__(self, device: int = 0, hbm_budget: float = 150e9, max_batch_jobs: int = 64,
                 precision: int = PRECISION_FP32C):
        self.L = _lib.load()
        self.srv = C.c_void_p()
        rc = self.L.bsq_server_create(C.byref(self.srv), device, int(hbm_budget), max_batch_jobs, precision)
        if rc != 0:
            raise _lib.BsqError(rc, "bsq_server_create failed")
        self._jobs = {}

    def submit(self, sample, settings: ImSettings | None = None, deletion_propagation_cutoff=None,
               deletion_seed_cutoff=None, hist_capacity=8192, n_read_files=None, n_quality=None,
               view=None) -> int:
        """Queue one job; `sample` (or the prepared abi.SampleView `view`) stays referenced until
        the job is released."""
        view = view or abi.SampleView(sample)
        R = n_read_files or sample.n_read_files
        Q = n_quality or sample.n_quality
        ec = abi.EcParams(n_read_files=R, n_quality=Q, do_coverage=1, do_errors=1, preprocess_stage=0,
                          unmatched_end_minimum_read_length=50, unmatched_end_length_factor=0.1)
        im, keep = im_params(sample, settings or ImSettings(), deletion_propagation_cutoff, deletion_seed_cutoff,
                             PRECISION_FP32C, R, Q)
        job = abi.Job(ref=C.pointer(view.ref), reads=C.pointer(view.reads), ec=ec, im=im, hist_capacity=hist_capacity)
        jid = C.c_uint64()
        rc = self.L.bsq_server_submit(self.srv, C.byref(job), C.byref(jid))
        if rc != 0:
            raise _lib.BsqError(rc, self.L.bsq_server_last_error(self.srv).decode())
        self._jobs[jid.value] = (sample, view, keep, job, R, Q, hist_capacity)
        return jid.value

    @staticmethod
    def _info(i: abi.JobInfo) -> dict:
        return {k: getattr(i, k) for k, _ in abi.JobInfo._fields_}

    def wait(self, jid: int, timeout_ms: int = -1) -> dict:
        info = abi.JobInfo()
        rc = self.L.bsq_server_wait(self.srv, jid, timeout_ms, C.byref(info))
        if rc != 0:
            raise _lib.BsqError(rc, "wait failed")
        d = self._info(info)
        if d["state"] < 0:
            raise _lib.BsqError(d["state"], self.L.bsq_server_job_error(self.srv, jid).decode())
        return d

    def result(self, jid: int) -> dict:
        """Pass-1 and pass-2 results of a finished job (waits for it)."""
        info = self.wait(jid)
        sample, _, _, _, R, Q, cap = self._jobs[jid]
        G = sample.n_coverage_groups
        counts = np.zeros(R * 25 * Q, dtype=np.uint64)
        hist = np.zeros((G, cap), dtype=np.uint64)
        hsize = np.zeros(G, dtype=np.uint32)
        rc = self.L.bsq_server_error_counts(self.srv, jid, abi.ptr(counts, C.c_uint64), abi.ptr(hist, C.c_uint64),
                                            abi.ptr(hsize, C.c_uint32))
        if rc != 0:
            raise _lib.BsqError(rc, "error counts unavailable")
        ra = (abi.RaRecord * max(1, info["n_ra"]))()
        mc = (abi.McRecord * max(1, info["n_mc"]))()
        un = (abi.UnRecord * max(1, info["n_un"]))()
        rc = self.L.bsq_server_results(self.srv, jid, C.cast(ra, C.c_void_p), info["n_ra"], C.cast(mc, C.c_void_p),
                                       info["n_mc"], C.cast(un, C.c_void_p), info["n_un"])
        if rc != 0:
            raise _lib.BsqError(rc, "results unavailable")
        return dict(counts=counts, hist=hist, hist_size=hsize, ra=abi.ra_to_dicts(ra[:info["n_ra"]]),
                    mc=abi.mc_to_dicts(mc[:info["n_mc"]]), un=abi.un_to_dicts(un[:info["n_un"]]), info=info)

    def release(self, jid: int):
        self.L.bsq_server_release(self.srv, jid)
        self._jobs.pop(jid, None)

    def set_tuning(self, **kw):
        """Launch shapes for the server's passes (keys of abi.Tuning); applied before the next round."""
        t = abi.Tuning(**kw)
        rc = self.L.bsq_server_set_tuning(self.srv, C.byref(t))
        if rc != 0:
            raise _lib.BsqError(rc, "bsq_server_set_tuning failed")

    def stats(self) -> dict:
        st = abi.ServerStats()
        self.L.bsq_server_get_stats(self.srv, C.byref(st))
        out = {k: getattr(st, k) for k, _ in abi.ServerStats._fields_}
        out["phase_ms"] = dict(zip(("pass1", "tables", "pass2", "results", "free"), list(st.phase_ms)))
        return out

    def close(self):
        if self.srv:
            self.L.bsq_server_destroy(self.srv)
            self.srv = C.c_void_p()
            self._jobs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Bam:
    """An uploaded, inflated BAM file (bsq_bam_open); decode() and load() make it a sample."""

    def __init__(self, scorer: Scorer, handle):
        self.sc, self.h = scorer, handle
        self.counts = None

    def header(self) -> dict:
        text, tl, n = C.c_char_p(), C.c_uint64(), C.c_uint32()
        names, lens = C.POINTER(C.c_char_p)(), C.POINTER(C.c_uint32)()
        self.sc._check(self.sc.L.bsq_bam_header(self.h, C.byref(text), C.byref(tl), C.byref(n), C.byref(names),
                                                C.byref(lens)))
        return dict(text=C.string_at(text, tl.value).decode(), names=[names[i].decode() for i in range(n.value)],
                    lengths=[lens[i] for i in range(n.value)])

    def decode(self, groups=None):
        """groups: (ids, file_base, file_count) as breseq resolves read groups, or None."""
        g, keep = None, []
        if groups is not None:
            ids, base, count = groups
            arr_ids = (C.c_char_p * len(ids))(*[x.encode() for x in ids])
            b = np.ascontiguousarray(base, dtype=np.uint32)
            c = np.ascontiguousarray(count, dtype=np.uint32)
            keep = [arr_ids, b, c]
            g = abi.BamGroups(n_groups=len(ids), ids=arr_ids, file_base=abi.ptr(b, C.c_uint32),
                              file_count=abi.ptr(c, C.c_uint32))
        n, nc, nb = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.sc._check(self.sc.L.bsq_bam_decode(self.sc.ctx, self.h, C.byref(g) if g is not None else None,
                                                C.byref(n), C.byref(nc), C.byref(nb)))
        self.counts = (n.value, nc.value, nb.value)
        return self.counts

    def records(self) -> dict:
        """The decoded records as numpy arrays in the bsq_read_soa layout."""
        nb = C.c_uint64()
        self.sc._check(self.sc.L.bsq_bam_name_bytes(self.sc.ctx, self.h, C.byref(nb)))
        arrs, st = abi.read_arrays(*self.counts, nb.value)
        self.sc._check(self.sc.L.bsq_bam_copy_records(self.sc.ctx, self.h, C.byref(st)))
        arrs["qname"] = arrs["qname"][: nb.value]
        return arrs

    def load(self, reference_sample) -> int:
        view = abi.SampleView(reference_sample)
        sid = C.c_int32()
        n_rg = sum(1 for line in self.header()["text"].splitlines() if line.startswith("@RG"))
        self.sc._check(self.sc.L.bsq_bam_load(self.sc.ctx, self.h, C.byref(view.ref), C.byref(sid)))
        self.sc._views[sid.value] = (reference_sample, view)
        self.sc._rg_count[sid.value] = n_rg
        return sid.value

    def close(self):
        if self.h:
            self.sc.L.bsq_bam_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
