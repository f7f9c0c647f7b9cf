"""ctypes mirror of include/breseq_gb300.h (structs only; the function bindings live in _lib.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

P = C.POINTER


class Reference(C.Structure):
    _fields_ = [
        ("n_targets", C.c_uint32),
        ("target_offset", P(C.c_uint64)),
        ("seq", C.c_char_p),
        ("coverage_group", P(C.c_uint32)),
        ("n_coverage_groups", C.c_uint32),
        ("target_order", P(C.c_uint32)),
        ("n_target_order", C.c_uint32),
    ]


class ReadSoA(C.Structure):
    _fields_ = [
        ("n_reads", C.c_uint64),
        ("tid", P(C.c_int32)),
        ("pos", P(C.c_int32)),
        ("flag", P(C.c_uint16)),
        ("mapq", P(C.c_uint8)),
        ("x1", P(C.c_uint32)),
        ("xl", P(C.c_int32)),
        ("xr", P(C.c_int32)),
        ("read_file", P(C.c_uint8)),
        ("read_group", P(C.c_uint16)),
        ("l_qseq", P(C.c_uint32)),
        ("seq_off", P(C.c_uint64)),
        ("cigar_off", P(C.c_uint64)),
        ("n_cigar", P(C.c_uint16)),
        ("cigar", P(C.c_uint32)),
        ("seq", P(C.c_uint8)),
        ("qual", P(C.c_uint8)),
        ("n_cigar_total", C.c_uint64),
        ("n_bases_total", C.c_uint64),
        ("xj", P(C.c_uint8)),
        ("isize", P(C.c_int32)),
        ("xp", P(C.c_uint8)),
        ("qname_off", P(C.c_uint64)),
        ("qname", C.c_void_p),
        ("mtid", P(C.c_int32)),
        ("mpos", P(C.c_int32)),
    ]


XP_CODES = {"FR": 0, "RF": 1, "FF": 2}
XP_NONE = 3


class PairParams(C.Structure):
    _fields_ = [
        ("n_read_groups", C.c_uint32),
        ("dp_group", P(C.c_int32)),
        ("n_dp_groups", C.c_uint32),
        ("window_width", P(C.c_double)),
        ("r1_name_prefix", P(C.c_uint32)),
        ("r2_name_prefix", P(C.c_uint32)),
        ("discordant_pair_seed", C.c_int32),
        ("predict_missing_pairs", C.c_int32),
        ("missing_pair_seed", C.c_int32),
        ("missing_pair_seed_fraction", C.c_double),
        ("deletion_propagation_cutoff", P(C.c_double)),
        ("predict_pair_distance", C.c_int32),
        ("pd_cdf", P(P(C.c_int64))),
        ("pd_cdf_len", P(C.c_uint32)),
        ("pd_orientation", P(C.c_uint8)),
        ("pd_max_span", C.c_int32),
        ("pd_z_seed", C.c_double),
        ("pair_distance_seed", C.c_int32),
        ("pair_distance_tail_quantile", C.c_double),
        ("pd_mean_covering_gap", C.c_double),
        ("total_reference_length", C.c_uint64),
    ]


class PdRegion(C.Structure):
    _fields_ = [
        ("target", C.c_uint32),
        ("start", C.c_uint32),
        ("end", C.c_uint32),
        ("direction", C.c_char),
        ("reserved", C.c_char * 3),
        ("peak_position", C.c_uint32),
        ("peak_covering", C.c_int32),
        ("peak_tail", C.c_int32),
        ("reserved2", C.c_uint32),
        ("peak_z", C.c_double),
    ]


class PdSummary(C.Structure):
    _fields_ = [
        ("mean_covering_gap", C.c_double),
        ("n_effective_tests", C.c_double),
        ("seed_z_used", C.c_double),
        ("z_iqr_inflation", C.c_double),
        ("region_tail_fit_ok", C.c_int32),
        ("reserved", C.c_int32),
        ("region_tail_log_intercept", C.c_double),
        ("region_tail_sigma", C.c_double),
        ("region_tail_fit_lo", C.c_double),
        ("region_tail_fit_hi", C.c_double),
        ("ladder", C.c_uint64 * 21),
        ("regions_seeded", C.c_uint64),
    ]


class PairRegion(C.Structure):
    _fields_ = [
        ("target", C.c_uint32),
        ("start", C.c_uint32),
        ("end", C.c_uint32),
        ("strand", C.c_char),
        ("orientation", C.c_char * 3),
        ("max_count", C.c_uint32),
        ("max_total", C.c_uint32),
        ("redundant", C.c_uint32),
        ("reserved", C.c_uint32),
        ("text_off", C.c_uint64),
        ("text_len", C.c_uint64),
    ]


class ScParams(C.Structure):
    _fields_ = [
        ("minimum_clipped_bases", C.c_uint32),
        ("consensus_base_fraction", C.c_double),
        ("dispersion_trim_frequency", C.c_double),
        ("maximum_dispersion", C.c_double),
        ("minimum_rate", C.c_double),
        ("target_name_order", P(C.c_uint32)),
    ]


class ScSummary(C.Structure):
    _fields_ = [
        ("total_spanning_read_bases", C.c_uint64),
        ("total_clipped_read_ends", C.c_uint64),
        ("total_agreeing_clipped_read_ends", C.c_uint64),
        ("soft_clipping_rate", C.c_double),
        ("null_rate", C.c_double),
        ("null_rate_raw", C.c_double),
        ("dispersion", C.c_double),
        ("dispersion_raw", C.c_double),
        ("pearson_phi", C.c_double),
        ("tested_positions", C.c_uint64),
        ("trimmed_positions", C.c_uint64),
        ("mean_tested_reads", C.c_double),
        ("n_positions", C.c_uint64),
    ]


class ScPosition(C.Structure):
    _fields_ = [
        ("target", C.c_uint32),
        ("position", C.c_uint32),
        ("direction", C.c_int32),
        ("clipped_count", C.c_uint32),
        ("total_count", C.c_uint32),
        ("agree_count", C.c_uint32),
        ("clipped_sequence", C.c_char * 24),
    ]


class EcParams(C.Structure):
    _fields_ = [
        ("n_read_files", C.c_uint32),
        ("n_quality", C.c_uint32),
        ("do_coverage", C.c_int32),
        ("do_errors", C.c_int32),
        ("preprocess_stage", C.c_int32),
        ("unmatched_end_minimum_read_length", C.c_uint32),
        ("unmatched_end_length_factor", C.c_double),
    ]


class EcResult(C.Structure):
    _fields_ = [
        ("counts", P(C.c_uint64)),
        ("coverage_hist", P(C.c_uint64)),
        ("hist_capacity", C.c_uint32),
        ("hist_size", P(C.c_uint32)),
        ("no_pos_hash_pr", P(C.c_double)),
    ]


class ImParams(C.Structure):
    _fields_ = [
        ("n_read_files", C.c_uint32),
        ("n_quality", C.c_uint32),
        ("base_quality_cutoff", C.c_uint32),
        ("mutation_cutoff", C.c_double),
        ("polymorphism_cutoff", C.c_double),
        ("polymorphism_precision_decimal", C.c_double),
        ("polymorphism_precision_places", C.c_uint32),
        ("skip_missing_coverage_prediction", C.c_int32),
        ("log10_ref_length", C.c_double),
        ("deletion_propagation_cutoff", P(C.c_double)),
        ("deletion_seed_cutoff", P(C.c_double)),
        ("precision", C.c_int32),
        ("n_read_groups", C.c_uint32),
        ("dp_group", P(C.c_int32)),
    ]


class RaRecord(C.Structure):
    _fields_ = [
        ("tid", C.c_uint32), ("position", C.c_uint32), ("insert_position", C.c_uint32),
        ("ref_base", C.c_char), ("new_base", C.c_char), ("major_base", C.c_char), ("minor_base", C.c_char),
        ("score", C.c_double), ("consensus_score", C.c_double), ("f", C.c_double * 5),
        ("major_frequency", C.c_double), ("frequency", C.c_double),
        ("frequency_lower", C.c_double), ("frequency_upper", C.c_double),
        ("fisher_strand_p", C.c_double), ("ks_quality_p", C.c_double),
        ("ref_cov", C.c_int32 * 2), ("new_cov", C.c_int32 * 2), ("major_cov", C.c_int32 * 2),
        ("minor_cov", C.c_int32 * 2), ("total_cov", C.c_int32 * 2),
        ("n", C.c_uint32), ("passed_consensus", C.c_uint8), ("passed_polymorphism", C.c_uint8),
        ("pad", C.c_uint8 * 2),
    ]


class RaRaw(C.Structure):
    _fields_ = [
        ("column", C.c_uint32), ("insert_position", C.c_uint32), ("score", C.c_double),
        ("consensus_score", C.c_double), ("f", C.c_double * 5), ("frequency_lower", C.c_double),
        ("frequency_upper", C.c_double), ("pos_info", (C.c_uint32 * 2) * 5), ("n", C.c_uint32),
        ("ref_idx", C.c_uint8), ("var_idx", C.c_uint8), ("major_idx", C.c_uint8), ("minor_idx", C.c_uint8),
        ("passed_consensus", C.c_uint8), ("passed_polymorphism", C.c_uint8), ("pad", C.c_uint8 * 2),
    ]


class RaSettings(C.Structure):
    _fields_ = [
        ("polymorphism_prediction", C.c_int32), ("polymorphism_precision_places", C.c_uint32),
        ("mutation_log10_e_value_cutoff", C.c_double), ("consensus_frequency_cutoff", C.c_double),
        ("consensus_minimum_variant_coverage", C.c_double), ("consensus_minimum_total_coverage", C.c_double),
        ("consensus_minimum_variant_coverage_each_strand", C.c_double),
        ("consensus_minimum_total_coverage_each_strand", C.c_double),
        ("consensus_reject_indel_homopolymer_length", C.c_uint32),
        ("consensus_reject_surrounding_homopolymer_length", C.c_uint32),
        ("polymorphism_log10_e_value_cutoff", C.c_double), ("polymorphism_frequency_cutoff", C.c_double),
        ("polymorphism_minimum_variant_coverage", C.c_double), ("polymorphism_minimum_total_coverage", C.c_double),
        ("polymorphism_minimum_variant_coverage_each_strand", C.c_double),
        ("polymorphism_minimum_total_coverage_each_strand", C.c_double),
        ("polymorphism_reject_indel_homopolymer_length", C.c_uint32),
        ("polymorphism_reject_surrounding_homopolymer_length", C.c_uint32),
        ("polymorphism_fisher_strand_p_value_cutoff", C.c_double),
        ("polymorphism_ks_quality_p_value_cutoff", C.c_double), ("polymorphism_no_indels", C.c_int32),
    ]


class RaCall(C.Structure):
    _fields_ = [("prediction", C.c_char * 16), ("reject", C.c_char * 96), ("consensus_reject", C.c_char * 96),
                ("polymorphism_reject", C.c_char * 96), ("deleted", C.c_uint8), ("pad", C.c_uint8 * 7)]


class McRecord(C.Structure):
    _fields_ = [
        ("tid", C.c_uint32), ("start", C.c_uint32), ("end", C.c_uint32), ("start_range", C.c_uint32),
        ("end_range", C.c_uint32), ("pad", C.c_uint32),
        ("left_outside_cov", C.c_double), ("left_inside_cov", C.c_double),
        ("right_inside_cov", C.c_double), ("right_outside_cov", C.c_double),
    ]


class UnRecord(C.Structure):
    _fields_ = [("tid", C.c_uint32), ("start", C.c_uint32), ("end", C.c_uint32)]


class PositionArrays(C.Structure):
    _fields_ = [
        ("unique_top", P(C.c_uint32)), ("unique_bot", P(C.c_uint32)),
        ("redundant_top", P(C.c_double)), ("redundant_bot", P(C.c_double)),
        ("raw_redundant_top", P(C.c_uint32)), ("raw_redundant_bot", P(C.c_uint32)),
        ("consensus_score", P(C.c_double)), ("best_base", P(C.c_uint8)), ("n_scored", P(C.c_uint32)),
    ]


def ptr(a: np.ndarray, ctype):
    assert a.flags["C_CONTIGUOUS"], "arrays handed to the library must be contiguous"
    return a.ctypes.data_as(P(ctype))


class Tuning(C.Structure):
    _fields_ = [("ec_read_chunk", C.c_uint32), ("ec_blocks_per_sm", C.c_uint32), ("col_blocks_per_sm", C.c_uint32),
                ("cand_warps_per_sm", C.c_uint32), ("bound_warps_per_sm", C.c_uint32), ("use_graphs", C.c_int32)]


class Job(C.Structure):
    _fields_ = [("ref", C.POINTER(Reference)), ("reads", C.POINTER(ReadSoA)), ("ec", EcParams), ("im", ImParams),
                ("hist_capacity", C.c_uint32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("round_jobs", C.c_uint32), ("footprint", C.c_uint64), ("n_ra", C.c_uint64),
                ("n_mc", C.c_uint64), ("n_un", C.c_uint64), ("read_bases", C.c_uint64), ("submit_ms", C.c_double),
                ("admit_ms", C.c_double), ("ready_ms", C.c_double), ("start_ms", C.c_double), ("done_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("jobs_done", C.c_uint64), ("rounds", C.c_uint64), ("budget", C.c_uint64), ("in_use", C.c_uint64),
                ("peak_in_use", C.c_uint64), ("max_round_jobs", C.c_uint32), ("max_resident_jobs", C.c_uint32),
                ("gpu_busy_ms", C.c_double), ("phase_ms", C.c_double * 5)]


class SampleView:
    """Builds the Reference / ReadSoA structs over a synth.Sample (or any object with the same
    array attributes) and keeps every array it points into alive."""

    def __init__(self, s):
        self._keep = []

        def k(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a

        toff = k(s.target_offset, np.uint64)
        seq = k(s.ref_seq, np.uint8)
        cg = k(s.coverage_group, np.uint32)
        order = k(s.target_order, np.uint32)
        self.ref = Reference(
            n_targets=len(toff) - 1, target_offset=ptr(toff, C.c_uint64),
            seq=C.cast(seq.ctypes.data, C.c_char_p), coverage_group=ptr(cg, C.c_uint32),
            n_coverage_groups=int(s.n_coverage_groups), target_order=ptr(order, C.c_uint32),
            n_target_order=len(order))
        fields = dict(tid=(np.int32, C.c_int32), pos=(np.int32, C.c_int32), flag=(np.uint16, C.c_uint16),
                      mapq=(np.uint8, C.c_uint8), x1=(np.uint32, C.c_uint32), xl=(np.int32, C.c_int32),
                      xr=(np.int32, C.c_int32), read_file=(np.uint8, C.c_uint8),
                      read_group=(np.uint16, C.c_uint16), l_qseq=(np.uint32, C.c_uint32),
                      seq_off=(np.uint64, C.c_uint64), cigar_off=(np.uint64, C.c_uint64),
                      n_cigar=(np.uint16, C.c_uint16), cigar=(np.uint32, C.c_uint32),
                      seq=(np.uint8, C.c_uint8), qual=(np.uint8, C.c_uint8))
        kw = {}
        for name, (dt, ct) in fields.items():
            kw[name] = ptr(k(getattr(s, name), dt), ct)
        xj = getattr(s, "xj", None)
        if xj is not None:
            kw["xj"] = ptr(k(xj, np.uint8), C.c_uint8)
        if getattr(s, "xp", None) is not None:
            kw["isize"] = ptr(k(s.isize, np.int32), C.c_int32)
            kw["xp"] = ptr(k(s.xp, np.uint8), C.c_uint8)
            kw["qname_off"] = ptr(k(s.qname_off, np.uint64), C.c_uint64)
            kw["qname"] = k(np.frombuffer(bytes(s.qname), dtype=np.uint8) if not isinstance(s.qname, np.ndarray)
                            else s.qname, np.uint8).ctypes.data
        if getattr(s, "mtid", None) is not None:
            kw["mtid"] = ptr(k(s.mtid, np.int32), C.c_int32)
            kw["mpos"] = ptr(k(s.mpos, np.int32), C.c_int32)
        self.reads = ReadSoA(n_reads=int(len(s.tid)), n_cigar_total=int(len(s.cigar)),
                             n_bases_total=int(len(s.qual)), **kw)


def sc_summary_dict(s: ScSummary) -> dict:
    return {name: getattr(s, name) for name, _ in ScSummary._fields_}


class BamGroups(C.Structure):
    _fields_ = [
        ("n_groups", C.c_uint32),
        ("ids", P(C.c_char_p)),
        ("file_base", P(C.c_uint32)),
        ("file_count", P(C.c_uint32)),
    ]


READ_ARRAY_FIELDS = (("tid", np.int32), ("pos", np.int32), ("flag", np.uint16), ("mapq", np.uint8), ("x1", np.uint32),
                     ("xl", np.int32), ("xr", np.int32), ("read_file", np.uint8), ("read_group", np.uint16),
                     ("l_qseq", np.uint32), ("seq_off", np.uint64), ("cigar_off", np.uint64), ("n_cigar", np.uint16),
                     ("cigar", np.uint32), ("seq", np.uint8), ("qual", np.uint8), ("xj", np.uint8),
                     ("isize", np.int32), ("xp", np.uint8), ("qname_off", np.uint64), ("qname", np.uint8),
                     ("mtid", np.int32), ("mpos", np.int32))
_CT = {np.int32: C.c_int32, np.uint16: C.c_uint16, np.uint8: C.c_uint8, np.uint32: C.c_uint32, np.uint64: C.c_uint64}


class ReadArrays(C.Structure):
    _fields_ = [(name, P(_CT[dt])) for name, dt in READ_ARRAY_FIELDS]


def read_arrays(n: int, n_cigar: int, n_bases: int, n_name_bytes: int = 0):
    """Numpy arrays for decoded records and the bsq_read_arrays struct pointing at them."""
    size = {"cigar": n_cigar, "seq": n_bases // 2, "qual": n_bases, "qname_off": n + 1, "qname": n_name_bytes}
    arrs = {name: np.zeros(max(1, size.get(name, n)), dtype=dt) for name, dt in READ_ARRAY_FIELDS}
    st = ReadArrays(**{name: ptr(arrs[name], _CT[dt]) for name, dt in READ_ARRAY_FIELDS})
    return arrs, st


class CovColumns(C.Structure):
    _fields_ = [
        ("unique_top", P(C.c_uint32)),
        ("unique_bot", P(C.c_uint32)),
        ("redundant_top", P(C.c_double)),
        ("redundant_bot", P(C.c_double)),
        ("raw_redundant_top", P(C.c_uint32)),
        ("raw_redundant_bot", P(C.c_uint32)),
        ("unique_top_begin", P(C.c_uint32)),
        ("unique_bot_begin", P(C.c_uint32)),
    ]


POSITION_CTYPES = dict(unique_top=C.c_uint32, unique_bot=C.c_uint32, redundant_top=C.c_double,
                       redundant_bot=C.c_double, raw_redundant_top=C.c_uint32, raw_redundant_bot=C.c_uint32,
                       consensus_score=C.c_double, best_base=C.c_uint8, n_scored=C.c_uint32)


def position_arrays_view(arrs: dict):
    """A PositionArrays over a dict of per-position arrays (keys of POSITION_CTYPES; absent ones stay NULL)
    and the contiguous arrays it points into, which the caller keeps alive across the call."""
    keep = {}
    for k, t in POSITION_CTYPES.items():
        if k in arrs and arrs[k] is not None:
            keep[k] = np.ascontiguousarray(arrs[k], dtype=np.dtype(t))
    return PositionArrays(**{k: ptr(v, POSITION_CTYPES[k]) for k, v in keep.items()}), keep


def cov_columns(n: int):
    """Numpy arrays for one region of n positions and the bsq_cov_columns struct pointing at them."""
    arrs = {name: np.zeros(n, dtype=np.float64 if "redundant_" in name and "raw" not in name else np.uint32)
            for name, _ in CovColumns._fields_}
    st = CovColumns(**{k: ptr(v, C.c_double if v.dtype == np.float64 else C.c_uint32) for k, v in arrs.items()})
    return arrs, st


class CoverageFit(C.Structure):
    _fields_ = [
        ("nbinom_size", C.c_double),
        ("nbinom_mean", C.c_double),
        ("nbinom_prob", C.c_double),
        ("nbinom_variance", C.c_double),
        ("nbinom_relative_variance", C.c_double),
        ("average", C.c_double),
        ("variance", C.c_double),
        ("relative_variance", C.c_double),
        ("deletion_coverage_propagation_cutoff", C.c_double),
        ("nbinom_scale", C.c_double),
        ("censor_start", C.c_uint32),
        ("censor_end", C.c_uint32),
        ("restarts_converged", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


def coverage_fit_dict(f: CoverageFit) -> dict:
    return {name: getattr(f, name) for name, _ in CoverageFit._fields_ if name != "reserved"}


SC_ROW_DTYPE = np.dtype([("target", np.uint32), ("position", np.uint32), ("direction", np.int32),
                         ("clipped_count", np.uint32), ("total_count", np.uint32), ("agree_count", np.uint32),
                         ("clipped_sequence", "S24")])


def sc_rows_array(rows, n: int) -> np.ndarray:
    """The first n bsq_sc_position entries of a ctypes array as a numpy structured array."""
    assert SC_ROW_DTYPE.itemsize == C.sizeof(ScPosition)
    if n == 0:
        return np.zeros(0, dtype=SC_ROW_DTYPE)
    return np.frombuffer(bytes(memoryview(rows).cast("B")[:n * C.sizeof(ScPosition)]), dtype=SC_ROW_DTYPE).copy()


def ra_to_dicts(arr) -> list:
    out = []
    for r in arr:
        out.append(dict(
            tid=r.tid, position=r.position, insert_position=r.insert_position,
            ref_base=r.ref_base.decode(), new_base=r.new_base.decode(), major_base=r.major_base.decode(),
            minor_base=r.minor_base.decode(), score=r.score, consensus_score=r.consensus_score,
            f=list(r.f), major_frequency=r.major_frequency, frequency=r.frequency,
            frequency_lower=r.frequency_lower, frequency_upper=r.frequency_upper,
            fisher_strand_p=r.fisher_strand_p, ks_quality_p=r.ks_quality_p,
            ref_cov=tuple(r.ref_cov), new_cov=tuple(r.new_cov), major_cov=tuple(r.major_cov),
            minor_cov=tuple(r.minor_cov), total_cov=tuple(r.total_cov), n=r.n,
            passed_consensus=r.passed_consensus, passed_polymorphism=r.passed_polymorphism))
    return out


def ra_from_dicts(recs):
    arr = (RaRecord * max(1, len(recs)))()
    for i, d in enumerate(recs):
        r = arr[i]
        for k in ("tid", "position", "insert_position", "score", "consensus_score", "major_frequency", "frequency",
                  "frequency_lower", "frequency_upper", "fisher_strand_p", "ks_quality_p", "n",
                  "passed_consensus", "passed_polymorphism"):
            setattr(r, k, d[k])
        for k in ("ref_base", "new_base", "major_base", "minor_base"):
            setattr(r, k, d[k].encode())
        for b in range(5):
            r.f[b] = d["f"][b]
        for k in ("ref_cov", "new_cov", "major_cov", "minor_cov", "total_cov"):
            getattr(r, k)[0], getattr(r, k)[1] = d[k]
    return arr


def mc_from_dicts(recs):
    arr = (McRecord * max(1, len(recs)))()
    for i, d in enumerate(recs):
        for k, v in d.items():
            setattr(arr[i], k, v)
    return arr


def un_from_dicts(recs):
    arr = (UnRecord * max(1, len(recs)))()
    for i, d in enumerate(recs):
        for k, v in d.items():
            setattr(arr[i], k, v)
    return arr


def mc_to_dicts(arr) -> list:
    return [dict(tid=m.tid, start=m.start, end=m.end, start_range=m.start_range, end_range=m.end_range,
                 left_outside_cov=m.left_outside_cov, left_inside_cov=m.left_inside_cov,
                 right_inside_cov=m.right_inside_cov, right_outside_cov=m.right_outside_cov) for m in arr]


def un_to_dicts(arr) -> list:
    return [dict(tid=u.tid, start=u.start, end=u.end) for u in arr]
