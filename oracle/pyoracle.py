"""ctypes front end of the CPU oracle (test infrastructure only: tests/, the smoke test and the CPU
baseline leg of bench.py use it to check and time the CUDA path)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from breseq_gb300 import abi
from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.OUT
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        L.oracle_error_count.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.POINTER(abi.EcParams),
                                         C.POINTER(abi.EcResult), C.c_int, C.c_char_p, C.c_int]
        L.oracle_counts_to_log10_prob.argtypes = [C.POINTER(C.c_uint64), C.c_uint32, C.c_uint32, C.POINTER(C.c_double)]
        L.oracle_identify.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.POINTER(abi.ImParams),
                                      C.POINTER(C.c_double), C.POINTER(C.c_void_p), C.c_int, C.c_char_p, C.c_int]
        L.oracle_im_counts.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.oracle_im_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_im_positions.argtypes = [C.c_void_p, C.POINTER(abi.PositionArrays)]
        L.oracle_im_free.argtypes = [C.c_void_p]
        L.oracle_fisher_2x2.argtypes = [C.c_uint32] * 4
        L.oracle_fisher_2x2.restype = C.c_double
        L.oracle_ks_less.argtypes = [C.POINTER(C.c_double), C.c_uint32, C.POINTER(C.c_double), C.c_uint32]
        L.oracle_ks_less.restype = C.c_double
        L.oracle_soft_clipping.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.POINTER(C.c_char_p),
                                           C.POINTER(abi.ScParams), C.POINTER(C.c_void_p), C.c_char_p, C.c_int]
        L.oracle_sc_summary.argtypes = [C.c_void_p, C.POINTER(abi.ScSummary)]
        L.oracle_sc_rows.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_sc_free.argtypes = [C.c_void_p]
        L.oracle_pair_candidates.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.POINTER(abi.PairParams),
                                             C.POINTER(C.c_char_p), C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p,
                                             C.c_int]
        L.oracle_fit_coverage_distribution.argtypes = [C.POINTER(C.c_uint64), C.c_uint32, C.c_double,
                                                       C.POINTER(abi.CoverageFit)]
        for name, n in (("oracle_nbinom_pmf", 3), ("oracle_nbinom_cdf", 3), ("oracle_lgam", 1), ("oracle_lngamma", 1),
                        ("oracle_gamma", 1)):
            getattr(L, name).argtypes = [C.c_double] * n
            getattr(L, name).restype = C.c_double
        L.oracle_coverage_columns.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.c_uint32, C.c_uint32,
                                              C.c_uint32, C.POINTER(abi.CovColumns), C.POINTER(C.c_uint32), C.c_char_p,
                                              C.c_int]
        L.oracle_write_coverage_region.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.c_char_p,
                                                   C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                                   C.c_uint32, C.POINTER(C.c_double), C.c_char_p, C.c_int]
        L.oracle_write_coverage_region_rg.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.c_char_p,
                                                      C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                                      C.c_uint32, C.POINTER(C.c_double), C.c_uint32, C.c_char_p,
                                                      C.c_int]
        L.oracle_im_coverage_columns.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.c_uint32,
                                                 C.c_uint32, C.c_uint32, C.c_int32, C.c_int, C.c_uint32,
                                                 C.POINTER(C.c_int32), C.POINTER(abi.CovColumns), C.c_char_p, C.c_int]
        L.oracle_write_coverage_table_rg.argtypes = [C.POINTER(abi.Reference), C.POINTER(abi.ReadSoA), C.c_char_p,
                                                     C.c_uint32, C.POINTER(abi.PositionArrays), C.c_uint32, C.c_int,
                                                     C.POINTER(C.c_int32), C.c_char_p, C.c_int]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def error_count(sample, n_threads=os.cpu_count() or 1, do_coverage=True, do_errors=True, preprocess=False,
                hist_capacity=None, n_quality=None):
    view = abi.SampleView(sample)
    R, Q = sample.n_read_files, n_quality or sample.n_quality
    G = sample.n_coverage_groups
    cap = hist_capacity or 4096
    counts = np.zeros(R * 25 * Q, dtype=np.uint64)
    hist = np.zeros(G * cap, dtype=np.uint64)
    hsize = np.zeros(G, dtype=np.uint32)
    pr = np.zeros(len(sample.target_offset) - 1, dtype=np.float64)
    p = abi.EcParams(n_read_files=R, n_quality=Q, do_coverage=int(do_coverage), do_errors=int(do_errors),
                     preprocess_stage=int(preprocess), unmatched_end_minimum_read_length=50,
                     unmatched_end_length_factor=0.1)
    out = abi.EcResult(counts=abi.ptr(counts, C.c_uint64), coverage_hist=abi.ptr(hist, C.c_uint64),
                       hist_capacity=cap, hist_size=abi.ptr(hsize, C.c_uint32), no_pos_hash_pr=abi.ptr(pr, C.c_double))
    err = C.create_string_buffer(256)
    rc = lib().oracle_error_count(C.byref(view.ref), C.byref(view.reads), C.byref(p), C.byref(out), n_threads, err, 256)
    if rc != 0:
        raise OracleError(f"oracle_error_count failed ({rc}): {err.value.decode()}")
    return dict(counts=counts, hist=hist.reshape(G, cap), hist_size=hsize, no_pos_hash_pr=pr)


def counts_to_log10_prob(counts, R, Q):
    out = np.zeros(R * 25 * Q, dtype=np.float64)
    c = np.ascontiguousarray(counts, dtype=np.uint64)
    lib().oracle_counts_to_log10_prob(abi.ptr(c, C.c_uint64), R, Q, abi.ptr(out, C.c_double))
    return out


def default_im_params(sample, polymorphism_mode=False, prop_cutoff=None, seed_cutoff=None, dp_group=()):
    """Settings defaults of breseq (src/breseq/settings.cpp:857-950, 1335); dp_group: the DP group of
    each read group (identify_mutations.cpp:883-911), empty for none."""
    T = len(sample.target_offset) - 1
    total = float(sample.target_offset[-1])
    prop = np.broadcast_to(np.asarray(5.0 if prop_cutoff is None else prop_cutoff, dtype=np.float64), (T,)).copy()
    seed = np.broadcast_to(np.asarray(0.0 if seed_cutoff is None else seed_cutoff, dtype=np.float64), (T,)).copy()
    return dict(n_read_files=sample.n_read_files, n_quality=sample.n_quality, base_quality_cutoff=3,
                mutation_cutoff=10.0, polymorphism_cutoff=2.0 if polymorphism_mode else 10.0,
                polymorphism_precision_decimal=1e-6,
                polymorphism_precision_places=8 if polymorphism_mode else 3,
                skip_missing_coverage_prediction=0, log10_ref_length=float(np.log10(total)),
                deletion_propagation_cutoff=np.ascontiguousarray(prop, dtype=np.float64),
                deletion_seed_cutoff=np.ascontiguousarray(seed, dtype=np.float64), precision=0,
                dp_group=np.ascontiguousarray(list(dp_group), dtype=np.int32))


def make_im_params(d):
    dpg = np.ascontiguousarray(d.get("dp_group", np.zeros(0, np.int32)), dtype=np.int32)
    keep = [d["deletion_propagation_cutoff"], d["deletion_seed_cutoff"], dpg if len(dpg) else np.full(1, -1, np.int32)]
    skip = ("deletion_propagation_cutoff", "deletion_seed_cutoff", "dp_group")
    p = abi.ImParams(**{k: v for k, v in d.items() if k not in skip},
                     deletion_propagation_cutoff=abi.ptr(keep[0], C.c_double),
                     deletion_seed_cutoff=abi.ptr(keep[1], C.c_double),
                     n_read_groups=len(dpg), dp_group=abi.ptr(keep[2], C.c_int32))
    return p, keep


def identify(sample, log10_table, params: dict, n_threads=os.cpu_count() or 1, positions=True):
    view = abi.SampleView(sample)
    p, keep = make_im_params(params)
    tab = np.ascontiguousarray(log10_table, dtype=np.float64)
    handle = C.c_void_p()
    err = C.create_string_buffer(256)
    rc = lib().oracle_identify(C.byref(view.ref), C.byref(view.reads), C.byref(p), abi.ptr(tab, C.c_double),
                               C.byref(handle), n_threads, err, 256)
    if rc != 0:
        raise OracleError(f"oracle_identify failed ({rc}): {err.value.decode()}")
    try:
        n_ra, n_mc, n_un = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().oracle_im_counts(handle, C.byref(n_ra), C.byref(n_mc), C.byref(n_un))
        ra = (abi.RaRecord * max(1, n_ra.value))()
        mc = (abi.McRecord * max(1, n_mc.value))()
        un = (abi.UnRecord * max(1, n_un.value))()
        lib().oracle_im_copy(handle, C.cast(ra, C.c_void_p), C.cast(mc, C.c_void_p), C.cast(un, C.c_void_p))
        out = dict(ra=abi.ra_to_dicts(ra[:n_ra.value]), mc=abi.mc_to_dicts(mc[:n_mc.value]),
                   un=abi.un_to_dicts(un[:n_un.value]))
        if positions:
            n = int(sample.target_offset[-1])
            arrs = dict(unique_top=np.zeros(n, np.uint32), unique_bot=np.zeros(n, np.uint32),
                        redundant_top=np.zeros(n, np.float64), redundant_bot=np.zeros(n, np.float64),
                        raw_redundant_top=np.zeros(n, np.uint32), raw_redundant_bot=np.zeros(n, np.uint32),
                        consensus_score=np.zeros(n, np.float64), best_base=np.zeros(n, np.uint8),
                        n_scored=np.zeros(n, np.uint32))
            ctypes_map = dict(unique_top=C.c_uint32, unique_bot=C.c_uint32, redundant_top=C.c_double,
                              redundant_bot=C.c_double, raw_redundant_top=C.c_uint32, raw_redundant_bot=C.c_uint32,
                              consensus_score=C.c_double, best_base=C.c_uint8, n_scored=C.c_uint32)
            pa = abi.PositionArrays(**{k: abi.ptr(v, ctypes_map[k]) for k, v in arrs.items()})
            lib().oracle_im_positions(handle, C.byref(pa))
            out["positions"] = arrs
        return out
    finally:
        lib().oracle_im_free(handle)


def fisher_2x2(a, b, c, d):
    return lib().oracle_fisher_2x2(a, b, c, d)


def ks_less(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().oracle_ks_less(abi.ptr(x, C.c_double), len(x), abi.ptr(y, C.c_double), len(y))


def soft_clipping(sample, minimum_clipped_bases=12, consensus_base_fraction=0.95, dispersion_trim_frequency=0.25,
                  maximum_dispersion=0.005, minimum_rate=1e-5):
    """tabulate_soft_clipping_counts restated on the CPU: dict(summary, rows) in the library's format.
    The row order comes from the oracle's own std::map over the target names."""
    view = abi.SampleView(sample)
    names = (C.c_char_p * len(sample.target_names))(*[n.encode() for n in sample.target_names])
    p = abi.ScParams(minimum_clipped_bases=minimum_clipped_bases, consensus_base_fraction=consensus_base_fraction,
                     dispersion_trim_frequency=dispersion_trim_frequency, maximum_dispersion=maximum_dispersion,
                     minimum_rate=minimum_rate)
    h = C.c_void_p()
    err = C.create_string_buffer(256)
    rc = lib().oracle_soft_clipping(C.byref(view.ref), C.byref(view.reads), names, C.byref(p), C.byref(h), err, 256)
    if rc != 0:
        raise OracleError(f"oracle_soft_clipping failed ({rc}): {err.value.decode()}")
    try:
        s = abi.ScSummary()
        lib().oracle_sc_summary(h, C.byref(s))
        rows = (abi.ScPosition * max(1, s.n_positions))()
        lib().oracle_sc_rows(h, rows)
        return dict(summary=abi.sc_summary_dict(s), rows=abi.sc_rows_array(rows, s.n_positions))
    finally:
        lib().oracle_sc_free(h)


def coverage_columns(sample, tid, start, end):
    """coverage_output::pileup_callback restated on the CPU for positions start..end of target tid."""
    view = abi.SampleView(sample)
    arrs, st = abi.cov_columns(end - start + 1)
    last = C.c_uint32()
    err = C.create_string_buffer(256)
    rc = lib().oracle_coverage_columns(C.byref(view.ref), C.byref(view.reads), tid, start, end, C.byref(st),
                                       C.byref(last), err, 256)
    if rc != 0:
        raise OracleError(f"oracle_coverage_columns failed ({rc}): {err.value.decode()}")
    arrs["last"] = last.value
    return arrs


def im_coverage_columns(sample, tid, start, end, read_group=-1, coverage_fit_failed=False, dp_group=()):
    """identify_mutations' coverage tally (main loop at insert position 0, or tabulate_position_coverage for
    a failed coverage fit) restated on the CPU for positions start..end of target tid.  dp_group: per read
    group its discordant-pair group or -1."""
    view = abi.SampleView(sample)
    arrs, st = abi.cov_columns(end - start + 1)
    err = C.create_string_buffer(256)
    dp = np.ascontiguousarray(dp_group, dtype=np.int32)
    rc = lib().oracle_im_coverage_columns(C.byref(view.ref), C.byref(view.reads), tid, start, end, read_group,
                                          1 if coverage_fit_failed else 0, len(dp),
                                          abi.ptr(dp, C.c_int32) if len(dp) else None, C.byref(st), err, 256)
    if rc != 0:
        raise OracleError(f"oracle_im_coverage_columns failed ({rc}): {err.value.decode()}")
    return arrs


def write_coverage_table(sample, path, tid, positions, n_read_groups=None, coverage_fit_failed=False, dp_group=()):
    """<seq_id>.coverage.tsv from the aggregate per-position arrays plus each read group's columns."""
    view = abi.SampleView(sample)
    if n_read_groups is None:
        n_read_groups = int(np.max(sample.read_group)) + 1 if len(sample.read_group) else 1
    dp = np.full(max(1, n_read_groups), -1, np.int32)
    dp[:min(len(dp_group), len(dp))] = np.asarray(dp_group, dtype=np.int32)[:len(dp)]
    pa, keep = abi.position_arrays_view(positions)
    err = C.create_string_buffer(256)
    rc = lib().oracle_write_coverage_table_rg(C.byref(view.ref), C.byref(view.reads), path.encode(), tid,
                                              C.byref(pa), n_read_groups, 1 if coverage_fit_failed else 0,
                                              abi.ptr(dp, C.c_int32), err, 256)
    del keep
    if rc != 0:
        raise OracleError(f"oracle_write_coverage_table_rg failed ({rc}): {err.value.decode()}")


def write_coverage_region(sample, path, tid, start, end, resolution=600, total_only=False, csv=False,
                          reference_average=None, per_read_group=False, n_read_groups=None):
    view = abi.SampleView(sample)
    flags = (1 if total_only else 0) | (2 if csv else 0) | (4 if per_read_group else 0)
    avg = C.byref(C.c_double(reference_average)) if reference_average is not None else None
    if n_read_groups is None:
        n_read_groups = int(np.max(sample.read_group)) + 1 if len(sample.read_group) else 1
    err = C.create_string_buffer(256)
    rc = lib().oracle_write_coverage_region_rg(C.byref(view.ref), C.byref(view.reads), path.encode(),
                                               sample.target_names[tid].encode(), tid, start, end, resolution, flags,
                                               avg, n_read_groups, err, 256)
    if rc != 0:
        raise OracleError(f"oracle_write_coverage_region failed ({rc}): {err.value.decode()}")


def fit_coverage_distribution(hist, deletion_propagation_pr_cutoff):
    """CoverageDistribution::fit on a unique-only histogram hist[0 .. size-1] (single-threaded)."""
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    out = abi.CoverageFit()
    lib().oracle_fit_coverage_distribution(abi.ptr(h, C.c_uint64), h.size, float(deletion_propagation_pr_cutoff),
                                           C.byref(out))
    return abi.coverage_fit_dict(out)


def special(name, *args):
    """nbinom_pmf / nbinom_cdf / lgam / lngamma / gamma of the restatement."""
    return getattr(lib(), "oracle_" + name)(*[float(a) for a in args])


def pair_candidates(sample, settings, dp_path, mp_path, deletion_propagation_cutoff=None, pd_path=None):
    """The DP / MP candidate-region files of a sample with pair annotations (breseq_gb300.synth.with_pairs);
    settings: a breseq_gb300.api.PairSettings."""
    from breseq_gb300.api import pair_params
    view = abi.SampleView(sample)
    p, keep = pair_params(sample, settings, deletion_propagation_cutoff)
    names = (C.c_char_p * len(sample.target_names))(*[n.encode() for n in sample.target_names])
    err = C.create_string_buffer(256)
    rc = lib().oracle_pair_candidates(C.byref(view.ref), C.byref(view.reads), C.byref(p), names,
                                      dp_path.encode() if dp_path else None, mp_path.encode() if mp_path else None,
                                      pd_path.encode() if pd_path else None, err, 256)
    if rc != 0:
        raise RuntimeError(f"oracle_pair_candidates failed: {err.value.decode()}")


# ----------------------------------------------------------------- pair-distance setup, restated in Python
# pd_load_weighted_histogram (src/breseq/pd_evidence.cpp:56-97), pd_build_cdf
# (src/breseq/identify_mutations.cpp:112-141) and Cephes ndtri (src/breseq/stats.cpp:1747-1791); Python
# floats are IEEE doubles and math.log / math.sqrt are the C library's, so results are bit-identical.
_ND_P0 = (-5.99633501014107895267E1, 9.80010754185999661536E1, -5.66762857469070293439E1, 1.39312609387279679503E1,
          -1.23916583867381258016E0)
_ND_Q0 = (1.95448858338141759834E0, 4.67627912898881538453E0, 8.63602421390890590575E1, -2.25462687854119370527E2,
          2.00260212380060660359E2, -8.20372256168333339912E1, 1.59056225126211695515E1, -1.18331621121330003142E0)
_ND_P1 = (4.05544892305962419923E0, 3.15251094599893866154E1, 5.71628192246421288162E1, 4.40805073893200834700E1,
          1.46849561928858024014E1, 2.18663306850790267539E0, -1.40256079171354495875E-1, -3.50424626827848203418E-2,
          -8.57456785154685413611E-4)
_ND_Q1 = (1.57799883256466749731E1, 4.53907635128879210584E1, 4.13172038254672030440E1, 1.50425385692907503408E1,
          2.50464946208309415979E0, -1.42182922854787788574E-1, -3.80806407691578277194E-2, -9.33259480895457427372E-4)
_ND_P2 = (3.23774891776946035970E0, 6.91522889068984211695E0, 3.93881025292474443415E0, 1.33303460815807542389E0,
          2.01485389549179081538E-1, 1.23716634817820021358E-2, 3.01581553508235416007E-4, 2.65806974686737550832E-6,
          6.23974539184983293730E-9)
_ND_Q2 = (6.02427039364742014255E0, 3.67983563856160859403E0, 1.37702099489081330271E0, 2.16236993594496635890E-1,
          1.34204006088543189037E-2, 3.28014464682127739104E-4, 2.89247864745380683936E-6, 6.79019408009981274425E-9)


def _polevl(x, c):
    a = c[0]
    for v in c[1:]:
        a = a * x + v
    return a


def _p1evl(x, c):
    a = x + c[0]
    for v in c[1:]:
        a = a * x + v
    return a


def ndtri(y0):
    import math
    if y0 <= 0.0:
        return -1.79769313486231570815E308
    if y0 >= 1.0:
        return 1.79769313486231570815E308
    code, y = 1, y0
    if y > (1.0 - 0.13533528323661269189):
        y, code = 1.0 - y, 0
    if y > 0.13533528323661269189:
        y = y - 0.5
        y2 = y * y
        x = y + y * (y2 * _polevl(y2, _ND_P0) / _p1evl(y2, _ND_Q0))
        return x * 2.50662827463100050242E0
    x = math.sqrt(-2.0 * math.log(y))
    x0 = x - math.log(x) / x
    z = 1.0 / x
    x1 = z * _polevl(z, _ND_P1) / _p1evl(z, _ND_Q1) if x < 8.0 else z * _polevl(z, _ND_P2) / _p1evl(z, _ND_Q2)
    x = x0 - x1
    return -x if code != 0 else x


def pd_build_null(distance, count, trunc, max_distance):
    weighted, total = [], 0.0
    for d, n in zip(distance, count):
        d, n = int(d), float(n)
        if d < 0 or n <= 0.0:
            continue
        if max_distance > 0 and d > max_distance:
            continue
        w = float(d - trunc)
        if w <= 0.0:
            continue
        if len(weighted) <= d:
            weighted += [0.0] * (d + 1 - len(weighted))
        weighted[d] = n * w
        total += weighted[d]
    if total <= 0.0:
        return None, 0.0
    cdf, below, gap = [], 0.0, 0.0
    for d, w in enumerate(weighted):
        mid = (below + 0.5 * w) / total
        below += w
        gap += w * (float(d) - float(trunc))
        scaled = min(max(int(mid * 1048576.0 + 0.5), 0), 1048576)
        cdf.append(scaled)
    return np.array(cdf, dtype=np.int64), gap / total


def pd_seed_z(seed_z, gap, total_length):
    if seed_z > 0.0:
        return seed_z
    a = 0.005
    if gap > 0.0 and total_length > 0:
        a *= gap / float(total_length)
    a = min(max(a, 1e-12), 0.5)
    return max(min(ndtri(1.0 - a), 2.5), 1.0)
