"""ctypes binding of libbsq_gb300.so.  There is no fallback: if the library was not built, or the
CUDA runtime cannot create a context, every call raises."""
from __future__ import annotations

import ctypes as C
import os

from . import abi

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libbsq_gb300.so")
_lib = None


class BsqError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"breseq_gb300 error {code}: {msg}")
        self.code = code


def load():
    """Load the in-tree library (build it first with breseq_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BsqError(-1, f"{LIB_PATH} is missing: run `python -m breseq_gb300.build` (needs nvcc)")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER
    L.bsq_create.argtypes = [P(C.c_void_p), C.c_int]
    L.bsq_destroy.argtypes = [C.c_void_p]
    L.bsq_destroy.restype = None
    L.bsq_last_error.argtypes = [C.c_void_p]
    L.bsq_last_error.restype = C.c_char_p
    L.bsq_version.restype = C.c_char_p
    L.bsq_load_sample.argtypes = [C.c_void_p, P(abi.Reference), P(abi.ReadSoA), P(C.c_int32)]
    L.bsq_free_sample.argtypes = [C.c_void_p, C.c_int32]
    L.bsq_sample_footprint.argtypes = [P(abi.Reference), P(abi.ReadSoA)]
    L.bsq_sample_footprint.restype = C.c_uint64
    L.bsq_error_count.argtypes = [C.c_void_p, C.c_int32, P(abi.EcParams), P(abi.EcResult)]
    L.bsq_error_count_batch.argtypes = [C.c_void_p, C.c_uint32, P(C.c_int32), P(abi.EcParams), P(abi.EcResult)]
    L.bsq_identify_mutations_batch.argtypes = [C.c_void_p, C.c_uint32, P(C.c_int32), P(abi.ImParams),
                                               P(P(C.c_double)), P(P(abi.PositionArrays))]
    L.bsq_im_batch_result_counts.argtypes = [C.c_void_p, C.c_uint32, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64)]
    L.bsq_im_batch_result_copy.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                           C.c_void_p, C.c_uint64]
    L.bsq_counts_to_log10_prob.argtypes = [P(C.c_uint64), C.c_uint32, C.c_uint32, P(C.c_double)]
    L.bsq_identify_mutations.argtypes = [C.c_void_p, C.c_int32, P(abi.ImParams), P(C.c_double), P(abi.PositionArrays)]
    L.bsq_im_result_counts.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_uint64), P(C.c_uint64)]
    L.bsq_im_result_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]
    L.bsq_last_pass_stats.argtypes = [C.c_void_p, P(C.c_double), P(C.c_uint32), P(C.c_double)]
    L.bsq_timer_start.argtypes = [C.c_void_p]
    L.bsq_timer_stop.argtypes = [C.c_void_p, P(C.c_double)]
    L.bsq_host_register.argtypes = [C.c_void_p, C.c_uint64]
    L.bsq_host_unregister.argtypes = [C.c_void_p]
    L.bsq_score_positions_noalloc.argtypes = [C.c_void_p, C.c_int32, P(abi.ImParams), P(C.c_double), C.c_void_p,
                                              C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    L.bsq_default_ra_settings.argtypes = [C.c_int, P(abi.RaSettings)]
    L.bsq_test_ra_evidence.argtypes = [C.c_void_p, C.c_uint64, P(abi.RaSettings), P(abi.Reference), P(C.c_char_p), C.c_void_p]
    L.bsq_write_error_rates.argtypes = [C.c_char_p, P(C.c_uint64), C.c_uint32, C.c_uint32]
    L.bsq_write_base_qual_error_prob.argtypes = [C.c_char_p, P(C.c_char_p), P(C.c_uint64), C.c_uint32, C.c_uint32]
    L.bsq_write_coverage_distribution.argtypes = [C.c_char_p, P(C.c_uint64), C.c_uint32]
    L.bsq_write_coverage_table.argtypes = [C.c_char_p, C.c_char_p, P(abi.Reference), C.c_uint32, P(abi.PositionArrays)]
    L.bsq_format_ra.argtypes = [C.c_void_p, C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint64]
    L.bsq_write_gd.argtypes = [C.c_char_p, P(abi.Reference), P(C.c_char_p), P(C.c_double), C.c_uint32, C.c_void_p,
                               C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]
    L.bsq_counts_to_log10_prob_batch.argtypes = [C.c_uint32, P(P(C.c_uint64)), P(C.c_uint32), P(C.c_uint32),
                                                 P(P(C.c_double))]
    L.bsq_last_pass_bytes.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_uint64)]
    L.bsq_get_tuning.argtypes = [C.c_void_p, P(abi.Tuning)]
    L.bsq_set_tuning.argtypes = [C.c_void_p, P(abi.Tuning)]
    L.bsq_autotune.argtypes = [C.c_void_p, C.c_uint32, P(C.c_int32), P(abi.EcParams), P(abi.ImParams),
                               P(P(C.c_double)), P(abi.Tuning)]
    L.bsq_job_footprint.argtypes = [P(abi.Reference), P(abi.ReadSoA)]
    L.bsq_job_footprint.restype = C.c_uint64
    L.bsq_server_create.argtypes = [P(C.c_void_p), C.c_int, C.c_uint64, C.c_uint32, C.c_int32]
    L.bsq_server_destroy.argtypes = [C.c_void_p]
    L.bsq_server_destroy.restype = None
    L.bsq_server_last_error.argtypes = [C.c_void_p]
    L.bsq_server_last_error.restype = C.c_char_p
    L.bsq_server_submit.argtypes = [C.c_void_p, P(abi.Job), P(C.c_uint64)]
    L.bsq_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, P(abi.JobInfo)]
    L.bsq_server_job_info.argtypes = [C.c_void_p, C.c_uint64, P(abi.JobInfo)]
    L.bsq_server_job_error.argtypes = [C.c_void_p, C.c_uint64]
    L.bsq_server_job_error.restype = C.c_char_p
    L.bsq_server_error_counts.argtypes = [C.c_void_p, C.c_uint64, P(C.c_uint64), P(C.c_uint64), P(C.c_uint32)]
    L.bsq_server_results.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                     C.c_void_p, C.c_uint64]
    L.bsq_server_release.argtypes = [C.c_void_p, C.c_uint64]
    L.bsq_server_get_stats.argtypes = [C.c_void_p, P(abi.ServerStats)]
    L.bsq_server_set_tuning.argtypes = [C.c_void_p, P(abi.Tuning)]
    L.bsq_default_sc_params.argtypes = [P(abi.ScParams)]
    L.bsq_soft_clipping.argtypes = [C.c_void_p, C.c_int32, P(abi.ScParams), P(abi.ScSummary)]
    L.bsq_sc_result_copy.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
    L.bsq_write_soft_clipping_counts.argtypes = [C.c_char_p, P(C.c_char_p), P(abi.ScParams), P(abi.ScSummary),
                                                 C.c_void_p, C.c_uint64]
    L.bsq_coverage_columns.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, P(abi.CovColumns),
                                       P(C.c_uint32)]
    L.bsq_write_coverage_region.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_char_p, C.c_uint32, C.c_uint32,
                                            C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_double)]
    L.bsq_coverage_columns_rg.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32,
                                          P(abi.CovColumns), P(C.c_uint32)]
    L.bsq_write_coverage_region_rg.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_char_p, C.c_uint32, C.c_uint32,
                                               C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_double), C.c_uint32]
    L.bsq_im_coverage_columns_rg.argtypes = [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32,
                                             C.c_int, C.c_uint32, P(C.c_int32), P(abi.CovColumns)]
    L.bsq_write_coverage_table_rg.argtypes = [C.c_void_p, C.c_int32, C.c_char_p, C.c_char_p, P(abi.Reference),
                                              C.c_uint32, P(abi.PositionArrays), C.c_uint32, C.c_int, P(C.c_int32)]
    L.bsq_intervals_from_positions.argtypes = [P(abi.Reference), P(abi.PositionArrays), P(abi.ImParams), C.c_void_p,
                                               C.c_uint64, P(C.c_uint64), C.c_void_p, C.c_uint64, P(C.c_uint64)]
    L.bsq_bam_open.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, P(C.c_void_p)]
    L.bsq_bam_close.argtypes = [C.c_void_p]
    L.bsq_bam_close.restype = None
    L.bsq_bam_header.argtypes = [C.c_void_p, P(C.c_char_p), P(C.c_uint64), P(C.c_uint32), P(P(C.c_char_p)),
                                 P(P(C.c_uint32))]
    L.bsq_bam_decode.argtypes = [C.c_void_p, C.c_void_p, P(abi.BamGroups), P(C.c_uint64), P(C.c_uint64), P(C.c_uint64)]
    L.bsq_bam_copy_records.argtypes = [C.c_void_p, C.c_void_p, P(abi.ReadArrays)]
    L.bsq_bam_load.argtypes = [C.c_void_p, C.c_void_p, P(abi.Reference), P(C.c_int32)]
    L.bsq_bam_name_bytes.argtypes = [C.c_void_p, C.c_void_p, P(C.c_uint64)]
    L.bsq_pair_candidates.argtypes = [C.c_void_p, C.c_int32, P(abi.PairParams), P(C.c_uint64), P(C.c_uint64),
                                      P(C.c_uint64)]
    L.bsq_pair_result_copy.argtypes = [C.c_void_p, P(abi.PairRegion), C.c_uint64, P(abi.PairRegion), C.c_uint64,
                                       C.c_char_p, C.c_uint64]
    L.bsq_pd_result.argtypes = [C.c_void_p, P(C.c_uint64), P(abi.PdRegion), C.c_uint64, P(abi.PdSummary)]
    L.bsq_write_pd_candidate_regions.argtypes = [C.c_char_p, P(C.c_char_p), P(abi.PdRegion), C.c_uint64,
                                                 P(abi.PdSummary)]
    L.bsq_pd_build_null.argtypes = [P(C.c_int32), P(C.c_double), C.c_uint64, C.c_int32, C.c_int32, P(C.c_int64),
                                    C.c_uint32, P(C.c_uint32), P(C.c_double)]
    L.bsq_pd_max_span.argtypes = [C.c_int32, P(C.c_double), C.c_uint32]
    L.bsq_pd_max_span.restype = C.c_int32
    L.bsq_pd_seed_z.argtypes = [C.c_double, C.c_double, C.c_uint64]
    L.bsq_pd_seed_z.restype = C.c_double
    L.bsq_ndtri.argtypes = [C.c_double]
    L.bsq_ndtri.restype = C.c_double
    for fn in (L.bsq_write_dp_candidate_regions, L.bsq_write_mp_candidate_regions):
        fn.argtypes = [C.c_char_p, P(C.c_char_p), P(abi.PairRegion), C.c_uint64, C.c_char_p]
    L.bsq_fit_coverage_distribution.argtypes = [P(C.c_uint64), C.c_uint32, C.c_double, C.c_int, P(abi.CoverageFit)]
    L.bsq_fit_negative_binomial.argtypes = [P(C.c_double), C.c_uint32, C.c_int, P(C.c_double), P(C.c_double)]
    L.bsq_nbinom_pmf.argtypes = [C.c_double, C.c_double, C.c_double]
    L.bsq_nbinom_pmf.restype = C.c_double
    L.bsq_nbinom_cdf.argtypes = [C.c_double, C.c_double, C.c_double]
    L.bsq_nbinom_cdf.restype = C.c_double
    L.bsq_nbinom_quantile.argtypes = [C.c_double, C.c_double, C.c_double, P(C.c_uint64)]
    _lib = L
    return L


EXPORTED = ("bsq_create", "bsq_destroy", "bsq_last_error", "bsq_version", "bsq_load_sample", "bsq_free_sample",
            "bsq_sample_footprint", "bsq_error_count", "bsq_counts_to_log10_prob", "bsq_identify_mutations",
            "bsq_im_result_counts", "bsq_im_result_copy",
            "bsq_error_count_batch", "bsq_identify_mutations_batch", "bsq_im_batch_result_counts",
            "bsq_im_batch_result_copy", "bsq_counts_to_log10_prob_batch", "bsq_last_pass_bytes", "bsq_get_tuning", "bsq_set_tuning", "bsq_autotune",
            "bsq_job_footprint", "bsq_server_create", "bsq_server_destroy",
            "bsq_server_last_error", "bsq_server_submit", "bsq_server_wait", "bsq_server_job_info",
            "bsq_server_job_error", "bsq_server_error_counts", "bsq_server_results", "bsq_server_release",
            "bsq_server_get_stats", "bsq_server_set_tuning", "bsq_last_pass_stats", "bsq_timer_start",
            "bsq_timer_stop", "bsq_host_register", "bsq_host_unregister", "bsq_score_positions_noalloc",
            "bsq_default_ra_settings", "bsq_test_ra_evidence", "bsq_write_error_rates", "bsq_write_base_qual_error_prob",
            "bsq_write_coverage_distribution", "bsq_write_coverage_table", "bsq_format_ra", "bsq_write_gd",
            "bsq_default_sc_params", "bsq_soft_clipping", "bsq_sc_result_copy", "bsq_write_soft_clipping_counts",
            "bsq_coverage_columns", "bsq_write_coverage_region", "bsq_bam_open", "bsq_bam_close", "bsq_bam_header",
            "bsq_bam_decode", "bsq_bam_copy_records", "bsq_bam_load", "bsq_fit_coverage_distribution",
            "bsq_fit_negative_binomial", "bsq_nbinom_pmf", "bsq_nbinom_cdf", "bsq_nbinom_quantile",
            "bsq_bam_name_bytes", "bsq_pair_candidates", "bsq_pair_result_copy", "bsq_write_dp_candidate_regions",
            "bsq_write_mp_candidate_regions", "bsq_pd_result",
            "bsq_write_pd_candidate_regions", "bsq_coverage_columns_rg", "bsq_write_coverage_region_rg",
            "bsq_pd_build_null", "bsq_pd_max_span", "bsq_pd_seed_z", "bsq_ndtri", "bsq_im_coverage_columns_rg",
            "bsq_write_coverage_table_rg", "bsq_intervals_from_positions")
