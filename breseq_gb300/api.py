"""Host API over the C ABI, mirroring breseq's two entry points of the scoring path.

    error_count(...)         <- breseq::error_count          (src/breseq/error_count.h:44-56)
    identify_mutations(...)  <- breseq::identify_mutations   (src/breseq/identify_mutations.h:46-60)

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
class ImSettings:
    """The Settings fields identify_mutations reads, with breseq's defaults."""
    polymorphism_prediction: bool = False
    base_quality_cutoff: int = 3
    mutation_log10_e_value_cutoff: float = 10.0
    polymorphism_log10_e_value_cutoff: float | None = None   # 2 (polymorphism mode) / 10 (consensus mode)
    polymorphism_precision_decimal: float = 1e-6
    polymorphism_precision_places: int | None = None          # 8 / 3
    skip_missing_coverage_prediction: bool = False

    def resolved(self):
        poly = self.polymorphism_log10_e_value_cutoff
        if poly is None:
            poly = 2.0 if self.polymorphism_prediction else 10.0
        places = self.polymorphism_precision_places
        if places is None:
            places = 8 if self.polymorphism_prediction else 3
        return poly, places


class Scorer:
    """One library context on one GPU; samples stay resident until freed."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        self.ctx = C.c_void_p()
        rc = self.L.bsq_create(C.byref(self.ctx), device)
        if rc != 0:
            raise _lib.BsqError(rc, "bsq_create failed (no CUDA device?)")
        self._views = {}

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
        return sid.value

    def free_sample(self, sid: int):
        self._check(self.L.bsq_free_sample(self.ctx, sid))
        self._views.pop(sid, None)

    def sample(self, sid):
        return self._views[sid][0]

    # ------------------------------------------------------------------ pass 1
    def error_count(self, sid: int, n_read_files=None, n_quality=None, do_coverage=True, do_errors=True,
                    preprocess=False, unmatched_end_minimum_read_length=50, unmatched_end_length_factor=0.1,
                    hist_capacity=8192):
        s = self.sample(sid)
        R = n_read_files or s.n_read_files
        Q = n_quality or s.n_quality
        G = s.n_coverage_groups
        counts = np.zeros(R * 25 * Q, dtype=np.uint64)
        hist = np.zeros(G * hist_capacity, dtype=np.uint64)
        hsize = np.zeros(G, dtype=np.uint32)
        pr = np.zeros(len(s.target_offset) - 1, dtype=np.float64)
        p = abi.EcParams(n_read_files=R, n_quality=Q, do_coverage=int(do_coverage), do_errors=int(do_errors),
                         preprocess_stage=int(preprocess),
                         unmatched_end_minimum_read_length=unmatched_end_minimum_read_length,
                         unmatched_end_length_factor=unmatched_end_length_factor)
        out = abi.EcResult(counts=abi.ptr(counts, C.c_uint64), coverage_hist=abi.ptr(hist, C.c_uint64),
                           hist_capacity=hist_capacity, hist_size=abi.ptr(hsize, C.c_uint32),
                           no_pos_hash_pr=abi.ptr(pr, C.c_double))
        self._check(self.L.bsq_error_count(self.ctx, sid, C.byref(p), C.byref(out)))
        return dict(counts=counts, hist=hist.reshape(G, hist_capacity), hist_size=hsize, no_pos_hash_pr=pr)

    def counts_to_log10_prob(self, counts, R, Q):
        out = np.zeros(R * 25 * Q, dtype=np.float64)
        c = np.ascontiguousarray(counts, dtype=np.uint64)
        self._check(self.L.bsq_counts_to_log10_prob(abi.ptr(c, C.c_uint64), R, Q, abi.ptr(out, C.c_double)))
        return out

    # ------------------------------------------------------------------ pass 2
    def identify_mutations(self, sid: int, log10_table, settings: ImSettings | None = None,
                           deletion_propagation_cutoff=None, deletion_seed_cutoff=None,
                           precision=PRECISION_FP32C, positions=False, n_read_files=None, n_quality=None):
        s = self.sample(sid)
        st = settings or ImSettings()
        poly, places = st.resolved()
        T = len(s.target_offset) - 1
        prop = np.broadcast_to(np.asarray(5.0 if deletion_propagation_cutoff is None else deletion_propagation_cutoff,
                                          dtype=np.float64), (T,)).copy()
        seed = np.broadcast_to(np.asarray(0.0 if deletion_seed_cutoff is None else deletion_seed_cutoff,
                                          dtype=np.float64), (T,)).copy()
        tab = np.ascontiguousarray(log10_table, dtype=np.float64)
        p = abi.ImParams(n_read_files=n_read_files or s.n_read_files, n_quality=n_quality or s.n_quality,
                         base_quality_cutoff=st.base_quality_cutoff,
                         mutation_cutoff=st.mutation_log10_e_value_cutoff, polymorphism_cutoff=poly,
                         polymorphism_precision_decimal=st.polymorphism_precision_decimal,
                         polymorphism_precision_places=places,
                         skip_missing_coverage_prediction=int(st.skip_missing_coverage_prediction),
                         log10_ref_length=float(np.log10(float(s.target_offset[-1]))),
                         deletion_propagation_cutoff=abi.ptr(prop, C.c_double),
                         deletion_seed_cutoff=abi.ptr(seed, C.c_double), precision=precision)
        arrs = None
        pa = None
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
        self._check(self.L.bsq_identify_mutations(self.ctx, sid, C.byref(p), abi.ptr(tab, C.c_double),
                                                  C.byref(pa) if pa is not None else None))
        n_ra, n_mc, n_un = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.L.bsq_im_result_counts(self.ctx, C.byref(n_ra), C.byref(n_mc), C.byref(n_un)))
        ra = (abi.RaRecord * max(1, n_ra.value))()
        mc = (abi.McRecord * max(1, n_mc.value))()
        un = (abi.UnRecord * max(1, n_un.value))()
        self._check(self.L.bsq_im_result_copy(self.ctx, C.cast(ra, C.c_void_p), n_ra.value, C.cast(mc, C.c_void_p),
                                              n_mc.value, C.cast(un, C.c_void_p), n_un.value))
        out = dict(ra=abi.ra_to_dicts(ra[:n_ra.value]), mc=abi.mc_to_dicts(mc[:n_mc.value]),
                   un=abi.un_to_dicts(un[:n_un.value]))
        if arrs is not None:
            out["positions"] = arrs
        return out

    def timer_start(self):
        self._check(self.L.bsq_timer_start(self.ctx))

    def timer_stop(self) -> float:
        ms = C.c_double()
        self._check(self.L.bsq_timer_stop(self.ctx, C.byref(ms)))
        return ms.value

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
