"""The C-ABI library builds, loads without a GPU, exports every function the header declares, and its
host-only entry points agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from breseq_gb300 import _lib, abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "breseq_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bsq_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    assert set(declared_functions()) >= set(_lib.EXPORTED)


def test_version_and_no_device_error(built_lib):
    L = _lib.load()
    assert b"sm_103a" in L.bsq_version()
    ctx = C.c_void_p()
    rc = L.bsq_create(C.byref(ctx), 0)
    if rc != 0:           # no GPU here: a clean error code, never a crash
        assert rc in (-1, -2)
    else:
        L.bsq_destroy(ctx)


@pytest.mark.parametrize("seed", range(12))
def test_counts_to_log10_prob_matches_oracle(built_lib, oracle_lib, seed):
    """The library rounds to six significant digits without text; the oracle prints with %.6g and
    parses back.  Bit-exact over tables from sparse to 10^12-deep counts."""
    from oracle import pyoracle as po
    rng = np.random.default_rng(seed)
    R, Q = (1, 42) if seed % 3 == 0 else (2, 64)
    top = [10**3, 10**7, 10**12][seed % 3]
    counts = rng.integers(0, top, size=R * 25 * Q).astype(np.uint64)
    counts[rng.random(counts.size) < 0.3] = 0
    out = np.zeros(R * 25 * Q)
    L = _lib.load()
    assert L.bsq_counts_to_log10_prob(abi.ptr(counts, C.c_uint64), R, Q, abi.ptr(out, C.c_double)) == 0
    assert np.array_equal(out, po.counts_to_log10_prob(counts, R, Q))


def test_struct_sizes_match_header():
    # bsq_ra_record layout shared by the library, the oracle and the bindings
    assert C.sizeof(abi.RaRecord) == 4 * 3 + 4 + 8 * 2 + 8 * 5 + 8 * 6 + 4 * 10 + 4 + 4
    assert C.sizeof(abi.McRecord) == 6 * 4 + 4 * 8


def test_counts_to_log10_prob_batch_equals_single(built_lib):
    rng = np.random.default_rng(11)
    L = _lib.load()
    shapes = [(1, 42), (2, 42), (2, 64), (3, 30)]
    counts = [rng.integers(0, 10**6, size=R * 25 * Q).astype(np.uint64) for R, Q in shapes]
    outs = [np.zeros(R * 25 * Q) for R, Q in shapes]
    n = len(shapes)
    rc = L.bsq_counts_to_log10_prob_batch(n, (C.POINTER(C.c_uint64) * n)(*[abi.ptr(c, C.c_uint64) for c in counts]),
                                          (C.c_uint32 * n)(*[R for R, _ in shapes]), (C.c_uint32 * n)(*[Q for _, Q in shapes]),
                                          (C.POINTER(C.c_double) * n)(*[abi.ptr(o, C.c_double) for o in outs]))
    assert rc == 0
    for (R, Q), c, o in zip(shapes, counts, outs):
        single = np.zeros(R * 25 * Q)
        assert L.bsq_counts_to_log10_prob(abi.ptr(c, C.c_uint64), R, Q, abi.ptr(single, C.c_double)) == 0
        assert np.array_equal(o, single)
