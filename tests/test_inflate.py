"""The library's DEFLATE decoder (breseq_gb300/csrc/bsq_inflate.cuh), compiled for the host, against
zlib (the inflater htslib uses under breseq) on random, repetitive and sequence-like data at every
compression level and strategy, and on truncated or corrupted input, which must fail cleanly."""
import ctypes as C
import os
import random
import subprocess
import zlib

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "inflate_host.cpp")
OUT = os.path.join(ROOT, "tests", "native", "_build", "libinflate_host.so")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT])
    L = C.CDLL(OUT)
    L.host_inflate.argtypes = [C.c_char_p, C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32)]
    return L


def payload(rng, n, kind):
    if kind == 0:
        return bytes(rng.getrandbits(8) for _ in range(n))
    if kind == 1:
        return bytes(rng.choice(b"ACGT") for _ in range(n))
    if kind == 2:
        return (b"ACGTTGCA" * (n // 8 + 1))[:n]
    return bytes(rng.choice(b"!#%&'()*+,-./0123456789:;<=>?@ABCDEFGHIJ") for _ in range(n))


def deflate(raw, level, strategy):
    co = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy)
    return co.compress(raw) + co.flush()


STRATEGIES = [zlib.Z_DEFAULT_STRATEGY, zlib.Z_FIXED, zlib.Z_HUFFMAN_ONLY, zlib.Z_RLE]


@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("strategy", STRATEGIES, ids=["default", "fixed", "huffman", "rle"])
def test_matches_zlib(lib, level, strategy):
    rng = random.Random(level * 10 + strategy)
    for n in [0, 1, 7, 300, 5000, 65536]:
        for kind in range(4):
            raw = payload(rng, n, kind)
            comp = deflate(raw, level, strategy)
            out = C.create_string_buffer(max(1, n))
            got = C.c_uint32()
            assert lib.host_inflate(comp, len(comp), out, n, C.byref(got)) == 0
            assert got.value == n and out.raw[:n] == raw


def test_bad_input_fails_cleanly(lib):
    rng = random.Random(5)
    raw = payload(rng, 20000, 3)
    comp = deflate(raw, 6, zlib.Z_DEFAULT_STRATEGY)
    out = C.create_string_buffer(65536)
    got = C.c_uint32()
    # truncated: runs out of input
    assert lib.host_inflate(comp[: len(comp) // 2], len(comp) // 2, out, 65536, C.byref(got)) != 0
    # output larger than the capacity
    assert lib.host_inflate(comp, len(comp), out, 1000, C.byref(got)) == 5
    # block type 3
    assert lib.host_inflate(bytes([0x07]), 1, out, 65536, C.byref(got)) == 2
    # stored block whose length and complement disagree
    assert lib.host_inflate(bytes([0x01, 0x05, 0x00, 0x00, 0x00]), 5, out, 65536, C.byref(got)) == 3
    # bit flips: an error or some output, never anything else
    for _ in range(200):
        b = bytearray(comp)
        for _ in range(2):
            b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
        assert lib.host_inflate(bytes(b), len(b), out, 65536, C.byref(got)) in range(0, 8)
