"""The library's DEFLATE decoders (breseq_gb300/csrc/bsq_inflate.cuh: the bit-by-bit one and the
two-phase one the device runs, one block per thread into tokens and the tokens into bytes, here both
phases on one thread), compiled for the host, against
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
    L.host_inflate_tokens.argtypes = L.host_inflate.argtypes
    L.host_crc_combine.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64]
    L.host_crc_combine.restype = C.c_uint32
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


def run(lib, fn, comp, out, cap, got):
    return getattr(lib, fn)(comp, len(comp), out, cap, C.byref(got))


@pytest.mark.parametrize("fn", ["host_inflate", "host_inflate_tokens"])
@pytest.mark.parametrize("level", [0, 1, 6, 9])
@pytest.mark.parametrize("strategy", STRATEGIES, ids=["default", "fixed", "huffman", "rle"])
def test_matches_zlib(lib, fn, level, strategy):
    rng = random.Random(level * 10 + strategy)
    for n in [0, 1, 7, 300, 5000, 65536]:
        for kind in range(4):
            raw = payload(rng, n, kind)
            comp = deflate(raw, level, strategy)
            out = C.create_string_buffer(max(1, n))
            got = C.c_uint32()
            assert run(lib, fn, comp, out, n, got) == 0
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


def test_two_phase_bad_input(lib):
    rng = random.Random(12)
    raw = payload(rng, 30000, 3)
    comp = deflate(raw, 6, zlib.Z_DEFAULT_STRATEGY)
    out = C.create_string_buffer(65536)
    got = C.c_uint32()
    assert lib.host_inflate_tokens(comp[: len(comp) // 2], len(comp) // 2, out, 30000, C.byref(got)) != 0
    assert lib.host_inflate_tokens(comp, len(comp), out, 1000, C.byref(got)) == 5
    assert lib.host_inflate_tokens(comp, len(comp), out, 30001, C.byref(got)) == 5     # short of the size
    for _ in range(300):
        b = bytearray(comp)
        for _ in range(rng.randrange(1, 3)):
            b[rng.randrange(len(b))] ^= 1 << rng.randrange(8)
        assert lib.host_inflate_tokens(bytes(b), len(b), out, 30000, C.byref(got)) in range(0, 8)


def test_crc_combine(lib):
    # crc(AB) from crc(A), crc(B) and |B|, as the device combines the 32 lanes' slices
    rng = random.Random(3)
    for _ in range(200):
        a = payload(rng, rng.randrange(0, 3000), rng.randrange(4))
        b = payload(rng, rng.randrange(0, 3000), rng.randrange(4))
        assert lib.host_crc_combine(zlib.crc32(a), zlib.crc32(b), len(b)) == zlib.crc32(a + b)
