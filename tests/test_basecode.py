"""The class bytes (breseq_gb300/csrc/bsq_basecode.cuh: quality * 5 + base, four bases in the bytes of a
word) and pass 1's reference-match mask (same_as_reference8, eight bases a word), compiled for the
host and checked against the per-base rules on every (nibble, quality) and (read nibble, reference
code) pair and on random words."""
import ctypes as C
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "native", "basecode_host.cpp")
OUT = os.path.join(ROOT, "tests", "native", "_build", "libbasecode_host.so")


def test_class_bytes_match_the_per_base_rule():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT])
    L = C.CDLL(OUT)
    L.basecode_selftest.argtypes = [C.c_uint]
    assert L.basecode_selftest(7) == 0
