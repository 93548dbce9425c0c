"""The fixed-point value behind the mixed form's digit split
(strassen_gb300/csrc/bsg_digits.h, oz_fixed_bits): the header is compiled for
the host with g++ and checked against exact integer rounding (ties to even)
of v 2^(K - e), on random values of every magnitude and on the cases where
rounding is delicate: right shifts of 1..55 bits (either side of the 32-bit
word boundary and past the 53-bit significand), exact ties, subnormals and
zeros."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "strassen_gb300", "csrc")

_SRC = r"""
#include "bsg_digits.h"
extern "C" void split(const unsigned long long *bits, const int *e, const int *K, long long *out, unsigned long n) {
    for (unsigned long i = 0; i < n; ++i) out[i] = bsg::oz_fixed_bits(bits[i], e[i], K[i]);
}
"""


@pytest.fixture(scope="module")
def split(tmp_path_factory):
    d = tmp_path_factory.mktemp("split")
    src, lib = d / "split.cpp", d / "split.so"
    src.write_text(_SRC)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(lib)])
    f = C.CDLL(str(lib)).split
    f.restype = None

    def run(bits, e, K):
        bits = np.ascontiguousarray(bits, dtype=np.uint64)
        e = np.ascontiguousarray(e, dtype=np.int32)
        K = np.ascontiguousarray(K, dtype=np.int32)
        out = np.zeros(len(bits), dtype=np.int64)
        f(bits.ctypes.data, e.ctypes.data, K.ctypes.data, out.ctypes.data, C.c_ulong(len(bits)))
        return out

    return run


def _exact(bits, e, K):
    """round(v 2^(K - e)) ties to even, with Python integers"""
    E = (bits >> 52) & 0x7FF
    M = (bits & ((1 << 52) - 1)) | ((1 << 52) if E else 0)
    sh = (E if E else 1) - 1075 + K - e
    if sh >= 0:
        N = M << sh
    else:
        q, r = divmod(M, 1 << -sh)
        half = 1 << (-sh - 1)
        N = q + (1 if r > half or (r == half and q & 1) else 0)
    return -N if bits >> 63 else N


def _check(split, bits, e, K):
    got = split(bits, e, K)
    for b, ee, k, g in zip(bits.tolist(), e.tolist(), K.tolist(), got.tolist()):
        assert g == _exact(b, ee, k), (hex(b), ee, k, g)


def _exp_of(bits):
    """the frexp exponent of |v| (max < 2^e), as the row maxima give it"""
    E = (bits >> 52) & 0x7FF
    if E:
        return E - 1022
    m = bits & ((1 << 52) - 1)
    return (m.bit_length() - 1) - 1074 + 1 if m else 0


def test_random_values_every_digit_count(split):
    rng = np.random.default_rng(11)
    n = 60000
    bits = rng.integers(0, 1 << 63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    # exponents from the whole range, most near 1
    E = np.where(rng.random(n) < 0.8, rng.integers(990, 1060, n), rng.integers(0, 2047, n)).astype(np.uint64)
    bits = (bits & ~np.uint64(0x7FF << 52)) | (E << np.uint64(52))
    # row exponents at or above the value's own: shifts from 1 to past 60 bits
    e = np.array([_exp_of(int(b) & ((1 << 63) - 1)) for b in bits.tolist()]) + rng.integers(0, 48, n)
    K = 7 + 8 * (rng.integers(2, 8, n) - 1)  # 2 .. 7 digits
    _check(split, bits, e.astype(np.int32), K.astype(np.int32))


def test_word_boundaries_and_ties(split):
    bits, es, Ks = [], [], []
    rng = np.random.default_rng(12)
    for K in (15, 23, 31, 39, 47, 55):
        for s in list(range(1, 56)):
            for _ in range(6):
                E = int(rng.integers(900, 1100))
                m = int(rng.integers(0, 1 << 52))
                if s <= 52 and rng.random() < 0.5:
                    # an exact tie: the s shifted-out bits are 100..0
                    m = (m >> s << s) | (1 << (s - 1)) if s <= 52 else m
                    m &= (1 << 52) - 1
                b = (E << 52) | m | (int(rng.integers(0, 2)) << 63)
                # e from s: s = 1075 - E - K + e
                bits.append(b)
                es.append(s - 1075 + E + K)
                Ks.append(K)
    _check(split, np.array(bits, dtype=np.uint64), np.array(es, dtype=np.int32), np.array(Ks, dtype=np.int32))


def test_zeros_and_subnormals(split):
    bits = [0, 1 << 63, 1, 3, (1 << 52) - 1, (1 << 51) + 5, (1 << 63) | 12345]
    es = [0, 0, -1073, -1072, -1022, -1022, -1060]
    for K in (15, 39, 55):
        _check(split, np.array(bits, dtype=np.uint64), np.array(es, dtype=np.int32), np.full(len(bits), K, np.int32))
