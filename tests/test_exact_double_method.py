"""The method of the importance smoothing's integer arithmetic (csrc/k_adaptive.cu, xd_*),
restated in Python integers and checked against IEEE 754 double arithmetic (numpy float64):
products of floats and sums of nonnegative doubles, rounded to nearest-even, on random operands
across wide exponent ranges and on constructed ties. The CUDA kernel itself is compared with the
double-precision instructions in tests/test_gpu_smoothing.py."""
from __future__ import annotations

import struct

import numpy as np

M64 = (1 << 64) - 1


def xd_from_float(f: float) -> tuple[int, int]:
    b = struct.unpack("<I", struct.pack("<f", f))[0]
    if b == 0:
        return (0, 0)
    eb = b >> 23
    if eb:
        return (((b & 0x7FFFFF) | 0x800000) << 29, eb - 179)
    sh = (64 - b.bit_length()) - 11
    return (b << sh, -149 - sh)


def xd_round(r: int, rem: int, half: int, e: int) -> tuple[int, int]:
    if rem > half or (rem == half and (r & 1)):
        r += 1
        if r == 1 << 53:
            r >>= 1
            e += 1
    return (r, e)


def xd_mul(a, b):
    if a[0] == 0 or b[0] == 0:
        return (0, 0)
    p = a[0] * b[0]
    lo, hi = p & M64, p >> 64
    s = 53 if (hi >> 41) else 52
    r = ((hi << (64 - s)) & M64) | (lo >> s)
    return xd_round(r, lo & ((1 << s) - 1), 1 << (s - 1), a[1] + b[1] + s)


def xd_add(a, b):
    if b[0] == 0:
        return a
    if a[0] == 0:
        return b
    if a[1] < b[1]:
        a, b = b, a
    d = a[1] - b[1]
    if d >= 54:
        return a
    A, B = a[0] << 10, b[0] << 10
    if d:
        B = (B >> d) | (1 if B & ((1 << d) - 1) else 0)
    S = A + B
    assert S < 1 << 64
    k = 11 if (S >> 63) else 10
    return xd_round(S >> k, S & ((1 << k) - 1), 1 << (k - 1), a[1] - 10 + k)


def value(x) -> float:
    return float(x[0]) * 2.0 ** x[1] if x[0] else 0.0


def xd_from_double(d: float) -> tuple[int, int]:
    if d == 0:
        return (0, 0)
    m, e = np.frexp(d)
    return (int(m * 2**53), int(e) - 53)


def random_float(rng) -> float:
    k = int(rng.integers(0, 6))
    if k == 0:
        return float(np.float32(rng.uniform(0, 1)))
    if k == 1:
        return float(np.float32(rng.integers(0, 64) / 64.0))
    if k == 2:
        return float(np.float32(10.0 ** rng.uniform(-30, 3)))
    if k == 3:
        return float(np.float32(1.0) / np.float32(1 + rng.integers(0, 20)))  # the spatial weights
    if k == 4:
        return float(np.float32(rng.integers(1, 1 << 24)) * np.float32(2.0 ** rng.integers(-40, 0)))
    return float(np.float32(rng.uniform(0, 4)))


def test_products_and_sums_match_ieee_double():
    rng = np.random.default_rng(7)
    for _ in range(20000):
        a, b, c, d = (random_float(rng) for _ in range(4))
        want_w = (np.float64(a) * np.float64(b)) * np.float64(c)
        got_w = xd_mul(xd_mul(xd_from_float(a), xd_from_float(b)), xd_from_float(c))
        assert value(got_w) == want_w, (a, b, c)
        assert value(xd_mul(got_w, xd_from_float(d))) == want_w * np.float64(d), (a, b, c, d)
        acc, xacc = np.float64(0.0), (0, 0)
        for _ in range(int(rng.integers(1, 10))):
            v = np.float64(random_float(rng)) * np.float64(random_float(rng)) * np.float64(random_float(rng))
            acc = acc + v
            xacc = xd_add(xacc, xd_from_double(v))
            assert value(xacc) == acc


def test_subnormal_floats_convert_exactly():
    for bits in (1, 2, 3, 0x400000, 0x7FFFFF):
        f = struct.unpack("<f", struct.pack("<I", bits))[0]
        assert value(xd_from_float(f)) == np.float64(f)


def test_ties_round_to_even():
    rng = np.random.default_rng(11)
    for _ in range(20000):
        e = int(rng.integers(-60, 10))
        a = np.float64(int(rng.integers(1 << 52, 1 << 53))) * 2.0**e
        k = int(rng.integers(1, 60))
        b = np.float64(int(rng.integers(1 << 52, 1 << 53))) * 2.0 ** (e - k)
        half = np.float64(2.0 ** (e - 1))
        for bb in (b, half, 3 * half, half * (1 + 2.0**-52), half * (1 - 2.0**-53)):
            assert value(xd_add(xd_from_double(a), xd_from_double(bb))) == a + bb, (a, bb)
