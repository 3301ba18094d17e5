"""The importance smoothing's integer arithmetic (csrc/k_adaptive.cu: float_parts, xd_mul24,
xd_exact48, quotient_to_float) restated in Python integers and checked against IEEE 754
arithmetic (numpy float64 and float32): the weight products of three floats, the products with
the importance (summed as doubles, as the kernel sums them) and the final float(accum /
weight_sum), on operands across wide exponent ranges and on quotients at float midpoints. The
kernel itself is compared with the double-precision path in tests/test_gpu_smoothing.py."""
from __future__ import annotations

import struct

import numpy as np

M64 = (1 << 64) - 1


def float_parts(f: float):
    b = struct.unpack("<I", struct.pack("<f", f))[0]
    eb = b >> 23
    return ((b & 0x7FFFFF) | 0x800000, eb - 150, eb != 0 and eb < 255)


def xd_round(r: int, rem: int, half: int, e: int):
    if rem > half or (rem == half and (r & 1)):
        r += 1
        if r == 1 << 53:
            r >>= 1
            e += 1
    return (r, e)


def clz64(v: int) -> int:
    return 64 - v.bit_length()


def xd_mul24(a: int, b: int, e: int):
    lo1 = (a & 0xFFFFFFFF) * b
    mid = (a >> 32) * b
    lo = (lo1 + (mid << 32)) & M64
    hi = (mid >> 32) + (1 if lo < lo1 else 0)
    assert (1 << 5) <= hi < (1 << 13)
    s = 75 - clz64(hi)
    r = ((hi << (64 - s)) & M64) | (lo >> s)
    return xd_round(r, lo & ((1 << s) - 1), 1 << (s - 1), e + s)


def xd_exact48(a: int, e: int):
    sh = clz64(a) - 11
    return (a << sh, e - sh)


def quotient_to_float(am: int, ae: int, wm: int, we: int):
    q0 = np.float32(np.float32(am >> 29) / np.float32(wm >> 29))
    qb = struct.unpack("<I", struct.pack("<f", float(q0)))[0]
    qm, qe = (qb & 0x7FFFFF) | 0x800000, (qb >> 23) - 150
    r = ((am << (-qe)) - qm * wm) & M64
    r = r - (1 << 64) if r >> 63 else r
    assert abs(r) < 8 * wm
    u = np.float32(np.float32(r) / np.float32(wm))
    n = np.rint(u)
    if abs(abs(float(u - n)) - 0.5) < 1.0 / 256.0:
        return None
    M = qm + int(n)
    if M < (1 << 23) or M >= (1 << 24):
        return None
    be = qe + ae - we + 150
    if be < 1 or be > 254:
        return None
    return struct.unpack("<f", struct.pack("<I", (be << 23) | (M & 0x7FFFFF)))[0]


def value(x) -> float:
    return float(x[0]) * 2.0 ** x[1] if x[0] else 0.0


def parts_of_double(d: float):
    b = struct.unpack("<Q", struct.pack("<d", d))[0]
    return ((b & ((1 << 52) - 1)) | (1 << 52), ((b >> 52) & 0x7FF) - 1075)


def weight(sw: float, nw: float, dw: float):
    sm, se, _ = float_parts(sw)
    nm, ne, _ = float_parts(nw)
    dm, de, _ = float_parts(dw)
    if sm == 0x800000:
        return xd_exact48(nm * dm, ne + de + se + 23)
    return xd_mul24(sm * nm, dm, se + ne + de)


def rnd(rng, lo, hi):
    return float(np.float32(rng.uniform(lo, hi)))


def test_weights_and_products_match_ieee_double():
    rng = np.random.default_rng(7)
    spatial = [float(np.float32(1.0) / np.float32(1.0 + d2)) for d2 in (0, 1, 2, 4, 5, 8, 9, 10, 13, 18)]
    for _ in range(5000):
        acc, xacc = np.float64(0.0), np.float64(0.0)
        for _ in range(int(rng.integers(1, 10))):
            sw = spatial[int(rng.integers(len(spatial)))]
            nw = rnd(rng, 2.0**-25, 1.0) if rng.random() < 0.9 else float(np.float32(rng.integers(1, 64) / 64.0))
            dw = float(np.float32(np.exp(np.float32(-4.0 * rng.uniform(0, 2)))))
            imp = float(np.float32(10.0 ** rng.uniform(-4, 0.7)))
            wn = weight(sw, nw, dw)
            want_w = (np.float64(sw) * np.float64(nw)) * np.float64(dw)
            assert value(wn) == want_w, (sw, nw, dw)
            im, ie, _ = float_parts(imp)
            pv = xd_mul24(wn[0], im, wn[1] + ie)
            assert value(pv) == want_w * np.float64(imp)
            acc = acc + want_w * np.float64(imp)
            xacc = xacc + np.float64(value(pv))
            assert xacc == acc


def test_quotient_matches_double_then_float_rounding():
    rng = np.random.default_rng(13)
    fallbacks = 0
    trials = 40000
    for i in range(trials):
        if i % 4 == 0:  # quotients on or next to float midpoints
            q = np.float32(rng.uniform(0.1, 4.0))
            w = np.float64(rng.uniform(0.5, 9.0))
            a = (np.float64(q) + np.float64(np.spacing(q)) * rng.choice([0.5, 0.5 + 2.0**-30, 0.5 - 2.0**-30, 0.0])) * w
        else:
            a, w = np.float64(10.0 ** rng.uniform(-4, 2)), np.float64(10.0 ** rng.uniform(-2, 1))
        am, ae = parts_of_double(float(a))
        wm, we = parts_of_double(float(w))
        got = quotient_to_float(am, ae, wm, we)
        want = np.float32(a / w)
        if got is None:
            fallbacks += 1
        else:
            assert np.float32(got) == want, (a, w, got, want)
    assert fallbacks < trials // 4 + trials // 50  # the constructed midpoints and about 1/128 of the rest

