// Exact IEEE 754 double-precision arithmetic on nonnegative values in integer instructions, for
// kernels that must reproduce the reference's double-precision products, sums and quotients bit
// for bit: GB300 issues double-precision instructions at 2 per SM per clock, integer and
// single-precision ones at up to 128. A positive double is m * 2^e with m in [2^52, 2^53); every
// operation forms its exact result and rounds it to nearest-even as IEEE 754 does. Callers keep
// the values positive, normal and finite (anything else goes to the double-precision operations).
#pragma once

#include <cstdint>

namespace rpd {

struct XD {
    uint64_t m;
    int e;
};

__device__ __forceinline__ XD xd_round(uint64_t r, uint64_t rem, uint64_t half, int e) {
    if (rem > half || (rem == half && (r & 1ull))) {
        ++r;
        if (r == (1ull << 53)) {
            r >>= 1;
            ++e;
        }
    }
    return XD{r, e};
}

// A positive normal float as m * 2^e with m in [2^23, 2^24); false for zero, subnormals,
// negative values, infinities and NaN.
__device__ __forceinline__ bool float_parts(float f, uint32_t& m, int& e) {
    const uint32_t b = __float_as_uint(f);
    const uint32_t eb = b >> 23;  // the sign bit makes a negative value's eb >= 256
    m = (b & 0x7fffffu) | 0x800000u;
    e = int(eb) - 150;
    return eb != 0u && eb < 255u;
}

// a * b * 2^e rounded to 53 bits, for a product a * b in [2^69, 2^77) (a < 2^53, b < 2^24)
__device__ __forceinline__ XD xd_mul24(uint64_t a, uint32_t b, int e) {
    const uint64_t lo1 = (a & 0xffffffffull) * b;
    const uint64_t mid = (a >> 32) * b;
    const uint64_t lo = lo1 + (mid << 32);
    const uint64_t hi = (mid >> 32) + (lo < lo1 ? 1ull : 0ull);  // in [2^5, 2^13)
    const int s = 75 - __clzll(static_cast<long long>(hi));      // top bit - 52, 17..24
    const uint64_t r = (hi << (64 - s)) | (lo >> s);
    return xd_round(r, lo & ((1ull << s) - 1ull), 1ull << (s - 1), e + s);
}

// an exact product a * 2^e of at most 53 bits (a in [2^46, 2^48)) in normal form
__device__ __forceinline__ XD xd_exact48(uint64_t a, int e) {
    const int sh = __clzll(static_cast<long long>(a)) - 11;
    return XD{a << sh, e - sh};
}

__device__ __forceinline__ double xd_to_double(XD a) {
    if (a.m == 0ull) return 0.0;
    return __longlong_as_double((static_cast<long long>(a.e + 1075) << 52) | static_cast<long long>(a.m - (1ull << 52)));
}

// float(a / w) with the quotient rounded to double first, a = am * 2^ae and w = wm * 2^we
// (am, wm in [2^52, 2^53)). A single-precision quotient q0 = qm * 2^qe is within a few ulps of
// t = am / wm; the remainder am * 2^-qe - qm * wm is exact in 64-bit integers, and its ratio to
// wm places t between the float grid points. Where t lies within 2^-8 of an ulp of a midpoint,
// or the result leaves q0's binade or the normal range, it returns false.
__device__ __forceinline__ bool quotient_to_float(uint64_t am, int ae, uint64_t wm, int we, float& out) {
    const float q0 = float(uint32_t(am >> 29)) / float(uint32_t(wm >> 29));
    const uint32_t qb = __float_as_uint(q0);
    const uint32_t qm = (qb & 0x7fffffu) | 0x800000u;
    const int qe = int(qb >> 23) - 150;                                     // -25 .. -22
    const long long r = static_cast<long long>((am << (-qe)) - uint64_t(qm) * wm);  // |r| < 8 wm
    const float u = float(r) / float(wm);
    const float n = rintf(u);
    if (fabsf(fabsf(u - n) - 0.5f) < 1.0f / 256.0f) return false;
    const long long M = static_cast<long long>(qm) + static_cast<long long>(n);
    if (M < (1ll << 23) || M >= (1ll << 24)) return false;
    const int be = qe + ae - we + 150;
    if (be < 1 || be > 254) return false;
    out = __uint_as_float((uint32_t(be) << 23) | (uint32_t(M) & 0x7fffffu));
    return true;
}


// a + b for nonnegative normalised operands (b may be 0)
__device__ __forceinline__ XD xd_add(XD a, XD b) {
    if (b.m == 0ull) return a;
    if (a.m == 0ull) return b;
    if (a.e < b.e) {
        const XD t = a;
        a = b;
        b = t;
    }
    const int d = a.e - b.e;
    if (d >= 54) return a;  // b is below half an ulp of a
    const uint64_t A = a.m << 10;
    uint64_t B = b.m << 10;
    if (d) B = (B >> d) | ((B & ((1ull << d) - 1ull)) ? 1ull : 0ull);  // bits shifted out: sticky
    const uint64_t S = A + B;                                        // below 2^64
    const int k = (S >> 63) ? 11 : 10;
    return xd_round(S >> k, S & ((1ull << k) - 1ull), 1ull << (k - 1), a.e - 10 + k);
}

// the parts of a positive normal double
__device__ __forceinline__ XD xd_of_double(double v) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
    return XD{(b & ((1ull << 52) - 1ull)) | (1ull << 52), int((b >> 52) & 0x7ffull) - 1075};
}

}  // namespace rpd
