// Device-side scalar helpers with the reference's semantics.
//
// The denoise stage is compiled with -fmad=false and IEEE division / square root, so
// every float and double expression below rounds exactly like the reference's x86-64
// build: no fused multiply-add, operations in source order. std::max / std::min /
// std::clamp keep their NaN behaviour ((a < b) ? b : a and so on), and 3-vector
// reductions use Eigen's scalar order c0 + (c1 + c2).
#pragma once

#include <cstdint>

namespace rpd {

__device__ __forceinline__ float fmaxs(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float fmins(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float fclamps(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
__device__ __forceinline__ double dmaxs(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double dclamps(double v, double lo, double hi) {
    return (v < lo) ? lo : ((hi < v) ? hi : v);
}
__device__ __forceinline__ int imaxs(int a, int b) { return (a < b) ? b : a; }
__device__ __forceinline__ int imins(int a, int b) { return (b < a) ? b : a; }
__device__ __forceinline__ int iclamps(int v, int lo, int hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

// The template lerp of shared/global.h:45-48, which the reference calls for Vec3f only
// (main.cpp:1115).
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }
// The reference's lerp(float, float, float) calls (main.cpp:196,869-879, core/buffers.h:84-86,
// core/stats.h:90) resolve to std::lerp: stb_image.h (included with its implementation by
// shared/image.h:10-11) includes <math.h>, whose C++20 libstdc++ form exports std::lerp to
// the global namespace, and the non-template float overload wins. The C++20 algorithm
// (P0811R3) as libstdc++ evaluates it: t*b + (1-t)*a when a and b do not share a sign, b
// exactly at t == 1, otherwise a + t*(b-a) kept from passing b.
__device__ __forceinline__ float lerp_std(float a, float b, float t) {
    if ((a <= 0.0f && b >= 0.0f) || (a >= 0.0f && b <= 0.0f)) return __fadd_rn(__fmul_rn(t, b), __fmul_rn(1.0f - t, a));
    if (t == 1.0f) return b;
    const float x = __fadd_rn(a, __fmul_rn(t, b - a));
    if ((t > 1.0f) == (b > a)) return (b < x) ? x : b;
    return (b > x) ? x : b;
}

__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
    return a0 * b0 + (a1 * b1 + a2 * b2);
}
__device__ __forceinline__ float norm3(float a0, float a1, float a2) { return sqrtf(dot3(a0, a1, a2, a0, a1, a2)); }

// calc_luminance (core/common.h:39-41)
__device__ __forceinline__ float luminance(float r, float g, float b) {
    return 0.2126f * r + 0.7152f * g + 0.0722f * b;
}

// relative_depth_delta (main.cpp:266-268): |a-b| / max({|a|, |b|, EPS_SMALL})
__device__ __forceinline__ float relative_depth_delta(float a, float b) {
    float m = fabsf(a);
    if (m < fabsf(b)) m = fabsf(b);
    if (m < 1e-8f) m = 1e-8f;
    return fabsf(a - b) / m;
}

__device__ __forceinline__ bool finite3(float a, float b, float c) {
    return isfinite(a) && isfinite(b) && isfinite(c);
}

}  // namespace rpd
