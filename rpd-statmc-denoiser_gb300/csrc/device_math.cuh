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

// lerp (shared/global.h:45-48)
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + (b - a) * t; }

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
