// Encoders of the compact per-sample form (rpd_sample_soa16, include/rpd_gb300.h), shared by
// rpd_encode_samples16 and the serving loop's sample synthesis.
#pragma once

#include <cuda_fp16.h>

#include <cstdint>

namespace rpd {

__device__ __forceinline__ uint16_t f2h(float v) { return __half_as_ushort(__float2half_rn(v)); }

// sqrt(max(L, 0)) keeps a non-finite radiance non-finite (the sample is then dropped, as the
// reference drops it, main.cpp:707)
__device__ __forceinline__ uint16_t enc_sqrt_radiance(float L) {
    if (!(L == L)) return f2h(L);  // NaN
    return f2h(sqrtf(fmaxf(L, 0.0f)));
}
// snorm16 of a normal component; a NaN component encodes as 0
__device__ __forceinline__ int16_t enc_snorm16(float n) {
    if (!(n == n)) return 0;
    return int16_t(__float2int_rn(fminf(fmaxf(n, -1.0f), 1.0f) * 32767.0f));
}
// unorm16 of a random dimension in [0, 1): floor(u * 65536), clamped to [0, 65535] (a value
// outside [0, 1) lands in the bin the reference's clamp gives it); NaN encodes as 0
__device__ __forceinline__ uint16_t enc_unorm16(float u) {
    if (!(u == u)) return 0;
    const float v = floorf(u * 65536.0f);
    return uint16_t(fminf(fmaxf(v, 0.0f), 65535.0f));
}

}  // namespace rpd
