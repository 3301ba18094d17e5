// rpd_encode_samples16: device-side conversion of rpd_sample_soa planes into the compact
// rpd_sample_soa16 form (include/rpd_gb300.h) that rpd_job_push_samples16 decodes.
#include <cuda_fp16.h>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "compact.cuh"

namespace rpd {

namespace {

__global__ void k_encode_samples16(DeviceSamples in, int64_t n_samples, DeviceSamples16 out) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n_samples) return;
    for (int c = 0; c < 3; ++c) {
        const_cast<uint16_t*>(out.sqrt_radiance[c])[k] = enc_sqrt_radiance(in.radiance[c][k]);
        const_cast<int16_t*>(out.normal[c])[k] = enc_snorm16(in.normal[c][k]);
    }
    const_cast<uint16_t*>(out.depth)[k] = f2h(in.depth[k] / out.depth_scale);
    for (int c = 0; c < 2; ++c) {
        if (in.pixel_u[0]) const_cast<uint16_t*>(out.pixel_u[c])[k] = enc_unorm16(in.pixel_u[c][k]);
        if (in.lens_u[0]) const_cast<uint16_t*>(out.lens_u[c])[k] = enc_unorm16(in.lens_u[c][k]);
        if (in.brdf_u[0]) const_cast<uint16_t*>(out.brdf_u[c])[k] = enc_unorm16(in.brdf_u[c][k]);
        if (in.light_u[0]) const_cast<uint16_t*>(out.light_u[c])[k] = enc_unorm16(in.light_u[c][k]);
        if (in.env_u[0]) const_cast<uint16_t*>(out.env_u[c])[k] = enc_unorm16(in.env_u[c][k]);
    }
}

__global__ void k_encode_albedo16(const float* a0, const float* a1, const float* a2, int64_t n_pixels,
                                  DeviceSamples16 out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_pixels) return;
    const_cast<uint16_t*>(out.pixel_albedo[0])[i] = f2h(a0[i]);
    const_cast<uint16_t*>(out.pixel_albedo[1])[i] = f2h(a1[i]);
    const_cast<uint16_t*>(out.pixel_albedo[2])[i] = f2h(a2[i]);
}

}  // namespace

cudaError_t launch_encode_samples16(const DeviceSamples& in, int64_t n_samples, int64_t n_pixels,
                                    const DeviceSamples16& out, cudaStream_t stream) {
    if (n_samples > 0) k_encode_samples16<<<grid_for(n_samples, 256), 256, 0, stream>>>(in, n_samples, out);
    if (n_pixels > 0 && in.pixel_albedo[0] && out.pixel_albedo[0])
        k_encode_albedo16<<<grid_for(n_pixels, 256), 256, 0, stream>>>(in.pixel_albedo[0], in.pixel_albedo[1],
                                                                       in.pixel_albedo[2], n_pixels, out);
    return cudaGetLastError();
}

}  // namespace rpd
