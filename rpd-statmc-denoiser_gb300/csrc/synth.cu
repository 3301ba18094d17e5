// Device fill of the synthetic per-sample generator (include/rpd_synth.h). The same
// header-only code runs on the host (oracle/synth_host.c, rpd_synth_fill with host
// memory) and here; built without FMA contraction, both produce identical samples.
#include "rpd_internal.h"
#include "device_math.cuh"
#include "rpd_synth.h"

namespace rpd {

namespace {

struct SynthOut {
    float* radiance[3];
    float* normal[3];
    float* depth;
    float* albedo[3];
    float* pixel_albedo[3];
    float* pixel_u[2];
    float* lens_u[2];
    float* brdf_u[2];
    float* light_u[2];
    uint8_t* flags;
    uint8_t* category;
};

__global__ void k_synth_pixels(rpd_synth_params prm, const rpd_synth_region* table, int64_t first, int64_t count,
                               int32_t* region_of, SynthOut o) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int64_t pix = first + i;
    const int x = int(pix % prm.width), y = int(pix / prm.width);
    const int r = rpd_synth_pixel_region(&prm, table, x, y);
    region_of[i] = r;
    if (o.pixel_albedo[0])
        for (int c = 0; c < 3; ++c) o.pixel_albedo[c][i] = table[r].albedo[c];
}

// One thread per sample; the owning pixel is found by binary search over the offsets.
__global__ void k_synth_samples(rpd_synth_params prm, const rpd_synth_region* table, int64_t first, int64_t count,
                                const int64_t* offsets, const int32_t* start_n, const int32_t* region_of,
                                SynthOut o) {
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = offsets[count];
    if (k >= total) return;
    int64_t lo = 0, hi = count - 1;
    while (lo < hi) {  // last pixel whose offset <= k
        const int64_t mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= k) lo = mid; else hi = mid - 1;
    }
    const int64_t i = lo;
    const int64_t pix = first + i;
    const int x = int(pix % prm.width), y = int(pix / prm.width);
    const rpd_synth_region* reg = &table[region_of[i]];
    const uint32_t ordinal = uint32_t(start_n ? start_n[i] : 0) + uint32_t(k - offsets[i]);
    rpd_synth_sample s;
    rpd_synth_sample_make(&prm, reg, x, y, ordinal, &s);
    for (int c = 0; c < 3; ++c) {
        o.radiance[c][k] = s.radiance[c];
        o.normal[c][k] = s.normal[c];
    }
    o.depth[k] = s.depth;
    for (int c = 0; c < 2; ++c) {
        o.pixel_u[c][k] = s.pixel_u[c];
        o.lens_u[c][k] = s.lens_u[c];
        o.brdf_u[c][k] = s.brdf_u[c];
        o.light_u[c][k] = s.light_u[c];
    }
    o.flags[k] = s.flags;
    o.category[k] = s.category;
    if (o.albedo[0])
        for (int c = 0; c < 3; ++c) o.albedo[c][k] = reg->albedo[c];
}

}  // namespace

// Generates samples for pixels [first, first+count) into device planes. offsets holds
// count+1 exclusive offsets in HBM; region_of is count int32 of scratch.
cudaError_t launch_synth(const rpd_synth_params& prm, const rpd_synth_region* d_table, int64_t first, int64_t count,
                         const int64_t* d_offsets, int64_t total, const int32_t* d_start_n, int32_t* d_region_of,
                         const rpd_sample_soa& out, cudaStream_t stream) {
    SynthOut o;
    for (int c = 0; c < 3; ++c) {
        o.radiance[c] = const_cast<float*>(out.radiance[c]);
        o.normal[c] = const_cast<float*>(out.normal[c]);
        o.albedo[c] = const_cast<float*>(out.albedo[c]);
        o.pixel_albedo[c] = const_cast<float*>(out.pixel_albedo[c]);
    }
    o.depth = const_cast<float*>(out.depth);
    for (int c = 0; c < 2; ++c) {
        o.pixel_u[c] = const_cast<float*>(out.pixel_u[c]);
        o.lens_u[c] = const_cast<float*>(out.lens_u[c]);
        o.brdf_u[c] = const_cast<float*>(out.brdf_u[c]);
        o.light_u[c] = const_cast<float*>(out.light_u[c]);
    }
    o.flags = const_cast<uint8_t*>(out.flags);
    o.category = const_cast<uint8_t*>(out.category);
    k_synth_pixels<<<grid_for(count, 256), 256, 0, stream>>>(prm, d_table, first, count, d_region_of, o);
    if (total > 0)
        k_synth_samples<<<grid_for(total, 256), 256, 0, stream>>>(prm, d_table, first, count, d_offsets, d_start_n,
                                                                  d_region_of, o);
    return cudaGetLastError();
}

}  // namespace rpd
