// The two standalone post-filters of denoising/.
//
//   k_atrous_pass      atrous_filter_pass (denoising/atrous_wavelet.cpp:54-149): 25-tap B3
//                      spline at step 2^iter with luminance, normal-angle and albedo
//                      edge stopping, clamp-to-edge; the host ping-pongs `iterations` passes
//                      (185-197).
//   k_joint_bilateral  the filter() loop of denoising/joint_bilateral.cpp:43-132: one
//                      (2r+1)^2 pass, r = max(1, ceil(3 sigma_p)), writing the gaussian,
//                      colour-bilateral and joint outputs together.
// Both read interleaved RGB float images (the HDR layout of the reference) and keep its
// single-precision arithmetic; exp/acos are CUDA's (within 2 ulp of the C library's).
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ void filt_normalize(float& x, float& y, float& z) {
    const float len_sq = x * x + y * y + z * z;
    if (len_sq > 1e-8f) {
        const float inv_len = 1.0f / sqrtf(len_sq);
        x *= inv_len;
        y *= inv_len;
        z *= inv_len;
    }
}

__constant__ float c_h[5] = {1 / 16.0f, 1 / 4.0f, 3 / 8.0f, 1 / 4.0f, 1 / 16.0f};

__global__ void k_atrous_pass(const float* __restrict__ input, float* __restrict__ output,
                              const float* __restrict__ normal, const float* __restrict__ albedo, int w, int h,
                              int step_width, float sigma_c, float sigma_n, float sigma_a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const int idx = y * w + x;
    const float c_r = input[3 * idx], c_g = input[3 * idx + 1], c_b = input[3 * idx + 2];
    const float c_lum = luminance(c_r, c_g, c_b);
    float n_r = normal[3 * idx], n_g = normal[3 * idx + 1], n_b = normal[3 * idx + 2];
    filt_normalize(n_r, n_g, n_b);
    const float a_r = albedo[3 * idx], a_g = albedo[3 * idx + 1], a_b = albedo[3 * idx + 2];
    const float inv_c = 2.0f * sigma_c * sigma_c;
    const float inv_n = 2.0f * sigma_n * sigma_n;
    const float inv_a = 2.0f * sigma_a * sigma_a;
    float sum_r = 0.0f, sum_g = 0.0f, sum_b = 0.0f, sum_weight = 0.0f;
    for (int k = 0; k < 25; ++k) {
        const int kx = k % 5 - 2, ky = k / 5 - 2;
        const int nx = iclamps(x + kx * step_width, 0, w - 1);
        const int ny = iclamps(y + ky * step_width, 0, h - 1);
        const int n_idx = ny * w + nx;
        const float p_r = input[3 * n_idx], p_g = input[3 * n_idx + 1], p_b = input[3 * n_idx + 2];
        const float p_lum = luminance(p_r, p_g, p_b);
        float pn_r = normal[3 * n_idx], pn_g = normal[3 * n_idx + 1], pn_b = normal[3 * n_idx + 2];
        filt_normalize(pn_r, pn_g, pn_b);
        const float w_spatial = c_h[ky + 2] * c_h[kx + 2];
        const float lum_diff = c_lum - p_lum;
        const float w_color = expf(-lum_diff * lum_diff / inv_c);
        float dot_n = n_r * pn_r + n_g * pn_g + n_b * pn_b;
        dot_n = fclamps(dot_n, -1.0f, 1.0f);
        const float angle = acosf(dot_n);
        const float w_normal = expf(-angle * angle / inv_n);
        const float da_r = a_r - albedo[3 * n_idx], da_g = a_g - albedo[3 * n_idx + 1], da_b = a_b - albedo[3 * n_idx + 2];
        const float dist_sq_albedo = da_r * da_r + da_g * da_g + da_b * da_b;
        const float w_albedo = expf(-dist_sq_albedo / inv_a);
        const float weight = w_spatial * w_color * w_normal * w_albedo;
        sum_r += weight * p_r;
        sum_g += weight * p_g;
        sum_b += weight * p_b;
        sum_weight += weight;
    }
    if (sum_weight > 1e-8f) {
        output[3 * idx] = sum_r / sum_weight;
        output[3 * idx + 1] = sum_g / sum_weight;
        output[3 * idx + 2] = sum_b / sum_weight;
    } else {
        output[3 * idx] = c_r;
        output[3 * idx + 1] = c_g;
        output[3 * idx + 2] = c_b;
    }
}

__global__ void k_joint_bilateral(const float* __restrict__ raw, const float* __restrict__ normal,
                                  const float* __restrict__ albedo, int w, int h, int radius, float sigma_c,
                                  float sigma_n, float sigma_p, float sigma_a, float* __restrict__ gaussian,
                                  float* __restrict__ bilateral, float* __restrict__ joint) {
    const int jx = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (jx >= w || i >= h) return;
    const int ci = 3 * (i * w + jx);
    const float red = raw[ci], green = raw[ci + 1], blue = raw[ci + 2];
    float n_i_r = normal[ci] * 2.0f - 1.0f;
    float n_i_g = normal[ci + 1] * 2.0f - 1.0f;
    float n_i_b = normal[ci + 2] * 2.0f - 1.0f;
    filt_normalize(n_i_r, n_i_g, n_i_b);
    const float a_i_r = albedo[ci], a_i_g = albedo[ci + 1], a_i_b = albedo[ci + 2];
    const float sp = 2.0f * sigma_p * sigma_p;
    const float sc = 2.0f * sigma_c * sigma_c;
    const float sn = 2.0f * sigma_n * sigma_n;
    const float sa = 2.0f * sigma_a * sigma_a;
    float ws_g = 0.0f, vr_g = 0.0f, vg_g = 0.0f, vb_g = 0.0f;
    float ws_c = 0.0f, vr_c = 0.0f, vg_c = 0.0f, vb_c = 0.0f;
    float ws_j = 0.0f, vr_j = 0.0f, vg_j = 0.0f, vb_j = 0.0f;
    for (int y = i - radius; y < i + radius + 1; ++y) {
        for (int x = jx - radius; x < jx + radius + 1; ++x) {
            const int c = int(fmins(fmaxs(0.0f, float(y)), float(h) - 1));
            const int r = int(fmins(fmaxs(0.0f, float(x)), float(w) - 1));
            const float dist_square_pixel = float((i - c) * (i - c) + (jx - r) * (jx - r));
            const int q = 3 * (c * w + r);
            const float rr = raw[q], rg = raw[q + 1], rb = raw[q + 2];
            const float red_diff = red - rr, green_diff = green - rg, blue_diff = blue - rb;
            float dist_square_color = red_diff * red_diff + green_diff * green_diff + blue_diff * blue_diff;
            dist_square_color *= 0.5f;
            float n_j_r = normal[q] * 2.0f - 1.0f;
            float n_j_g = normal[q + 1] * 2.0f - 1.0f;
            float n_j_b = normal[q + 2] * 2.0f - 1.0f;
            filt_normalize(n_j_r, n_j_g, n_j_b);
            const float ar = a_i_r - albedo[q], ag = a_i_g - albedo[q + 1], ab = a_i_b - albedo[q + 2];
            const float dist_square_albedo = ar * ar + ag * ag + ab * ab;
            float dot_product = n_i_r * n_j_r + n_i_g * n_j_g + n_i_b * n_j_b;
            dot_product = fclamps(dot_product, -1.0f, 1.0f);
            const float n_val = acosf(dot_product);
            float n_val_square = n_val * n_val;
            n_val_square *= 1.5f;
            const float e_p = -dist_square_pixel / sp;
            const float weight_gauss = expf(e_p);
            const float e_c = e_p - dist_square_color / sc;
            const float weight_color = expf(e_c);
            const float weight_joint = expf(e_c - n_val_square / sn - dist_square_albedo / sa);
            vr_g += weight_gauss * rr;
            vg_g += weight_gauss * rg;
            vb_g += weight_gauss * rb;
            vr_c += weight_color * rr;
            vg_c += weight_color * rg;
            vb_c += weight_color * rb;
            vr_j += weight_joint * rr;
            vg_j += weight_joint * rg;
            vb_j += weight_joint * rb;
            ws_g += weight_gauss;
            ws_c += weight_color;
            ws_j += weight_joint;
        }
    }
    gaussian[ci] = vr_g / ws_g;
    gaussian[ci + 1] = vg_g / ws_g;
    gaussian[ci + 2] = vb_g / ws_g;
    bilateral[ci] = vr_c / ws_c;
    bilateral[ci + 1] = vg_c / ws_c;
    bilateral[ci + 2] = vb_c / ws_c;
    joint[ci] = vr_j / ws_j;
    joint[ci + 1] = vg_j / ws_j;
    joint[ci + 2] = vb_j / ws_j;
}

}  // namespace

cudaError_t launch_atrous(const float* raw, const float* normal, const float* albedo, int w, int h, float sigma_c,
                          float sigma_n, float sigma_a, int iterations, float* buf_a, float* buf_b, float** result,
                          cudaStream_t stream, uint64_t* launches) {
    const dim3 block(32, 8);
    const dim3 grid((w + 31) / 32, (h + 7) / 8);
    const float* in = raw;
    float* out = buf_a;
    float* other = buf_b;
    *result = const_cast<float*>(raw);
    for (int it = 0; it < iterations; ++it) {
        k_atrous_pass<<<grid, block, 0, stream>>>(in, out, normal, albedo, w, h, 1 << it, sigma_c, sigma_n, sigma_a);
        *launches += 1;
        *result = out;
        in = out;
        float* t = out;
        out = other;
        other = t;
    }
    return cudaGetLastError();
}

cudaError_t launch_joint_bilateral(const float* raw, const float* normal, const float* albedo, int w, int h,
                                   float sigma_c, float sigma_n, float sigma_p, float sigma_a, float* gaussian,
                                   float* bilateral, float* joint, cudaStream_t stream, uint64_t* launches) {
    const int radius = std::max(1, int(std::ceil(3.0f * sigma_p)));
    const dim3 block(32, 8);
    const dim3 grid((w + 31) / 32, (h + 7) / 8);
    k_joint_bilateral<<<grid, block, 0, stream>>>(raw, normal, albedo, w, h, radius, sigma_c, sigma_n, sigma_p, sigma_a,
                                                  gaussian, bilateral, joint);
    *launches += 1;
    return cudaGetLastError();
}

}  // namespace rpd
