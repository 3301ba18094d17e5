// variance_denoise (main.cpp:1166-1268): Jacobi iterations of the gated neighbour mean
// with the upward-only update, ping-ponging two planes, then max with the raw variance.
// Single precision throughout, in the reference's order, so the result is bit-identical.
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ float pixel_variance(float m2, int n) { return (n > 1) ? m2 / float(n - 1) : 0.0f; }

__global__ void k_var_init(PixelPlanes p, int64_t np, float max_variance, float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float v = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(v)) v = 1e-8f;
    curr[i] = fclamps(v, 1e-8f, max_variance);
}

struct VarParams {
    int w, h, radius;
    float normal_threshold, depth_threshold, compat_sigma, shrinkage_k;
};

// rpf::conservative_variance_update (core/stats.h:85-91)
__device__ __forceinline__ float conservative_variance_update(float value, float neighbor, float stabilizer) {
    const float blend = fclamps(fmaxs(0.0f, neighbor - value) / fmaxs(1e-8f, value + neighbor + stabilizer), 0.0f, 1.0f);
    return lerp_std(value, neighbor, blend);
}

__global__ void k_var_smooth(PixelPlanes p, VarParams prm, const float* src, float* dst) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(prm.w) * prm.h) return;
    if (p.hit_count[idx] == 0) {
        dst[idx] = src[idx];
        return;
    }
    const int y = int(idx / prm.w), x = int(idx % prm.w);
    const float ni0 = p.f_normal[0][idx], ni1 = p.f_normal[1][idx], ni2 = p.f_normal[2][idx];
    const float depth_i = p.f_depth[idx];
    const float var_i = fmaxs(1e-8f, src[idx]);
    float weight_sum = 0.0f, weighted_sum = 0.0f;
    for (int dy = -prm.radius; dy <= prm.radius; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= prm.h) continue;
        for (int dx = -prm.radius; dx <= prm.radius; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= prm.w || (dx == 0 && dy == 0)) continue;
            const int64_t jn = int64_t(yy) * prm.w + xx;
            if (p.hit_count[jn] == 0) continue;
            if (dot3(ni0, ni1, ni2, p.f_normal[0][jn], p.f_normal[1][jn], p.f_normal[2][jn]) < prm.normal_threshold)
                continue;
            if (relative_depth_delta(depth_i, p.f_depth[jn]) > prm.depth_threshold) continue;
            const float var_j = fmaxs(1e-8f, src[jn]);
            const float relative_difference = fabsf(var_i - var_j) / fmaxs(1e-8f, sqrtf(var_i * var_j));
            if (relative_difference > prm.compat_sigma) continue;
            const float dist2 = float(dx * dx + dy * dy);
            const float w_j = 1.0f / (1.0f + dist2);
            weighted_sum += w_j * var_j;
            weight_sum += w_j;
        }
    }
    float neighbor_mean = var_i;
    if (weight_sum > 1e-8f) neighbor_mean = weighted_sum / weight_sum;
    dst[idx] = conservative_variance_update(var_i, neighbor_mean, prm.shrinkage_k);
}

__global__ void k_var_final(PixelPlanes p, int64_t np, float max_variance, const float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float raw = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(raw)) raw = 1e-8f;
    raw = fclamps(raw, 1e-8f, max_variance);
    p.variance_denoised[i] = fmaxs(curr[i], raw);
}

}  // namespace

cudaError_t launch_variance(Job& j) {
    KernelScope ks(j, RPD_KERNEL_VARIANCE);
    const int64_t np = j.g.np;
    const float max_variance = j.cfg.adaptive_sigma_max * j.cfg.adaptive_sigma_max;
    float* curr = j.p.var_ping;
    float* next = j.p.var_pong;
    k_var_init<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, max_variance, curr);
    VarParams prm{j.g.w, j.g.h, j.cfg.var_window_radius, j.cfg.var_normal_threshold, j.cfg.var_depth_threshold,
                  j.cfg.var_compat_sigma, j.cfg.var_shrinkage_k};
    for (int it = 0; it < j.cfg.var_iterations; ++it) {
        k_var_smooth<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, prm, curr, next);
        float* t = curr;
        curr = next;
        next = t;
    }
    k_var_final<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, max_variance, curr);
    j.launches += 2 + j.cfg.var_iterations;
    return cudaGetLastError();
}

}  // namespace rpd
