// statmc_denoise (main.cpp:957-1162): the per-channel square-root-domain Welch
// compatibility window with the RPD relaxation.
//
//   k_sqrt_var_mean    sqrt-domain variance of the mean, floored at EPS_SMALL (972-980)
//   k_sqrt_var_stable  max with its 3x3 inverse-distance average (981-990)
//   k_statmc_window    the (2r+1)^2 window (998-1127) — one thread per pixel, the
//                      reference's operations in its order (double where it uses double),
//                      so every gate and the q > 25 test decide exactly as the reference.
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

__constant__ float c_t05[30] = {
    12.706f, 4.303f, 3.182f, 2.776f, 2.571f, 2.447f, 2.365f, 2.306f, 2.262f, 2.228f,
    2.201f, 2.179f, 2.160f, 2.145f, 2.131f, 2.120f, 2.110f, 2.101f, 2.093f, 2.086f,
    2.080f, 2.074f, 2.069f, 2.064f, 2.060f, 2.056f, 2.052f, 2.048f, 2.045f, 2.042f};
__constant__ float c_t01[30] = {
    63.657f, 9.925f, 5.841f, 4.604f, 4.032f, 3.707f, 3.499f, 3.355f, 3.250f, 3.169f,
    3.106f, 3.055f, 3.012f, 2.977f, 2.947f, 2.921f, 2.898f, 2.878f, 2.861f, 2.845f,
    2.831f, 2.819f, 2.807f, 2.797f, 2.787f, 2.779f, 2.771f, 2.763f, 2.756f, 2.750f};

__device__ __forceinline__ float interpolate_table(const float* table, float df) {
    const int lo = iclamps(int(floorf(df)), 1, 30);
    const int hi = iclamps(int(ceilf(df)), 1, 30);
    if (lo == hi) return table[lo - 1];
    return lerpf(table[lo - 1], table[hi - 1], (df - float(lo)) / float(hi - lo));
}

// lookup_t_critical (main.cpp:188-231)
__device__ float lookup_t_critical(float df, float alpha) {
    df = fmaxs(df, 1.0f);
    alpha = fclamps(alpha, 1e-8f, 0.999999f);
    if (df < 30.5f && fabsf(alpha - 0.05f) < 1e-4f) return interpolate_table(c_t05, df);
    if (df < 30.5f && fabsf(alpha - 0.01f) < 1e-4f) return interpolate_table(c_t01, df);
    float z;
    if (alpha <= 0.001f) z = 3.29f;
    else if (alpha <= 0.005f) z = 2.81f;
    else if (alpha <= 0.01f) z = 2.58f;
    else if (alpha <= 0.02f) z = 2.33f;
    else if (alpha <= 0.05f) z = 1.96f;
    else if (alpha <= 0.10f) z = 1.64f;
    else z = 1.28f;
    if (df < 30.0f) {
        const float adj = sqrtf(df / fmaxs(1.0f, df - 1.0f));
        z *= adj;
    }
    return z;
}

__device__ __forceinline__ float pixel_variance(float m2, int n) {  // core/stats.h:14-16
    return (n > 1) ? m2 / float(n - 1) : 0.0f;
}

__global__ void k_sqrt_var_mean(PixelPlanes p, int64_t np) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int n = p.n[i];
    for (int c = 0; c < 3; ++c) {
        const float var = (n <= 1) ? 0.0f : p.sqrt_sq[c][i] / float(n - 1);
        p.sqrt_var_mean[c][i] = fmaxs(var / float(imaxs(1, n)), 1e-8f);
    }
}

__global__ void k_sqrt_var_stable(PixelPlanes p, int w, int h) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(w) * h) return;
    const int cy = int(i / w), cx = int(i % w);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, weight_sum = 0.0;
    for (int dy = -1; dy <= 1; ++dy) {
        const int y = iclamps(cy + dy, 0, h - 1);
        for (int dx = -1; dx <= 1; ++dx) {
            const int x = iclamps(cx + dx, 0, w - 1);
            const double weight = 1.0 / (1.0 + double(dx * dx + dy * dy));
            const int64_t q = int64_t(y) * w + x;
            a0 += double(p.sqrt_var_mean[0][q]) * weight;
            a1 += double(p.sqrt_var_mean[1][q]) * weight;
            a2 += double(p.sqrt_var_mean[2][q]) * weight;
            weight_sum += weight;
        }
    }
    const float avg[3] = {float(a0 / weight_sum), float(a1 / weight_sum), float(a2 / weight_sum)};
    for (int c = 0; c < 3; ++c) p.sqrt_var_stable[c][i] = fmaxs(p.sqrt_var_mean[c][i], avg[c]);
}

struct StatmcParams {
    int w, h, r;
    float normal_threshold, depth_threshold, rpd_scale, alpha, var2_max;
};

__global__ void __launch_bounds__(128) k_statmc_window(PixelPlanes p, StatmcParams prm) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(prm.w) * prm.h) return;
    const int y = int(idx / prm.w), x = int(idx % prm.w);
    const int n_raw = p.n[idx];
    const float m2_i = p.square_diff[idx];
    if (p.hit_count[idx] == 0) {
        for (int c = 0; c < 3; ++c) p.denoised[c][idx] = p.color_mean[c][idx];
        p.uncertainty[idx] = pixel_variance(m2_i, n_raw) / float(imaxs(1, n_raw));
        p.alpha[idx] = 1.0f;
        return;
    }
    const float ni0 = p.f_normal[0][idx], ni1 = p.f_normal[1][idx], ni2 = p.f_normal[2][idx];
    const float depth_i = p.f_depth[idx];
    const float ai0 = p.f_albedo[0][idx], ai1 = p.f_albedo[1][idx], ai2 = p.f_albedo[2][idx];
    float var_i = pixel_variance(m2_i, n_raw);
    if (!isfinite(var_i)) var_i = 1e-8f;
    var_i = fclamps(var_i, 1e-8f, prm.var2_max);
    const int n_i = imaxs(1, n_raw);
    float rpd_i[6];
    for (int c = 0; c < 6; ++c) rpd_i[c] = p.rpd[c][idx];
    const float var_mean_i = fmaxs(1e-8f, var_i / float(n_i));
    const float smi[3] = {p.sqrt_mean[0][idx], p.sqrt_mean[1][idx], p.sqrt_mean[2][idx]};
    const float svi[3] = {p.sqrt_var_stable[0][idx], p.sqrt_var_stable[1][idx], p.sqrt_var_stable[2][idx]};
    p.var_total[idx] = var_i;
    p.var_eff[idx] = var_mean_i;
    p.var_ratio[idx] = (var_i > 1e-8f) ? (var_mean_i * float(n_i)) / var_i : 0.0f;

    double weight_sum = 0.0, weight_square_sum = 0.0, weighted_variance_sum = 0.0;
    double cs0 = 0.0, cs1 = 0.0, cs2 = 0.0, accepted = 0.0;
    const double center_weight = 1.0;
    const int r = prm.r;
    for (int dy = -r; dy <= r; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= prm.h) continue;
        for (int dx = -r; dx <= r; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= prm.w) continue;
            const int64_t jn = int64_t(yy) * prm.w + xx;
            if (p.hit_count[jn] == 0) continue;
            if (dot3(ni0, ni1, ni2, p.f_normal[0][jn], p.f_normal[1][jn], p.f_normal[2][jn]) < prm.normal_threshold)
                continue;
            if (relative_depth_delta(depth_i, p.f_depth[jn]) > prm.depth_threshold) continue;
            if (norm3(ai0 - p.f_albedo[0][jn], ai1 - p.f_albedo[1][jn], ai2 - p.f_albedo[2][jn]) > 0.12f) continue;
            const int n_rawj = p.n[jn];
            float var_j = pixel_variance(p.square_diff[jn], n_rawj);
            if (!isfinite(var_j)) var_j = 1e-8f;
            var_j = fclamps(var_j, 1e-8f, prm.var2_max);
            const int n_j = imaxs(1, n_rawj);
            const float var_mean_j = fmaxs(1e-8f, var_j / float(n_j));
            double max_t2 = 0.0;
            for (int c = 0; c < 3; ++c) {
                const double v_i = double(svi[c]);
                const double v_j = double(p.sqrt_var_stable[c][jn]);
                const double variance_sum = v_i + v_j;
                const double mean_diff = double(smi[c] - p.sqrt_mean[c][jn]);
                const double t2 = mean_diff * mean_diff / dmaxs(double(1e-8f), variance_sum);
                const double denom_df = (v_i * v_i) / dmaxs(double(n_i - 1), 1.0) +
                                        (v_j * v_j) / dmaxs(double(n_j - 1), 1.0);
                const double df = (denom_df > double(1e-8f)) ? (variance_sum * variance_sum) / denom_df
                                                             : double(n_i + n_j - 2);
                const double t_crit = double(lookup_t_critical(float(df), prm.alpha));
                max_t2 = dmaxs(max_t2, t2 / (t_crit * t_crit));
            }
            // rpf::shared_reliability + relax_compatibility (core/stats.h:56-78)
            float shared = 0.0f;
            for (int c = 0; c < 6; ++c) shared = fmaxs(shared, fmins(rpd_i[c], p.rpd[c][jn]));
            shared = fclamps(shared, 0.0f, 1.0f);
            const float adjustment = fclamps(prm.rpd_scale * shared, 0.0f, 1.0f);
            const double q = max_t2 / (1.0 + double(adjustment));
            if (q > 25.0) continue;
            const double dist2 = double(dx * dx + dy * dy);
            const double spatial_w = 1.0 / (1.0 + dist2);
            const double weight_j = spatial_w * exp(-0.5 * q);
            cs0 += double(p.color_mean[0][jn]) * weight_j;
            cs1 += double(p.color_mean[1][jn]) * weight_j;
            cs2 += double(p.color_mean[2][jn]) * weight_j;
            weight_sum += weight_j;
            weight_square_sum += weight_j * weight_j;
            weighted_variance_sum += weight_j * weight_j * double(var_mean_j);
            if ((dx != 0 || dy != 0) && weight_j > 0.05 * spatial_w) accepted += 1.0;
        }
    }
    const float cmi[3] = {p.color_mean[0][idx], p.color_mean[1][idx], p.color_mean[2][idx]};
    float mean_nb[3] = {cmi[0], cmi[1], cmi[2]};
    double var_neighbors = double(var_mean_i);
    if (weight_sum > double(1e-8f)) {
        mean_nb[0] = float(cs0 / weight_sum);
        mean_nb[1] = float(cs1 / weight_sum);
        mean_nb[2] = float(cs2 / weight_sum);
        var_neighbors = weighted_variance_sum / (weight_sum * weight_sum);
    }
    const double effective = weight_sum * weight_sum / dmaxs(double(1e-8f), weight_square_sum);
    const double blend = (accepted >= 2.0 && weight_sum >= 1.1 * center_weight)
                             ? dclamps(1.0 - 1.0 / sqrt(effective), 0.0, 0.8) : 0.0;
    const float alpha = float(1.0 - blend);
    const float fb = float(blend);
    for (int c = 0; c < 3; ++c) p.denoised[c][idx] = lerpf(cmi[c], mean_nb[c], fb);
    const float uncertainty = float(double(alpha) * double(alpha) * double(var_mean_i) +
                                    blend * blend * var_neighbors +
                                    2.0 * double(alpha) * blend * (center_weight / dmaxs(weight_sum, double(1e-8f))) *
                                        double(var_mean_i));
    p.alpha[idx] = alpha;
    p.uncertainty[idx] = uncertainty;
}

}  // namespace

cudaError_t launch_statmc(Job& j) {
    const int64_t np = j.g.np;
    {
        KernelScope ks(j, RPD_KERNEL_SQRT_VARIANCE);
        k_sqrt_var_mean<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np);
        k_sqrt_var_stable<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, j.g.w, j.g.h);
    }
    KernelScope ks(j, RPD_KERNEL_STATMC_WINDOW);
    StatmcParams prm{j.g.w, j.g.h, j.cfg.color_window_radius, j.cfg.color_normal_threshold,
                     j.cfg.color_depth_threshold, j.cfg.rpf_shrinkage_scale, j.cfg.color_compat_alpha,
                     j.cfg.color_sigma_max * j.cfg.color_sigma_max};
    k_statmc_window<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, prm);
    j.launches += 3;
    return cudaGetLastError();
}

}  // namespace rpd
