// statmc_denoise (main.cpp:957-1162): the per-channel square-root-domain Welch
// compatibility window with the RPD relaxation.
//
//   k_sqrt_var_mean    sqrt-domain variance of the mean, floored at EPS_SMALL (972-980)
//   k_sqrt_var_stable  max with its 3x3 inverse-distance average (981-990); the same pass packs
//                      every pixel's neighbour record into six float4 planes (p.win):
//                        W_GATE (unit normal xyz, depth)      the normal / depth gates
//                        W_ALB  (albedo xyz, 1/max(n-1, 1))   the albedo gate; 0 marks a pixel
//                                                             without a primary hit
//                        W_SM   (sqrt mean rgb, rpd[4])       Welch means
//                        W_SV   (stabilised sqrt var rgb, rpd[5])
//                        W_RPD  (rpd[0..3])                   the RPD relaxation
//                        W_CM   (colour mean rgb, var of the mean) the weighted sums; for a
//                                                             pixel without a hit, its pass-through
//                                                             uncertainty instead
//   k_statmc_tma       the (2r+1)^2 window (998-1127), fast path. A 32 x BY block stages its
//                      (32+2r) x (BY+2r) halo tile of the six planes into shared memory with
//                      one tensor copy (cp.async.bulk.tensor, completion on an mbarrier; the
//                      copy's zero fill past the image edges marks those neighbours invalid)
//                      and evaluates every neighbour in single precision:
//                        * the normal / depth / albedo gates are decided exactly as the
//                          reference decides them (identical float operations; the depth
//                          quotient is only rounded exactly when it lies within 2^-20 of the
//                          threshold; the albedo norm is compared through the exact squared
//                          threshold of the correctly rounded sqrt);
//                        * the Welch t^2, Welch-Satterthwaite df, t critical value and RPD
//                          relaxation run in float with approximate reciprocals (relative
//                          error below 3e-6), and whenever q lies within the guard band
//                          (2^-15 relative by default) of a decision point — q = 25 (reject),
//                          q = 2 ln 20 (the accepted-neighbour count), the df of the t-table /
//                          normal-quantile switch, or the 1e-8 df-denominator test — the
//                          pixel goes on a list for k_statmc_slow (none on the uniform 16-spp
//                          frame; about 0.1 % of the pixels after three adaptive passes, where
//                          mixed counts put some df near the t-table switch);
//                        * each block picks a specialised loop from the range of 1/(n-1) over
//                          its halo: when every pair's df lies below the t-table switch
//                          (df <= (n_i - 1) + (n_j - 1)) no neighbour needs the switch test, and
//                          when every df lies above it (df >= min(n_i, n_j) - 1 >= 31) the t
//                          critical value is the normal quantile and df is not formed at all.
//                      Weights are summed in float per window row and across rows. The blend's
//                      weight_sum >= 1.1 test has its own guard band; a pixel inside it goes
//                      on the list too.
//   k_statmc_slow      the listed pixels, one warp each: the window again with every banded
//                      neighbour's q recomputed in double exactly as the reference computes
//                      it, then the whole pixel in double if its weight sum is still inside
//                      the 1.1 test's band.
//   k_statmc_window    the whole window in double, the reference's operations in its order
//                      (the exact mode, and the path for radii whose halo tile would not fit in
//                      shared memory and for depth thresholds below 1e-21).

#include <algorithm>
#include <cmath>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "exact_arith.cuh"
#include "tma.cuh"

namespace rpd {

namespace {

// The two-sided t critical values of lookup_t_critical (main.cpp:199-212), df = 1..30.
#define RPD_T05                                                                                   \
    12.706f, 4.303f, 3.182f, 2.776f, 2.571f, 2.447f, 2.365f, 2.306f, 2.262f, 2.228f, 2.201f, 2.179f, \
        2.160f, 2.145f, 2.131f, 2.120f, 2.110f, 2.101f, 2.093f, 2.086f, 2.080f, 2.074f, 2.069f,      \
        2.064f, 2.060f, 2.056f, 2.052f, 2.048f, 2.045f, 2.042f
#define RPD_T01                                                                                   \
    63.657f, 9.925f, 5.841f, 4.604f, 4.032f, 3.707f, 3.499f, 3.355f, 3.250f, 3.169f, 3.106f, 3.055f, \
        3.012f, 2.977f, 2.947f, 2.921f, 2.898f, 2.878f, 2.861f, 2.845f, 2.831f, 2.819f, 2.807f,      \
        2.797f, 2.787f, 2.779f, 2.771f, 2.763f, 2.756f, 2.750f
__constant__ float c_t05[30] = {RPD_T05};
__constant__ float c_t01[30] = {RPD_T01};
constexpr float kT05[30] = {RPD_T05};
constexpr float kT01[30] = {RPD_T01};

__device__ __forceinline__ float interpolate_table(const float* table, float df) {
    const int lo = iclamps(int(floorf(df)), 1, 30);
    const int hi = iclamps(int(ceilf(df)), 1, 30);
    if (lo == hi) return table[lo - 1];
    return lerp_std(table[lo - 1], table[hi - 1], (df - float(lo)) / float(hi - lo));
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

// sample_vec3_local_average (main.cpp:170-184) of the sqrt variance of the mean, then the
// component max (981-990). The reference accumulates in double: v * weight with weights 1/3
// (corners, 1.0 / 3.0 rounded), 1/2 and 1 (both exact), nine additions in (dy, dx) order, one
// division by the summed weights. A 32 x 8 block stages, per pixel of its (clamped) 34 x 10 halo,
// the three products each channel can need (v, v * 0.5, v * (1.0 / 3.0)) in double once. Of a
// pixel's three channels, the first's nine additions run exactly in integer instructions
// (exact_arith.cuh) and the others' as double additions, so the integer and double pipes share
// the work; each quotient is rounded to float through a single-precision estimate and an exact
// integer remainder (the double division only where that cannot decide). The values are
// positive: sqrt_var_mean is floored at 1e-8.
enum WinPlane { W_GATE = 0, W_ALB, W_SM, W_SV, W_RPD, W_CM, W_COUNT };

// The neighbour record of pixel i (the planes of p.win) and the window's debug planes
// (main.cpp:1010-1023). Records of pixels without a primary hit are zero but for W_CM, which
// holds what the window writes for them (main.cpp:1001-1006): the colour mean and the
// unclamped variance over n.
__device__ __forceinline__ void pack_window_record(const PixelPlanes& p, int64_t np, int64_t i, const float sv[3],
                                                   float var2_max) {
    float4* win = p.win;
    const int n_raw = p.n[i];
    const float m2 = p.square_diff[i];
    const float4 cm = make_float4(p.color_mean[0][i], p.color_mean[1][i], p.color_mean[2][i], 0.0f);
    if (p.hit_count[i] == 0) {
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        for (int k = W_GATE; k < W_CM; ++k) win[k * np + i] = z;
        win[W_CM * np + i] = make_float4(cm.x, cm.y, cm.z, pixel_variance(m2, n_raw) / float(imaxs(1, n_raw)));
        return;
    }
    float var = pixel_variance(m2, n_raw);
    if (!isfinite(var)) var = 1e-8f;
    var = fclamps(var, 1e-8f, var2_max);
    const int n = imaxs(1, n_raw);
    const float vm = fmaxs(1e-8f, var / float(n));
    p.var_total[i] = var;
    p.var_eff[i] = vm;
    p.var_ratio[i] = (var > 1e-8f) ? (vm * float(n)) / var : 0.0f;
    const float rp = 1.0f / fmaxf(float(n - 1), 1.0f);
    win[W_GATE * np + i] = make_float4(p.f_normal[0][i], p.f_normal[1][i], p.f_normal[2][i], p.f_depth[i]);
    win[W_ALB * np + i] = make_float4(p.f_albedo[0][i], p.f_albedo[1][i], p.f_albedo[2][i], rp);
    win[W_SM * np + i] = make_float4(p.sqrt_mean[0][i], p.sqrt_mean[1][i], p.sqrt_mean[2][i], p.rpd[4][i]);
    win[W_SV * np + i] = make_float4(sv[0], sv[1], sv[2], p.rpd[5][i]);
    win[W_RPD * np + i] = make_float4(p.rpd[0][i], p.rpd[1][i], p.rpd[2][i], p.rpd[3][i]);
    win[W_CM * np + i] = make_float4(cm.x, cm.y, cm.z, vm);
}

constexpr int kSvTx = 32, kSvTy = 8;
__global__ void __launch_bounds__(kSvTx * kSvTy) k_sqrt_var_stable(PixelPlanes p, int w, int h, double weight_sum,
                                                                  float var2_max) {
    __shared__ double tile[3][3][(kSvTy + 2) * (kSvTx + 2)];  // [channel][v, v/2, v/3][pixel]
    const int tw = kSvTx + 2, tn = (kSvTy + 2) * (kSvTx + 2);
    const int x0 = blockIdx.x * kSvTx, y0 = blockIdx.y * kSvTy;
    const int tid = threadIdx.y * kSvTx + threadIdx.x;
    const double third = 1.0 / (1.0 + 2.0);
    for (int e = tid; e < tn; e += kSvTx * kSvTy) {
        const int gx = iclamps(x0 - 1 + e % tw, 0, w - 1), gy = iclamps(y0 - 1 + e / tw, 0, h - 1);
        const int64_t q = int64_t(gy) * w + gx;
        for (int c = 0; c < 3; ++c) {
            const double v = double(p.sqrt_var_mean[c][q]);
            tile[c][0][e] = v;
            tile[c][1][e] = v * 0.5;
            tile[c][2][e] = v * third;
        }
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= w || y >= h) return;
    const int64_t i = int64_t(y) * w + x;
    const int e = (threadIdx.y + 1) * tw + threadIdx.x + 1;
    const XD wsum = xd_of_double(weight_sum);
    float sv[3];
    for (int c = 0; c < 3; ++c) {
        const double* t1 = tile[c][0];
        const double* th = tile[c][1];
        const double* tt = tile[c][2];
        // the reference's nine double additions in its order, each rounded as the double-precision
        // add rounds it, in integer arithmetic (GB300's double-precision pipe is the scarce one)
        XD x = xd_of_double(tt[e - tw - 1]);
        x = xd_add(x, xd_of_double(th[e - tw]));
        x = xd_add(x, xd_of_double(tt[e - tw + 1]));
        x = xd_add(x, xd_of_double(th[e - 1]));
        x = xd_add(x, xd_of_double(t1[e]));
        x = xd_add(x, xd_of_double(th[e + 1]));
        x = xd_add(x, xd_of_double(tt[e + tw - 1]));
        x = xd_add(x, xd_of_double(th[e + tw]));
        x = xd_add(x, xd_of_double(tt[e + tw + 1]));
        const double a = xd_to_double(x);
        const XD ax = xd_of_double(a);
        float q;
        if (!quotient_to_float(ax.m, ax.e, wsum.m, wsum.e, q)) q = float(a / weight_sum);
        sv[c] = fmaxs(p.sqrt_var_mean[c][i], q);
        p.sqrt_var_stable[c][i] = sv[c];
    }
    pack_window_record(p, int64_t(w) * h, i, sv, var2_max);
}

struct StatmcParams {
    int w, h, r;
    float normal_threshold, depth_threshold, rpd_scale, alpha, var2_max;
    float albedo_sq_threshold;  // smallest float s with fl(sqrt(s)) > 0.12f
    int table;                  // 0: alpha 0.05 table, 1: alpha 0.01 table, 2: normal quantile
    float z;                    // normal quantile of the alpha
    float inv_z2;               // 1 / z^2
    float df_break;             // 30.5 with a table, 30 with the quantile
    float band;                 // relative guard band of the q and df decisions
    float ws_band;              // relative guard band of the weight_sum >= 1.1 test
    float den_lim;              // 1e-8 (1 + band): the df denominator's band edge
    float df_lim;               // df_break * band
    float q25_lim;              // 25 * band
    float qacc_lim;             // 2 ln 20 * band
    float rp_below;             // a block whose smallest 1/(n-1) is at least this has every df below df_break
    float rp_above;             // a block whose largest 1/(n-1) is at most this has every df at or above 31
    int by;                     // block rows of the generic-radius tiled kernel
};

// The Welch compatibility q of one (i, j) pair in double, the reference's operations in
// its order (main.cpp:1063-1082).
__device__ double exact_q(const float* svi, const float* smi, int n_i, const float* svj, const float* smj, int n_j,
                          float alpha, float adjustment) {
    double max_t2 = 0.0;
    for (int c = 0; c < 3; ++c) {
        const double v_i = double(svi[c]);
        const double v_j = double(svj[c]);
        const double variance_sum = v_i + v_j;
        const double mean_diff = double(smi[c] - smj[c]);
        const double t2 = mean_diff * mean_diff / dmaxs(double(1e-8f), variance_sum);
        const double denom_df = (v_i * v_i) / dmaxs(double(n_i - 1), 1.0) + (v_j * v_j) / dmaxs(double(n_j - 1), 1.0);
        const double df = (denom_df > double(1e-8f)) ? (variance_sum * variance_sum) / denom_df
                                                     : double(n_i + n_j - 2);
        const double t_crit = double(lookup_t_critical(float(df), alpha));
        max_t2 = dmaxs(max_t2, t2 / (t_crit * t_crit));
    }
    return max_t2 / (1.0 + double(adjustment));
}

// One pixel of statmc_denoise entirely in double (main.cpp:999-1127).
__device__ __noinline__ void exact_pixel(const PixelPlanes& p, const StatmcParams& prm, int64_t idx) {
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
            const float smj[3] = {p.sqrt_mean[0][jn], p.sqrt_mean[1][jn], p.sqrt_mean[2][jn]};
            const float svj[3] = {p.sqrt_var_stable[0][jn], p.sqrt_var_stable[1][jn], p.sqrt_var_stable[2][jn]};
            // rpf::shared_reliability + relax_compatibility (core/stats.h:56-78)
            float shared = 0.0f;
            for (int c = 0; c < 6; ++c) shared = fmaxs(shared, fmins(rpd_i[c], p.rpd[c][jn]));
            shared = fclamps(shared, 0.0f, 1.0f);
            const float adjustment = fclamps(prm.rpd_scale * shared, 0.0f, 1.0f);
            const double q = exact_q(svi, smi, n_i, svj, smj, n_j, prm.alpha, adjustment);
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
    const float uncertainty = float(double(alpha) * double(alpha) * double(var_mean_i) + blend * blend * var_neighbors +
                                    2.0 * double(alpha) * blend * (center_weight / dmaxs(weight_sum, double(1e-8f))) *
                                        double(var_mean_i));
    p.alpha[idx] = alpha;
    p.uncertainty[idx] = uncertainty;
}

__global__ void __launch_bounds__(128) k_statmc_window(PixelPlanes p, StatmcParams prm) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(prm.w) * prm.h) return;
    exact_pixel(p, prm, idx);
}

// ---- fast tiled path ------------------------------------------------------------------------

constexpr int kTileX = 32;
constexpr int kRows = 8;                          // block rows of the fixed-radius kernels
constexpr float kQAccept = 5.991464547107979f;   // 2 ln 20: exp(-q/2) > 0.05 (main.cpp:1093)
constexpr float kDepthBand = 1.0f / 1048576.0f;  // 2^-20: depth quotient decided by a product

// t critical value per half unit of df for the t-table alphas: k = floor(2 df) (df clamped to
// 31.75) selects a line, t = v[k].y * df + v[k].x. k < 2: df below 1, which lookup_t_critical
// raises to 1 (t[0]); k in [2, 59]: the interpolation between t[lo-1] and t[lo], lo = k / 2;
// k = 60: df in [30, 30.5), t[29]; k >= 61: df >= 30.5, the normal quantile z.
struct LineTable {
    float2 v[64];
};

// a / b as a times the PTX approximate reciprocal of b (rcp.approx: at most 1 ulp from 1/b over
// the full range, subnormal b flushed); every decision taken on a quotient has a guard band
// thousands of ulps wide.
__device__ __forceinline__ float div_approx(float a, float b) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
    return a * r;
}

// e^x as 2^(x log2 e) with the PTX base-2 exponential (ex2.approx, relative error about 2^-22):
// the weights exp(-q/2) carry no decision (the decisions are taken on q), so the stage's 1e-4
// bar is far away. x = -q/2 is formed as q * (-log2(e) / 2) in one multiplication.
constexpr float kNegHalfLog2e = -0.72134752044448170368f;
__device__ __forceinline__ float exp_neg_half(float q) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(q * kNegHalfLog2e));
    return r;
}
// sw * e^(-q/2) as one base-2 exponential, with l2sw = log2(sw)
__device__ __forceinline__ float weight_of(float q, float l2sw) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__fmaf_rn(q, kNegHalfLog2e, l2sw)));
    return r;
}

// The centre pixel's record, held in registers through its window.
struct Pix {
    float n0, n1, n2;        // unit normal
    float d, dm;             // depth, max(|depth|, EPS_SMALL)
    float a0, a1, a2;        // albedo
    float sm0, sm1, sm2;     // sqrt colour mean
    float sv0, sv1, sv2;     // stabilised sqrt variance of the mean
    float v0, v1, v2;        // sv^2 / max(n - 1, 1)
    float r0, r1, r2, r3, r4, r5;  // RPD components
};

// t critical value of a neighbour's df. MODE 0-2: an alpha with a t table (0.05, 0.01): the
// line of the half-step table, t = v.y * df + v.x; lines 61-63 hold the normal quantile, so the
// table also covers df at or above the switch. MODE 3: any other alpha, the normal quantile
// scaled by sqrt(df / (df - 1)) below df = 30 (main.cpp:214-225).
template <int MODE>
__device__ __forceinline__ float t_crit(float df, const float2* __restrict__ line, const StatmcParams& prm) {
    if constexpr (MODE != 3) {
        // MODE 1: every df is at most (n_i - 1) + (n_j - 1) <= 30, inside the table already
        const float dfc = MODE == 1 ? df : fminf(df, 31.75f);
        // 2 dfc is exact, so one rounding down of 2 dfc + 1.5 * 2^23 leaves floor(2 dfc) in the low bits
        const float fl = __fmaf_rd(dfc, 2.0f, 12582912.0f);
        const float2 l = line[__float_as_int(fl) - 0x4B400000];
        return __fmaf_rn(l.y, dfc, l.x);
    } else {
        const float dfc = fmaxf(df, 1.0f);
        if (dfc < 30.0f) {
            const float x = div_approx(dfc, fmaxf(1.0f, dfc - 1.0f));
            return prm.z * (x * rsqrtf(x));
        }
        return prm.z;
    }
}

// One neighbour of the window: gates, Welch q, relaxation, weight, accumulation. MODE 0: any
// df (t table); 1: every df of the block below the switch (t table); 2: every df at or above
// 31 (t = z); 3: any df, normal-quantile alpha.
// Straight-line: the gates are folded into one predicate (each written as the negation of the
// reference's `continue` test, so a NaN passes a gate as it does there) and only the
// accumulation is conditional, so a warp whose lanes leave at different gates runs one path.
template <int MODE>
__device__ __forceinline__ void visit(const float4* __restrict__ T, int tn, int e, float l2sw, int dx, int dy,
                                      const StatmcParams& prm, const Pix& P, const float2* __restrict__ line,
                                      float row[6], int& accepted, bool& slow) {
    const float4 G = T[W_GATE * tn + e];
    const float4 A = T[W_ALB * tn + e];
    bool ok = !(dot3(P.n0, P.n1, P.n2, G.x, G.y, G.z) < prm.normal_threshold);
    ok = ok && A.w > 0.0f;  // outside the image or no primary hit
    {
        // relative_depth_delta(d_i, d_j) > threshold: fl(|d_i - d_j| / m) against the threshold,
        // decided by the product threshold * m away from it and by the IEEE quotient near it
        float m = P.dm;
        const float dj = fabsf(G.w);
        if (m < dj) m = dj;
        const float num = fabsf(P.d - G.w);
        const float tm = prm.depth_threshold * m;
        const float dl = num - tm;
        bool far;
        // tm >= 1e-30 here: thresholds below 1e-21 take the exact window (m >= 1e-8)
        if (fabsf(dl) <= tm * kDepthBand) far = __fdiv_rn(num, m) > prm.depth_threshold;
        else far = dl > 0.0f;
        ok = ok && !far;
    }
    const float da0 = P.a0 - A.x, da1 = P.a1 - A.y, da2 = P.a2 - A.z;
    ok = ok && !(dot3(da0, da1, da2, da0, da1, da2) >= prm.albedo_sq_threshold);

    const float4 S = T[W_SM * tn + e], V = T[W_SV * tn + e];
    bool exact = false;
    const float vs0 = P.sv0 + V.x, vs1 = P.sv1 + V.y, vs2 = P.sv2 + V.z;
    const float md0 = P.sm0 - S.x, md1 = P.sm1 - S.y, md2 = P.sm2 - S.z;
    float qmax;
    if constexpr (MODE == 2) {
        qmax = fmaxf(fmaxf(div_approx(md0 * md0, vs0), div_approx(md1 * md1, vs1)), div_approx(md2 * md2, vs2)) *
               prm.inv_z2;
    } else {
        const float rpj = A.w;
        const float den0 = __fmaf_rn(V.x * V.x, rpj, P.v0);
        const float den1 = __fmaf_rn(V.y * V.y, rpj, P.v1);
        const float den2 = __fmaf_rn(V.z * V.z, rpj, P.v2);
        // MODE 1 blocks have every denominator above the band (their smallest term is)
        if constexpr (MODE != 1) exact |= fminf(fminf(den0, den1), den2) <= prm.den_lim;
        const float df0 = div_approx(vs0 * vs0, den0);
        const float df1 = div_approx(vs1 * vs1, den1);
        const float df2 = div_approx(vs2 * vs2, den2);
        if constexpr (MODE == 0 || MODE == 3) {
            exact |= fabsf(df0 - prm.df_break) <= prm.df_lim;
            exact |= fabsf(df1 - prm.df_break) <= prm.df_lim;
            exact |= fabsf(df2 - prm.df_break) <= prm.df_lim;
        }
        const float t0 = t_crit<MODE>(df0, line, prm);
        const float t1 = t_crit<MODE>(df1, line, prm);
        const float t2 = t_crit<MODE>(df2, line, prm);
        qmax = fmaxf(fmaxf(div_approx(md0 * md0, vs0 * (t0 * t0)), div_approx(md1 * md1, vs1 * (t1 * t1))),
                     div_approx(md2 * md2, vs2 * (t2 * t2)));
    }
    // rpf::shared_reliability + relax_compatibility (core/stats.h:56-78)
    const float4 RJ = T[W_RPD * tn + e];
    float shared = fmaxf(fmaxf(fminf(P.r0, RJ.x), fminf(P.r1, RJ.y)), fmaxf(fminf(P.r2, RJ.z), fminf(P.r3, RJ.w)));
    shared = __saturatef(fmaxf(shared, fmaxf(fminf(P.r4, S.w), fminf(P.r5, V.w))));
    const float adjustment = __saturatef(prm.rpd_scale * shared);
    const float q = div_approx(qmax, 1.0f + adjustment);
    const bool center = dx == 0 && dy == 0;
    exact |= fabsf(q - 25.0f) <= prm.q25_lim;
    exact |= !center && fabsf(q - kQAccept) <= prm.qacc_lim;
    // a decision inside a guard band hands the pixel to the slow pass (k_statmc_slow)
    slow = slow || (ok && exact);
    if (ok && !(q > 25.0f)) {
        if (!center && q < kQAccept) ++accepted;
        const float wj = weight_of(q, l2sw);
        const float4 CM = T[W_CM * tn + e];
        const float w2 = wj * wj;
        row[0] = __fmaf_rn(wj, CM.x, row[0]);
        row[1] = __fmaf_rn(wj, CM.y, row[1]);
        row[2] = __fmaf_rn(wj, CM.z, row[2]);
        row[3] += wj;
        row[4] += w2;
        row[5] = __fmaf_rn(w2, CM.w, row[5]);
    }
}

template <int RC, int MODE>
__device__ __forceinline__ void window_rows(const float4* __restrict__ T, int tn, int tw, int r,
                                            const float* __restrict__ spatial, const float2* __restrict__ line,
                                            const StatmcParams& prm, const Pix& P, int ei, float acc[6],
                                            int& accepted, bool& slow) {
    const int side = 2 * r + 1;
    for (int dy = -r; dy <= r; ++dy) {
        float row[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        const int erow = ei + dy * tw;
        const float* srow = spatial + (dy + r) * side + r;
        if constexpr (RC > 0) {
#pragma unroll
            for (int dx = -RC; dx <= RC; ++dx)
                visit<MODE>(T, tn, erow + dx, srow[dx], dx, dy, prm, P, line, row, accepted, slow);
        } else {
#pragma unroll 1
            for (int dx = -r; dx <= r; ++dx)
                visit<MODE>(T, tn, erow + dx, srow[dx], dx, dy, prm, P, line, row, accepted, slow);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) acc[k] += row[k];
    }
}

// The blend of a pixel from its window's sums (main.cpp:1099-1126) in single precision.
__device__ __forceinline__ void write_blend(const PixelPlanes& p, int64_t idx, float4 cmi, const float acc[6],
                                            int accepted) {
    const float weight_sum = acc[3];
    const float var_mean_i = cmi.w;
    float mean_nb[3] = {cmi.x, cmi.y, cmi.z};
    float var_neighbors = var_mean_i;
    if (weight_sum > 1e-8f) {
        const float inv = 1.0f / weight_sum;
        mean_nb[0] = acc[0] * inv;
        mean_nb[1] = acc[1] * inv;
        mean_nb[2] = acc[2] * inv;
        var_neighbors = acc[5] * inv * inv;
    }
    const float effective = weight_sum * weight_sum / fmaxf(1e-8f, acc[4]);
    const float blend =
        (accepted >= 2 && weight_sum >= 1.1f) ? fminf(fmaxf(1.0f - rsqrtf(effective), 0.0f), 0.8f) : 0.0f;
    const float alpha = 1.0f - blend;
    p.denoised[0][idx] = lerpf(cmi.x, mean_nb[0], blend);
    p.denoised[1][idx] = lerpf(cmi.y, mean_nb[1], blend);
    p.denoised[2][idx] = lerpf(cmi.z, mean_nb[2], blend);
    const float uncertainty = alpha * alpha * var_mean_i + blend * blend * var_neighbors +
                              2.0f * alpha * blend * (1.0f / fmaxf(weight_sum, 1e-8f)) * var_mean_i;
    p.alpha[idx] = alpha;
    p.uncertainty[idx] = uncertainty;
}

// ---- slow pass -----------------------------------------------------------------------------

// The pixels the fast loop hands over (a decision inside a guard band, or the weight sum inside
// the band of the 1.1 test), one warp per pixel, the window's neighbours split over the lanes
// and read from the packed records in HBM. Every neighbour is evaluated in single precision as
// the fast loop evaluates it, except that a neighbour whose q (or df) lies in a band has its q
// recomputed in double exactly as the reference computes it (main.cpp:1055-1097) and its
// rejection, weight and acceptance taken from that; a pixel whose summed weight lies inside
// the 1.1 test's band is then recomputed wholly in double (exact_pixel). Run as its own
// launch, the rare pixel costs one warp's share of a short pass instead of holding the 31
// other lanes of its warp in the fast loop.
constexpr int kSlowThreads = 256;
constexpr int kSlowBlocks = 152 * 2;  // two blocks on each of GB300's 152 SMs

__global__ void __launch_bounds__(kSlowThreads) k_statmc_slow(PixelPlanes p, StatmcParams prm, LineTable lt) {
    __shared__ float2 s_line[64];
    const int64_t np = int64_t(prm.w) * prm.h;
    unsigned long long count = p.counters[RPD_COUNTER_WINDOW_SLOW_PIXELS];
    if (count == 0) return;  // the usual case on uniform sample counts: the whole block leaves
    if (count > (unsigned long long)np) count = (unsigned long long)np;
    if (threadIdx.x < 64) s_line[threadIdx.x] = lt.v[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int r = prm.r, side = 2 * r + 1, visits = side * side;
    const float4* win = p.win;
    const unsigned long long warps = (unsigned long long)gridDim.x * (kSlowThreads / 32);
    for (unsigned long long k = (unsigned long long)blockIdx.x * (kSlowThreads / 32) + threadIdx.x / 32; k < count;
         k += warps) {
        const int64_t idx = p.slow[k];
        const int y = int(idx / prm.w), x = int(idx % prm.w);
        const float4 gi = win[W_GATE * np + idx], ai = win[W_ALB * np + idx], si = win[W_SM * np + idx];
        const float4 vi = win[W_SV * np + idx], ri = win[W_RPD * np + idx];
        float dm = fabsf(gi.w);
        if (dm < 1e-8f) dm = 1e-8f;
        const float smi[3] = {si.x, si.y, si.z}, svi[3] = {vi.x, vi.y, vi.z};
        const float vi0 = vi.x * vi.x * ai.w, vi1 = vi.y * vi.y * ai.w, vi2 = vi.z * vi.z * ai.w;
        const int n_i = imaxs(1, p.n[idx]);
        float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        int accepted = 0, pairs = 0;
        for (int v = lane; v < visits; v += 32) {
            const int dx = v % side - r, dy = v / side - r;
            const int xx = x + dx, yy = y + dy;
            if (xx < 0 || xx >= prm.w || yy < 0 || yy >= prm.h) continue;  // the zero record: no neighbour
            const int64_t jn = int64_t(yy) * prm.w + xx;
            const float4 G = win[W_GATE * np + jn];
            if (dot3(gi.x, gi.y, gi.z, G.x, G.y, G.z) < prm.normal_threshold) continue;
            const float4 A = win[W_ALB * np + jn];
            if (!(A.w > 0.0f)) continue;
            {
                float m = dm;
                const float dj = fabsf(G.w);
                if (m < dj) m = dj;
                const float num = fabsf(gi.w - G.w);
                const float tm = prm.depth_threshold * m;
                const float dl = num - tm;
                bool far;
                if (fabsf(dl) <= tm * kDepthBand || !(tm >= 1e-30f)) far = __fdiv_rn(num, m) > prm.depth_threshold;
                else far = dl > 0.0f;
                if (far) continue;
            }
            const float da0 = ai.x - A.x, da1 = ai.y - A.y, da2 = ai.z - A.z;
            if (dot3(da0, da1, da2, da0, da1, da2) >= prm.albedo_sq_threshold) continue;
            const float4 S = win[W_SM * np + jn], V = win[W_SV * np + jn], RJ = win[W_RPD * np + jn];
            const float vs[3] = {vi.x + V.x, vi.y + V.y, vi.z + V.z};
            const float md[3] = {si.x - S.x, si.y - S.y, si.z - S.z};
            const float den[3] = {__fmaf_rn(V.x * V.x, A.w, vi0), __fmaf_rn(V.y * V.y, A.w, vi1),
                                  __fmaf_rn(V.z * V.z, A.w, vi2)};
            bool exact = fminf(fminf(den[0], den[1]), den[2]) <= prm.den_lim;
            float qmax = 0.0f;
            for (int c = 0; c < 3; ++c) {
                const float df = div_approx(vs[c] * vs[c], den[c]);
                exact |= fabsf(df - prm.df_break) <= prm.df_lim;
                const float t = prm.table < 2 ? t_crit<0>(df, s_line, prm) : t_crit<3>(df, s_line, prm);
                qmax = fmaxf(qmax, div_approx(md[c] * md[c], vs[c] * (t * t)));
            }
            float shared = fmaxf(fmaxf(fminf(ri.x, RJ.x), fminf(ri.y, RJ.y)), fmaxf(fminf(ri.z, RJ.z), fminf(ri.w, RJ.w)));
            shared = __saturatef(fmaxf(shared, fmaxf(fminf(si.w, S.w), fminf(vi.w, V.w))));
            const float adjustment = __saturatef(prm.rpd_scale * shared);
            const float q = div_approx(qmax, 1.0f + adjustment);
            const bool center = dx == 0 && dy == 0;
            exact |= fabsf(q - 25.0f) <= prm.q25_lim;
            exact |= !center && fabsf(q - kQAccept) <= prm.qacc_lim;
            float wj;
            if (exact) {
                ++pairs;
                const float smj[3] = {S.x, S.y, S.z}, svj[3] = {V.x, V.y, V.z};
                const double qx = exact_q(svi, smi, n_i, svj, smj, imaxs(1, p.n[jn]), prm.alpha, adjustment);
                if (qx > 25.0) continue;
                const double sw = 1.0 / (1.0 + double(dx * dx + dy * dy));
                const double wd = sw * exp(-0.5 * qx);
                if (!center && wd > 0.05 * sw) ++accepted;
                wj = float(wd);
            } else {
                if (q > 25.0f) continue;
                if (!center && q < kQAccept) ++accepted;
                wj = __frcp_rn(1.0f + float(dx * dx + dy * dy)) * exp_neg_half(q);
            }
            const float4 CM = win[W_CM * np + jn];
            const float w2 = wj * wj;
            acc[0] = __fmaf_rn(wj, CM.x, acc[0]);
            acc[1] = __fmaf_rn(wj, CM.y, acc[1]);
            acc[2] = __fmaf_rn(wj, CM.z, acc[2]);
            acc[3] += wj;
            acc[4] += w2;
            acc[5] = __fmaf_rn(w2, CM.w, acc[5]);
        }
        // the lanes' sums in a fixed butterfly order: the same bits on every run
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
            accepted += __shfl_xor_sync(0xffffffffu, accepted, o);
            pairs += __shfl_xor_sync(0xffffffffu, pairs, o);
        }
        if (lane == 0) {
            if (pairs > 0) atomicAdd(p.counters + RPD_COUNTER_WINDOW_PAIR_RECHECKS, (unsigned long long)pairs);
            if (accepted >= 2 && fabsf(acc[3] - 1.1f) <= 1.1f * prm.ws_band) {
                atomicAdd(p.counters + RPD_COUNTER_WINDOW_PIXEL_RECHECKS, 1ull);
                exact_pixel(p, prm, idx);
            } else {
                write_blend(p, idx, win[W_CM * np + idx], acc, accepted);
            }
        }
        __syncwarp();
    }
}

// RC > 0: radius RC and kRows block rows fixed at compile time; RC == 0: prm.r and prm.by.
template <int RC>
__global__ void __launch_bounds__(kTileX * kRows, 3)
    k_statmc_tma(PixelPlanes p, StatmcParams prm, LineTable lt, const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ float2 s_line[64];
    __shared__ unsigned s_rpmin, s_rpmax, s_dmin;
    __shared__ int s_fail;
    const int r = RC > 0 ? RC : prm.r;
    const int by = RC > 0 ? kRows : prm.by;
    const int tw = kTileX + 2 * r, th = by + 2 * r, tn = tw * th, side = 2 * r + 1;
    // the tile copy's destination, 128-byte aligned
    const uint32_t pad = (128u - (smem_addr(smem_raw) & 127u)) & 127u;
    float4* T = reinterpret_cast<float4*>(smem_raw + pad);
    float* spatial = reinterpret_cast<float*>(T + W_COUNT * tn);  // side * side
    const int tid = threadIdx.y * kTileX + threadIdx.x;
    const int nthreads = kTileX * by;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * by;
    const uint32_t bar_a = smem_addr(&bar);

    if (tid == 0) {
        mbar_init(bar_a, 1);
        s_rpmin = 0x7f800000u;  // +inf
        s_rpmax = 0u;
        s_dmin = 0x7f800000u;
        s_fail = 0;
    }
    __syncthreads();
    if (tid == 0) {
        tile_load(T, &tmap, x0, y0, r, tw, th, W_COUNT, bar_a);
    }
    if (tid < 64) s_line[tid] = lt.v[tid];
    for (int e = tid; e < side * side; e += nthreads) {
        const int dx = e % side - r, dy = e / side - r;
        // log2 of 1 / (1 + d^2) (main.cpp:1094): the weight is then one base-2 exponential
        spatial[e] = log2f(__frcp_rn(1.0f + float(dx * dx + dy * dy)));
    }
    if (!mbar_wait_bounded(bar_a, 0)) s_fail = 1;
    __syncthreads();
    if (s_fail) {
        // the copy did not land in time: report it, and let the copy finish (bounded) before the
        // block's shared memory is released
        if (tid == 0) {
            atomicAdd(p.counters + RPD_COUNTER_DEVICE_WAIT_TIMEOUTS, 1ull);
            mbar_wait_bounded(bar_a, 0);
        }
        return;
    }

    // the halo's range of 1/max(n-1, 1) selects the block's loop; so does the smallest term
    // fl(fl(sv^2) * rp) of a df denominator: every denominator fl(sv_j^2 * rp_j + v_i) is at
    // least its neighbour's term, so above the band when the smallest term is
    float lmin = __uint_as_float(0x7f800000u), lmax = 0.0f, dmin = __uint_as_float(0x7f800000u);
    for (int e = tid; e < tn; e += nthreads) {
        const float rp = T[W_ALB * tn + e].w;
        if (rp > 0.0f) {
            const float4 v = T[W_SV * tn + e];
            lmin = fminf(lmin, rp);
            lmax = fmaxf(lmax, rp);
            dmin = fminf(dmin, fminf(fminf((v.x * v.x) * rp, (v.y * v.y) * rp), (v.z * v.z) * rp));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
        lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        dmin = fminf(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    }
    if ((tid & 31) == 0) {
        atomicMin(&s_rpmin, __float_as_uint(lmin));  // non-negative floats order as their bits
        atomicMax(&s_rpmax, __float_as_uint(lmax));
        atomicMin(&s_dmin, __float_as_uint(dmin));
    }
    __syncthreads();
    const int mode = __uint_as_float(s_rpmax) <= prm.rp_above                                     ? 2
                     : prm.table == 2                                                              ? 3
                     : __uint_as_float(s_rpmin) >= prm.rp_below && __uint_as_float(s_dmin) > prm.den_lim ? 1
                                                                                                   : 0;

    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t idx = int64_t(y) * prm.w + x;
    const int ei = (threadIdx.y + r) * tw + threadIdx.x + r;
    const float4 cmi = T[W_CM * tn + ei];
    const float4 ali = T[W_ALB * tn + ei];
    if (!(ali.w > 0.0f)) {  // no primary hit: the pixel passes through (main.cpp:1001-1006)
        p.denoised[0][idx] = cmi.x;
        p.denoised[1][idx] = cmi.y;
        p.denoised[2][idx] = cmi.z;
        p.uncertainty[idx] = cmi.w;
        p.alpha[idx] = 1.0f;
        return;
    }
    Pix P;
    {
        const float4 g = T[W_GATE * tn + ei], s = T[W_SM * tn + ei], v = T[W_SV * tn + ei], rr = T[W_RPD * tn + ei];
        P.n0 = g.x;
        P.n1 = g.y;
        P.n2 = g.z;
        P.d = g.w;
        P.dm = fabsf(g.w);
        if (P.dm < 1e-8f) P.dm = 1e-8f;
        P.a0 = ali.x;
        P.a1 = ali.y;
        P.a2 = ali.z;
        P.sm0 = s.x;
        P.sm1 = s.y;
        P.sm2 = s.z;
        P.sv0 = v.x;
        P.sv1 = v.y;
        P.sv2 = v.z;
        P.v0 = v.x * v.x * ali.w;
        P.v1 = v.y * v.y * ali.w;
        P.v2 = v.z * v.z * ali.w;
        P.r0 = rr.x;
        P.r1 = rr.y;
        P.r2 = rr.z;
        P.r3 = rr.w;
        P.r4 = s.w;
        P.r5 = v.w;
    }
    float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int accepted = 0;
    bool slow = false;
    if (mode == 2)
        window_rows<RC, 2>(T, tn, tw, r, spatial, s_line, prm, P, ei, acc, accepted, slow);
    else if (mode == 1)
        window_rows<RC, 1>(T, tn, tw, r, spatial, s_line, prm, P, ei, acc, accepted, slow);
    else if (mode == 3)
        window_rows<RC, 3>(T, tn, tw, r, spatial, s_line, prm, P, ei, acc, accepted, slow);
    else
        window_rows<RC, 0>(T, tn, tw, r, spatial, s_line, prm, P, ei, acc, accepted, slow);

    // the blend in single precision from the float sums (relative error ~1e-6, far inside the
    // plain-form bar); a pixel with a decision inside a guard band, or whose weight sum lies
    // inside the band of the 1.1 test, goes on the slow pass's list (each pixel at most once,
    // so the list never outgrows its W*H entries)
    if (slow || (accepted >= 2 && fabsf(acc[3] - 1.1f) <= 1.1f * prm.ws_band)) {
        const unsigned long long k = atomicAdd(p.counters + RPD_COUNTER_WINDOW_SLOW_PIXELS, 1ull);
        p.slow[k] = int32_t(idx);
        return;
    }
    write_blend(p, idx, cmi, acc, accepted);
}

// Smallest float s with fl(sqrt(s)) > t: the albedo gate sqrt(s) > 0.12 without a sqrt.
float sqrt_gate_threshold(float t) {
    uint32_t lo = 0, hi = 0x7f800000u;  // [0, +inf)
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        float s;
        std::memcpy(&s, &mid, 4);
        if (std::sqrt(s) > t) hi = mid;
        else lo = mid + 1;
    }
    float out;
    std::memcpy(&out, &lo, 4);
    return out;
}

size_t tile_bytes(int r, int by) {
    const size_t side = size_t(2 * r + 1);
    return 128 + size_t(kTileX + 2 * r) * size_t(by + 2 * r) * W_COUNT * sizeof(float4) + side * side * sizeof(float);
}

LineTable line_table(int table, float z) {
    const float* tab = table == 0 ? kT05 : kT01;
    LineTable lt{};
    for (int k = 0; k < 64; ++k) {
        if (k < 2) {
            lt.v[k] = make_float2(tab[0], 0.0f);
        } else if (k < 60) {
            const int lo = k >> 1;
            const float d = tab[lo] - tab[lo - 1];
            lt.v[k] = make_float2(float(double(tab[lo - 1]) - double(lo) * double(d)), d);
        } else if (k == 60) {
            lt.v[k] = make_float2(tab[29], 0.0f);
        } else {
            lt.v[k] = make_float2(z, 0.0f);
        }
    }
    return lt;
}

// The tensor map of the job's packed records for halo boxes of radius r and `by` block rows.
cudaError_t window_map(Job& j, int r, int by) {
    if (j.win_map_r == r && j.win_map_by == by) return cudaSuccess;
    const cudaError_t e = encode_record_map(reinterpret_cast<CUtensorMap*>(j.win_map), j.p.win, j.g.w, j.g.h, W_COUNT,
                                            kTileX + 2 * r, by + 2 * r);
    if (e != cudaSuccess) return e;
    j.win_map_r = r;
    j.win_map_by = by;
    return cudaSuccess;
}

template <int RC>
cudaError_t launch_tma(Job& j, const StatmcParams& prm, const LineTable& lt, int by) {
    const size_t smem = tile_bytes(prm.r, by);
    // the dynamic shared memory size this instantiation allows, per device
    static std::mutex mu;
    static std::unordered_map<int, size_t> configured;
    {
        std::lock_guard<std::mutex> lock(mu);
        size_t& allowed = configured[j.ctx->device];
        if (smem > allowed) {
            const cudaError_t e = cudaFuncSetAttribute(k_statmc_tma<RC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       int(smem));
            if (e != cudaSuccess) return e;
            allowed = smem;
        }
    }
    const cudaError_t e = window_map(j, prm.r, by);
    if (e != cudaSuccess) return e;
    CUtensorMap map;
    std::memcpy(&map, j.win_map, sizeof(map));
    const dim3 block(kTileX, by);
    const dim3 grid((j.g.w + kTileX - 1) / kTileX, (j.g.h + by - 1) / by);
    k_statmc_tma<RC><<<grid, block, smem, j.stream>>>(j.p, prm, lt, map);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_statmc(Job& j) {
    const int64_t np = j.g.np;
    const float var2_max = j.cfg.color_sigma_max * j.cfg.color_sigma_max;
    {
        KernelScope ks(j, RPD_KERNEL_SQRT_VARIANCE);
        k_sqrt_var_mean<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np);
        // the summed weights of the 3x3 average, accumulated as the reference accumulates them
        double weight_sum = 0.0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) weight_sum += 1.0 / (1.0 + double(dx * dx + dy * dy));
        const dim3 sgrid((j.g.w + kSvTx - 1) / kSvTx, (j.g.h + kSvTy - 1) / kSvTy);
        k_sqrt_var_stable<<<sgrid, dim3(kSvTx, kSvTy), 0, j.stream>>>(j.p, j.g.w, j.g.h, weight_sum, var2_max);
    }
    KernelScope ks(j, RPD_KERNEL_STATMC_WINDOW);
    StatmcParams prm{};
    prm.w = j.g.w;
    prm.h = j.g.h;
    prm.r = j.cfg.color_window_radius;
    prm.normal_threshold = j.cfg.color_normal_threshold;
    prm.depth_threshold = j.cfg.color_depth_threshold;
    prm.rpd_scale = j.cfg.rpf_shrinkage_scale;
    prm.alpha = j.cfg.color_compat_alpha;
    prm.var2_max = var2_max;
    static const float albedo_sq = sqrt_gate_threshold(0.12f);
    prm.albedo_sq_threshold = albedo_sq;
    // the branch of lookup_t_critical this alpha takes (main.cpp:189-225)
    const float a = std::min(std::max(prm.alpha, 1e-8f), 0.999999f);
    if (std::fabs(a - 0.05f) < 1e-4f) prm.table = 0;
    else if (std::fabs(a - 0.01f) < 1e-4f) prm.table = 1;
    else prm.table = 2;
    prm.z = a <= 0.001f ? 3.29f : a <= 0.005f ? 2.81f : a <= 0.01f ? 2.58f : a <= 0.02f ? 2.33f
          : a <= 0.05f ? 1.96f : a <= 0.10f ? 1.64f : 1.28f;
    prm.inv_z2 = float(1.0 / (double(prm.z) * double(prm.z)));
    prm.df_break = prm.table < 2 ? 30.5f : 30.0f;
    prm.band = std::ldexp(1.0f, -j.window_guard);
    prm.ws_band = std::ldexp(1.0f, -j.window_guard - 1);
    prm.den_lim = 1e-8f * (1.0f + prm.band);
    prm.df_lim = prm.df_break * prm.band;
    prm.q25_lim = 25.0f * prm.band;
    prm.qacc_lim = kQAccept * prm.band;
    // df <= (n_i - 1) + (n_j - 1) < 30.5 (table) / 30 (quantile) when every n - 1 <= 15 / 14;
    // df >= min(n_i, n_j) - 1 >= 31 when every n - 1 >= 31
    prm.rp_below = prm.table < 2 ? 1.0f / 15.0f : 1.0f / 14.0f;
    prm.rp_above = 1.0f / 31.0f;
    cudaError_t e = cudaSuccess;
    const int r = prm.r;
    // the fast window decides the depth gate through threshold * m, which for m >= 1e-8 stays a
    // normal float away from 0 only when the threshold is at least about 1e-21
    if (j.exact_window || r > 16 || !(prm.depth_threshold >= 1e-21f)) {
        k_statmc_window<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, prm);
        e = cudaGetLastError();
    } else {
        const LineTable lt = line_table(prm.table, prm.z);
        bool tiled = true;
        const size_t limit = size_t(200) * 1024;
        const bool fixed = (r == 3 || r == 5 || r == 7) && (j.statmc_by == 0 || j.statmc_by == kRows) &&
                           tile_bytes(r, kRows) <= limit;
        if (fixed) {
            prm.by = kRows;
            e = r == 5 ? launch_tma<5>(j, prm, lt, kRows) : r == 7 ? launch_tma<7>(j, prm, lt, kRows)
                                                               : launch_tma<3>(j, prm, lt, kRows);
        } else {
            int by = 0;
            for (int cand : {8, 4, 2})
                if (tile_bytes(r, cand) <= limit && (j.statmc_by == 0 || cand <= j.statmc_by)) {
                    by = cand;
                    break;
                }
            if (by == 0) {
                k_statmc_window<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, prm);
                e = cudaGetLastError();
                tiled = false;
            } else {
                prm.by = by;
                e = launch_tma<0>(j, prm, lt, by);
            }
        }
        if (tiled && e == cudaSuccess) {
            const int64_t blocks = std::min<int64_t>(kSlowBlocks, (np + kSlowThreads / 32 - 1) / (kSlowThreads / 32));
            k_statmc_slow<<<unsigned(blocks), kSlowThreads, 0, j.stream>>>(j.p, prm, lt);
            e = cudaGetLastError();
            j.launches += 1;
        }
    }
    j.launches += 3;
    return e;
}

}  // namespace rpd
