// statmc_denoise (main.cpp:957-1162): the per-channel square-root-domain Welch
// compatibility window with the RPD relaxation.
//
//   k_sqrt_var_mean    sqrt-domain variance of the mean, floored at EPS_SMALL (972-980)
//   k_sqrt_var_stable  max with its 3x3 inverse-distance average (981-990)
//   k_statmc_tile      the (2r+1)^2 window (998-1127), fast path. A 32 x BY block stages
//                      its (32+2r) x (BY+2r) halo tile of per-pixel records in shared memory
//                      (structure of arrays, so a warp reading 32 neighbours at one offset is
//                      bank-conflict free) and evaluates every neighbour in single precision:
//                        * the normal / depth / albedo gates are decided exactly as the
//                          reference decides them (identical float operations; the depth
//                          quotient is only rounded exactly when it lies within 2^-20 of the
//                          threshold; the albedo norm is compared through the exact squared
//                          threshold of the correctly rounded sqrt);
//                        * the Welch t^2, Welch-Satterthwaite df, t-table lookup and RPD
//                          relaxation run in float with approximate division. Their relative
//                          error is below 3e-6, so whenever q lies within 2^-15 (relative)
//                          of a decision point — q = 25 (reject), q = 2 ln 20 (the accepted-
//                          neighbour count), df = 30.5 / 30 (t-table branch) or the 1e-8
//                          df-denominator test — that neighbour's q is recomputed in double
//                          exactly as the reference computes it, and the decisions use it.
//                      Weights are accumulated in float per window row and in double-float
//                      across rows. The blend's weight_sum >= 1.1 test has its own guard
//                      band; a pixel inside it is recomputed wholly in double.
//   k_statmc_window    the whole window in double, the reference's operations in its order
//                      (the exact mode, the fallback of the fast path, and the path for
//                      radii whose halo tile would not fit in shared memory).
#include <algorithm>
#include <cmath>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "exact_arith.cuh"

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
constexpr int kSvTx = 32, kSvTy = 8;
__global__ void __launch_bounds__(kSvTx * kSvTy) k_sqrt_var_stable(PixelPlanes p, int w, int h, double weight_sum) {
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
    for (int c = 0; c < 3; ++c) {
        const double* t1 = tile[c][0];
        const double* th = tile[c][1];
        const double* tt = tile[c][2];
        double a;
        if (c == 0) {
            XD x = xd_of_double(tt[e - tw - 1]);
            x = xd_add(x, xd_of_double(th[e - tw]));
            x = xd_add(x, xd_of_double(tt[e - tw + 1]));
            x = xd_add(x, xd_of_double(th[e - 1]));
            x = xd_add(x, xd_of_double(t1[e]));
            x = xd_add(x, xd_of_double(th[e + 1]));
            x = xd_add(x, xd_of_double(tt[e + tw - 1]));
            x = xd_add(x, xd_of_double(th[e + tw]));
            x = xd_add(x, xd_of_double(tt[e + tw + 1]));
            a = xd_to_double(x);
        } else {
            a = 0.0;
            a += tt[e - tw - 1];
            a += th[e - tw];
            a += tt[e - tw + 1];
            a += th[e - 1];
            a += t1[e];
            a += th[e + 1];
            a += tt[e + tw - 1];
            a += th[e + tw];
            a += tt[e + tw + 1];
        }
        const XD ax = xd_of_double(a);
        float q;
        if (!quotient_to_float(ax.m, ax.e, wsum.m, wsum.e, q)) q = float(a / weight_sum);
        p.sqrt_var_stable[c][i] = fmaxs(p.sqrt_var_mean[c][i], q);
    }
}

struct StatmcParams {
    int w, h, r;
    float normal_threshold, depth_threshold, rpd_scale, alpha, var2_max;
    float albedo_sq_threshold;  // smallest float s with fl(sqrt(s)) > 0.12f
    int table;                  // 0: alpha 0.05 table, 1: alpha 0.01 table, 2: normal quantile
    float z;                    // normal quantile of the alpha (table == 2)
    float df_break;             // 30.5 with a table, 30 with the quantile
    int by;                     // block height of the tiled kernel
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
__device__ void exact_pixel(const PixelPlanes& p, const StatmcParams& prm, int64_t idx) {
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

// ---- fast tiled path ----------------------------------------------------------------------

// Halo tile planes, float4 per pixel (structure of float4 arrays: a warp reading 32
// neighbours at one offset reads 512 contiguous bytes, conflict free):
//   P_GATE (nx, ny, nz, depth)         normal / depth gates
//   P_ALB  (ax, ay, az, n)             albedo gate, sample count as float (0: outside the
//                                      image or no primary hit, which the reference skips)
//   P_SM   (sqrt mean rgb, rpd[4])     Welch means
//   P_SV   (sqrt var stable rgb, rpd[5]) Welch variances
//   P_A    (sv^2 / (n - 1) rgb, var of the mean)
//   P_RPD  (rpd[0..3])
//   P_CM   (colour mean rgb, 0)
enum TilePlane { P_GATE = 0, P_ALB, P_SM, P_SV, P_A, P_RPD, P_CM, P_COUNT };

constexpr int kTileX = 32;
constexpr float kBand = 1.0f / 32768.0f;          // 2^-15 relative guard band
constexpr float kQAccept = 5.991464547107979f;     // 2 ln 20: exp(-q/2) > 0.05
constexpr double kWsBand = 1.0 / 65536.0;          // guard band of weight_sum >= 1.1
constexpr float kDepthBand = 1.0f / 1048576.0f;    // 2^-20: depth quotient decided by a product

// t critical value of the fast path. The table branch interpolates (tab[lo-1], tab[lo]) with
// lo = round(df - 1/2) taken from the float's bits (df in [1, 30.5): no conversion unit); at
// an integer df this may pick the lower cell with fraction 1, the same value to an ulp. The
// pairs hold (tab[i], tab[i+1] - tab[i]) and (tab[29], 0), so df in [30, 30.5) gives tab[29]
// as lookup_t_critical does.
__device__ __forceinline__ float tile_t_lookup(const float2* pairs, float df, const StatmcParams& prm) {
    df = fmaxf(df, 1.0f);
    if (prm.table < 2 && df < 30.5f) {
        const float fl = (df - 0.5f) + 12582912.0f;  // 1.5 * 2^23: integer part in the low bits
        const int lo = imaxs(__float_as_int(fl) - 0x4B400000, 1);
        const float2 ab = pairs[lo - 1];
        return __fmaf_rn(ab.y, df - float(lo), ab.x);
    }
    float z = prm.z;
    if (df < 30.0f) z = z * sqrtf(__fdividef(df, fmaxf(1.0f, df - 1.0f)));
    return z;
}

__global__ void __launch_bounds__(256, 2) k_statmc_tile(PixelPlanes p, StatmcParams prm) {
    extern __shared__ float4 smem4[];
    const int r = prm.r;
    const int tw = kTileX + 2 * r, th = prm.by + 2 * r;
    const int tn = tw * th;
    const int side = 2 * r + 1;
    float4* T = smem4;                                                  // P_COUNT planes of tn
    float2* pairs = reinterpret_cast<float2*>(smem4 + P_COUNT * tn);    // 32 t-table pairs
    float* spatial_tab = reinterpret_cast<float*>(pairs + 32);          // side * side
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * prm.by;
    const int tid = threadIdx.y * kTileX + threadIdx.x;
    const int nthreads = kTileX * prm.by;

    if (tid < 32) {
        const float* tab = prm.table == 0 ? c_t05 : c_t01;
        pairs[tid] = tid < 29 ? make_float2(tab[tid], tab[tid + 1] - tab[tid])
                              : make_float2(tid == 29 ? tab[29] : 0.0f, 0.0f);
    }
    for (int e = tid; e < side * side; e += nthreads) {
        const int dx = e % side - r, dy = e / side - r;
        spatial_tab[e] = __frcp_rn(1.0f + float(dx * dx + dy * dy));  // 1 / (1 + d^2), main.cpp:1096
    }
    for (int e = tid; e < tn; e += nthreads) {
        const int gx = x0 - r + e % tw, gy = y0 - r + e / tw;
        bool inside = gx >= 0 && gx < prm.w && gy >= 0 && gy < prm.h;
        const int64_t q = inside ? int64_t(gy) * prm.w + gx : 0;
        const bool hit = inside && p.hit_count[q] > 0;
        T[P_GATE * tn + e] = hit ? make_float4(p.f_normal[0][q], p.f_normal[1][q], p.f_normal[2][q], p.f_depth[q])
                                 : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!hit) {
            T[P_ALB * tn + e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            continue;
        }
        const int n_raw = p.n[q];
        const int nj = imaxs(1, n_raw);
        float var = pixel_variance(p.square_diff[q], n_raw);
        if (!isfinite(var)) var = 1e-8f;
        var = fclamps(var, 1e-8f, prm.var2_max);
        const float nm1 = fmaxf(float(nj - 1), 1.0f);
        float sv[3];
        for (int c = 0; c < 3; ++c) sv[c] = p.sqrt_var_stable[c][q];
        T[P_ALB * tn + e] = make_float4(p.f_albedo[0][q], p.f_albedo[1][q], p.f_albedo[2][q], float(nj));
        T[P_SM * tn + e] = make_float4(p.sqrt_mean[0][q], p.sqrt_mean[1][q], p.sqrt_mean[2][q], p.rpd[4][q]);
        T[P_SV * tn + e] = make_float4(sv[0], sv[1], sv[2], p.rpd[5][q]);
        T[P_A * tn + e] = make_float4(__fdividef(sv[0] * sv[0], nm1), __fdividef(sv[1] * sv[1], nm1),
                                      __fdividef(sv[2] * sv[2], nm1), fmaxs(1e-8f, var / float(nj)));
        T[P_RPD * tn + e] = make_float4(p.rpd[0][q], p.rpd[1][q], p.rpd[2][q], p.rpd[3][q]);
        T[P_CM * tn + e] = make_float4(p.color_mean[0][q], p.color_mean[1][q], p.color_mean[2][q], 0.0f);
    }
    __syncthreads();

    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t idx = int64_t(y) * prm.w + x;
    if (p.hit_count[idx] == 0) {
        const int n_raw = p.n[idx];
        for (int c = 0; c < 3; ++c) p.denoised[c][idx] = p.color_mean[c][idx];
        p.uncertainty[idx] = pixel_variance(p.square_diff[idx], n_raw) / float(imaxs(1, n_raw));
        p.alpha[idx] = 1.0f;
        return;
    }
    const int ei = (threadIdx.y + r) * tw + threadIdx.x + r;
    const float4 gi = T[P_GATE * tn + ei], ali = T[P_ALB * tn + ei];
    const float4 smi4 = T[P_SM * tn + ei], svi4 = T[P_SV * tn + ei], ai4 = T[P_A * tn + ei], ri4 = T[P_RPD * tn + ei];
    const float smi[3] = {smi4.x, smi4.y, smi4.z}, svi[3] = {svi4.x, svi4.y, svi4.z};
    const float nif = ali.w;
    const int n_i = int(nif);
    {
        // the debug planes (main.cpp:1021-1023)
        const int n_raw = p.n[idx];
        float var_i = pixel_variance(p.square_diff[idx], n_raw);
        if (!isfinite(var_i)) var_i = 1e-8f;
        var_i = fclamps(var_i, 1e-8f, prm.var2_max);
        const float vm = fmaxs(1e-8f, var_i / float(n_i));
        p.var_total[idx] = var_i;
        p.var_eff[idx] = vm;
        p.var_ratio[idx] = (var_i > 1e-8f) ? (vm * float(n_i)) / var_i : 0.0f;
    }
    const float dthr = prm.depth_threshold;
    const float dabs_i = fabsf(gi.w);

    // double-float accumulators across rows: colour (3), weight, weight^2, weight^2*var
    float acc_hi[6] = {0, 0, 0, 0, 0, 0}, acc_lo[6] = {0, 0, 0, 0, 0, 0};
    int accepted = 0;
    for (int dy = -r; dy <= r; ++dy) {
        float row[6] = {0, 0, 0, 0, 0, 0};
        const int erow = (threadIdx.y + r + dy) * tw + threadIdx.x + r;
        const float* srow = spatial_tab + (dy + r) * side + r;
#pragma unroll 2
        for (int dx = -r; dx <= r; ++dx) {
            const int e = erow + dx;
            const float4 gj = T[P_GATE * tn + e];
            if (dot3(gi.x, gi.y, gi.z, gj.x, gj.y, gj.z) < prm.normal_threshold) continue;
            const float4 aj = T[P_ALB * tn + e];
            if (!(aj.w > 0.0f)) continue;  // outside the image or no primary hit
            // relative_depth_delta(di, dj) > threshold: fl(num / m) against dthr, decided by
            // the product dthr * m away from the threshold and by the IEEE quotient near it
            float m = dabs_i;
            if (m < fabsf(gj.w)) m = fabsf(gj.w);
            if (m < 1e-8f) m = 1e-8f;
            const float num = fabsf(gi.w - gj.w);
            const float tm = dthr * m;
            bool far;
            if (!(tm >= 1e-30f)) far = __fdiv_rn(num, m) > dthr;  // tiny or zero threshold: no product test
            else if (num > tm * (1.0f + kDepthBand)) far = true;
            else if (num < tm * (1.0f - kDepthBand)) far = false;
            else far = __fdiv_rn(num, m) > dthr;
            if (far) continue;
            const float da0 = ali.x - aj.x, da1 = ali.y - aj.y, da2 = ali.z - aj.z;
            if (dot3(da0, da1, da2, da0, da1, da2) >= prm.albedo_sq_threshold) continue;

            const float4 smj = T[P_SM * tn + e], svj = T[P_SV * tn + e], aaj = T[P_A * tn + e];
            const float njf = aj.w;
            bool exact = false;
            // per channel t^2 / t_crit^2 = md^2 / (vs * tc^2); the largest is found by cross
            // products and divided once, together with the RPD relaxation
            float qn = 0.0f, qd = 1.0f;
            {
                const float sj[3] = {smj.x, smj.y, smj.z}, vj[3] = {svj.x, svj.y, svj.z};
                const float aj3[3] = {aaj.x, aaj.y, aaj.z}, ai3[3] = {ai4.x, ai4.y, ai4.z};
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float vs = svi[c] + vj[c];
                    const float md = smi[c] - sj[c];
                    const float den = ai3[c] + aj3[c];
                    exact |= fabsf(den - 1e-8f) <= 1e-8f * kBand;
                    const float df = den > 1e-8f ? __fdividef(vs * vs, den) : nif + njf - 2.0f;
                    exact |= fabsf(df - prm.df_break) <= prm.df_break * kBand;
                    const float tc = tile_t_lookup(pairs, df, prm);
                    const float n2 = md * md, d2 = vs * tc * tc;
                    if (n2 * qd > qn * d2) {
                        qn = n2;
                        qd = d2;
                    }
                }
            }
            const float4 rj = T[P_RPD * tn + e];
            float shared = fmaxs(fmaxs(fmins(ri4.x, rj.x), fmins(ri4.y, rj.y)),
                                 fmaxs(fmins(ri4.z, rj.z), fmins(ri4.w, rj.w)));
            shared = fmaxs(shared, fmaxs(fmins(smi4.w, smj.w), fmins(svi4.w, svj.w)));
            shared = fclamps(shared, 0.0f, 1.0f);
            const float adjustment = fclamps(prm.rpd_scale * shared, 0.0f, 1.0f);
            const float q = __fdividef(qn, qd * (1.0f + adjustment));
            const bool center = dx == 0 && dy == 0;
            exact |= fabsf(q - 25.0f) <= 25.0f * kBand;
            exact |= !center && fabsf(q - kQAccept) <= kQAccept * kBand;
            float wj;
            if (exact) {
                const float sjx[3] = {smj.x, smj.y, smj.z}, vjx[3] = {svj.x, svj.y, svj.z};
                const double qx = exact_q(svi, smi, n_i, vjx, sjx, int(njf), prm.alpha, adjustment);
                if (qx > 25.0) continue;
                const double sw = 1.0 / (1.0 + double(dx * dx + dy * dy));
                const double wd = sw * exp(-0.5 * qx);
                if (!center && wd > 0.05 * sw) ++accepted;
                wj = float(wd);
            } else {
                if (q > 25.0f) continue;
                if (!center && q < kQAccept) ++accepted;
                wj = srow[dx] * __expf(-0.5f * q);
            }
            const float4 cmj = T[P_CM * tn + e];
            const float w2 = wj * wj;
            row[0] = __fmaf_rn(wj, cmj.x, row[0]);
            row[1] = __fmaf_rn(wj, cmj.y, row[1]);
            row[2] = __fmaf_rn(wj, cmj.z, row[2]);
            row[3] += wj;
            row[4] += w2;
            row[5] = __fmaf_rn(w2, aaj.w, row[5]);
        }
        for (int k = 0; k < 6; ++k) {  // TwoSum into the double-float accumulators
            const float s = acc_hi[k] + row[k];
            const float bb = s - acc_hi[k];
            const float err = (acc_hi[k] - (s - bb)) + (row[k] - bb);
            acc_hi[k] = s;
            acc_lo[k] += err;
        }
    }
    // the blend in single precision from the double-float sums (their relative error, ~1e-7,
    // is far inside the plain-form bar; the weight_sum >= 1.1 test keeps its guard band)
    const float cs0 = acc_hi[0] + acc_lo[0];
    const float cs1 = acc_hi[1] + acc_lo[1];
    const float cs2 = acc_hi[2] + acc_lo[2];
    const float weight_sum = acc_hi[3] + acc_lo[3];
    const float weight_square_sum = acc_hi[4] + acc_lo[4];
    const float weighted_variance_sum = acc_hi[5] + acc_lo[5];
    if (accepted >= 2 && fabsf(weight_sum - 1.1f) <= 1.1f * float(kWsBand)) {
        exact_pixel(p, prm, idx);
        return;
    }
    const float var_mean_i = ai4.w;
    const float4 cmi4 = T[P_CM * tn + ei];
    const float cmi[3] = {cmi4.x, cmi4.y, cmi4.z};
    float mean_nb[3] = {cmi[0], cmi[1], cmi[2]};
    float var_neighbors = var_mean_i;
    if (weight_sum > 1e-8f) {
        const float inv = 1.0f / weight_sum;
        mean_nb[0] = cs0 * inv;
        mean_nb[1] = cs1 * inv;
        mean_nb[2] = cs2 * inv;
        var_neighbors = weighted_variance_sum * inv * inv;
    }
    const float effective = weight_sum * weight_sum / fmaxf(1e-8f, weight_square_sum);
    const float blend = (accepted >= 2 && weight_sum >= 1.1f) ? fminf(fmaxf(1.0f - rsqrtf(effective), 0.0f), 0.8f)
                                                               : 0.0f;
    const float alpha = 1.0f - blend;
    for (int c = 0; c < 3; ++c) p.denoised[c][idx] = lerpf(cmi[c], mean_nb[c], blend);
    const float uncertainty = alpha * alpha * var_mean_i + blend * blend * var_neighbors +
                              2.0f * alpha * blend * (1.0f / fmaxf(weight_sum, 1e-8f)) * var_mean_i;
    p.alpha[idx] = alpha;
    p.uncertainty[idx] = uncertainty;
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
    return size_t(kTileX + 2 * r) * size_t(by + 2 * r) * P_COUNT * sizeof(float4) + 32 * sizeof(float2) +
           side * side * sizeof(float);
}

}  // namespace

cudaError_t launch_statmc(Job& j) {
    const int64_t np = j.g.np;
    {
        KernelScope ks(j, RPD_KERNEL_SQRT_VARIANCE);
        k_sqrt_var_mean<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np);
        // the summed weights of the 3x3 average, accumulated as the reference accumulates them
        double weight_sum = 0.0;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) weight_sum += 1.0 / (1.0 + double(dx * dx + dy * dy));
        const dim3 sgrid((j.g.w + kSvTx - 1) / kSvTx, (j.g.h + kSvTy - 1) / kSvTy);
        k_sqrt_var_stable<<<sgrid, dim3(kSvTx, kSvTy), 0, j.stream>>>(j.p, j.g.w, j.g.h, weight_sum);
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
    prm.var2_max = j.cfg.color_sigma_max * j.cfg.color_sigma_max;
    static const float albedo_sq = sqrt_gate_threshold(0.12f);
    prm.albedo_sq_threshold = albedo_sq;
    // the branch of lookup_t_critical this alpha takes (main.cpp:189-225)
    const float a = std::min(std::max(prm.alpha, 1e-8f), 0.999999f);
    if (std::fabs(a - 0.05f) < 1e-4f) prm.table = 0;
    else if (std::fabs(a - 0.01f) < 1e-4f) prm.table = 1;
    else prm.table = 2;
    prm.z = a <= 0.001f ? 3.29f : a <= 0.005f ? 2.81f : a <= 0.01f ? 2.58f : a <= 0.02f ? 2.33f
          : a <= 0.05f ? 1.96f : a <= 0.10f ? 1.64f : 1.28f;
    prm.df_break = prm.table < 2 ? 30.5f : 30.0f;
    int by = 0;
    for (int cand : {8, 4, 2}) {
        if (tile_bytes(prm.r, cand) <= size_t(110) * 1024) {
            by = cand;
            break;
        }
    }
    // a tuned tile height (RPD_TUNE_STATMC_ROWS) when its tile fits
    if (j.statmc_by > 0 && j.statmc_by <= by) by = j.statmc_by;
    if (j.exact_window || by == 0) {
        k_statmc_window<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, prm);
    } else {
        prm.by = by;
        const size_t smem = tile_bytes(prm.r, by);
        cudaError_t e = cudaFuncSetAttribute(k_statmc_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        const dim3 block(kTileX, by);
        const dim3 grid((j.g.w + kTileX - 1) / kTileX, (j.g.h + by - 1) / by);
        k_statmc_tile<<<grid, block, smem, j.stream>>>(j.p, prm);
    }
    j.launches += 3;
    return cudaGetLastError();
}

}  // namespace rpd
