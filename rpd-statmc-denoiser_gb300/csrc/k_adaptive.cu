// compute_adaptive_sample_counts (main.cpp:1273-1446).
//
//   k_importance        variance source and importance = sqrt (1303-1327)
//   k_smooth_importance edge-aware smoothing (1331-1368), its double-precision products carried
//                       out exactly in integer instructions
//   k_allocate_coop     the budget-preserving allocation (1329-1438) in parallel, with the
//                       reference's integers bit for bit (k_allocate.cu)
//   k_allocate_serial   the same allocation as one device thread in the reference's order. It
//                       runs behind the parallel kernel and returns at once unless that kernel
//                       flagged a case outside its method (or RPD_TUNE_ALLOCATOR selects it).
#include <algorithm>
#include <cfloat>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "exact_arith.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ float pixel_variance(float m2, int n) { return (n > 1) ? m2 / float(n - 1) : 0.0f; }

__global__ void k_importance(PixelPlanes p, int64_t np, float sigma_max) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float raw = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(raw)) raw = 1e-8f;
    raw = fmaxs(1e-8f, raw);
    float dsv = p.variance_denoised[i];
    if (!isfinite(dsv) || dsv <= 0.0f) dsv = raw;
    const float vs = fclamps(fmaxs(raw, dsv), 1e-8f, sigma_max * sigma_max);
    p.importance[i] = sqrtf(vs);
}

// The edge-aware smoothing of one pixel (main.cpp:1339-1366) in the reference's double-precision
// instructions.
__device__ float smooth_pixel_fp64(const PixelPlanes& p, int w, int h, int radius, const float* in, int x, int y,
                                   int64_t idx) {
    const float ni0 = p.f_normal[0][idx], ni1 = p.f_normal[1][idx], ni2 = p.f_normal[2][idx];
    const float di = p.f_depth[idx];
    double accum = 0.0, weight_sum = 0.0;
    for (int dy = -radius; dy <= radius; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= h) continue;
        for (int dx = -radius; dx <= radius; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= w) continue;
            const int64_t nidx = int64_t(yy) * w + xx;
            if (p.hit_count[nidx] == 0) continue;
            const float spatial_w = 1.0f / (1.0f + float(dx * dx + dy * dy));
            const float normal_w = fclamps(
                (dot3(ni0, ni1, ni2, p.f_normal[0][nidx], p.f_normal[1][nidx], p.f_normal[2][nidx]) + 1.0f) * 0.5f,
                0.0f, 1.0f);
            const float depth_w = expf(-4.0f * relative_depth_delta(di, p.f_depth[nidx]));
            const double w_neighbor = double(spatial_w) * double(normal_w) * double(depth_w);
            accum += w_neighbor * double(in[nidx]);
            weight_sum += w_neighbor;
        }
    }
    return (weight_sum > double(1e-8f)) ? float(accum / weight_sum) : in[idx];
}

// The same pixel with the products in integer instructions (XD) and the two sums as double
// additions of the products' bits: the same bits as smooth_pixel_fp64 with three of its five
// double-precision operations per neighbour, and none of its conversions, left out (the two sums
// in integer instructions as well measured slower: 0.53 -> 0.61 ms per 1920x1080 adaptive
// step, the integer additions cost more issue than the double pipe's wait). R > 0 fixes
// the radius at compile time (R = 0: `radius`). Returns false for inputs outside the integer
// form (negative, subnormal or non-finite weights or importances).
template <int R>
__device__ bool smooth_pixel_int(const PixelPlanes& p, int w, int h, int radius, const float* in, int x, int y,
                                 int64_t idx, float& out) {
    const int rad = R > 0 ? R : radius;
    const float ni0 = p.f_normal[0][idx], ni1 = p.f_normal[1][idx], ni2 = p.f_normal[2][idx];
    const float di = p.f_depth[idx];
    double accum = 0.0, weight_sum = 0.0;
    bool ok = true;
#pragma unroll
    for (int dy = -rad; dy <= rad; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= h) continue;
        const int64_t row = idx + int64_t(dy) * w;
#pragma unroll
        for (int dx = -rad; dx <= rad; ++dx) {
            const int xx = x + dx;
            if (xx < 0 || xx >= w) continue;
            const int64_t nidx = row + dx;
            if (p.hit_count[nidx] == 0) continue;
            const float spatial_w = 1.0f / (1.0f + float(dx * dx + dy * dy));
            const float normal_w = fclamps(
                (dot3(ni0, ni1, ni2, p.f_normal[0][nidx], p.f_normal[1][nidx], p.f_normal[2][nidx]) + 1.0f) * 0.5f,
                0.0f, 1.0f);
            const float depth_w = expf(-4.0f * relative_depth_delta(di, p.f_depth[nidx]));
            const float imp = in[nidx];
            uint32_t sm, nm, dm, im;
            int se, ne, de, ie;
            float_parts(spatial_w, sm, se);
            const bool nok = float_parts(normal_w, nm, ne), dok = float_parts(depth_w, dm, de);
            const bool iok = float_parts(imp, im, ie);
            if (!(nok && dok)) {
                // a zero normal weight (opposite normals) adds exact zeros to both sums
                if (normal_w == 0.0f && dok && (iok || imp == 0.0f)) continue;
                ok = false;
                continue;
            }
            // (spatial * normal) * depth: the first product is exact; the second is exact too
            // when the spatial weight is a power of two (then it is normal * depth scaled), else
            // rounded
            const XD wn = sm == 0x800000u ? xd_exact48(uint64_t(nm) * dm, ne + de + se + 23)
                                          : xd_mul24(uint64_t(sm) * nm, dm, se + ne + de);
            if (iok) accum += xd_to_double(xd_mul24(wn.m, im, wn.e + ie));
            else if (imp != 0.0f) ok = false;
            weight_sum += xd_to_double(wn);
        }
    }
    if (!ok) return false;
    if (!(weight_sum > double(1e-8f))) {
        out = in[idx];
        return true;
    }
    if (accum == 0.0) {
        out = 0.0f;
        return true;
    }
    const long long ab = __double_as_longlong(accum), wb = __double_as_longlong(weight_sum);
    const uint64_t am = (uint64_t(ab) & ((1ull << 52) - 1ull)) | (1ull << 52);
    const uint64_t wm = (uint64_t(wb) & ((1ull << 52) - 1ull)) | (1ull << 52);
    const int ae = int((ab >> 52) & 0x7ff) - 1075, we = int((wb >> 52) & 0x7ff) - 1075;
    if (!quotient_to_float(am, ae, wm, we, out)) out = float(accum / weight_sum);
    return true;
}

__global__ void k_smooth_importance(PixelPlanes p, int w, int h, int radius, const float* in, float* out,
                                    int fp64) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(w) * h) return;
    if (p.hit_count[idx] == 0) {
        out[idx] = in[idx];
        return;
    }
    const int y = int(idx / w), x = int(idx % w);
    float v = 0.0f;
    bool done = false;
    if (!fp64) {
        done = radius == 1 ? smooth_pixel_int<1>(p, w, h, radius, in, x, y, idx, v)
                           : smooth_pixel_int<0>(p, w, h, radius, in, x, y, idx, v);
    }
    if (!done) v = smooth_pixel_fp64(p, w, h, radius, in, x, y, idx);
    out[idx] = v;
}

// hash_u32 / hash_to_unit_float (main.cpp:270-281)
__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

struct AllocParams {
    int64_t np;
    int extra_sample_total;
    int reserved_samples;
    int max_extra_per_pixel;
    uint32_t seed;
};

__global__ void k_allocate_serial(PixelPlanes p, AllocParams a, const float* importance, const int* guard,
                                  int floor_per_pixel) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int64_t np = a.np;
    if (guard) {
        if (*(volatile const int*)guard == 0) return;  // the parallel allocation completed
        for (int64_t i = 0; i < np; ++i) p.counts[i] = floor_per_pixel;
    }
    double sum_importance = 0.0;
    for (int64_t i = 0; i < np; ++i) sum_importance = sum_importance + double(importance[i]);
    int remaining_samples = imaxs(0, a.extra_sample_total - a.reserved_samples);
    if (sum_importance <= 0.0 || remaining_samples <= 0) return;
    float* desired_add = p.desired_add;
    for (int64_t i = 0; i < np; ++i) desired_add[i] = 0.0f;
    int32_t* active = p.active_a;
    int32_t* next_active = p.active_b;
    int64_t n_active = np;
    for (int64_t i = 0; i < np; ++i) active[i] = int32_t(i);
    double remaining_importance = sum_importance;
    while (n_active > 0 && remaining_samples > 0 && remaining_importance > double(1e-8f)) {
        bool clipped = false;
        int64_t n_next = 0;
        for (int64_t k = 0; k < n_active; ++k) {
            const int32_t idx = active[k];
            const double share = double(importance[idx]) / remaining_importance;
            const double desired = share * double(remaining_samples);
            if (desired > double(a.max_extra_per_pixel)) {
                desired_add[idx] = float(a.max_extra_per_pixel);
                remaining_samples -= a.max_extra_per_pixel;
                remaining_importance -= double(importance[idx]);
                clipped = true;
            } else {
                next_active[n_next++] = idx;
            }
        }
        if (!clipped) {
            for (int64_t k = 0; k < n_next; ++k) {
                const int32_t idx = next_active[k];
                desired_add[idx] = float(double(importance[idx]) / remaining_importance * double(remaining_samples));
            }
            break;
        }
        int32_t* t = active;
        active = next_active;
        next_active = t;
        n_active = n_next;
    }
    int assigned = 0;
    double residual_sum = 0.0;
    for (int64_t i = 0; i < np; ++i) {
        const int add = int(floorf(desired_add[i]));
        p.counts[i] += add;
        assigned += add;
        p.residual[i] = fmaxs(0.0f, desired_add[i] - float(add));
        residual_sum += double(p.residual[i]);
    }
    const int remaining = imaxs(0, a.extra_sample_total - a.reserved_samples - assigned);
    if (remaining > 0 && residual_sum > double(1e-8f)) {
        const double offset = double(float(hash_u32(a.seed ^ 0x4d595df4u) & 0x00ffffffu) / float(0x01000000u));
        double cumulative = 0.0;
        int64_t cursor = 0;
        for (int k = 0; k < remaining; ++k) {
            const double target = ((double(k) + offset) / double(remaining)) * residual_sum;
            while (cursor < np && cumulative + double(p.residual[cursor]) < target) {
                cumulative += double(p.residual[cursor]);
                ++cursor;
            }
            if (cursor < np) p.counts[cursor]++;
        }
    }
}

__global__ void k_fill_counts(int32_t* counts, int64_t np, int value) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < np) counts[i] = value;
}

__global__ void k_copy(const float* src, float* dst, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

}  // namespace

namespace {

// The allocation from the final importance map in j.p.importance (main.cpp:1372-1438); the
// counts hold the floor already.
cudaError_t launch_allocation(Job& j, int extra_sample_total, int floor_per_pixel) {
    const int64_t np = j.g.np;
    const float* importance = j.p.importance;
    AllocParams a{np, extra_sample_total, floor_per_pixel * j.g.w * j.g.h,
                  std::max(4, 8 * std::max(1, j.cfg.adaptive_spp)), j.cfg.seed};
    const int* guard = nullptr;
    if (!j.serial_allocator) {
        const cudaError_t e = launch_allocate_parallel(j, importance, a.extra_sample_total, a.reserved_samples,
                                                       a.max_extra_per_pixel, a.seed, &guard);
        if (e != cudaSuccess) return e;
    }
    k_allocate_serial<<<1, 1, 0, j.stream>>>(j.p, a, importance, guard, floor_per_pixel);
    j.launches += 1;
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_adaptive(Job& j) {
    KernelScope ks(j, RPD_KERNEL_ADAPTIVE);
    const int64_t np = j.g.np;
    const int w = j.g.w, h = j.g.h;
    const int extra_sample_total = j.cfg.adaptive_spp * w * h;
    const int floor_per_pixel = std::clamp(j.cfg.adaptive_base_samples, 0, j.cfg.adaptive_spp);
    k_fill_counts<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p.counts, np, floor_per_pixel);
    j.launches += 1;
    if (extra_sample_total <= 0) return cudaGetLastError();
    k_importance<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, j.cfg.adaptive_sigma_max);
    j.launches += 1;
    const int radius = j.cfg.adaptive_importance_smoothing_radius;
    if (radius > 0) {
        k_smooth_importance<<<grid_for(np, 128), 128, 0, j.stream>>>(j.p, w, h, radius, j.p.importance,
                                                                     j.p.importance_tmp, j.smooth_fp64 ? 1 : 0);
        k_copy<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p.importance_tmp, j.p.importance, np);
        j.launches += 2;
    }
    return launch_allocation(j, extra_sample_total, floor_per_pixel);
}

cudaError_t launch_allocate_map(Job& j) {
    KernelScope ks(j, RPD_KERNEL_ADAPTIVE);
    const int64_t np = j.g.np;
    const int extra_sample_total = j.cfg.adaptive_spp * j.g.w * j.g.h;
    const int floor_per_pixel = std::clamp(j.cfg.adaptive_base_samples, 0, j.cfg.adaptive_spp);
    k_fill_counts<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p.counts, np, floor_per_pixel);
    j.launches += 1;
    if (extra_sample_total <= 0) return cudaGetLastError();
    return launch_allocation(j, extra_sample_total, floor_per_pixel);
}

}  // namespace rpd
