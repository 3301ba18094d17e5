// accumulate_rpf_sample_to_grid (main.cpp:329-376), fast path.
//
// One warp per (node, dimension group). Group 0 owns the `pixel` dependency; groups 1-6
// own a random dimension X (brdf, lens, light_uv, environment, light_select, rr) together
// with its screen comparator screen_X. The reference's per-sample double-precision
// accumulations are regrouped by what they depend on:
//   * the node weight w = fl(ax * ay) is a per-pixel product of an x factor and a y factor,
//     so every total of a dependency (w_sum, w2_sum, y_sum, y2_sum) is w times a per-pixel
//     class sum (count, sum y, sum y^2) that the statistics pass produced;
//   * the screen bin of a sample depends on the node and on where the sample lies in its
//     pixel; with a power-of-two support of at least 4 pixels every sample whose position
//     stays inside its pixel falls in the pixel's nominal bin, so a uniform pixel updates
//     one screen bin once (other pixels, and other supports, are binned sample by sample
//     exactly as the reference bins them);
//   * only the random-dimension bins are updated per sample, from the packed key the
//     statistics pass wrote.
// Phase A walks the node's support pixels (lanes over pixels); phase B walks the support's
// samples (lanes over consecutive samples of each support row: coalesced loads). Each lane
// owns private accumulators, combined across the warp at the end of each phase in a fixed
// order: deterministic, no atomics. Sums of y are double-float (pairs of floats, exact
// products via FMA; about 2^-44 relative — GB300 executes double precision at 1/55 of its
// single-precision rate). With a power-of-two node step every weight is an exact multiple
// of 1/step^2, so the bin weights are accumulated as exact integers.
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

constexpr int kGroups = 7;

__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (x - bb);
    hi = s;
}

// (hi, lo) += a * (bh + bl), with the product a*bh split exactly
__device__ __forceinline__ void df_add_scaled(float& hi, float& lo, float a, float bh, float bl) {
    const float p = a * bh;
    const float e = __fmaf_rn(a, bh, -p);
    df_add(hi, lo, p);
    lo += __fmaf_rn(a, bl, e);
}

struct DF {
    float h = 0.0f, l = 0.0f;
};

struct Totals {
    DF w, w2, y, y2;
};

// Dependency2D::add bin (core/stats.h:166-168)
__device__ __forceinline__ int bin2d(float u, float v) {
    const int x = iclamps(int(u * 4.0f), 0, 3);
    const int z = iclamps(int(v * 4.0f), 0, 3);
    return z * 4 + x;
}

__device__ __forceinline__ void add_class(Totals& t, float w, float c, float s1h, float s1l, float s2h, float s2l) {
    df_add_scaled(t.w.h, t.w.l, w, c, 0.0f);
    const float w2 = w * w;
    const float w2e = __fmaf_rn(w, w, -w2);
    df_add_scaled(t.w2.h, t.w2.l, c, w2, w2e);
    df_add_scaled(t.y.h, t.y.l, w, s1h, s1l);
    df_add_scaled(t.y2.h, t.y2.l, w, s2h, s2l);
}

__device__ __forceinline__ void add_sample(Totals& t, float w, float y) {
    df_add(t.w.h, t.w.l, w);
    const float w2 = w * w;
    df_add(t.w2.h, t.w2.l, w2);
    t.w2.l += __fmaf_rn(w, w, -w2);
    const float wy = w * y;
    const float wye = __fmaf_rn(w, y, -wy);
    df_add(t.y.h, t.y.l, wy);
    t.y.l += wye;
    const float p = wy * y;  // (w*y)*y with w*y = wy + wye
    const float pe = __fmaf_rn(wy, y, -p);
    df_add(t.y2.h, t.y2.l, p);
    t.y2.l += __fmaf_rn(wye, y, pe);
}

// Lane-private bins in shared memory, [slot][lane] of the warp's region (conflict free).
// INT_W: slots 0-15 hold the bin weights as exact integers w * step^2, 16-31 / 32-47 the
// double-float sums of w*y. Otherwise: weights double-float in 0-15 / 16-31, sums in
// 32-47 / 48-63.
template <bool INT_W>
struct LaneBins {
    static constexpr int kSlots = INT_W ? 48 : 64;
    static constexpr int kSy = INT_W ? 16 : 32;
    float* base;
    int lane;
    float wscale;  // step^2 (INT_W)
    __device__ float& at(int slot) { return base[slot * 32 + lane]; }
    __device__ void clear() {
        for (int k = 0; k < kSlots; ++k) at(k) = 0.0f;
    }
    __device__ void add_weight(int bin, float w, float c) {  // weight += w * c
        if (INT_W) {
            uint32_t* u = reinterpret_cast<uint32_t*>(&at(bin));
            *u += uint32_t(w * wscale) * uint32_t(c);
        } else {
            float wh = at(bin), wl = at(16 + bin);
            df_add_scaled(wh, wl, w, c, 0.0f);
            at(bin) = wh;
            at(16 + bin) = wl;
        }
    }
    __device__ void add_sum(int bin, float w, float sh, float sl) {  // sum_y += w * (sh + sl)
        float yh = at(kSy + bin), yl = at(kSy + 16 + bin);
        df_add_scaled(yh, yl, w, sh, sl);
        at(kSy + bin) = yh;
        at(kSy + 16 + bin) = yl;
    }
    // Sum the 32 lanes in a fixed (rotated) order; lane v owns value v: weight[v] for v < 16,
    // sum_y[v - 16] otherwise. Adds the result to acc[v].
    __device__ void reduce_into(double* acc) {
        __syncwarp();
        const int v = lane;
        double out;
        if (INT_W && v < 16) {
            uint64_t total = 0;
            for (int i = 0; i < 32; ++i) {
                const int src = (i + v) & 31;
                total += reinterpret_cast<const uint32_t*>(base)[v * 32 + src];
            }
            out = double(total) / double(wscale);
        } else {
            const int hi_slot = v < 16 ? v : kSy + (v - 16);
            float h = 0.0f, l = 0.0f;
            for (int i = 0; i < 32; ++i) {
                const int src = (i + v) & 31;  // rotated: the 32 lanes read 32 different banks
                df_add(h, l, base[hi_slot * 32 + src]);
                l += base[(hi_slot + 16) * 32 + src];
            }
            out = double(h) + double(l);
        }
        acc[v] += out;
        __syncwarp();
    }
};

__device__ void reduce_totals_into(Totals t, double* acc) {
    float v[8] = {t.w.h, t.w.l, t.w2.h, t.w2.l, t.y.h, t.y.l, t.y2.h, t.y2.l};
    for (int off = 16; off > 0; off >>= 1) {
        for (int q = 0; q < 4; ++q) {
            const float oh = __shfl_down_sync(0xffffffffu, v[2 * q], off);
            const float ol = __shfl_down_sync(0xffffffffu, v[2 * q + 1], off);
            df_add(v[2 * q], v[2 * q + 1], oh);
            v[2 * q + 1] += ol;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        acc[32] += double(v[0]) + double(v[1]);
        acc[33] += double(v[2]) + double(v[3]);
        acc[34] += double(v[4]) + double(v[5]);
        acc[35] += double(v[6]) + double(v[7]);
    }
}

struct GridParams {
    Geometry g;
    int64_t first, count;
    int uniform_ok;  // power-of-two support >= 4
    int pow2_step;   // the node step is a power of two: x / step is exact
    float inv_step;
    int spp;         // samples per pixel of the push, 0 when the counts vary
    float inv_spp;
};

// x (or y) factor of the bilinear weight of node n for coordinate c (main.cpp:332-346):
// (1 - t) when floor(c / step) is n, t when it is n - 1, 0 otherwise.
__device__ __forceinline__ float axis_factor(const GridParams& gp, int c, int n, int nodes) {
    const float gc = gp.pow2_step ? float(c) * gp.inv_step : float(c) / float(gp.g.step);
    const int c0 = iclamps(int(floorf(gc)), 0, nodes - 1);
    const int c1 = imins(c0 + 1, nodes - 1);
    const float t = fclamps(gc - float(c0), 0.0f, 1.0f);
    if (c0 == n) return 1.0f - t;
    if (c1 == n) return t;
    return 0.0f;
}

template <bool INT_W>
__global__ void __launch_bounds__(kGroups * 32) k_grid_fast(GridParams gpar, double* pass_grid, DeviceSamples s,
                                                            const int64_t* offsets, GridPrep gp) {
    extern __shared__ float sm[];
    const int lane = threadIdx.x & 31;
    const int grp = threadIdx.x >> 5;
    const int64_t node = blockIdx.x;
    const Geometry& g = gpar.g;
    const int nx = int(node % g.nodes_x), ny = int(node / g.nodes_x);
    LaneBins<INT_W> bins{sm + grp * LaneBins<INT_W>::kSlots * 32, lane, float(g.step) * float(g.step)};
    const uint32_t vbit = key_valid_bit(grp);
    const uint32_t pbit = key_valid_bit(0);
    int dep_x = D_PIXEL, dep_s = D_PIXEL;
    switch (grp) {
    case 1: dep_x = D_BRDF; dep_s = D_SCREEN_BRDF; break;
    case 2: dep_x = D_LENS; dep_s = D_SCREEN_LENS; break;
    case 3: dep_x = D_LIGHT_UV; dep_s = D_SCREEN_LIGHT_UV; break;
    case 4: dep_x = D_ENV; dep_s = D_SCREEN_ENV; break;
    case 5: dep_x = D_LIGHT_SELECT; dep_s = D_SCREEN_LIGHT_SELECT; break;
    case 6: dep_x = D_RR; dep_s = D_SCREEN_RR; break;
    default: break;
    }
    double* base = pass_grid + node * kDeps * kDepStride;
    const float support = float(g.support);
    const float half_support = 0.5f * support;
    const float support_left = float(nx * g.step) - half_support;
    const float support_top = float(ny * g.step) - half_support;
    const int xlo = imaxs(0, (nx - 1) * g.step - 1), xhi = imins(g.w - 1, (nx + 1) * g.step + 1);
    const int ylo = imaxs(0, (ny - 1) * g.step - 1), yhi = imins(g.h - 1, (ny + 1) * g.step + 1);
    const int cols = xhi - xlo + 1;
    const int npix = cols * (yhi - ylo + 1);

    // ---- phase A: per-pixel class sums -> totals and (uniform pixels) screen bins ---------
    bins.clear();
    Totals tot_x, tot_s;
    for (int q = lane; q < npix; q += 32) {
        const int x = xlo + q % cols, y = ylo + q / cols;
        const int64_t idx = int64_t(y) * g.w + x;
        if (idx < gpar.first || idx >= gpar.first + gpar.count) continue;
        const float w = axis_factor(gpar, x, nx, g.nodes_x) * axis_factor(gpar, y, ny, g.nodes_y);
        if (w <= 1e-8f) continue;  // BinnedDependency::add skips (core/stats.h:103)
        const float cnt = gp.cls[grp][0][idx];
        if (cnt == 0.0f) continue;
        const float s1h = gp.cls[grp][1][idx], s1l = gp.cls[grp][2][idx];
        const float s2h = gp.cls[grp][3][idx], s2l = gp.cls[grp][4][idx];
        const uint8_t pf = gp.pflags[idx];
        const bool mixed = grp > 0 && (pf & kPixMixed);
        add_class(tot_x, w, cnt, s1h, s1l, s2h, s2l);
        if (!mixed) add_class(tot_s, w, cnt, s1h, s1l, s2h, s2l);
        if (gpar.uniform_ok && (pf & kPixUniform) && !mixed) {
            const float su0 = fclamps((float(x) - support_left) / support, 0.0f, 1.0f);
            const float sv0 = fclamps((float(y) - support_top) / support, 0.0f, 1.0f);
            const int b = bin2d(su0, sv0);
            bins.add_weight(b, w, cnt);
            bins.add_sum(b, w, s1h, s1l);
            continue;
        }
        // screen bins sample by sample (and screen_X totals of mixed pixels)
        const int64_t local = idx - gpar.first;
        for (int64_t k = offsets[local]; k < offsets[local + 1]; ++k) {
            const uint32_t key = gp.key[k];
            if (!(key & pbit) || !(key & vbit)) continue;
            const float yv = gp.lum[k];
            const float su = fclamps((float(x) + s.pixel_u[0][k] - support_left) / support, 0.0f, 1.0f);
            const float sv = fclamps((float(y) + s.pixel_u[1][k] - support_top) / support, 0.0f, 1.0f);
            const int b = bin2d(su, sv);
            bins.add_weight(b, w, 1.0f);
            bins.add_sum(b, w, yv, 0.0f);
            if (mixed) add_sample(tot_s, w, yv);
        }
    }
    // screen bins and totals: `pixel` for group 0, screen_X (and X's totals) otherwise
    bins.reduce_into(base + dep_s * kDepStride);
    reduce_totals_into(tot_s, base + dep_s * kDepStride);
    if (grp == 0) return;
    reduce_totals_into(tot_x, base + dep_x * kDepStride);

    // ---- phase B: random-dimension bins, lanes over consecutive samples -------------------
    bins.clear();
    const int shift = grp == 6 ? 20 : key_bin_shift(grp);
    const uint32_t mask = grp == 6 ? 1u : 15u;
    // the columns this node draws from: x factor > 0
    int xa = xhi + 1, xb = xlo - 1;
    for (int x = xlo; x <= xhi; ++x)
        if (axis_factor(gpar, x, nx, g.nodes_x) > 0.0f) {
            xa = imins(xa, x);
            xb = imaxs(xb, x);
        }
    for (int y = ylo; y <= yhi; ++y) {
        const float ay = axis_factor(gpar, y, ny, g.nodes_y);
        if (ay <= 0.0f || xa > xb) continue;
        int64_t p0 = int64_t(y) * g.w + xa, p1 = int64_t(y) * g.w + xb + 1;
        p0 = p0 < gpar.first ? gpar.first : p0;
        p1 = p1 > gpar.first + gpar.count ? gpar.first + gpar.count : p1;
        if (p0 >= p1) continue;
        const int64_t k0 = offsets[p0 - gpar.first], k1 = offsets[p1 - gpar.first];
        const int xrow0 = int(p0 - int64_t(y) * g.w);
        for (int64_t k = k0 + lane; k < k1; k += 32) {
            const uint32_t key = gp.key[k];
            if (!(key & vbit)) continue;
            const float yv = gp.lum[k];
            int64_t pl;  // the sample's pixel within the row segment
            if (gpar.spp > 0) {
                pl = int64_t(__float2int_rz((float(k - k0) + 0.5f) * gpar.inv_spp));
            } else {
                int64_t lo = 0, hi = p1 - p0 - 1;
                while (lo < hi) {
                    const int64_t mid = (lo + hi + 1) >> 1;
                    if (offsets[p0 - gpar.first + mid] <= k) lo = mid; else hi = mid - 1;
                }
                pl = lo;
            }
            const float w = axis_factor(gpar, xrow0 + int(pl), nx, g.nodes_x) * ay;
            if (w <= 1e-8f) continue;
            const int rb = int((key >> shift) & mask);
            bins.add_weight(rb, w, 1.0f);
            bins.add_sum(rb, w, yv, 0.0f);
        }
    }
    bins.reduce_into(base + dep_x * kDepStride);
}

}  // namespace

cudaError_t launch_grid_fast(Job& j, const DeviceSamples& s, int64_t first, int64_t count, const GridPrep& gp,
                             int32_t spp, int32_t max_count) {
    KernelScope ks(j, RPD_KERNEL_GRID);
    const int step = j.g.step;
    const bool pow2 = (step & (step - 1)) == 0;
    GridParams gpar{j.g, first, count, 0, pow2 ? 1 : 0, 1.0f / float(step), spp, spp > 0 ? 1.0f / float(spp) : 0.0f};
    const int sup = j.g.support;
    gpar.uniform_ok = (sup >= 4 && (sup & (sup - 1)) == 0) ? 1 : 0;
    // exact integer bin weights need a power-of-two step and a per-bin total below 2^32:
    // at most support^2 pixels * max_count samples * step^2
    const double bound = double(sup + 3) * double(sup + 3) * double(std::max(max_count, 1)) * double(step) * double(step);
    cudaError_t e;
    if (pow2 && bound < 4.0e9) {
        const size_t smem = size_t(kGroups) * LaneBins<true>::kSlots * 32 * sizeof(float);
        e = cudaFuncSetAttribute(k_grid_fast<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        k_grid_fast<true><<<unsigned(j.g.nn), kGroups * 32, smem, j.stream>>>(gpar, j.n.pass_grid, s, j.offsets, gp);
    } else {
        const size_t smem = size_t(kGroups) * LaneBins<false>::kSlots * 32 * sizeof(float);
        e = cudaFuncSetAttribute(k_grid_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
        k_grid_fast<false><<<unsigned(j.g.nn), kGroups * 32, smem, j.stream>>>(gpar, j.n.pass_grid, s, j.offsets, gp);
    }
    j.launches += 1;
    return cudaGetLastError();
}

}  // namespace rpd
