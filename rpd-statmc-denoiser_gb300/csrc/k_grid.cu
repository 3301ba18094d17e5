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
// k_grid_fast walks the node's support pixels (lanes over pixels) for the totals and the
// screen bins; k_grid_random walks the support's samples (lanes over consecutive samples of
// each support row: coalesced loads) for the random-dimension bins. Each lane owns private
// accumulators, combined in a fixed order at the end: deterministic, no atomics. Sums of y are double-float (pairs of floats, exact
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

    // ---- per-pixel class sums -> totals and (uniform pixels) screen bins ------------------
    bins.clear();
    Totals tot_x, tot_s;
    for (int q0 = 0; q0 < npix; q0 += 32) {
        const int q = q0 + lane;
        bool slow = false;
        int x = 0, y = 0;
        int64_t idx = 0;
        float w = 0.0f;
        bool mixed = false;
        if (q < npix) {
            x = xlo + q % cols;
            y = ylo + q / cols;
            idx = int64_t(y) * g.w + x;
            if (idx >= gpar.first && idx < gpar.first + gpar.count) {
                w = axis_factor(gpar, x, nx, g.nodes_x) * axis_factor(gpar, y, ny, g.nodes_y);
                const float cnt = w > 1e-8f ? gp.cls[grp][0][idx] : 0.0f;  // core/stats.h:103 skips w <= 1e-8
                if (cnt != 0.0f) {
                    const float s1h = gp.cls[grp][1][idx], s1l = gp.cls[grp][2][idx];
                    const float s2h = gp.cls[grp][3][idx], s2l = gp.cls[grp][4][idx];
                    const uint8_t pf = gp.pflags[idx];
                    mixed = grp > 0 && (pf & kPixMixed);
                    add_class(tot_x, w, cnt, s1h, s1l, s2h, s2l);
                    if (!mixed) add_class(tot_s, w, cnt, s1h, s1l, s2h, s2l);
                    if (gpar.uniform_ok && (pf & kPixUniform) && !mixed) {
                        const float su0 = fclamps((float(x) - support_left) / support, 0.0f, 1.0f);
                        const float sv0 = fclamps((float(y) - support_top) / support, 0.0f, 1.0f);
                        const int b = bin2d(su0, sv0);
                        bins.add_weight(b, w, cnt);
                        bins.add_sum(b, w, s1h, s1l);
                    } else {
                        slow = true;
                    }
                }
            }
        }
        // pixels binned sample by sample (and the screen_X totals of mixed pixels): the whole
        // warp walks each such pixel's samples, every lane into its own bins
        unsigned pending = __ballot_sync(0xffffffffu, slow);
        while (pending) {
            const int src = __ffs(pending) - 1;
            pending &= pending - 1;
            const int64_t pidx = __shfl_sync(0xffffffffu, idx, src);
            const float pw = __shfl_sync(0xffffffffu, w, src);
            const bool pmixed = __shfl_sync(0xffffffffu, int(mixed), src) != 0;
            const float fx = float(__shfl_sync(0xffffffffu, x, src));
            const float fy = float(__shfl_sync(0xffffffffu, y, src));
            const int64_t local = pidx - gpar.first;
            const int64_t kend = offsets[local + 1];
            for (int64_t k = offsets[local] + lane; k < kend; k += 32) {
                const uint32_t key = gp.key[k];
                if (!(key & pbit) || !(key & vbit)) continue;
                const float yv = gp.lum[k];
                const float su = fclamps((fx + s.pixel_u[0][k] - support_left) / support, 0.0f, 1.0f);
                const float sv = fclamps((fy + s.pixel_u[1][k] - support_top) / support, 0.0f, 1.0f);
                const int b = bin2d(su, sv);
                bins.add_weight(b, pw, 1.0f);
                bins.add_sum(b, pw, yv, 0.0f);
                if (pmixed) add_sample(tot_s, pw, yv);
            }
        }
    }
    // screen bins and totals: `pixel` for group 0, screen_X (and X's totals) otherwise
    bins.reduce_into(base + dep_s * kDepStride);
    reduce_totals_into(tot_s, base + dep_s * kDepStride);
    if (grp == 0) return;
    reduce_totals_into(tot_x, base + dep_x * kDepStride);
}

// ---- random-dimension bins (Dependency2D::add / BinnedDependency::add of brdf, lens,
// light_uv, environment, light_select and rr; main.cpp:356-375) --------------------------
//
// One block per node, NW warps splitting the node's support rows. A lane walks consecutive
// samples of a row segment (coalesced key/luminance loads) and updates, for each sample, the
// bins of all six random dimensions at once: the key, the luminance and the node weight are
// read and formed once per sample. Every lane owns private bins in shared memory
// ([slot][lane], conflict free); the block combines warps and lanes in a fixed order at the
// end, so the result is deterministic.
constexpr int kRandDims = 6;
constexpr int kRandSlots = 5 * 16 + 2;  // brdf, lens, light_uv, environment, light_select; rr has 2 bins
__host__ __device__ constexpr int rand_slot0(int d) { return d * 16; }
// d: 0 brdf, 1 lens, 2 light_uv, 3 environment, 4 light_select, 5 rr (grid group d + 1)
__host__ __device__ constexpr int rand_dep(int d) {
    return d == 0 ? D_BRDF : d == 1 ? D_LENS : d == 2 ? D_LIGHT_UV : d == 3 ? D_ENV : d == 4 ? D_LIGHT_SELECT : D_RR;
}
constexpr uint32_t kRandValidMask = (0x3fu << 22);  // key valid bits of the six dimensions

struct RandParams {
    GridParams gp;
    uint32_t spp_magic;  // floor(k / spp) == umulhi(k, magic) for every in-segment k (0: search)
    int spp_shift;       // spp is 2^shift (-1: not a power of two)
    int cols;            // support columns of a node, 2 * step + 3 (shared-memory tables)
};

template <bool INT_W>
struct RandLayout {
    // per warp: weights [kRandSlots][32] (u32 exact integers or float2 double-float), then
    // sums [kRandSlots][32] float2
    static constexpr int kWeightBytes = kRandSlots * 32 * (INT_W ? 4 : 8);
    static constexpr int kWarpBytes = kWeightBytes + kRandSlots * 32 * 8;
};

template <bool INT_W, int NW>
__global__ void __launch_bounds__(NW * 32) k_grid_random(RandParams rp, double* pass_grid, const int64_t* offsets,
                                                         GridPrep gp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using L = RandLayout<INT_W>;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const GridParams& gpar = rp.gp;
    const Geometry& g = gpar.g;
    const int64_t node = blockIdx.x;
    const int nx = int(node % g.nodes_x), ny = int(node / g.nodes_x);
    unsigned char* wbase = smem_raw + warp * L::kWarpBytes;
    uint32_t* wint = reinterpret_cast<uint32_t*>(wbase);
    float2* wdf = reinterpret_cast<float2*>(wbase);
    float2* sums = reinterpret_cast<float2*>(wbase + L::kWeightBytes);
    // column factors of the support (x factor * step, exact for a power-of-two step), and the
    // offsets of each warp's current row segment (varying counts)
    int64_t* seg = reinterpret_cast<int64_t*>(smem_raw + NW * L::kWarpBytes);
    int64_t* myseg = seg + warp * (rp.cols + 1);
    float* xf = reinterpret_cast<float*>(seg + NW * (rp.cols + 1));

    const int xlo = imaxs(0, (nx - 1) * g.step - 1), xhi = imins(g.w - 1, (nx + 1) * g.step + 1);
    const int ylo = imaxs(0, (ny - 1) * g.step - 1), yhi = imins(g.h - 1, (ny + 1) * g.step + 1);
    for (int c = threadIdx.x; c < rp.cols; c += NW * 32)
        xf[c] = (xlo + c <= xhi) ? axis_factor(gpar, xlo + c, nx, g.nodes_x) : 0.0f;
    for (int k = 0; k < kRandSlots; ++k) {
        if (INT_W) wint[k * 32 + lane] = 0u;
        else wdf[k * 32 + lane] = make_float2(0.0f, 0.0f);
        sums[k * 32 + lane] = make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    int xa = xhi + 1, xb = xlo - 1;  // the columns with x factor > 0
    for (int x = xlo; x <= xhi; ++x)
        if (xf[x - xlo] > 0.0f) {
            xa = imins(xa, x);
            xb = imaxs(xb, x);
        }
    const float wscale = float(g.step) * float(g.step);
    const float inv_wscale = 1.0f / wscale;

    for (int y = ylo + warp; y <= yhi; y += NW) {
        const float ay = axis_factor(gpar, y, ny, g.nodes_y);
        if (ay <= 0.0f || xa > xb) continue;
        int64_t p0 = int64_t(y) * g.w + xa, p1 = int64_t(y) * g.w + xb + 1;
        p0 = p0 < gpar.first ? gpar.first : p0;
        p1 = p1 > gpar.first + gpar.count ? gpar.first + gpar.count : p1;
        if (p0 >= p1) continue;
        const int npx = int(p1 - p0);
        const int64_t* off = offsets + (p0 - gpar.first);
        if (rp.spp_magic == 0u && rp.spp_shift < 0) {
            __syncwarp();
            for (int q = lane; q <= npx; q += 32) myseg[q] = off[q];
            __syncwarp();
        }
        const int64_t k0 = off[0], k1 = off[npx];
        const int col0 = int(p0 - int64_t(y) * g.w) - xlo;  // xf index of the segment's first pixel
        const int n = int(k1 - k0);
        constexpr int U = 4;  // samples per lane in flight
        for (int kb = lane; kb < n; kb += 32 * U) {
            uint32_t keys[U];
            float ys[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int kk = kb + 32 * u;
                keys[u] = kk < n ? gp.key[k0 + kk] : 0u;
                ys[u] = kk < n ? gp.lum[k0 + kk] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t key = keys[u];
                if (!(key & kRandValidMask)) continue;
                const int kk = kb + 32 * u;
                int pl;
                if (rp.spp_shift >= 0) {
                    pl = kk >> rp.spp_shift;
                } else if (rp.spp_magic) {
                    pl = int(__umulhi(uint32_t(kk), rp.spp_magic));
                } else {
                    int lo = 0, hi = npx - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (myseg[mid] - k0 <= kk) lo = mid; else hi = mid - 1;
                    }
                    pl = lo;
                }
                const float w = xf[col0 + pl] * ay;
                if (w <= 1e-8f) continue;  // BinnedDependency::add skips (core/stats.h:103)
                const uint32_t iw = INT_W ? uint32_t(w * wscale) : 0u;
                const float wy = w * ys[u];
                const float wye = __fmaf_rn(w, ys[u], -wy);
                // the six dimensions own disjoint slot ranges: load all, update, store all
                int slot[kRandDims];
                bool on[kRandDims];
                uint32_t wi[kRandDims];
                float2 wd[kRandDims], sy[kRandDims];
#pragma unroll
                for (int d = 0; d < kRandDims; ++d) {
                    on[d] = (key & key_valid_bit(d + 1)) != 0;
                    const uint32_t bin = (key >> (d == 5 ? 20 : key_bin_shift(d + 1))) & (d == 5 ? 1u : 15u);
                    slot[d] = (rand_slot0(d) + int(bin)) * 32 + lane;
                }
#pragma unroll
                for (int d = 0; d < kRandDims; ++d) {
                    if (!on[d]) continue;
                    if (INT_W) wi[d] = wint[slot[d]];
                    else wd[d] = wdf[slot[d]];
                    sy[d] = sums[slot[d]];
                }
#pragma unroll
                for (int d = 0; d < kRandDims; ++d) {
                    if (!on[d]) continue;
                    if (INT_W) wi[d] += iw;
                    else df_add(wd[d].x, wd[d].y, w);
                    df_add(sy[d].x, sy[d].y, wy);
                    sy[d].y += wye;
                }
#pragma unroll
                for (int d = 0; d < kRandDims; ++d) {
                    if (!on[d]) continue;
                    if (INT_W) wint[slot[d]] = wi[d];
                    else wdf[slot[d]] = wd[d];
                    sums[slot[d]] = sy[d];
                }
            }
        }
    }
    __syncthreads();
    // combine: thread t owns values v = t, t + NW*32, ... of [weights(kRandSlots), sums(kRandSlots)],
    // summed over warps in order and over lanes in a rotated order (32 different banks)
    for (int v = threadIdx.x; v < 2 * kRandSlots; v += NW * 32) {
        const bool is_w = v < kRandSlots;
        const int slot = is_w ? v : v - kRandSlots;
        int d = 0;
        while (d < kRandDims - 1 && slot >= rand_slot0(d + 1)) ++d;
        const int bin = slot - rand_slot0(d);
        double out;
        if (is_w && INT_W) {
            uint64_t total = 0;
            for (int wi = 0; wi < NW; ++wi) {
                const uint32_t* src = reinterpret_cast<const uint32_t*>(smem_raw + wi * L::kWarpBytes) + slot * 32;
                for (int i = 0; i < 32; ++i) total += src[(i + v) & 31];
            }
            out = double(total) * double(inv_wscale);
        } else {
            // four interleaved double-float partial sums, then combined in a fixed order
            float h[4] = {0.0f, 0.0f, 0.0f, 0.0f}, l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int wi = 0; wi < NW; ++wi) {
                const unsigned char* b = smem_raw + wi * L::kWarpBytes;
                const float2* src = reinterpret_cast<const float2*>(is_w ? b : b + L::kWeightBytes) + slot * 32;
                for (int i = 0; i < 32; i += 4) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float2 q = src[(i + j + v) & 31];
                        df_add(h[j], l[j], q.x);
                        l[j] += q.y;
                    }
                }
            }
            for (int j = 1; j < 4; ++j) {
                df_add(h[0], l[0], h[j]);
                l[0] += l[j];
            }
            out = double(h[0]) + double(l[0]);
        }
        if (out != 0.0) pass_grid[(node * kDeps + rand_dep(d)) * kDepStride + (is_w ? bin : 16 + bin)] += out;
    }
}

}  // namespace

namespace {

// floor(k / spp) through a multiply-high: magic = ceil(2^32 / spp), checked for every k a
// row segment can hold (returns 0 when it does not hold, and the kernel searches instead)
uint32_t spp_magic_for(int spp, int max_k) {
    if (spp <= 0) return 0u;
    const uint64_t m = ((uint64_t(1) << 32) + uint64_t(spp) - 1) / uint64_t(spp);
    if (m > 0xffffffffull) return 0u;
    for (int k = 0; k < max_k; ++k)
        if (int((uint64_t(k) * m) >> 32) != k / spp) return 0u;
    return uint32_t(m);
}

template <bool INT_W, int NW>
cudaError_t launch_random(Job& j, const RandParams& rp, const GridPrep& gp) {
    const size_t smem = size_t(NW) * RandLayout<INT_W>::kWarpBytes + size_t(NW) * (rp.cols + 1) * 8 +
                        size_t(rp.cols) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_grid_random<INT_W, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem));
    if (e != cudaSuccess) return e;
    k_grid_random<INT_W, NW><<<unsigned(j.g.nn), NW * 32, smem, j.stream>>>(rp, j.n.pass_grid, j.offsets, gp);
    j.launches += 1;
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_grid_fast(Job& j, const DeviceSamples& s, int64_t first, int64_t count, const GridPrep& gp,
                             int32_t spp, int32_t max_count) {
    const int step = j.g.step;
    const bool pow2 = (step & (step - 1)) == 0;
    GridParams gpar{j.g, first, count, 0, pow2 ? 1 : 0, 1.0f / float(step), spp, spp > 0 ? 1.0f / float(spp) : 0.0f};
    const int sup = j.g.support;
    gpar.uniform_ok = (sup >= 4 && sup <= 2048 && (sup & (sup - 1)) == 0) ? 1 : 0;
    // exact integer bin weights need a power-of-two step and a per-bin total below 2^32:
    // at most support^2 pixels * max_count samples * step^2
    const double bound = double(sup + 3) * double(sup + 3) * double(std::max(max_count, 1)) * double(step) * double(step);
    const bool int_w = pow2 && bound < 4.0e9;
    cudaError_t e;
    {
        KernelScope ks(j, RPD_KERNEL_GRID);
        if (int_w) {
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
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    KernelScope ks(j, RPD_KERNEL_GRID_RANDOM);
    RandParams rp{gpar, 0u, -1, 2 * step + 3};
    if (spp > 0) {
        if ((spp & (spp - 1)) == 0) {
            int sh = 0;
            while ((1 << sh) < spp) ++sh;
            rp.spp_shift = sh;
        } else {
            rp.spp_magic = spp_magic_for(spp, (2 * step + 3) * spp);
        }
    }
    return int_w ? launch_random<true, 2>(j, rp, gp) : launch_random<false, 2>(j, rp, gp);
}

}  // namespace rpd
