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
#include <cmath>
#include <type_traits>

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

// The fast path's pass grid holds every entry as a double-float (hi, lo) pair in the 8 bytes
// of a double; the merge into the frame grid turns it into a double (k_merge_grid).
__device__ __forceinline__ void df_accum(float2* e, float h, float l) {
    float2 v = *e;
    df_add(v.x, v.y, h);
    v.y += l;
    *e = v;
}

// An integer bin weight (a multiple of 1/step^2, below 2^32 by the launch's bound) as a
// double-float: the float of the integer plus the float of its remainder, scaled exactly.
__device__ __forceinline__ float2 int_weight_df(uint64_t total, float inv_wscale) {
    const uint32_t t = uint32_t(total);
    const float hi = __uint2float_rz(t);          // an integer <= t
    const uint32_t rem = t - __float2uint_rz(hi);  // below 2^8, exact in float
    return make_float2(hi * inv_wscale, float(rem) * inv_wscale);
}

struct Totals {
    DF w, w2, y, y2;
};

// The screen position (pixel_u) of sample k, from either sample-plane format.
__device__ __forceinline__ float sample_pu(const DeviceSamples& s, int c, int64_t k) {
    return s.compact ? float(s.c16.pixel_u[c][k]) * (1.0f / 65536.0f) : s.pixel_u[c][k];
}

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
    // sum_y[v - 16] otherwise. Returns the lane's value as a double-float.
    __device__ float2 reduce_value() {
        __syncwarp();
        const int v = lane;
        float2 out;
        if (INT_W && v < 16) {
            uint64_t total = 0;
            for (int i = 0; i < 32; ++i) total += reinterpret_cast<const uint32_t*>(base)[v * 32 + ((i + v) & 31)];
            out = int_weight_df(total, 1.0f / wscale);
        } else {
            const int hi_slot = v < 16 ? v : kSy + (v - 16);
            float h = 0.0f, l = 0.0f;
            for (int i = 0; i < 32; ++i) {
                const int src = (i + v) & 31;  // rotated: the 32 lanes read 32 different banks
                df_add(h, l, base[hi_slot * 32 + src]);
                l += base[(hi_slot + 16) * 32 + src];
            }
            out = make_float2(h, l);
        }
        __syncwarp();
        return out;
    }
    // As reduce_value, adding the result to the pass-grid entry acc[v].
    __device__ void reduce_into(float2* acc) {
        const float2 out = reduce_value();
        if (out.x != 0.0f || out.y != 0.0f) df_accum(acc + lane, out.x, out.y);
    }
};

// Warp sum of the lanes' totals (fixed shuffle tree); the result is valid in lane 0 as
// double-floats (w_sum, w2_sum, y_sum, y2_sum).
__device__ void reduce_totals(Totals t, float2* out4) {
    float v[8] = {t.w.h, t.w.l, t.w2.h, t.w2.l, t.y.h, t.y.l, t.y2.h, t.y2.l};
    for (int off = 16; off > 0; off >>= 1) {
        for (int q = 0; q < 4; ++q) {
            const float oh = __shfl_down_sync(0xffffffffu, v[2 * q], off);
            const float ol = __shfl_down_sync(0xffffffffu, v[2 * q + 1], off);
            df_add(v[2 * q], v[2 * q + 1], oh);
            v[2 * q + 1] += ol;
        }
    }
    for (int q = 0; q < 4; ++q) out4[q] = make_float2(v[2 * q], v[2 * q + 1]);
}

// v[q] for a lane-dependent q in 0-3, without indexing the registers
__device__ __forceinline__ float2 pick4(const float2* v, int q) {
    return q == 0 ? v[0] : q == 1 ? v[1] : q == 2 ? v[2] : v[3];
}

// As reduce_totals, adding the result to the pass-grid entries acc[32..35].
__device__ void reduce_totals_into(Totals t, float2* acc) {
    float2 r[4];
    reduce_totals(t, r);
    if ((threadIdx.x & 31) == 0) {
        for (int q = 0; q < 4; ++q)
            if (r[q].x != 0.0f || r[q].y != 0.0f) df_accum(acc + 32 + q, r[q].x, r[q].y);
    }
}

struct GridParams {
    Geometry g;
    int64_t first, count;
    int64_t node0;        // first node of the launch (the node rows whose supports meet the push)
    int64_t count_nodes;  // nodes of the launch
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

// A pixel's pattern sums, pattern and flags (see GridPrep).
struct PixPattern {
    float c, s1h, s1l, s2h, s2l;
    uint8_t pat, pf;
};
__device__ __forceinline__ PixPattern load_pattern(const GridPrep& gp, int64_t idx) {
    const float4 a = gp.pat4[idx];
    const float2 b = gp.pat2[idx];
    const uint32_t bits = __float_as_uint(b.y);
    return PixPattern{a.x, a.y, a.z, a.w, b.x, uint8_t(bits & 0xffu), uint8_t(bits >> 8)};
}

// The (count, sum y hi/lo, sum y^2 hi/lo) of class c for pixel idx (see GridPrep).
__device__ __forceinline__ void class_sums(const GridPrep& gp, int c, int64_t idx, const PixPattern& pp,
                                           float* out) {
    if (pp.pf & kPixDeviant) {
        for (int f = 0; f < 5; ++f) out[f] = gp.cls[c][f][idx];
    } else if (pp.pat & class_bit(c)) {
        out[0] = pp.c;
        out[1] = pp.s1h;
        out[2] = pp.s1l;
        out[3] = pp.s2h;
        out[4] = pp.s2l;
    } else {
        for (int f = 0; f < 5; ++f) out[f] = 0.0f;
    }
}

template <bool INT_W>
__global__ void __launch_bounds__(kGroups * 32) k_grid_fast(GridParams gpar, float2* pass_grid, DeviceSamples s,
                                                            const int64_t* offsets, GridPrep gp) {
    extern __shared__ float sm[];
    const int lane = threadIdx.x & 31;
    const int grp = threadIdx.x >> 5;
    const int64_t node = gpar.node0 + blockIdx.x;
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
    float2* base = pass_grid + node * kDeps * kDepStride;
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
                const PixPattern pp = load_pattern(gp, idx);
                const uint8_t pf = pp.pf;
                float cs[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                if (w > 1e-8f) class_sums(gp, grp, idx, pp, cs);  // core/stats.h:103 skips w <= 1e-8
                const float cnt = cs[0];
                if (cnt != 0.0f) {
                    const float s1h = cs[1], s1l = cs[2], s2h = cs[3], s2l = cs[4];
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
                const float su = fclamps((fx + sample_pu(s, 0, k) - support_left) / support, 0.0f, 1.0f);
                const float sv = fclamps((fy + sample_pu(s, 1, k) - support_top) / support, 0.0f, 1.0f);
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

// ---- totals and screen bins, pattern form (the default) ----------------------------------
//
// One warp per node. Pixels of the node's pattern P0 (the pattern of its first non-deviant
// support pixel) carry the same class sums for every class in P0, so their totals are formed
// once (TP) and their screen bins once (bins A: per pixel for uniform pixels, sample by sample
// otherwise); each class then takes TP and bins A if it is in P0. Every other pixel (deviant,
// or of another pattern) goes to a list handled class by class as the per-class kernel does
// (bins B). All sums are lane-private and combined in a fixed order: deterministic.
__device__ __forceinline__ int axis_ifactor(int c, int n, int nodes, int sh) {
    // x factor * step of a power-of-two step (c < (nodes - 1) * step for every image pixel)
    const int c0 = imins(c >> sh, nodes - 1);
    const int t = c - (c0 << sh);
    return c0 == n ? (1 << sh) - t : (c0 + 1 == n ? t : 0);
}

template <bool INT_W>
__global__ void __launch_bounds__(32) k_grid_screen(GridParams gpar, float2* pass_grid, DeviceSamples s,
                                                    const int64_t* offsets, GridPrep gp) {
    extern __shared__ float sm[];
    constexpr int kS = LaneBins<INT_W>::kSlots;
    const int lane = threadIdx.x;
    const int64_t node = gpar.node0 + blockIdx.x;
    const Geometry& g = gpar.g;
    const int nx = int(node % g.nodes_x), ny = int(node / g.nodes_x);
    const float wscale = float(g.step) * float(g.step);
    LaneBins<INT_W> binsA{sm, lane, wscale};
    int* xlist = reinterpret_cast<int*>(sm + kS * 32);
    float2* base = pass_grid + node * kDeps * kDepStride;
    const float support = float(g.support);
    const float half_support = 0.5f * support;
    const float support_left = float(nx * g.step) - half_support;
    const float support_top = float(ny * g.step) - half_support;
    const int xlo = imaxs(0, (nx - 1) * g.step - 1), xhi = imins(g.w - 1, (nx + 1) * g.step + 1);
    const int ylo = imaxs(0, (ny - 1) * g.step - 1), yhi = imins(g.h - 1, (ny + 1) * g.step + 1);
    const int cols = xhi - xlo + 1;
    const int npix = cols * (yhi - ylo + 1);
    const int sh = __ffs(g.step) - 1;                 // log2(step) when the step is a power of two
    const int bsh = __ffs(g.support) - 3;             // log2(support / 4) when uniform_ok
    const int sl = nx * g.step - g.support / 2, st = ny * g.step - g.support / 2;  // integer when uniform_ok
    const float inv_wscale = 1.0f / wscale;
    const uint32_t pbit = key_valid_bit(0);

    auto weight = [&](int x, int y) -> float {
        if (gpar.pow2_step)
            return float(axis_ifactor(x, nx, g.nodes_x, sh) * axis_ifactor(y, ny, g.nodes_y, sh)) * inv_wscale;
        return axis_factor(gpar, x, nx, g.nodes_x) * axis_factor(gpar, y, ny, g.nodes_y);
    };
    // the pixel's nominal screen bin (every sample's, for a uniform pixel)
    auto uniform_bin = [&](int x, int y) -> int {
        const int dx = x - sl, dy = y - st;
        const int bx = dx < 0 ? 0 : imins(dx >> bsh, 3), by = dy < 0 ? 0 : imins(dy >> bsh, 3);
        return by * 4 + bx;
    };
    // samples of pixel (px, py) binned one by one by the whole warp (main.cpp:349-357): every
    // lane into its own bins; also the screen totals of a mixed pixel (samples with the
    // position and the class)
    auto bin_samples = [&](LaneBins<INT_W>& bins, int64_t pidx, float pw, int px, int py, uint32_t vbit,
                           bool pmixed, Totals& ts) {
        const float fx = float(px), fy = float(py);
        const int64_t local = pidx - gpar.first;
        const int64_t kend = offsets[local + 1];
        for (int64_t k = offsets[local] + lane; k < kend; k += 32) {
            const uint32_t key = gp.key[k];
            if (!(key & pbit) || !(key & vbit)) continue;
            const float yv = gp.lum[k];
            const float su = fclamps((fx + sample_pu(s, 0, k) - support_left) / support, 0.0f, 1.0f);
            const float sv = fclamps((fy + sample_pu(s, 1, k) - support_top) / support, 0.0f, 1.0f);
            const int b = bin2d(su, sv);
            bins.add_weight(b, pw, 1.0f);
            bins.add_sum(b, pw, yv, 0.0f);
            if (pmixed) add_sample(ts, pw, yv);
        }
    };

    // ---- P0: the pattern of the first non-deviant support pixel with a pattern ----
    uint8_t P0 = 0;
    for (int q0 = 0; q0 < npix; q0 += 32) {
        const int q = q0 + lane;
        uint8_t pat = 0;
        if (q < npix) {
            const int64_t idx = int64_t(ylo + q / cols) * g.w + xlo + q % cols;
            if (idx >= gpar.first && idx < gpar.first + gpar.count) {
                const uint32_t bits = __float_as_uint(gp.pat2[idx].y);
                if (!((bits >> 8) & kPixDeviant)) pat = uint8_t(bits & 0xffu);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, pat != 0);
        if (m) {
            P0 = uint8_t(__shfl_sync(0xffffffffu, int(pat), __ffs(m) - 1));
            break;
        }
    }
    const bool p0pix = (P0 & RPD_SAMPLE_PIXEL_VALID) != 0;

    // ---- main pass: P0 pixels into TP / bins A, the rest into the list ----
    binsA.clear();
    Totals TP, unused;
    int nlist = 0;
    int x = xlo + lane % cols, y = ylo + lane / cols;  // position of q = q0 + lane
    // the pattern record of q, loaded one iteration ahead so the loads overlap the work
    auto fetch = [&](int q, int px, int py, PixPattern& pp, bool& in) {
        const int64_t idx = int64_t(py) * g.w + px;
        in = q < npix && idx >= gpar.first && idx < gpar.first + gpar.count;
        if (in) pp = load_pattern(gp, idx);
        else pp = PixPattern{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, 0};
    };
    PixPattern nxt;
    bool nin;
    fetch(lane, x, y, nxt, nin);
    for (int q0 = 0; q0 < npix; q0 += 32) {
        const PixPattern pp = nxt;
        const bool in = nin;
        const int cx = x, cy = y;
        x += 32;
        while (x > xhi) {
            x -= cols;
            ++y;
        }
        if (q0 + 32 < npix) fetch(q0 + 32 + lane, x, y, nxt, nin);
        bool exc = false, slow = false;
        const int64_t idx = int64_t(cy) * g.w + cx;
        float w = 0.0f;
        if (in) {
            w = weight(cx, cy);
            if (w > 1e-8f) {  // BinnedDependency::add skips w <= 1e-8 (core/stats.h:103)
                const bool dev = (pp.pf & kPixDeviant) != 0;
                if (!dev && pp.pat == P0 && pp.pat != 0) {
                    add_class(TP, w, pp.c, pp.s1h, pp.s1l, pp.s2h, pp.s2l);
                    if (p0pix) {
                        if (gpar.uniform_ok && (pp.pf & kPixUniform)) {
                            const int b = uniform_bin(cx, cy);
                            binsA.add_weight(b, w, pp.c);
                            binsA.add_sum(b, w, pp.s1h, pp.s1l);
                        } else {
                            slow = true;
                        }
                    }
                } else if (dev || pp.pat != 0) {
                    exc = true;
                }
            }
        }
        const int q = q0 + lane;
        const unsigned me = __ballot_sync(0xffffffffu, exc);
        if (exc) xlist[nlist + __popc(me & ((1u << lane) - 1))] = q;
        nlist += __popc(me);
        unsigned pending = __ballot_sync(0xffffffffu, slow);
        while (pending) {
            const int src = __ffs(pending) - 1;
            pending &= pending - 1;
            const int64_t pidx = __shfl_sync(0xffffffffu, idx, src);
            const float pw = __shfl_sync(0xffffffffu, w, src);
            const int px = __shfl_sync(0xffffffffu, cx, src), py = __shfl_sync(0xffffffffu, cy, src);
            bin_samples(binsA, pidx, pw, px, py, pbit, false, unused);
        }
    }
    __syncwarp();
    float2 tp[4];
    reduce_totals(TP, tp);
    // lane k of 0-7 adds total k & 3 of P0's pixels (the sums are lane 0's)
#pragma unroll
    for (int k = 0; k < 4; ++k) tp[k] = make_float2(__shfl_sync(0xffffffffu, tp[k].x, 0), __shfl_sync(0xffffffffu, tp[k].y, 0));
    const float2 tpq = pick4(tp, lane & 3);
    const float2 va = binsA.reduce_value();
    LaneBins<INT_W>& binsB = binsA;  // bins A are folded into va: reuse their storage

    // ---- class by class: P0's share plus the listed pixels ----
    for (int cl = 0; cl < kClasses; ++cl) {
        const bool inP0 = (P0 & class_bit(cl)) != 0;
        const bool p0screen = inP0 && p0pix;  // P0 pixels enter the screen sums of this class
        const uint32_t vbit = key_valid_bit(cl);
        Totals tx, ts;
        float2 vb = make_float2(0.0f, 0.0f);
        if (nlist > 0) {
            binsB.clear();
            for (int i0 = 0; i0 < nlist; i0 += 32) {
                const int i = i0 + lane;
                bool slow = false, mixed = false;
                int px = 0, py = 0;
                int64_t idx = 0;
                float w = 0.0f;
                if (i < nlist) {
                    const int q = xlist[i];
                    px = xlo + q % cols;
                    py = ylo + q / cols;
                    idx = int64_t(py) * g.w + px;
                    w = weight(px, py);
                    const PixPattern pp = load_pattern(gp, idx);
                    const uint8_t pf = pp.pf;
                    float cs[5];
                    class_sums(gp, cl, idx, pp, cs);
                    if (cs[0] != 0.0f) {
                        mixed = cl > 0 && (pf & kPixMixed);
                        add_class(tx, w, cs[0], cs[1], cs[2], cs[3], cs[4]);
                        if (!mixed) add_class(ts, w, cs[0], cs[1], cs[2], cs[3], cs[4]);
                        if (gpar.uniform_ok && (pf & kPixUniform) && !mixed) {
                            const int b = uniform_bin(px, py);
                            binsB.add_weight(b, w, cs[0]);
                            binsB.add_sum(b, w, cs[1], cs[2]);
                        } else {
                            slow = true;
                        }
                    }
                }
                unsigned pending = __ballot_sync(0xffffffffu, slow);
                while (pending) {
                    const int src = __ffs(pending) - 1;
                    pending &= pending - 1;
                    const int64_t pidx = __shfl_sync(0xffffffffu, idx, src);
                    const float pw = __shfl_sync(0xffffffffu, w, src);
                    const bool pmixed = __shfl_sync(0xffffffffu, int(mixed), src) != 0;
                    const int sx = __shfl_sync(0xffffffffu, px, src), sy = __shfl_sync(0xffffffffu, py, src);
                    bin_samples(binsB, pidx, pw, sx, sy, vbit, pmixed, ts);
                }
            }
            vb = binsB.reduce_value();
        }
        int dep_x = D_PIXEL, dep_s = D_PIXEL;
        switch (cl) {
        case 1: dep_x = D_BRDF; dep_s = D_SCREEN_BRDF; break;
        case 2: dep_x = D_LENS; dep_s = D_SCREEN_LENS; break;
        case 3: dep_x = D_LIGHT_UV; dep_s = D_SCREEN_LIGHT_UV; break;
        case 4: dep_x = D_ENV; dep_s = D_SCREEN_ENV; break;
        case 5: dep_x = D_LIGHT_SELECT; dep_s = D_SCREEN_LIGHT_SELECT; break;
        case 6: dep_x = D_RR; dep_s = D_SCREEN_RR; break;
        default: break;
        }
        // screen bins (the pixel dependency for class 0): lane v owns bin value v
        float bh = vb.x, bl = vb.y;
        if (p0screen) {
            df_add(bh, bl, va.x);
            bl += va.y;
        }
        // the class's totals, one entry per lane: lanes 0-3 the screen dependency's (32-35),
        // lanes 4-7 the random dimension's (classes 1-6); with no listed pixel the list's part is
        // zero on every lane (nothing to reduce)
        float th = 0.0f, tl = 0.0f;
        float2* te = nullptr;
        {
            float2 t4s[4] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f),
                             make_float2(0.0f, 0.0f)};
            float2 t4x[4] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f),
                             make_float2(0.0f, 0.0f)};
            if (nlist > 0) {
                reduce_totals(ts, t4s);
                if (cl > 0) reduce_totals(tx, t4x);
#pragma unroll
                for (int k = 0; k < 4; ++k) {  // the sums are lane 0's
                    t4s[k] = make_float2(__shfl_sync(0xffffffffu, t4s[k].x, 0), __shfl_sync(0xffffffffu, t4s[k].y, 0));
                    t4x[k] = make_float2(__shfl_sync(0xffffffffu, t4x[k].x, 0), __shfl_sync(0xffffffffu, t4x[k].y, 0));
                }
            }
            if (lane < 4 || (lane < 8 && cl > 0)) {
                const bool scr = lane < 4;
                const float2 ps = pick4(t4s, lane & 3), px = pick4(t4x, lane & 3);
                const float2 t = scr ? ps : px;
                th = t.x;
                tl = t.y;
                if (scr ? p0screen : inP0) {
                    df_add(th, tl, tpq.x);
                    tl += tpq.y;
                }
                te = base + (scr ? dep_s : dep_x) * kDepStride + 32 + (lane & 3);
            }
        }
        // both read-modify-writes of the lane with their loads issued first
        const bool bw = bh != 0.0f || bl != 0.0f;
        const bool tw = te != nullptr && (th != 0.0f || tl != 0.0f);
        float2* be = base + dep_s * kDepStride + lane;
        float2 bv = make_float2(0.0f, 0.0f), tv = make_float2(0.0f, 0.0f);
        if (bw) bv = *be;
        if (tw) tv = *te;
        if (bw) {
            df_add(bv.x, bv.y, bh);
            bv.y += bl;
            *be = bv;
        }
        if (tw) {
            df_add(tv.x, tv.y, th);
            tv.y += tl;
            *te = tv;
        }
    }
}

// ---- random-dimension bins (Dependency2D::add / BinnedDependency::add of brdf, lens,
// light_uv, environment, light_select and rr; main.cpp:356-375) --------------------------
//
// One block per node: RW row groups x DS dimension sets of warps. A warp walks the samples of
// its row group's support rows as one flat stream (lanes over consecutive samples: coalesced,
// 16-byte loads of 4 samples when possible) and updates, for each sample, the bins of the
// dimensions of its set. Every lane owns private bins in shared memory ([slot][lane], conflict
// free; a dimension the sample does not carry updates a per-lane trash slot instead, so the
// update has no branches). The block combines row groups and lanes in a fixed order at the
// end: deterministic, no atomics.
constexpr int kRandDims = 6;
constexpr int kAllDims = 0x3f, kNoEnvDims = 0x37;  // dimension masks (bit d: dimension d)
constexpr int kRandSlots = 5 * 16 + 2;  // brdf, lens, light_uv, environment, light_select; rr has 2 bins
// d: 0 brdf, 1 lens, 2 light_uv, 3 environment, 4 light_select, 5 rr (grid group d + 1)
__host__ __device__ constexpr int rand_slot0(int d) { return d * 16; }
__host__ __device__ constexpr int rand_dep(int d) {
    return d == 0 ? D_BRDF : d == 1 ? D_LENS : d == 2 ? D_LIGHT_UV : d == 3 ? D_ENV : d == 4 ? D_LIGHT_SELECT : D_RR;
}
__host__ __device__ constexpr int rand_shift(int d) { return d == 5 ? 20 : key_bin_shift(d + 1); }
__host__ __device__ constexpr uint32_t rand_mask(int d) { return d == 5 ? 1u : 15u; }

// The six dimensions split into DS sets (one warp of a row group each): fewer private bins per
// warp (more resident warps) at the price of walking the samples once per set.
template <int DS>
__host__ __device__ constexpr int dim_set(int d) {
    return DS == 1 ? 0 : DS == 2 ? ((d == 0 || d == 1 || d == 5) ? 0 : 1)
                                 : ((d == 0 || d == 5) ? 0 : (d == 1 || d == 4) ? 1 : 2);
}
// first slot of dimension d within its set's region
template <int DS>
__host__ __device__ constexpr int dim_slot0(int d) {
    return DS == 1 ? d * 16 : DS == 2 ? (d == 0 ? 0 : d == 1 ? 16 : d == 5 ? 32 : d == 2 ? 0 : d == 3 ? 16 : 32)
                                      : ((d == 0 || d == 1 || d == 2) ? 0 : 16);
}
// slots of the largest set, plus the trash slot
template <int DS>
__host__ __device__ constexpr int set_slots() { return DS == 1 ? kRandSlots : DS == 2 ? 48 : 32; }

struct RandParams {
    GridParams gp;
    uint32_t spp_magic;  // floor(k / spp) == umulhi(k, magic) for every in-segment k (0: search)
    int spp_shift;       // spp is 2^shift (-1: not a power of two)
    int cols;            // support columns of a node, 2 * step + 3 (shared-memory tables)
    // a launch that runs only when the push's largest per-pixel count (*max_count, in device
    // memory) is at most (max_mode 1) or above (max_mode 2) max_limit; max_mode 0: always runs
    const int64_t* max_count;
    int64_t max_limit;
    int max_mode;
    float2* target;  // the grid the pass adds to (the pass grid or, in pairs, the frame grid)
};

template <int WB, int DS>
struct RandLayout {
    // per warp: weights [slots][32] (WB bytes each: u16 or u32 exact integers, or float2
    // double-float), then sums [slots][32] float2; slot kTrash absorbs the updates of absent
    // dimensions
    static constexpr int kTrash = set_slots<DS>();
    static constexpr int kSlots = kTrash + 1;
    static constexpr int kWeightBytes = kSlots * 32 * WB;
    static constexpr int kWarpBytes = kWeightBytes + kSlots * 32 * 8;
};

// Per-warp table of the row segments a warp walks (one chunk of up to 32 support rows).
struct RowTable {
    int64_t k0[32];    // first sample of the segment
    int base[33];      // prefix of the segment lengths (flat sample index of the segment start)
    int col0[32];      // column-factor index of the segment's first pixel
    float ay[32];      // the row's y factor
    int p0[32];        // first pixel of the segment, relative to the push (varying counts)
    int npx[32];       // pixels in the segment
    int len[32];       // samples in the segment
};

// Everything a warp's walk needs.
template <int WB, int DS>
struct WalkCtx {
    std::conditional_t<WB == 2, uint16_t, uint32_t>* wint;
    float2* wdf;
    float2* sums;
    RowTable* rt;
    const float* xf;
    int lane;
    int xlo;          // image column of xf[0]
    float wscale;
};

// One sample: add w (weights) and w*y (sums) to the bin of every dimension of set SET the
// sample carries; dimensions outside the mask DIMS are never valid in the push's keys (their
// sample planes are absent) and are skipped. Absent dimensions (and w <= 1e-8, which BinnedDependency::add skips,
// core/stats.h:103) go to the trash slot with the same arithmetic.
template <int WB, int DS, int SET, int DIMS>
__device__ __forceinline__ void rand_update(const WalkCtx<WB, DS>& c, uint32_t key, float w, uint32_t iw,
                                            float y) {
    constexpr bool INT_W = WB != 8;
    using L = RandLayout<WB, DS>;
    const bool wok = w > 1e-8f;
    const float wy = w * y;
    const float wye = __fmaf_rn(w, y, -wy);
    int slot[kRandDims];
    uint32_t wi[kRandDims];
    float2 wd[kRandDims], sy[kRandDims];
#pragma unroll
    for (int d = 0; d < kRandDims; ++d) {
        if (dim_set<DS>(d) != SET || !((DIMS >> d) & 1)) continue;
        const bool on = wok && (key & key_valid_bit(d + 1)) != 0;
        const int bin = int((key >> rand_shift(d)) & rand_mask(d));
        slot[d] = (on ? dim_slot0<DS>(d) + bin : L::kTrash) * 32 + c.lane;
    }
    // the dimensions own disjoint slot ranges (the trash slot is only ever a sink): load all,
    // update, store all
#pragma unroll
    for (int d = 0; d < kRandDims; ++d) {
        if (dim_set<DS>(d) != SET || !((DIMS >> d) & 1)) continue;
        if (INT_W) wi[d] = c.wint[slot[d]];
        else wd[d] = c.wdf[slot[d]];
        sy[d] = c.sums[slot[d]];
    }
#pragma unroll
    for (int d = 0; d < kRandDims; ++d) {
        if (dim_set<DS>(d) != SET || !((DIMS >> d) & 1)) continue;
        if (INT_W) wi[d] += iw;
        else df_add(wd[d].x, wd[d].y, w);
        df_add(sy[d].x, sy[d].y, wy);
        sy[d].y += wye;
    }
#pragma unroll
    for (int d = 0; d < kRandDims; ++d) {
        if (dim_set<DS>(d) != SET || !((DIMS >> d) & 1)) continue;
        if (INT_W) c.wint[slot[d]] = wi[d];
        else c.wdf[slot[d]] = wd[d];
        c.sums[slot[d]] = sy[d];
    }
}

// Walk modes: samples one by one (0); quads of 4 samples of one pixel (1, uniform counts); aligned
// quads of 4 consecutive samples of the push with each sample's column (2, per-pixel counts).
constexpr int kWalkScalar = 0, kWalkPixelQuads = 1, kWalkColumnQuads = 2;

// The flat walk of one row-segment chunk (total samples, or total quads in the quad modes) for
// dimension set SET.
template <int WB, int DS, int SET, int MODE, int DIMS>
__device__ __forceinline__ void rand_walk(const WalkCtx<WB, DS>& c, const RandParams& rp, const GridPrep& gp,
                                          const int64_t* offsets, int total) {
    constexpr bool INT_W = WB != 8;
    const RowTable* rt = c.rt;
    const int lane = c.lane;
    int r = 0;  // current segment of this lane (monotone along its walk)
    if (MODE == kWalkColumnQuads) {
        // Quads of the push's samples 4Q .. 4Q+3 (16-byte loads of keys and luminances, 8 bytes of
        // columns; the sample planes are padded to a multiple of 64 samples). A quad may start
        // before the segment or run past it: those samples weigh nothing (the trash slot). The
        // weights are formed when the quad is processed, one batch after its loads were issued.
        constexpr int U = 2;
        const int nq = total;
        auto fetchq = [&](int q, uint4& kq, float4& yq, uint2& cq, int64_t& k4, int& seg) {
            kq = make_uint4(0u, 0u, 0u, 0u);
            yq = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            cq = make_uint2(0u, 0u);
            k4 = 0;
            seg = -1;
            if (q >= nq) return;
            while (q >= rt->base[r + 1]) ++r;
            k4 = ((rt->k0[r] >> 2) + (q - rt->base[r])) << 2;
            kq = *reinterpret_cast<const uint4*>(gp.key + k4);
            yq = *reinterpret_cast<const float4*>(gp.lum + k4);
            cq = *reinterpret_cast<const uint2*>(gp.col + k4);
            seg = r;
        };
        uint4 nk[U];
        float4 nyv[U];
        uint2 ncq[U];
        int64_t nk4[U];
        int nseg[U];
#pragma unroll
        for (int u = 0; u < U; ++u) fetchq(lane + 32 * u, nk[u], nyv[u], ncq[u], nk4[u], nseg[u]);
        for (int q0 = 0; q0 < nq; q0 += 32 * U) {
            uint4 ck[U];
            float4 cy[U];
            uint2 ccq[U];
            int64_t ck4[U];
            int cseg[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ck[u] = nk[u];
                cy[u] = nyv[u];
                ccq[u] = ncq[u];
                ck4[u] = nk4[u];
                cseg[u] = nseg[u];
            }
            if (q0 + 32 * U < nq) {
#pragma unroll
                for (int u = 0; u < U; ++u) fetchq(q0 + 32 * U + lane + 32 * u, nk[u], nyv[u], ncq[u], nk4[u], nseg[u]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (cseg[u] >= 0) {
                    const int64_t ks = rt->k0[cseg[u]], ke = ks + rt->len[cseg[u]];
                    const float ay = rt->ay[cseg[u]];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int64_t k = ck4[u] + i;
                        const int ci = int(((i < 2 ? ccq[u].x : ccq[u].y) >> (16 * (i & 1))) & 0xffffu) - c.xlo;
                        if (k >= ks && k < ke && unsigned(ci) < unsigned(rp.cols)) w[i] = c.xf[ci] * ay;
                    }
                }
                rand_update<WB, DS, SET, DIMS>(c, ck[u].x, w[0], INT_W ? uint32_t(w[0] * c.wscale) : 0u, cy[u].x);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].y, w[1], INT_W ? uint32_t(w[1] * c.wscale) : 0u, cy[u].y);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].z, w[2], INT_W ? uint32_t(w[2] * c.wscale) : 0u, cy[u].z);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].w, w[3], INT_W ? uint32_t(w[3] * c.wscale) : 0u, cy[u].w);
            }
        }
    } else if (MODE == kWalkPixelQuads) {
        // quads of 4 consecutive samples of one pixel (the samples per pixel are a power of two
        // >= 4 and every segment starts 16-byte aligned): one 16-byte load of keys and one of
        // luminances per quad, 2 quads per lane in flight
        constexpr int U = 2;
        const int nq = total >> 2;
        auto fetchq = [&](int q, uint4& kq, float4& yq, float& w) {
            kq = make_uint4(0u, 0u, 0u, 0u);
            yq = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            w = 0.0f;
            if (q >= nq) return;
            const int t = q << 2;
            while (t >= rt->base[r + 1]) ++r;
            const int kk = t - rt->base[r];
            const int64_t k = rt->k0[r] + kk;
            kq = *reinterpret_cast<const uint4*>(gp.key + k);
            yq = *reinterpret_cast<const float4*>(gp.lum + k);
            w = c.xf[rt->col0[r] + (kk >> rp.spp_shift)] * rt->ay[r];
        };
        uint4 nk[U];
        float4 nyv[U];
        float nw[U];
#pragma unroll
        for (int u = 0; u < U; ++u) fetchq(lane + 32 * u, nk[u], nyv[u], nw[u]);
        for (int q0 = 0; q0 < nq; q0 += 32 * U) {
            uint4 ck[U];
            float4 cy[U];
            float cw[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ck[u] = nk[u];
                cy[u] = nyv[u];
                cw[u] = nw[u];
            }
            if (q0 + 32 * U < nq) {
#pragma unroll
                for (int u = 0; u < U; ++u) fetchq(q0 + 32 * U + lane + 32 * u, nk[u], nyv[u], nw[u]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const uint32_t iw = INT_W ? uint32_t(cw[u] * c.wscale) : 0u;
                rand_update<WB, DS, SET, DIMS>(c, ck[u].x, cw[u], iw, cy[u].x);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].y, cw[u], iw, cy[u].y);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].z, cw[u], iw, cy[u].z);
                rand_update<WB, DS, SET, DIMS>(c, ck[u].w, cw[u], iw, cy[u].w);
            }
        }
    } else {
        // A fetch returns the sample's column-factor index and row factor, not its weight: with
        // per-pixel counts the index comes from a load, and looking the factor up at fetch time
        // would wait for that load before the samples already fetched are processed.
        constexpr int U = 4;  // samples per lane in flight
        auto fetch = [&](int t, uint32_t& key, float& y, int& ci, float& ay) {
            key = 0u;
            y = 0.0f;
            ci = -1;
            ay = 0.0f;
            if (t >= total) return;
            while (t >= rt->base[r + 1]) ++r;
            const int kk = t - rt->base[r];
            const int64_t k = rt->k0[r] + kk;
            key = gp.key[k];
            y = gp.lum[k];
            ay = rt->ay[r];
            if (gp.col) {  // per-pixel counts: the statistics pass stored each sample's column
                ci = int(gp.col[k]) - c.xlo;
                return;
            }
            int pl;
            if (rp.spp_shift >= 0) {
                pl = kk >> rp.spp_shift;
            } else if (rp.spp_magic) {
                pl = int(__umulhi(uint32_t(kk), rp.spp_magic));
            } else {
                const int64_t* off = offsets + rt->p0[r];
                int lo = 0, hi = rt->npx[r] - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (off[mid] <= k) lo = mid; else hi = mid - 1;
                }
                pl = lo;
            }
            ci = rt->col0[r] + pl;
        };
        uint32_t nk[U];
        float nyv[U], nay[U];
        int nci[U];
#pragma unroll
        for (int u = 0; u < U; ++u) fetch(lane + 32 * u, nk[u], nyv[u], nci[u], nay[u]);
        for (int t0 = 0; t0 < total; t0 += 32 * U) {
            uint32_t ck[U];
            float cy[U], cw[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ck[u] = nk[u];
                cy[u] = nyv[u];
                cw[u] = unsigned(nci[u]) < unsigned(rp.cols) ? c.xf[nci[u]] * nay[u] : 0.0f;
            }
            if (t0 + 32 * U < total) {
#pragma unroll
                for (int u = 0; u < U; ++u) fetch(t0 + 32 * U + lane + 32 * u, nk[u], nyv[u], nci[u], nay[u]);
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                rand_update<WB, DS, SET, DIMS>(c, ck[u], cw[u], INT_W ? uint32_t(cw[u] * c.wscale) : 0u, cy[u]);
        }
    }
}

template <int WB, int RW, int DS, int MODE, int DIMS>
__global__ void __launch_bounds__(RW * DS * 32) k_grid_random(RandParams rp, float2* pass_grid,
                                                              const int64_t* offsets, GridPrep gp) {
    constexpr bool INT_W = WB != 8;
    using WT = std::conditional_t<WB == 2, uint16_t, uint32_t>;
    constexpr int NW = RW * DS;
    constexpr int VPT = (2 * kRandSlots + NW * 32 - 1) / (NW * 32);  // combined values per thread
    if (rp.max_mode != 0 && ((*rp.max_count <= rp.max_limit) != (rp.max_mode == 1))) return;  // the other form runs
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using L = RandLayout<WB, DS>;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int dset = warp % DS;     // the dimension set of this warp
    const int rgroup = warp / DS;   // its row group
    const GridParams& gpar = rp.gp;
    const Geometry& g = gpar.g;
    const int64_t node = rp.gp.node0 + blockIdx.x;
    const int nx = int(node % g.nodes_x), ny = int(node / g.nodes_x);
    unsigned char* wbase = smem_raw + warp * L::kWarpBytes;
    WalkCtx<WB, DS> c;
    c.wint = reinterpret_cast<WT*>(wbase);
    c.wdf = reinterpret_cast<float2*>(wbase);
    c.sums = reinterpret_cast<float2*>(wbase + L::kWeightBytes);
    c.rt = reinterpret_cast<RowTable*>(smem_raw + NW * L::kWarpBytes) + warp;
    float* xf = reinterpret_cast<float*>(reinterpret_cast<RowTable*>(smem_raw + NW * L::kWarpBytes) + NW);
    c.xf = xf;
    c.lane = lane;
    c.wscale = float(g.step) * float(g.step);
    RowTable* rt = c.rt;

    // the grid entries this thread adds to at the end, read now so the loads overlap the walk
    float2 prev[VPT];
    int64_t gidx[VPT];
#pragma unroll
    for (int vi = 0; vi < VPT; ++vi) {
        const int v = threadIdx.x + vi * NW * 32;
        gidx[vi] = -1;
        prev[vi] = make_float2(0.0f, 0.0f);
        if (v < 2 * kRandSlots) {
            const bool is_w = v < kRandSlots;
            const int gslot = is_w ? v : v - kRandSlots;
            int d = 0;
            while (d < kRandDims - 1 && gslot >= rand_slot0(d + 1)) ++d;
            const int bin = gslot - rand_slot0(d);
            gidx[vi] = (node * kDeps + rand_dep(d)) * kDepStride + (is_w ? bin : 16 + bin);
            prev[vi] = pass_grid[gidx[vi]];
        }
    }
    const int xlo = imaxs(0, (nx - 1) * g.step - 1), xhi = imins(g.w - 1, (nx + 1) * g.step + 1);
    const int ylo = imaxs(0, (ny - 1) * g.step - 1), yhi = imins(g.h - 1, (ny + 1) * g.step + 1);
    c.xlo = xlo;
    for (int col = threadIdx.x; col < rp.cols; col += NW * 32)
        xf[col] = (xlo + col <= xhi) ? axis_factor(gpar, xlo + col, nx, g.nodes_x) : 0.0f;
    for (int k = 0; k < L::kSlots; ++k) {
        if (INT_W) c.wint[k * 32 + lane] = 0u;
        else c.wdf[k * 32 + lane] = make_float2(0.0f, 0.0f);
        c.sums[k * 32 + lane] = make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    int xa = xhi + 1, xb = xlo - 1;  // the columns with x factor > 0
    for (int x = xlo; x <= xhi; ++x)
        if (xf[x - xlo] > 0.0f) {
            xa = imins(xa, x);
            xb = imaxs(xb, x);
        }
    const int nrows = (yhi - ylo) / RW + 1;  // rows ylo + rgroup + RW * j

    for (int c0 = 0; c0 < nrows; c0 += 32) {
        // ---- this chunk's row segments, one lane per row ----
        const int y = ylo + rgroup + RW * (c0 + lane);
        int n = 0;  // the walk's units in the segment: samples, or quads in the column-quad mode
        if (c0 + lane < nrows && y <= yhi && xa <= xb) {
            const float ay = axis_factor(gpar, y, ny, g.nodes_y);
            int64_t p0 = int64_t(y) * g.w + xa, p1 = int64_t(y) * g.w + xb + 1;
            p0 = p0 < gpar.first ? gpar.first : p0;
            p1 = p1 > gpar.first + gpar.count ? gpar.first + gpar.count : p1;
            if (ay > 0.0f && p0 < p1) {
                const int64_t k0 = offsets[p0 - gpar.first];
                const int len = int(offsets[p1 - gpar.first] - k0);
                n = MODE == kWalkColumnQuads ? (len > 0 ? int(((k0 + len - 1) >> 2) - (k0 >> 2) + 1) : 0) : len;
                rt->k0[lane] = k0;
                rt->len[lane] = len;
                rt->col0[lane] = int(p0 - int64_t(y) * g.w) - xlo;
                rt->ay[lane] = ay;
                rt->p0[lane] = int(p0 - gpar.first);
                rt->npx[lane] = int(p1 - p0);
            }
        }
        int incl = n;  // inclusive scan of the segment lengths
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += v;
        }
        rt->base[lane + 1] = incl;
        if (lane == 0) rt->base[0] = 0;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        if (dset == 0) rand_walk<WB, DS, 0, MODE, DIMS>(c, rp, gp, offsets, total);
        if (DS > 1 && dset == 1) rand_walk<WB, DS, 1, MODE, DIMS>(c, rp, gp, offsets, total);
        if (DS > 2 && dset == 2) rand_walk<WB, DS, 2, MODE, DIMS>(c, rp, gp, offsets, total);
        __syncwarp();
    }
    __syncthreads();

    // combine: thread t owns values v = t + vi * NW*32 of [weights(kRandSlots), sums(kRandSlots)],
    // each summed over the row groups in order and over the 32 lanes in a rotated order
    // (32 different banks), two interleaved double-float chains per value
    int vslot[VPT], vset[VPT];
    bool vw[VPT];
#pragma unroll
    for (int vi = 0; vi < VPT; ++vi) {
        const int v = threadIdx.x + vi * NW * 32;
        const bool is_w = v < kRandSlots;
        const int gslot = is_w ? v : v - kRandSlots;
        int d = 0;
        while (d < kRandDims - 1 && gslot >= rand_slot0(d + 1)) ++d;
        vslot[vi] = dim_slot0<DS>(d) + (gslot - rand_slot0(d));
        vset[vi] = dim_set<DS>(d);
        vw[vi] = is_w;
    }
    uint64_t itot[VPT];
    float h[VPT][2], l[VPT][2];
#pragma unroll
    for (int vi = 0; vi < VPT; ++vi) {
        itot[vi] = 0;
        h[vi][0] = h[vi][1] = l[vi][0] = l[vi][1] = 0.0f;
    }
    for (int rg = 0; rg < RW; ++rg) {
        for (int i = 0; i < 32; i += 2) {
#pragma unroll
            for (int vi = 0; vi < VPT; ++vi) {
                if (gidx[vi] < 0) continue;
                const unsigned char* b = smem_raw + (rg * DS + vset[vi]) * L::kWarpBytes;
                const int v = threadIdx.x + vi * NW * 32;
                if (vw[vi] && INT_W) {
                    const WT* src = reinterpret_cast<const WT*>(b) + vslot[vi] * 32;
                    itot[vi] += uint64_t(src[(i + v) & 31]) + uint64_t(src[(i + 1 + v) & 31]);
                } else {
                    const float2* src =
                        reinterpret_cast<const float2*>(vw[vi] ? b : b + L::kWeightBytes) + vslot[vi] * 32;
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        const float2 q = src[(i + j + v) & 31];
                        df_add(h[vi][j], l[vi][j], q.x);
                        l[vi][j] += q.y;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int vi = 0; vi < VPT; ++vi) {
        if (gidx[vi] < 0) continue;
        float oh, ol;
        if (vw[vi] && INT_W) {
            const float2 t = int_weight_df(itot[vi], 1.0f / c.wscale);
            oh = t.x;
            ol = t.y;
        } else {
            df_add(h[vi][0], l[vi][0], h[vi][1]);
            l[vi][0] += l[vi][1];
            oh = h[vi][0];
            ol = l[vi][0];
        }
        if (oh != 0.0f || ol != 0.0f) {
            float2 e = prev[vi];
            df_add(e.x, e.y, oh);
            e.y += ol;
            pass_grid[gidx[vi]] = e;
        }
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

template <int WB, int RW, int DS, int MODE, int DIMS>
cudaError_t launch_random_vec(Job& j, const RandParams& rp, const GridPrep& gp) {
    constexpr int NW = RW * DS;
    const size_t smem = size_t(NW) * RandLayout<WB, DS>::kWarpBytes + size_t(NW) * sizeof(RowTable) +
                        size_t(rp.cols) * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_grid_random<WB, RW, DS, MODE, DIMS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    const unsigned nblocks = unsigned(rp.gp.count_nodes);
    k_grid_random<WB, RW, DS, MODE, DIMS><<<nblocks, NW * 32, smem, j.stream>>>(rp, rp.target, j.offsets, gp);
    j.launches += 1;
    return cudaGetLastError();
}

// Pixel quads need samples per pixel a multiple of 4 (and a power of two, for the shift) with
// 16-byte aligned key and luminance planes; column quads need the per-sample columns (per-pixel
// counts) with 16-byte aligned key and luminance planes and an 8-byte aligned column plane.
template <int WB, int RW, int DS, int DIMS = kAllDims>
cudaError_t launch_random(Job& j, const RandParams& rp, const GridPrep& gp) {
    const bool aligned = (reinterpret_cast<uintptr_t>(gp.key) & 15u) == 0 && (reinterpret_cast<uintptr_t>(gp.lum) & 15u) == 0;
    if (rp.spp_shift >= 2 && aligned) return launch_random_vec<WB, RW, DS, kWalkPixelQuads, DIMS>(j, rp, gp);
    if (gp.col && aligned && (reinterpret_cast<uintptr_t>(gp.col) & 7u) == 0)
        return launch_random_vec<WB, RW, DS, kWalkColumnQuads, DIMS>(j, rp, gp);
    return launch_random_vec<WB, RW, DS, kWalkScalar, DIMS>(j, rp, gp);
}

// WB: bytes of a lane-private bin weight (8 double-float, 4 or 2 exact integers); the 2-byte
// form is built for the default shape only (the caller checks that the lane sums fit)
template <int WB>
cudaError_t launch_random_shape(Job& j, const RandParams& rp, const GridPrep& gp, int shape, bool env) {
    if constexpr (WB == 2) {
        return env ? launch_random<2, 1, 1>(j, rp, gp) : launch_random<2, 1, 1, kNoEnvDims>(j, rp, gp);
    } else {
        switch (shape) {
        case 1: return launch_random<WB, 2, 1>(j, rp, gp);
        case 2: return launch_random<WB, 2, 2>(j, rp, gp);
        case 3: return launch_random<WB, 2, 3>(j, rp, gp);
        case 4: return launch_random<WB, 1, 2>(j, rp, gp);
        case 5: return launch_random<WB, 1, 3>(j, rp, gp);
        default: return launch_random<WB, 1, 1>(j, rp, gp);
        }
    }
}

}  // namespace

// Where a fast-mode push adds its bins. The reference adds each pass's grid to the frame grid at the
// end of the pass; with the frame grid in double-float pairs (or still empty) the push adds its
// pairs straight into it instead (the pairs' sums differ from pass-then-merge only in the rounding
// of the low words), and the end of the pass has nothing to merge. Otherwise the pass grid
// collects the pass as in the reference.
static cudaError_t grid_target(Job& j, float2** out) {
    const int64_t n = j.g.nn * kDeps * kDepStride;
    if (j.cfg.rpf_shrinkage_scale > 0.0f && (j.grid_fresh || j.grid_pairs)) {
        if (j.grid_fresh) {
            const cudaError_t e = cudaMemsetAsync(j.n.grid, 0, size_t(n) * sizeof(double), j.stream);
            if (e != cudaSuccess) return e;
            j.grid_fresh = false;
            j.grid_pairs = true;
        }
        j.pass_direct = true;
        *out = reinterpret_cast<float2*>(j.n.grid);
    } else {
        j.pass_indirect = true;
        *out = reinterpret_cast<float2*>(j.n.pass_grid);
    }
    return cudaSuccess;
}

cudaError_t launch_grid_fast(Job& j, const DeviceSamples& s, int64_t first, int64_t count, const GridPrep& gp,
                             int32_t spp, int32_t max_count, int64_t total_samples, const int64_t* d_max_count) {
    float2* target = nullptr;
    if (const cudaError_t e0 = grid_target(j, &target); e0 != cudaSuccess) return e0;
    const int step = j.g.step;
    const bool pow2 = (step & (step - 1)) == 0;
    GridParams gpar{j.g, first, count, 0, 0, 0, pow2 ? 1 : 0, 1.0f / float(step), spp, spp > 0 ? 1.0f / float(spp) : 0.0f};
    {
        // node rows whose support rows (ny-1)*step-1 .. (ny+1)*step+1 meet the push's rows
        const int y0 = int(first / j.g.w), y1 = int((first + count - 1) / j.g.w);
        const int ny0 = std::max(0, (y0 - 1) / step - 1), ny1 = std::min(j.g.nodes_y - 1, (y1 + 1) / step + 1);
        gpar.node0 = int64_t(ny0) * j.g.nodes_x;
        gpar.count_nodes = int64_t(ny1 - ny0 + 1) * j.g.nodes_x;
    }
    const unsigned nblocks = unsigned(gpar.count_nodes);
    const int sup = j.g.support;
    gpar.uniform_ok = (sup >= 4 && sup <= 2048 && (sup & (sup - 1)) == 0) ? 1 : 0;
    // exact integer bin weights need a power-of-two step and a per-bin total below 2^32:
    // at most support^2 pixels * max_count samples * step^2
    const double bound = double(sup + 3) * double(sup + 3) * double(std::max(max_count, 1)) * double(step) * double(step);
    // a bin's weight sum is at most the push's samples times step^2 units as well
    const double total_bound = double(std::max<int64_t>(total_samples, 1)) * double(step) * double(step);
    const bool int_w = pow2 && (bound < 4.0e9 || total_bound < 4.0e9);
    cudaError_t e;
    {
        KernelScope ks(j, RPD_KERNEL_GRID);
        const int side = 2 * step + 3;
        const size_t list_bytes = size_t(side) * size_t(side) * sizeof(int);
        if (list_bytes <= size_t(64) * 1024) {
            // pattern form: one warp per node
            const size_t smem = size_t(int_w ? LaneBins<true>::kSlots : LaneBins<false>::kSlots) * 32 * sizeof(float) +
                                list_bytes;
            if (int_w) {
                e = cudaFuncSetAttribute(k_grid_screen<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                k_grid_screen<true><<<nblocks, 32, smem, j.stream>>>(gpar, target, s, j.offsets, gp);
            } else {
                e = cudaFuncSetAttribute(k_grid_screen<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
                if (e != cudaSuccess) return e;
                k_grid_screen<false><<<nblocks, 32, smem, j.stream>>>(gpar, target, s, j.offsets, gp);
            }
        } else if (int_w) {
            const size_t smem = size_t(kGroups) * LaneBins<true>::kSlots * 32 * sizeof(float);
            e = cudaFuncSetAttribute(k_grid_fast<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
            k_grid_fast<true><<<nblocks, kGroups * 32, smem, j.stream>>>(gpar, target, s, j.offsets, gp);
        } else {
            const size_t smem = size_t(kGroups) * LaneBins<false>::kSlots * 32 * sizeof(float);
            e = cudaFuncSetAttribute(k_grid_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
            k_grid_fast<false><<<nblocks, kGroups * 32, smem, j.stream>>>(gpar, target, s, j.offsets, gp);
        }
        j.launches += 1;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    KernelScope ks(j, RPD_KERNEL_GRID_RANDOM);
    RandParams rp{gpar, 0u, -1, 2 * step + 3, nullptr, 0, 0, target};
    // the statistics pass clears a dimension's valid bit when the push has no plane for it: without
    // environment planes (a closed scene) the form without the environment dimension runs
    const bool env = s.compact ? s.c16.env_u[0] != nullptr : s.env_u[0] != nullptr;
    if (spp > 0) {
        if ((spp & (spp - 1)) == 0) {
            int sh = 0;
            while ((1 << sh) < spp) ++sh;
            rp.spp_shift = sh;
        } else {
            rp.spp_magic = spp_magic_for(spp, (2 * step + 3) * spp);
        }
    }
    // 16-bit lane sums (smaller bins, more resident warps) when no lane's sum can reach 2^16. Each
    // sample adds at most step^2 units. Uniform push: a lane takes at most 1/32 of a node's quads
    // (plus two partial quads per row segment). Per-pixel counts of at most M: a node's support
    // holds at most side^2 M samples, a segment of len samples spans at most len/4 + 1.5 quads, and
    // a lane takes at most 1/32 of a chunk's (up to 32 segments) quads plus one, so at most
    // side^2 M / 32 + 10 samples per chunk of 32 support rows.
    const bool default_shape = j.grid_shape == 0 || j.grid_shape == 6;
    const double side = double(2 * step + 3), units = double(step) * double(step);
    const double chunks = std::ceil(side / 32.0);
    auto counts_fit = [&](double m) { return (side * side * m / 32.0 + 10.0 * chunks) * units < 65536.0; };
    if (int_w && default_shape) {
        if (spp > 0) {
            if ((double(sup + 3) * double(sup + 3) * double(spp) / 32.0 + 8.0) * units < 65536.0)
                return launch_random_shape<2>(j, rp, gp, j.grid_shape, env);
        } else if (max_count != INT32_MAX) {
            if (counts_fit(double(std::max(max_count, 1)))) return launch_random_shape<2>(j, rp, gp, j.grid_shape, env);
        } else if (d_max_count) {
            // the largest count is known on the device only: launch both forms, each block of the
            // one that does not apply returns at once
            int64_t lim = int64_t(std::max(0.0, (65536.0 / units - 10.0 * chunks) * 32.0 / (side * side)));
            while (lim > 0 && !counts_fit(double(lim))) --lim;
            if (lim > 0) {
                RandParams r16 = rp;
                r16.max_count = d_max_count;
                r16.max_limit = lim;
                r16.max_mode = 1;
                if ((e = launch_random_shape<2>(j, r16, gp, j.grid_shape, env)) != cudaSuccess) return e;
                RandParams r32 = r16;
                r32.max_mode = 2;
                return launch_random_shape<4>(j, r32, gp, j.grid_shape, env);
            }
        }
    }
    return int_w ? launch_random_shape<4>(j, rp, gp, j.grid_shape, env) : launch_random_shape<8>(j, rp, gp, j.grid_shape, env);
}

}  // namespace rpd
