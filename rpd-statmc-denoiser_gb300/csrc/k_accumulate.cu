// Per-sample accumulation: pixel statistics, primary-hit features and the RPD grid.
//
//   k_accumulate_pixels  accumulate_sample (core/stats.h:25-41) and the feature / radiance
//                        sums of the render loops (main.cpp:572-576, 706-717), one thread
//                        per pixel walking its samples in order — bit-identical to the
//                        reference, whose pixel is also owned by a single thread.
//   k_grid_ordered       accumulate_rpf_sample_to_grid (main.cpp:329-376) regrouped by
//                        owner: one thread per (node, dependency) visits the node's support
//                        pixels in row-major order and their samples in order, which is the
//                        reference's summation order with one OpenMP thread, so the grid is
//                        bit-identical to that run. No atomics; deterministic.
//   k_merge_grid         merge_rpf_grids_into (main.cpp:378-388).
//   k_feature_cache      ensure_feature_cache (main.cpp:94-122).
//   k_finalize           FrameBuffers::finalize (core/buffers.h:152-167).
#include <cuda_fp16.h>

#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

constexpr int kScanBlock = 1024;

__global__ void k_offsets_uniform(int64_t* offsets, int64_t count, int32_t spp) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i <= count) offsets[i] = i * int64_t(spp);
}

// Three-phase exclusive scan of int32 counts into int64 offsets[0..count]: per-block sums, a
// scan of the block sums by one block, and the per-block scans shifted by them. Warp-shuffle
// scans, so each phase is a few steps per element.
__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int64_t t = __shfl_up_sync(0xffffffffu, v, off);
        if (lane >= off) v += t;
    }
    return v;
}

// inclusive scan over the block (blockDim.x == kScanBlock); `total` gets the block's sum
__device__ __forceinline__ int64_t block_incl_scan(int64_t v, int64_t* total) {
    __shared__ int64_t warp_tot[kScanBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_incl_scan(v);
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int64_t t = warp_incl_scan(warp_tot[lane]);
        warp_tot[lane] = t;
    }
    __syncthreads();
    if (warp > 0) v += warp_tot[warp - 1];
    if (total) *total = warp_tot[kScanBlock / 32 - 1];
    __syncthreads();
    return v;
}

// largest count of the block (counts are >= 0; 0 for an empty block)
__device__ __forceinline__ int32_t block_max(int32_t v) {
    __shared__ int32_t warp_max[kScanBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = __reduce_max_sync(0xffffffffu, v);
    if (lane == 0) warp_max[warp] = v;
    __syncthreads();
    if (warp == 0) v = __reduce_max_sync(0xffffffffu, warp_max[lane]);
    __syncthreads();
    return v;
}

// per block: the sum of its counts (block_sums) and their maximum (block_max)
__global__ void __launch_bounds__(kScanBlock) k_scan_block_sums(const int32_t* counts, int64_t count, int64_t* block_sums,
                                                              int64_t* block_maxima) {
    const int64_t i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
    const int32_t c = (i < count) ? counts[i] : 0;
    int64_t total;
    block_incl_scan(int64_t(c), &total);
    const int32_t m = block_max(c < 0 ? 0 : c);
    if (threadIdx.x == 0) {
        block_sums[blockIdx.x] = total;
        block_maxima[blockIdx.x] = m;
    }
}

// one block: block_sums[0..nblocks) -> exclusive offsets, block_sums[nblocks] = the total;
// block_maxima[nblocks] = the largest count
__global__ void __launch_bounds__(kScanBlock) k_scan_block_offsets(int64_t* block_sums, int64_t* block_maxima,
                                                                 int64_t nblocks) {
    int64_t carry = 0;
    int32_t mx = 0;
    for (int64_t b0 = 0; b0 < nblocks; b0 += kScanBlock) {
        const int64_t b = b0 + threadIdx.x;
        const int64_t v = b < nblocks ? block_sums[b] : 0;
        int64_t total;
        const int64_t incl = block_incl_scan(v, &total);
        if (b < nblocks) block_sums[b] = carry + incl - v;
        carry += total;
        mx = max(mx, block_max(b < nblocks ? int32_t(block_maxima[b]) : 0));
    }
    if (threadIdx.x == 0) {
        block_sums[nblocks] = carry;
        block_maxima[nblocks] = mx;
    }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_finish(const int32_t* counts, int64_t count, const int64_t* block_sums,
                                                           int64_t* offsets) {
    const int64_t i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
    const int64_t v = (i < count) ? int64_t(counts[i]) : 0;
    const int64_t incl = block_incl_scan(v, nullptr);
    const int64_t base = block_sums[blockIdx.x];
    if (i < count) offsets[i] = base + incl - v;
    if (i == count - 1) offsets[count] = base + incl;
}

// Dependency2D::add bin (core/stats.h:166-168)
__device__ __forceinline__ int bin2d_k(float u, float v) {
    const int x = iclamps(int(u * 4.0f), 0, 3);
    const int z = iclamps(int(v * 4.0f), 0, 3);
    return z * 4 + x;
}

// TwoSum of x into the double-float (hi, lo).
__device__ __forceinline__ void df_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (x - bb);
    hi = s;
}

// One traced sample as the statistics pass sees it.
struct SampleIn {
    float L[3], n[3], d, alb[3], pu[2], lu[2], bu[2], liu[2], eu[2];
    uint8_t f, cat;
    uint32_t bins;  // COMPACT_IN: the lens, BRDF, light and environment bins, 4 bits each
    float root[3];  // COMPACT_IN: sqrt(max(0, L)), known exactly (L is the square of a half)
};

// x / d correctly rounded from rd = 1/d (itself correctly rounded) by Markstein's correction
// (P. Markstein, "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Dev. 34(1), 1990): q = RN(x rd), the remainder x - d q is exact in a fused
// multiply-add, and RN(q + (x - d q) rd) is the correctly rounded x / d. It holds for a
// positive normal d whose mantissa is not all ones and a quotient, remainder and x in the
// normal range (or x = +0).
__device__ __forceinline__ float div_markstein(float x, float d, float rd) {
    const float q = __fmul_rn(x, rd);
    return __fmaf_rn(__fmaf_rn(-d, q, x), rd, q);
}
__device__ __forceinline__ bool markstein_ok(float x) { return x == 0.0f || fabsf(x) >= 5.42101086e-20f; }  // 2^-64

// Dependency2D::add's bin of a compact (unorm16) pair: u = q / 65536 exactly, so
// int(u * 4) = q >> 14, already within 0..3 (core/stats.h:166-168)
__device__ __forceinline__ uint32_t bin2d_q(uint16_t qu, uint16_t qv) { return uint32_t(qv >> 14) * 4u + uint32_t(qu >> 14); }

// Per-pixel running state of the statistics pass.
struct PixelAcc {
    float mean, m2;
    int n;
    float cm[3], sm[3], sq[3], rad[3], nor[3], alb[3], dep;
    int hits, nsamples;
    // validity-class sums for the grid pass: samples whose class bits equal the pixel's
    // pattern (the first nonzero class bits) share one set of sums; others go to per-class
    // sums and make the pixel deviant
    uint8_t pat;
    bool have_pat, dev;
    float pc, p1h, p1l, p2h, p2l;
    // the per-class sums [class][count, s1 hi, s1 lo, s2 hi, s2 lo] of a deviant pixel, in the
    // thread's local memory (written only once the pixel deviates, which is rare): held in
    // registers they would cost 35 registers through the whole sample loop
    float* cs;
    uint8_t pflags;
};

// COMPACT_IN: a sample decoded from the compact planes. Its radiance is the square of a
// non-negative half, so sqrt(max(0, L)) is exactly that half (in.root), no quotient's dividend is
// -0, and the random-dimension bins come with it (in.bins).
template <bool COMPACT_IN = false>
__device__ __forceinline__ void process_sample(PixelAcc& a, const SampleIn& in, bool per_sample_albedo,
                                               const float* palb, bool prep, uint8_t plane_mask, float fx,
                                               float fy, float& lum_out, uint32_t& key_out) {
    if (in.f & RPD_SAMPLE_HIT) {  // main.cpp:572-576
        ++a.hits;
        for (int c = 0; c < 3; ++c) a.nor[c] += in.n[c];
        for (int c = 0; c < 3; ++c) a.alb[c] += per_sample_albedo ? in.alb[c] : palb[c];
        a.dep += in.d;
    }
    if (!finite3(in.L[0], in.L[1], in.L[2])) {  // main.cpp:707
        lum_out = __int_as_float(0x7fc00000);  // NaN: dropped by the grid pass
        key_out = 0;
        return;
    }
    // accumulate_sample (core/stats.h:25-41)
    const float lum = luminance(in.L[0], in.L[1], in.L[2]);
    const float delta = lum - a.mean;
    ++a.n;
    if (COMPACT_IN) {
        // the seven quotients by n from one reciprocal, each still the IEEE quotient (the
        // dividends are known before any of the updates)
        const float fn = float(a.n);
        float cd[3], sd[3];
        bool fast = a.n < (1 << 23) && markstein_ok(delta);
        for (int c = 0; c < 3; ++c) {
            cd[c] = in.L[c] - a.cm[c];
            sd[c] = in.root[c] - a.sm[c];
            fast = fast && markstein_ok(cd[c]) && markstein_ok(sd[c]);
        }
        if (fast) {
            const float rn = 1.0f / fn;
            a.mean += div_markstein(delta, fn, rn);
            for (int c = 0; c < 3; ++c) a.cm[c] += div_markstein(cd[c], fn, rn);
            for (int c = 0; c < 3; ++c) a.sm[c] += div_markstein(sd[c], fn, rn);
        } else {
            a.mean += delta / fn;
            for (int c = 0; c < 3; ++c) a.cm[c] += cd[c] / fn;
            for (int c = 0; c < 3; ++c) a.sm[c] += sd[c] / fn;
        }
        const float delta2 = lum - a.mean;
        a.m2 += delta * delta2;
        for (int c = 0; c < 3; ++c) a.sq[c] += sd[c] * (in.root[c] - a.sm[c]);
    } else {
        a.mean += delta / float(a.n);
        const float delta2 = lum - a.mean;
        a.m2 += delta * delta2;
        for (int c = 0; c < 3; ++c) {
            const float cd = in.L[c] - a.cm[c];
            a.cm[c] += cd / float(a.n);
        }
        for (int c = 0; c < 3; ++c) {
            const float sc = sqrtf(fmaxs(0.0f, in.L[c]));
            const float sd = sc - a.sm[c];
            a.sm[c] += sd / float(a.n);
            a.sq[c] += sd * (sc - a.sm[c]);
        }
    }
    for (int c = 0; c < 3; ++c) a.rad[c] += in.L[c];
    ++a.nsamples;
    lum_out = lum;
    key_out = 0;
    if (!prep) return;
    const uint8_t fm = in.f & plane_mask;
    // packed random-dimension bins (Dependency2D::add, core/stats.h:166-168)
    uint32_t key = 0;
    if (COMPACT_IN) {
        key = in.bins & ((fm & RPD_SAMPLE_LENS_VALID ? 0x000fu : 0u) | (fm & RPD_SAMPLE_BRDF_VALID ? 0x00f0u : 0u) |
                         (fm & RPD_SAMPLE_LIGHT_VALID ? 0x0f00u : 0u) | (fm & RPD_SAMPLE_ENV_VALID ? 0xf000u : 0u));
    } else {
        if (fm & RPD_SAMPLE_LENS_VALID) key |= uint32_t(bin2d_k(in.lu[0], in.lu[1]));
        if (fm & RPD_SAMPLE_BRDF_VALID) key |= uint32_t(bin2d_k(in.bu[0], in.bu[1])) << 4;
        if (fm & RPD_SAMPLE_LIGHT_VALID) key |= uint32_t(bin2d_k(in.liu[0], in.liu[1])) << 8;
        if (fm & RPD_SAMPLE_ENV_VALID) key |= uint32_t(bin2d_k(in.eu[0], in.eu[1])) << 12;
    }
    key |= uint32_t(in.cat & RPD_CATEGORY_LIGHT_INDEX_MASK) << 16;
    key |= (in.cat & RPD_CATEGORY_RR_SURVIVED) ? (1u << 20) : 0u;
    key |= uint32_t(fm & 0xfe) << (kKeyValidShift - 1);
    key_out = key;
    const uint8_t cls_bits = fm & 0xfe;
    const float y2 = lum * lum;
    const float y2e = __fmaf_rn(lum, lum, -y2);
    if (cls_bits != 0 && !a.have_pat) {
        a.have_pat = true;
        a.pat = cls_bits;
    }
    if (cls_bits == 0) {
        // no validity class: nothing for the grid's totals
    } else if (cls_bits == a.pat) {
        a.pc += 1.0f;
        df_add(a.p1h, a.p1l, lum);
        df_add(a.p2h, a.p2l, y2);
        a.p2l += y2e;
    } else {
        if (!a.dev) {
            a.dev = true;
            for (int q = 0; q < kClasses * 5; ++q) a.cs[q] = 0.0f;
        }
        for (int c = 0; c < kClasses; ++c) {
            if (!(cls_bits & class_bit(c))) continue;
            float* e = a.cs + 5 * c;
            float h1 = e[1], l1 = e[2], h2 = e[3], l2 = e[4];
            df_add(h1, l1, lum);
            df_add(h2, l2, y2);
            l2 += y2e;
            e[0] += 1.0f;
            e[1] = h1;
            e[2] = l1;
            e[3] = h2;
            e[4] = l2;
        }
    }
    if (fm & RPD_SAMPLE_PIXEL_VALID) {
        // the screen position stays inside the pixel: with a power-of-two support 4 <= S <= 2^11
        // the screen bin is floor(fl(fl(x + u) - left) / (S/4)) (the division and the x4 are
        // power-of-two scalings; left is an integer), the pixel's own bin whenever
        // f = fl(x + u) - x lies in [0, 1 - 2^-12]: fl(X - left) is exact for left >= 0, and for
        // the first node row/column (left = -S/2, X + S/2 < 2^12) it moves by at most 2^-13
        // (main.cpp:352-356, core/stats.h:166-167)
        const float jx = (fx + in.pu[0]) - fx, jy = (fy + in.pu[1]) - fy;
        if (!(jx >= 0.0f && jx <= kUniformMax && jy >= 0.0f && jy <= kUniformMax)) a.pflags &= uint8_t(~kPixUniform);
    } else if (fm & (RPD_SAMPLE_LENS_VALID | RPD_SAMPLE_BRDF_VALID | RPD_SAMPLE_LIGHT_VALID | RPD_SAMPLE_ENV_VALID |
                     RPD_SAMPLE_LIGHT_SELECT_VALID | RPD_SAMPLE_RR_VALID)) {
        a.pflags |= kPixMixed;  // a random dimension without the screen position
    }
}

__device__ __forceinline__ float4 ld4(const float* p, int64_t k) { return *reinterpret_cast<const float4*>(p + k); }
__device__ __forceinline__ float lane4(const float4& v, int i) { return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w; }

// rpd_sample_soa16 decoding (include/rpd_gb300.h)
__device__ __forceinline__ float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }
__device__ __forceinline__ float snorm16(int16_t q) { return fmaxf(float(q) * (1.0f / 32767.0f), -1.0f); }
__device__ __forceinline__ float unorm16(uint16_t q) { return float(q) * (1.0f / 65536.0f); }
__device__ __forceinline__ float sq(float v) { return v * v; }

// A pixel's running state before its first sample of the push (the class sums start empty).
__device__ __forceinline__ void acc_init(PixelAcc& a) {
    a.pflags = kPixUniform;
    a.have_pat = false;
    a.dev = false;
    a.pat = 0;
    a.pc = a.p1h = a.p1l = a.p2h = a.p2l = 0.0f;  // the class sums are cleared when the pixel deviates
}

// The grid-pass sums of a pixel without samples in the push.
__device__ __forceinline__ void acc_store_empty(const GridPrep& gp, int64_t idx) {
    gp.pat4[idx] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    gp.pat2[idx] = make_float2(0.0f, __uint_as_float(uint32_t(kPixUniform) << 8));
}

__device__ __forceinline__ void acc_zero(PixelAcc& a) {
    a.mean = a.m2 = 0.0f;
    a.n = 0;
    for (int c = 0; c < 3; ++c) a.cm[c] = a.sm[c] = a.sq[c] = a.rad[c] = a.nor[c] = a.alb[c] = 0.0f;
    a.dep = 0.0f;
    a.hits = a.nsamples = 0;
}

__device__ __forceinline__ void acc_load(PixelAcc& a, const PixelPlanes& p, int64_t idx) {
    a.mean = p.mean[idx];
    a.m2 = p.square_diff[idx];
    a.n = p.n[idx];
    for (int c = 0; c < 3; ++c) {
        a.cm[c] = p.color_mean[c][idx];
        a.sm[c] = p.sqrt_mean[c][idx];
        a.sq[c] = p.sqrt_sq[c][idx];
        a.rad[c] = p.radiance[c][idx];
        a.nor[c] = p.normal[c][idx];
        a.alb[c] = p.albedo[c][idx];
    }
    a.dep = p.depth[idx];
    a.hits = p.hit_count[idx];
    a.nsamples = p.sample_count[idx];
}

// The pixel's statistics back to its planes, and its grid-pass sums: the pattern class's, and
// for a deviant pixel the full per-class sums.
__device__ __forceinline__ void acc_store(const PixelAcc& a, const PixelPlanes& p, const GridPrep& gp, int64_t idx,
                                          bool prep) {
    p.mean[idx] = a.mean;
    p.square_diff[idx] = a.m2;
    p.n[idx] = a.n;
    for (int c = 0; c < 3; ++c) {
        p.color_mean[c][idx] = a.cm[c];
        p.sqrt_mean[c][idx] = a.sm[c];
        p.sqrt_sq[c][idx] = a.sq[c];
        p.radiance[c][idx] = a.rad[c];
        p.normal[c][idx] = a.nor[c];
        p.albedo[c][idx] = a.alb[c];
    }
    p.depth[idx] = a.dep;
    p.hit_count[idx] = a.hits;
    p.sample_count[idx] = a.nsamples;
    if (prep) {
        gp.pat4[idx] = make_float4(a.pc, a.p1h, a.p1l, a.p2h);
        const uint32_t bits = uint32_t(a.have_pat ? a.pat : 0) |
                              (uint32_t(a.pflags | (a.dev ? kPixDeviant : 0)) << 8);
        gp.pat2[idx] = make_float2(a.p2l, __uint_as_float(bits));
        if (a.dev) {
            // full per-class sums: the deviating samples plus the pattern's
            for (int c = 0; c < kClasses; ++c) {
                const float* e = a.cs + 5 * c;
                float h1 = e[1], l1 = e[2], h2 = e[3], l2 = e[4], cnt = e[0];
                if (a.have_pat && (a.pat & class_bit(c))) {
                    cnt += a.pc;
                    df_add(h1, l1, a.p1h);
                    l1 += a.p1l;
                    df_add(h2, l2, a.p2h);
                    l2 += a.p2l;
                }
                gp.cls[c][0][idx] = cnt;
                gp.cls[c][1][idx] = h1;
                gp.cls[c][2][idx] = l1;
                gp.cls[c][3][idx] = h2;
                gp.cls[c][4][idx] = l2;
            }
        }
    }
}

// VEC4: every present plane is 16-byte aligned at the pixel's first sample and the pixel's
// sample count is a multiple of 4, so each plane is read four samples per load. COMPACT: the
// planes are rpd_sample_soa16's (s.c16), decoded to float here; WIDE reads them 8 samples (16
// bytes) per load. MINB: resident blocks per SM the register allocation must allow.
template <bool VEC4, bool COMPACT, bool WIDE, int MINB>
__global__ void __launch_bounds__(128, MINB) k_accumulate_pixels(PixelPlanes p, DeviceSamples s, const int64_t* offsets,
                                                           int32_t spp, int64_t first, int64_t count, GridPrep gp,
                                                           int fresh) {
    const int64_t local = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (local >= count) return;
    const int64_t idx = first + local;
    const int64_t k0 = offsets ? offsets[local] : local * spp;
    const int64_t k1 = offsets ? offsets[local + 1] : (local + 1) * spp;
    const bool prep = gp.lum != nullptr;
    const bool has_pu = COMPACT ? s.c16.pixel_u[0] != nullptr : s.pixel_u[0] != nullptr;
    const bool has_lu = COMPACT ? s.c16.lens_u[0] != nullptr : s.lens_u[0] != nullptr;
    const bool has_bu = COMPACT ? s.c16.brdf_u[0] != nullptr : s.brdf_u[0] != nullptr;
    const bool has_li = COMPACT ? s.c16.light_u[0] != nullptr : s.light_u[0] != nullptr;
    const bool has_eu = COMPACT ? s.c16.env_u[0] != nullptr : s.env_u[0] != nullptr;
    const uint8_t plane_mask = uint8_t(0xffu & ~((has_pu ? 0 : RPD_SAMPLE_PIXEL_VALID) |
                                                 (has_lu ? 0 : RPD_SAMPLE_LENS_VALID) |
                                                 (has_bu ? 0 : RPD_SAMPLE_BRDF_VALID) |
                                                 (has_li ? 0 : RPD_SAMPLE_LIGHT_VALID) |
                                                 (has_eu ? 0 : RPD_SAMPLE_ENV_VALID)));
    const float fx = float(idx % gp.width), fy = float(idx / gp.width);
    PixelAcc a;
    // the class sums' local array, addressed through an offset the compiler cannot fold, so that
    // it stays in local memory instead of registers
    float cls_local[kClasses * 5];
    a.cs = cls_local + (uint32_t(gp.width) >> 31);  // the width is positive: offset 0
    acc_init(a);
    if (k0 == k1) {
        if (prep) acc_store_empty(gp, idx);
        return;
    }
    // fresh: the frame's first push over every pixel, whose statistics the frame start zeroed
    if (fresh) acc_zero(a);
    else acc_load(a, p, idx);
    const bool per_sample_albedo = !COMPACT && s.albedo[0] != nullptr;
    float palb[3] = {0.0f, 0.0f, 0.0f};
    if (COMPACT) {
        if (s.c16.pixel_albedo[0])
            for (int c = 0; c < 3; ++c) palb[c] = h2f(s.c16.pixel_albedo[c][local]);
    } else if (!per_sample_albedo && s.pixel_albedo[0]) {
        for (int c = 0; c < 3; ++c) palb[c] = s.pixel_albedo[c][local];
    }
    const bool dims = prep;  // the random dimensions are only read for the grid pass

    if (COMPACT) {
        const DeviceSamples16& h = s.c16;
        const float dscale = h.depth_scale;
        if (VEC4) {
            // V samples per plane load: 8 (16-byte loads) when WIDE, else 4 (8-byte loads)
            constexpr int V = WIDE ? 8 : 4;
            constexpr int NW = V / 2;  // 32-bit words per load
            struct Wv { uint32_t w[NW]; };
            auto ldv = [](const void* ptr, int64_t k) {
                Wv r;
                if constexpr (WIDE) {
                    const uint4 v = *reinterpret_cast<const uint4*>(static_cast<const uint16_t*>(ptr) + k);
                    r.w[0] = v.x;
                    r.w[1] = v.y;
                    r.w[2] = v.z;
                    r.w[3] = v.w;
                } else {
                    const uint2 v = *reinterpret_cast<const uint2*>(static_cast<const uint16_t*>(ptr) + k);
                    r.w[0] = v.x;
                    r.w[1] = v.y;
                }
                return r;
            };
            auto lane16 = [](const Wv& v, int i) { return uint16_t(v.w[i >> 1] >> (16 * (i & 1))); };
            for (int64_t k = k0; k < k1; k += V) {
                Wv L[3], N[3], D, PU[2], LU[2], BU[2], LI[2], EU[2];
                for (int c = 0; c < 3; ++c) {
                    L[c] = ldv(h.sqrt_radiance[c], k);
                    N[c] = ldv(h.normal[c], k);
                }
                D = ldv(h.depth, k);
                Wv z;
                for (int q = 0; q < NW; ++q) z.w[q] = 0u;
                for (int c = 0; c < 2; ++c) {
                    PU[c] = (dims && has_pu) ? ldv(h.pixel_u[c], k) : z;
                    LU[c] = (dims && has_lu) ? ldv(h.lens_u[c], k) : z;
                    BU[c] = (dims && has_bu) ? ldv(h.brdf_u[c], k) : z;
                    LI[c] = (dims && has_li) ? ldv(h.light_u[c], k) : z;
                    EU[c] = (dims && has_eu) ? ldv(h.env_u[c], k) : z;
                }
                uint32_t F[NW / 2 > 0 ? NW / 2 : 1], Cg[NW / 2 > 0 ? NW / 2 : 1];
                for (int q = 0; q < V / 4; ++q) {
                    F[q] = *reinterpret_cast<const uint32_t*>(s.flags + k + 4 * q);
                    Cg[q] = (dims && s.category) ? *reinterpret_cast<const uint32_t*>(s.category + k + 4 * q) : 0u;
                }
                float lumv[V];
                uint32_t keyv[V];
                #pragma unroll
                for (int i = 0; i < V; ++i) {
                    SampleIn in;
                    for (int c = 0; c < 3; ++c) {
                        in.root[c] = fabsf(h2f(lane16(L[c], i)));
                        in.L[c] = sq(in.root[c]);
                        in.n[c] = snorm16(int16_t(lane16(N[c], i)));
                        in.alb[c] = 0.0f;
                    }
                    in.d = h2f(lane16(D, i)) * dscale;
                    for (int c = 0; c < 2; ++c) in.pu[c] = unorm16(lane16(PU[c], i));
                    in.bins = bin2d_q(lane16(LU[0], i), lane16(LU[1], i)) |
                              (bin2d_q(lane16(BU[0], i), lane16(BU[1], i)) << 4) |
                              (bin2d_q(lane16(LI[0], i), lane16(LI[1], i)) << 8) |
                              (bin2d_q(lane16(EU[0], i), lane16(EU[1], i)) << 12);
                    in.f = uint8_t(F[i >> 2] >> (8 * (i & 3)));
                    in.cat = uint8_t(Cg[i >> 2] >> (8 * (i & 3)));
                    process_sample<true>(a, in, false, palb, prep, plane_mask, fx, fy, lumv[i], keyv[i]);
                }
                if (prep) {
                    for (int q = 0; q < V / 4; ++q) {
                        *reinterpret_cast<float4*>(gp.lum + k + 4 * q) =
                            make_float4(lumv[4 * q], lumv[4 * q + 1], lumv[4 * q + 2], lumv[4 * q + 3]);
                        *reinterpret_cast<uint4*>(gp.key + k + 4 * q) =
                            make_uint4(keyv[4 * q], keyv[4 * q + 1], keyv[4 * q + 2], keyv[4 * q + 3]);
                    }
                }
            }
        } else {
            for (int64_t k = k0; k < k1; ++k) {
                SampleIn in;
                for (int c = 0; c < 3; ++c) {
                    in.root[c] = fabsf(h2f(h.sqrt_radiance[c][k]));
                    in.L[c] = sq(in.root[c]);
                    in.n[c] = snorm16(h.normal[c][k]);
                    in.alb[c] = 0.0f;
                }
                in.d = h2f(h.depth[k]) * dscale;
                uint16_t q[4][2];
                for (int c = 0; c < 2; ++c) {
                    in.pu[c] = (dims && has_pu) ? unorm16(h.pixel_u[c][k]) : 0.0f;
                    q[0][c] = (dims && has_lu) ? h.lens_u[c][k] : uint16_t(0);
                    q[1][c] = (dims && has_bu) ? h.brdf_u[c][k] : uint16_t(0);
                    q[2][c] = (dims && has_li) ? h.light_u[c][k] : uint16_t(0);
                    q[3][c] = (dims && has_eu) ? h.env_u[c][k] : uint16_t(0);
                }
                in.bins = bin2d_q(q[0][0], q[0][1]) | (bin2d_q(q[1][0], q[1][1]) << 4) |
                          (bin2d_q(q[2][0], q[2][1]) << 8) | (bin2d_q(q[3][0], q[3][1]) << 12);
                in.f = s.flags[k];
                in.cat = (dims && s.category) ? s.category[k] : 0;
                float lum;
                uint32_t key;
                process_sample<true>(a, in, false, palb, prep, plane_mask, fx, fy, lum, key);
                if (prep) {
                    gp.lum[k] = lum;
                    gp.key[k] = key;
                    if (gp.col) gp.col[k] = uint16_t(idx % gp.width);
                }
            }
        }
    } else if (VEC4) {
        for (int64_t k = k0; k < k1; k += 4) {
            float4 L[3], N[3], A[3], D, PU[2], LU[2], BU[2], LI[2], EU[2];
            for (int c = 0; c < 3; ++c) {
                L[c] = ld4(s.radiance[c], k);
                N[c] = ld4(s.normal[c], k);
                A[c] = per_sample_albedo ? ld4(s.albedo[c], k) : make_float4(0, 0, 0, 0);
            }
            D = ld4(s.depth, k);
            const float4 z4 = make_float4(0, 0, 0, 0);
            for (int c = 0; c < 2; ++c) {
                PU[c] = (dims && s.pixel_u[0]) ? ld4(s.pixel_u[c], k) : z4;
                LU[c] = (dims && s.lens_u[0]) ? ld4(s.lens_u[c], k) : z4;
                BU[c] = (dims && s.brdf_u[0]) ? ld4(s.brdf_u[c], k) : z4;
                LI[c] = (dims && s.light_u[0]) ? ld4(s.light_u[c], k) : z4;
                EU[c] = (dims && s.env_u[0]) ? ld4(s.env_u[c], k) : z4;
            }
            const uint32_t F4 = *reinterpret_cast<const uint32_t*>(s.flags + k);
            const uint32_t C4 = (dims && s.category) ? *reinterpret_cast<const uint32_t*>(s.category + k) : 0u;
            float lum4[4];
            uint32_t key4[4];
            #pragma unroll
            for (int i = 0; i < 4; ++i) {
                SampleIn in;
                for (int c = 0; c < 3; ++c) {
                    in.L[c] = lane4(L[c], i);
                    in.n[c] = lane4(N[c], i);
                    in.alb[c] = lane4(A[c], i);
                }
                in.d = lane4(D, i);
                for (int c = 0; c < 2; ++c) {
                    in.pu[c] = lane4(PU[c], i);
                    in.lu[c] = lane4(LU[c], i);
                    in.bu[c] = lane4(BU[c], i);
                    in.liu[c] = lane4(LI[c], i);
                    in.eu[c] = lane4(EU[c], i);
                }
                in.f = uint8_t(F4 >> (8 * i));
                in.cat = uint8_t(C4 >> (8 * i));
                process_sample(a, in, per_sample_albedo, palb, prep, plane_mask, fx, fy, lum4[i], key4[i]);
            }
            if (prep) {
                *reinterpret_cast<float4*>(gp.lum + k) = make_float4(lum4[0], lum4[1], lum4[2], lum4[3]);
                *reinterpret_cast<uint4*>(gp.key + k) = make_uint4(key4[0], key4[1], key4[2], key4[3]);
            }
        }
    } else {
        for (int64_t k = k0; k < k1; ++k) {
            SampleIn in;
            for (int c = 0; c < 3; ++c) {
                in.L[c] = s.radiance[c][k];
                in.n[c] = s.normal[c][k];
                in.alb[c] = per_sample_albedo ? s.albedo[c][k] : 0.0f;
            }
            in.d = s.depth[k];
            for (int c = 0; c < 2; ++c) {
                in.pu[c] = (dims && s.pixel_u[0]) ? s.pixel_u[c][k] : 0.0f;
                in.lu[c] = (dims && s.lens_u[0]) ? s.lens_u[c][k] : 0.0f;
                in.bu[c] = (dims && s.brdf_u[0]) ? s.brdf_u[c][k] : 0.0f;
                in.liu[c] = (dims && s.light_u[0]) ? s.light_u[c][k] : 0.0f;
                in.eu[c] = (dims && s.env_u[0]) ? s.env_u[c][k] : 0.0f;
            }
            in.f = s.flags[k];
            in.cat = (dims && s.category) ? s.category[k] : 0;
            float lum;
            uint32_t key;
            process_sample(a, in, per_sample_albedo, palb, prep, plane_mask, fx, fy, lum, key);
            if (prep) {
                gp.lum[k] = lum;
                gp.key[k] = key;
                if (gp.col) gp.col[k] = uint16_t(idx % gp.width);
            }
        }
    }

    acc_store(a, p, gp, idx, prep);
}

// Valid-flag bit each dependency needs, and whether it bins the screen position.
__device__ __forceinline__ uint8_t dep_flag(int d) {
    switch (d) {
    case D_PIXEL: return 0;
    case D_BRDF: case D_SCREEN_BRDF: return RPD_SAMPLE_BRDF_VALID;
    case D_LENS: case D_SCREEN_LENS: return RPD_SAMPLE_LENS_VALID;
    case D_LIGHT_UV: case D_SCREEN_LIGHT_UV: return RPD_SAMPLE_LIGHT_VALID;
    case D_ENV: case D_SCREEN_ENV: return RPD_SAMPLE_ENV_VALID;
    case D_LIGHT_SELECT: case D_SCREEN_LIGHT_SELECT: return RPD_SAMPLE_LIGHT_SELECT_VALID;
    default: return RPD_SAMPLE_RR_VALID;
    }
}
__device__ __forceinline__ bool dep_is_screen(int d) {
    return d == D_PIXEL || d == D_SCREEN_BRDF || d == D_SCREEN_LENS || d == D_SCREEN_LIGHT_UV ||
           d == D_SCREEN_ENV || d == D_SCREEN_LIGHT_SELECT || d == D_SCREEN_RR;
}

// Dependency2D::add bin (core/stats.h:166-168)
__device__ __forceinline__ int bin2d(float u, float v) {
    const int x = iclamps(int(u * 4.0f), 0, 3);
    const int z = iclamps(int(v * 4.0f), 0, 3);
    return z * 4 + x;
}

__global__ void __launch_bounds__(128) k_grid_ordered(Geometry g, double* pass_grid, DeviceSamples s,
                                                      const int64_t* offsets, int32_t spp, int64_t first,
                                                      int64_t count) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= g.nn * kDeps) return;
    const int node = int(t / kDeps);
    const int d = int(t % kDeps);
    const int nx = node % g.nodes_x, ny = node / g.nodes_x;
    const uint8_t need = dep_flag(d);
    const bool screen = dep_is_screen(d);
    const int bins = (d == D_RR) ? 2 : 16;
    // a NULL plane never validates its dependency
    const float* const* dims = nullptr;
    switch (d) {
    case D_BRDF: dims = s.brdf_u; break;
    case D_LENS: dims = s.lens_u; break;
    case D_LIGHT_UV: dims = s.light_u; break;
    case D_ENV: dims = s.env_u; break;
    default: break;
    }
    if (screen && !s.pixel_u[0]) return;
    if (dims && !dims[0]) return;
    if ((d == D_SCREEN_BRDF && !s.brdf_u[0]) || (d == D_SCREEN_LENS && !s.lens_u[0]) ||
        (d == D_SCREEN_LIGHT_UV && !s.light_u[0]) || (d == D_SCREEN_ENV && !s.env_u[0]))
        return;

    double* acc = pass_grid + int64_t(node) * kDeps * kDepStride + d * kDepStride;
    double wbin[16], ybin[16];
    for (int b = 0; b < 16; ++b) {
        wbin[b] = acc[b];
        ybin[b] = acc[16 + b];
    }
    double w_sum = acc[32], w2_sum = acc[33], y_sum = acc[34], y2_sum = acc[35];

    const float half_support = 0.5f * float(g.support);
    const float inv_dummy = 0.0f;
    (void)inv_dummy;
    // pixels whose bilinear footprint can reach this node
    const int xlo = imaxs(0, (nx - 1) * g.step - 1), xhi = imins(g.w - 1, (nx + 1) * g.step + 1);
    const int ylo = imaxs(0, (ny - 1) * g.step - 1), yhi = imins(g.h - 1, (ny + 1) * g.step + 1);
    for (int y = ylo; y <= yhi; ++y) {
        const float gy = float(y) / float(g.step);
        const int y0 = iclamps(int(floorf(gy)), 0, g.nodes_y - 1);
        const int y1 = imins(y0 + 1, g.nodes_y - 1);
        if (y0 != ny && y1 != ny) continue;
        const float ty = fclamps(gy - float(y0), 0.0f, 1.0f);
        for (int x = xlo; x <= xhi; ++x) {
            const int64_t idx = int64_t(y) * g.w + x;
            if (idx < first || idx >= first + count) continue;
            const float gx = float(x) / float(g.step);
            const int x0 = iclamps(int(floorf(gx)), 0, g.nodes_x - 1);
            const int x1 = imins(x0 + 1, g.nodes_x - 1);
            if (x0 != nx && x1 != nx) continue;
            const float tx = fclamps(gx - float(x0), 0.0f, 1.0f);
            // the four entries of main.cpp:341-346, in order; keep those naming this node
            float we[4];
            int ne = 0;
            if (x0 == nx && y0 == ny) we[ne++] = (1.0f - tx) * (1.0f - ty);
            if (x1 == nx && y0 == ny) we[ne++] = tx * (1.0f - ty);
            if (x0 == nx && y1 == ny) we[ne++] = (1.0f - tx) * ty;
            if (x1 == nx && y1 == ny) we[ne++] = tx * ty;
            bool any = false;
            for (int e = 0; e < ne; ++e) any |= we[e] > 1e-8f;
            if (!any) continue;
            const int64_t local = idx - first;
            const int64_t k0 = offsets ? offsets[local] : local * spp;
            const int64_t k1 = offsets ? offsets[local + 1] : (local + 1) * spp;
            const float support_left = float(nx * g.step) - half_support;
            const float support_top = float(ny * g.step) - half_support;
            for (int64_t k = k0; k < k1; ++k) {
                uint8_t f = s.flags ? s.flags[k] : 0;
                if (!s.pixel_u[0]) f &= uint8_t(~RPD_SAMPLE_PIXEL_VALID);
                if (!s.lens_u[0]) f &= uint8_t(~RPD_SAMPLE_LENS_VALID);
                if (!s.brdf_u[0]) f &= uint8_t(~RPD_SAMPLE_BRDF_VALID);
                if (!s.light_u[0]) f &= uint8_t(~RPD_SAMPLE_LIGHT_VALID);
                if (!s.env_u[0]) f &= uint8_t(~RPD_SAMPLE_ENV_VALID);
                const bool pixel_valid = (f & RPD_SAMPLE_PIXEL_VALID) != 0;
                if (screen && !pixel_valid) continue;
                if (need && !(f & need)) continue;
                // main.cpp:330 — samples without any captured dimension are skipped
                if (!(f & (RPD_SAMPLE_PIXEL_VALID | RPD_SAMPLE_LENS_VALID | RPD_SAMPLE_LIGHT_SELECT_VALID |
                           RPD_SAMPLE_BRDF_VALID | RPD_SAMPLE_LIGHT_VALID | RPD_SAMPLE_ENV_VALID |
                           RPD_SAMPLE_RR_VALID)))
                    continue;
                const float r = s.radiance[0][k], gch = s.radiance[1][k], b = s.radiance[2][k];
                if (!finite3(r, gch, b)) continue;
                const float lum = luminance(r, gch, b);
                int bin;
                if (screen) {
                    const float su = fclamps((float(x) + s.pixel_u[0][k] - support_left) / float(g.support), 0.0f, 1.0f);
                    const float sv = fclamps((float(y) + s.pixel_u[1][k] - support_top) / float(g.support), 0.0f, 1.0f);
                    bin = bin2d(su, sv);
                } else if (d == D_LIGHT_SELECT) {
                    bin = int(s.category[k] & RPD_CATEGORY_LIGHT_INDEX_MASK);
                } else if (d == D_RR) {
                    bin = (s.category[k] & RPD_CATEGORY_RR_SURVIVED) ? 1 : 0;
                } else {
                    bin = bin2d(dims[0][k], dims[1][k]);
                }
                bin = iclamps(bin, 0, bins - 1);
                const double yd = double(lum);
                for (int e = 0; e < ne; ++e) {
                    // BinnedDependency::add (core/stats.h:102-113)
                    if (we[e] <= 1e-8f) continue;
                    const double wd = double(we[e]);
                    wbin[bin] += wd;
                    ybin[bin] += wd * yd;
                    w_sum += wd;
                    w2_sum += wd * wd;
                    y_sum += wd * yd;
                    y2_sum += wd * yd * yd;
                }
            }
        }
    }
    for (int b = 0; b < 16; ++b) {
        acc[b] = wbin[b];
        acc[16 + b] = ybin[b];
    }
    acc[32] = w_sum;
    acc[33] = w2_sum;
    acc[34] = y_sum;
    acc[35] = y2_sum;
}

// float -> double from the bits (the conversion instruction runs on the double-precision pipe,
// 2 per SM per clock); zeros keep their sign, subnormals, infinities and NaN convert as usual.
__device__ __forceinline__ double widen(float f) {
    const uint32_t b = __float_as_uint(f);
    if ((b & 0x7fffffffu) == 0u) return __longlong_as_double(static_cast<long long>(uint64_t(b) << 32));
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return double(f);
    return __longlong_as_double(static_cast<long long>((uint64_t(b >> 31) << 63) | (uint64_t(e + 896u) << 52) |
                                                       (uint64_t(b & 0x7fffffu) << 29)));
}

// grid += pass (the first pass of a frame: grid = 0 + pass), then clear the pass grid. The pass
// grid holds double-float pairs (hi, lo) in the bytes of each double in the fast grid mode, doubles
// in the exact one. The frame grid takes the first merged pass's form: in the fast mode it stays
// pairs, each merge a double-float addition (about 2^-44 relative, within the grid's 1e-9 of the
// reference) with no double-precision instruction, which GB300 issues at 2 per SM per clock; a
// frame whose passes mix the modes ends in doubles.
enum MergeMode {
    kMergePairsFresh,     // pairs -> the frame's pairs
    kMergePairsPairs,     // frame pairs + pass pairs
    kMergeDoubleFresh,    // doubles -> the frame's doubles
    kMergeDoubleDouble,   // frame doubles + pass doubles
    kMergePairsIntoDouble,  // frame doubles + pass pairs
    kMergeDoubleIntoPairs   // frame pairs + pass doubles -> frame doubles
};
__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = ((a.x - (s - bb)) + (b.x - bb)) + (a.y + b.y);
    const float h = s + e;
    return make_float2(h, e - (h - s));
}

template <int MODE>
__global__ void k_merge_grid(double* grid, double* pass_grid, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float2* gp = reinterpret_cast<float2*>(grid);
    const float2* pp = reinterpret_cast<const float2*>(pass_grid);
    if (MODE == kMergePairsFresh) {
        gp[i] = pp[i];
    } else if (MODE == kMergePairsPairs) {
        gp[i] = pair_add(gp[i], pp[i]);
    } else {
        double v;
        if (MODE == kMergePairsIntoDouble) v = widen(pp[i].x) + widen(pp[i].y);
        else v = pass_grid[i];
        if (MODE == kMergeDoubleFresh) {
            // 0 + v without a double-precision add: the same value, with -0 turned into +0
            const long long b = __double_as_longlong(v);
            grid[i] = __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
        } else if (MODE == kMergeDoubleIntoPairs) {
            const float2 g = gp[i];
            grid[i] = (widen(g.x) + widen(g.y)) + v;
        } else {
            grid[i] = grid[i] + v;
        }
    }
    pass_grid[i] = 0.0;
}

// The frame grid as doubles (for reads): pairs widened and added.
__global__ void k_grid_pairs_to_double(const float2* pairs, double* out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 g = pairs[i];
    out[i] = widen(g.x) + widen(g.y);
}

__global__ void k_feature_cache(PixelPlanes p, int64_t np) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int hc = p.hit_count[i];
    if (hc > 0) {
        const float h = float(hc);
        float n0 = p.normal[0][i] / h, n1 = p.normal[1][i] / h, n2 = p.normal[2][i] / h;
        const float z = dot3(n0, n1, n2, n0, n1, n2);
        if (z > 1e-8f) {
            // Eigen normalize(): divide by sqrt(squaredNorm) when positive
            const float sn = sqrtf(z);
            n0 = n0 / sn;
            n1 = n1 / sn;
            n2 = n2 / sn;
        }
        p.f_normal[0][i] = n0;
        p.f_normal[1][i] = n1;
        p.f_normal[2][i] = n2;
        p.f_depth[i] = p.depth[i] / h;
        for (int c = 0; c < 3; ++c) p.f_albedo[c][i] = p.albedo[c][i] / h;
    } else {
        for (int c = 0; c < 3; ++c) p.f_normal[c][i] = p.normal[c][i];
        p.f_depth[i] = p.depth[i];
        for (int c = 0; c < 3; ++c) p.f_albedo[c][i] = p.albedo[c][i];
    }
}

__global__ void k_finalize(PixelPlanes p, int64_t np) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float samples = float(imaxs(1, p.sample_count[i]));
    const float hits = float(imaxs(1, p.hit_count[i]));
    for (int c = 0; c < 3; ++c) p.radiance[c][i] /= samples;
    for (int c = 0; c < 3; ++c) p.albedo[c][i] /= hits;
    float n0 = p.normal[0][i] / hits, n1 = p.normal[1][i] / hits, n2 = p.normal[2][i] / hits;
    const float z = dot3(n0, n1, n2, n0, n1, n2);
    if (z > 1e-8f) {
        const float sn = sqrtf(z);
        n0 = n0 / sn;
        n1 = n1 / sn;
        n2 = n2 / sn;
    }
    p.normal[0][i] = n0;
    p.normal[1][i] = n1;
    p.normal[2][i] = n2;
    p.depth[i] /= hits;
}

}  // namespace

cudaError_t launch_offsets_uniform(Job& j, int64_t count, int32_t spp) {
    KernelScope ks(j, RPD_KERNEL_OFFSETS);
    k_offsets_uniform<<<grid_for(count + 1, 256), 256, 0, j.stream>>>(j.offsets, count, spp);
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_offsets_scan(Job& j, const int32_t* d_counts, int64_t count) {
    KernelScope ks(j, RPD_KERNEL_OFFSETS);
    if (count <= 0) return cudaMemsetAsync(j.offsets, 0, sizeof(int64_t), j.stream);
    const int64_t nblocks = (count + kScanBlock - 1) / kScanBlock;
    // the offsets buffer reserves room for these after offsets[count]
    int64_t* block_sums = j.offsets + (count + 1);
    int64_t* block_maxima = block_sums + (nblocks + 1);
    k_scan_block_sums<<<unsigned(nblocks), kScanBlock, 0, j.stream>>>(d_counts, count, block_sums, block_maxima);
    k_scan_block_offsets<<<1, kScanBlock, 0, j.stream>>>(block_sums, block_maxima, nblocks);
    k_scan_finish<<<unsigned(nblocks), kScanBlock, 0, j.stream>>>(d_counts, count, block_sums, j.offsets);
    j.launches += 3;
    return cudaGetLastError();
}

const int64_t* offsets_count_max(const Job& j, int64_t count) {
    const int64_t nblocks = (count + kScanBlock - 1) / kScanBlock;
    return j.offsets + (count + 1) + (nblocks + 1) + nblocks;
}

// The statistics pass uses no shared memory: its launches ask for the whole unified array as L1,
// which keeps more of the sample sectors a thread reads again a step later (3 % more throughput
// on the served stream, where other requests' kernels share the SMs).
template <bool VEC4, bool COMPACT, bool WIDE, int MINB>
cudaError_t run_accumulate(Job& j, unsigned blocks, const DeviceSamples& s, int64_t first, int64_t count,
                           const GridPrep& gp, int fresh) {
    const cudaError_t e = cudaFuncSetAttribute(k_accumulate_pixels<VEC4, COMPACT, WIDE, MINB>,
                                               cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxL1);
    if (e != cudaSuccess) return e;
    k_accumulate_pixels<VEC4, COMPACT, WIDE, MINB><<<blocks, 128, 0, j.stream>>>(j.p, s, j.offsets, 0, first, count, gp,
                                                                              fresh);
    return cudaSuccess;
}

cudaError_t launch_accumulate_pixels(Job& j, const DeviceSamples& s, int64_t first, int64_t count,
                                     const GridPrep& gp, int32_t spp) {
    KernelScope ks(j, RPD_KERNEL_ACCUMULATE_PIXELS);
    // the frame's first push over every pixel starts from the zeros the frame start wrote
    // instead of reading them
    const int fresh = (j.acc_zero && first == 0 && count == j.g.np) ? 1 : 0;
    j.acc_zero = false;
    auto aligned = [](const void* ptr, uintptr_t a) { return (reinterpret_cast<uintptr_t>(ptr) & (a - 1)) == 0; };
    bool vec4 = spp > 0 && spp % 4 == 0 && aligned(s.flags, 16) && (!s.category || aligned(s.category, 16));
    if (s.compact) {
        const DeviceSamples16& h = s.c16;
        for (int c = 0; c < 3; ++c) vec4 = vec4 && aligned(h.sqrt_radiance[c], 8) && aligned(h.normal[c], 8);
        vec4 = vec4 && aligned(h.depth, 8);
        for (int c = 0; c < 2; ++c)
            vec4 = vec4 && (!h.pixel_u[0] || aligned(h.pixel_u[c], 8)) && (!h.lens_u[0] || aligned(h.lens_u[c], 8)) &&
                   (!h.brdf_u[0] || aligned(h.brdf_u[c], 8)) && (!h.light_u[0] || aligned(h.light_u[c], 8)) &&
                   (!h.env_u[0] || aligned(h.env_u[c], 8));
    } else {
        vec4 = vec4 && aligned(s.depth, 16);
        for (int c = 0; c < 3; ++c)
            vec4 = vec4 && aligned(s.radiance[c], 16) && aligned(s.normal[c], 16) && (!s.albedo[0] || aligned(s.albedo[c], 16));
        for (int c = 0; c < 2; ++c)
            vec4 = vec4 && (!s.pixel_u[0] || aligned(s.pixel_u[c], 16)) && (!s.lens_u[0] || aligned(s.lens_u[c], 16)) &&
                   (!s.brdf_u[0] || aligned(s.brdf_u[c], 16)) && (!s.light_u[0] || aligned(s.light_u[c], 16)) &&
                   (!s.env_u[0] || aligned(s.env_u[c], 16));
    }
    vec4 = vec4 && (!gp.lum || (aligned(gp.lum, 16) && aligned(gp.key, 16)));
    const unsigned blocks = grid_for(count, 128);
    // Shapes measured on GB300 at 1920x1080. Up to 16 samples per pixel, more resident pixels
    // hide the per-pixel latency (compact planes 4 blocks per SM, FP32 planes 3; per-pixel counts
    // 4 over compact planes, 5 over FP32 planes). From 32 on, a thread's sample run spans more bytes per plane than L1 keeps between its
    // loads, and a block's registers are not capped; from 64 on, compact planes are read 16 bytes
    // (8 samples) per load.
    const bool many = spp > 16;
    cudaError_t e;
    if (s.compact) {
        bool wide = vec4 && spp >= 64 && spp % 8 == 0;
        const DeviceSamples16& h = s.c16;
        for (int c = 0; c < 3; ++c) wide = wide && aligned(h.sqrt_radiance[c], 16) && aligned(h.normal[c], 16);
        wide = wide && aligned(h.depth, 16);
        for (int c = 0; c < 2; ++c)
            wide = wide && (!h.pixel_u[0] || aligned(h.pixel_u[c], 16)) && (!h.lens_u[0] || aligned(h.lens_u[c], 16)) &&
                   (!h.brdf_u[0] || aligned(h.brdf_u[c], 16)) && (!h.light_u[0] || aligned(h.light_u[c], 16)) &&
                   (!h.env_u[0] || aligned(h.env_u[c], 16));
        if (wide)
            e = run_accumulate<true, true, true, 1>(j, blocks, s, first, count, gp, fresh);
        else if (vec4 && many)
            e = run_accumulate<true, true, false, 1>(j, blocks, s, first, count, gp, fresh);
        else if (vec4)
            e = run_accumulate<true, true, false, 4>(j, blocks, s, first, count, gp, fresh);
        else
            e = run_accumulate<false, true, false, 4>(j, blocks, s, first, count, gp, fresh);
    } else {
        if (vec4 && many)
            e = run_accumulate<true, false, false, 1>(j, blocks, s, first, count, gp, fresh);
        else if (vec4)
            e = run_accumulate<true, false, false, 3>(j, blocks, s, first, count, gp, fresh);
        else
            e = run_accumulate<false, false, false, 5>(j, blocks, s, first, count, gp, fresh);
    }
    if (e != cudaSuccess) return e;
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_accumulate_grid(Job& j, const DeviceSamples& s, int64_t first, int64_t count) {
    KernelScope ks(j, RPD_KERNEL_GRID);
    const int64_t threads = j.g.nn * kDeps;
    k_grid_ordered<<<grid_for(threads, 128), 128, 0, j.stream>>>(j.g, j.n.pass_grid, s, j.offsets, 0, first, count);
    j.pass_indirect = true;
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_merge_grid(Job& j) {
    // pushes that added straight into the frame grid leave nothing in the pass grid
    const bool any = j.pass_indirect;
    j.pass_direct = j.pass_indirect = false;
    if (!any) return cudaSuccess;
    KernelScope ks(j, RPD_KERNEL_MERGE);
    const int64_t n = j.g.nn * kDeps * kDepStride;
    const bool pass_pairs = !j.exact_grid;  // the pass grid's form (k_grid_ordered writes doubles)
    const unsigned blocks = grid_for(n, 256);
    double* g = j.n.grid;
    double* pg = j.n.pass_grid;
    if (j.grid_fresh) {
        if (pass_pairs) k_merge_grid<kMergePairsFresh><<<blocks, 256, 0, j.stream>>>(g, pg, n);
        else k_merge_grid<kMergeDoubleFresh><<<blocks, 256, 0, j.stream>>>(g, pg, n);
        j.grid_pairs = pass_pairs;
    } else if (pass_pairs && j.grid_pairs) {
        k_merge_grid<kMergePairsPairs><<<blocks, 256, 0, j.stream>>>(g, pg, n);
    } else if (!pass_pairs && !j.grid_pairs) {
        k_merge_grid<kMergeDoubleDouble><<<blocks, 256, 0, j.stream>>>(g, pg, n);
    } else if (pass_pairs) {
        k_merge_grid<kMergePairsIntoDouble><<<blocks, 256, 0, j.stream>>>(g, pg, n);
    } else {
        k_merge_grid<kMergeDoubleIntoPairs><<<blocks, 256, 0, j.stream>>>(g, pg, n);
        j.grid_pairs = false;
    }
    j.grid_fresh = false;
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_grid_to_double(Job& j, double* out) {
    const int64_t n = j.g.nn * kDeps * kDepStride;
    k_grid_pairs_to_double<<<grid_for(n, 256), 256, 0, j.stream>>>(reinterpret_cast<const float2*>(j.n.grid), out, n);
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_feature_cache(Job& j) {
    KernelScope ks(j, RPD_KERNEL_FEATURES);
    k_feature_cache<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.p, j.g.np);
    j.launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_finalize(Job& j) {
    KernelScope ks(j, RPD_KERNEL_OTHER);
    k_finalize<<<grid_for(j.g.np, 256), 256, 0, j.stream>>>(j.p, j.g.np);
    j.launches += 1;
    return cudaGetLastError();
}

}  // namespace rpd
