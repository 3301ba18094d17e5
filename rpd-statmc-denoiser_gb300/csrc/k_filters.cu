// The two standalone post-filters of denoising/, as passes over per-pixel records.
//
// atrous_wavelet (denoising/atrous_wavelet.cpp:54-149, ping-ponged 185-197): `iterations`
// passes of the 5x5 B3-spline at step 2^i with luminance, normal-angle and albedo edge
// stopping, clamp-to-edge, centre kept when the weights vanish.
//   k_atrous_records  once per call: the unit normal (the stored normal renormalised when its
//                     squared length exceeds EPS_SMALL, atrous_wavelet.cpp:76-79) and the albedo
//                     of every pixel as float4 records, so no tap renormalises a neighbour;
//   k_atrous_pass     one pass. A thread owns one pixel; its 25 taps read the neighbour's
//                     colour (interleaved RGB, a warp reading 384 contiguous bytes per tap) and
//                     its 16-byte normal and albedo records, all served from L1/L2 after the
//                     first touch. The three edge-stopping factors exp(a) exp(b) exp(c) are one
//                     exponential of a + b + c.
//                     With records == nullptr the normals are renormalised at each tap instead
//                     (rpd_atrous_wavelet_noalloc, which has no scratch for records).
// joint_bilateral (denoising/joint_bilateral.cpp:15-132): one (2r+1)^2 window, r =
// max(1, ceil(3 sigma_p)), writing the gaussian, colour-bilateral and joint outputs at once.
//   k_bilateral_records  once per call: colour, the decoded unit normal (n * 2 - 1, then
//                     normalised, joint_bilateral.cpp:54-56,80-82) and albedo as float4 planes;
//   k_joint_bilateral a 32 x 8 block stages its (32 + 2r) x (8 + 2r) halo tile of the three
//                     planes in shared memory with one tensor copy (radius <= 16; larger radii
//                     read the records from global memory) and clamps each tap's coordinates
//                     into it, as the reference clamps them into the image. The pixel-distance
//                     term depends only on the (clamped) squared distance: its exponent and
//                     exponential come from a per-block table.
// Offsets are 64-bit. Single-precision arithmetic like the reference's; exp and acos are
// CUDA's, so outputs agree with the reference within the plain-form bar (1e-4 relative), not to
// the bit.
#include <algorithm>
#include <cmath>

#include "rpd_internal.h"
#include "device_math.cuh"
#include "tma.cuh"

namespace rpd {

namespace {

// The B3-spline taps h (atrous_wavelet.cpp:20); the spatial weight of tap (kx, ky) is
// h[ky] * h[kx], exact in single precision.
__constant__ float c_b3[5] = {1 / 16.0f, 1 / 4.0f, 3 / 8.0f, 1 / 4.0f, 1 / 16.0f};

// The reference's normalize(): scale by 1/sqrt(|v|^2) when |v|^2 > EPS_SMALL, operations in
// its order (the translation unit is compiled without contraction).
__device__ __forceinline__ float4 unit_or_same(float x, float y, float z) {
    const float len_sq = x * x + y * y + z * z;
    if (len_sq > 1e-8f) {
        const float inv_len = 1.0f / sqrtf(len_sq);
        x *= inv_len;
        y *= inv_len;
        z *= inv_len;
    }
    return make_float4(x, y, z, 0.0f);
}

__device__ __forceinline__ float dot_lr(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__global__ void k_atrous_records(const float* __restrict__ normal, const float* __restrict__ albedo, int64_t np,
                                 float4* __restrict__ nrm, float4* __restrict__ alb) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    nrm[i] = unit_or_same(normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]);
    alb[i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.0f);
}

// One a-trous pass. kc, kn, ka: 1 / (2 sigma^2) of the colour, normal and albedo terms.
template <bool kRecords>
__global__ void __launch_bounds__(256) k_atrous_pass(const float* __restrict__ in, float* __restrict__ out,
                                                     const float4* __restrict__ nrm, const float4* __restrict__ alb,
                                                     const float* __restrict__ normal, const float* __restrict__ albedo,
                                                     int w, int h, int step, float kc, float kn, float ka) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const int64_t i = int64_t(y) * w + x;
    const float cr = in[3 * i], cg = in[3 * i + 1], cb = in[3 * i + 2];
    const float c_lum = luminance(cr, cg, cb);
    float4 ni, ai;
    if constexpr (kRecords) {
        ni = nrm[i];
        ai = alb[i];
    } else {
        ni = unit_or_same(normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]);
        ai = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.0f);
    }
    int xs[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xs[k] = iclamps(x + (k - 2) * step, 0, w - 1);
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, sw = 0.0f;
#pragma unroll
    for (int ky = 0; ky < 5; ++ky) {
        const int64_t row = int64_t(iclamps(y + (ky - 2) * step, 0, h - 1)) * w;
#pragma unroll
        for (int kx = 0; kx < 5; ++kx) {
            const int64_t j = row + xs[kx];
            const float pr = in[3 * j], pg = in[3 * j + 1], pb = in[3 * j + 2];
            float4 nj, aj;
            if constexpr (kRecords) {
                nj = nrm[j];
                aj = alb[j];
            } else {
                nj = unit_or_same(normal[3 * j], normal[3 * j + 1], normal[3 * j + 2]);
                aj = make_float4(albedo[3 * j], albedo[3 * j + 1], albedo[3 * j + 2], 0.0f);
            }
            const float ld = c_lum - luminance(pr, pg, pb);
            const float angle = acosf(fclamps(dot_lr(ni, nj), -1.0f, 1.0f));
            const float da0 = ai.x - aj.x, da1 = ai.y - aj.y, da2 = ai.z - aj.z;
            const float dsa = da0 * da0 + da1 * da1 + da2 * da2;
            // w_color * w_normal * w_albedo (atrous_wavelet.cpp:122-139) as one exponential
            const float e = -__fmaf_rn(ld * ld, kc, __fmaf_rn(angle * angle, kn, dsa * ka));
            const float wt = (c_b3[ky] * c_b3[kx]) * __expf(e);
            sr = __fmaf_rn(wt, pr, sr);
            sg = __fmaf_rn(wt, pg, sg);
            sb = __fmaf_rn(wt, pb, sb);
            sw += wt;
        }
    }
    if (sw > 1e-8f) {
        const float inv = 1.0f / sw;
        out[3 * i] = sr * inv;
        out[3 * i + 1] = sg * inv;
        out[3 * i + 2] = sb * inv;
    } else {
        out[3 * i] = cr;
        out[3 * i + 1] = cg;
        out[3 * i + 2] = cb;
    }
}

enum BilateralPlane { B_COL = 0, B_NRM, B_ALB, B_COUNT };

__global__ void k_bilateral_records(const float* __restrict__ raw, const float* __restrict__ normal,
                                    const float* __restrict__ albedo, int64_t np, float4* __restrict__ rec) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    rec[B_COL * np + i] = make_float4(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2], 0.0f);
    rec[B_NRM * np + i] =
        unit_or_same(normal[3 * i] * 2.0f - 1.0f, normal[3 * i + 1] * 2.0f - 1.0f, normal[3 * i + 2] * 2.0f - 1.0f);
    rec[B_ALB * np + i] = make_float4(albedo[3 * i], albedo[3 * i + 1], albedo[3 * i + 2], 0.0f);
}

struct BilateralParams {
    int w, h, r;
    float kp, kc, kn, ka;   // 1 / (2 sigma^2) of the pixel-distance, colour, normal and albedo terms
};

constexpr int kBx = 32, kBy = 8;

// kTiled: the halo tile is in shared memory (one tensor copy); else the records are read from
// global memory (radius > 16).
template <bool kTiled>
__global__ void __launch_bounds__(kBx * kBy, 4)
    k_joint_bilateral(const float4* __restrict__ rec, BilateralParams prm, float* __restrict__ gaussian,
                      float* __restrict__ bilateral, float* __restrict__ joint, unsigned* fail,
                      const __grid_constant__ CUtensorMap tmap) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ int s_fail;
    const int r = prm.r;
    const int x0 = blockIdx.x * kBx, y0 = blockIdx.y * kBy;
    const int tid = threadIdx.y * kBx + threadIdx.x;
    const int tw = kBx + 2 * r, th = kBy + 2 * r;
    const int64_t np = int64_t(prm.w) * prm.h;
    const uint32_t pad = (128u - (smem_addr(smem_raw) & 127u)) & 127u;
    float4* T = reinterpret_cast<float4*>(smem_raw + pad);
    const int ntab = 2 * r * r + 1;  // squared distances 0 .. 2 r^2
    float* ep = reinterpret_cast<float*>(kTiled ? T + B_COUNT * tw * th : T);
    float* eg = ep + ntab;
    const uint32_t bar_a = smem_addr(&bar);
    if constexpr (kTiled) {
        if (tid == 0) {
            mbar_init(bar_a, 1);
            s_fail = 0;
        }
        __syncthreads();
        if (tid == 0) tile_load(T, &tmap, x0, y0, r, tw, th, B_COUNT, bar_a);
    }
    // weight_gauss = exp(-d / (2 sigma_p^2)) per squared distance d (joint_bilateral.cpp:100)
    for (int d = tid; d < ntab; d += kBx * kBy) {
        ep[d] = -float(d) * prm.kp;
        eg[d] = expf(ep[d]);
    }
    if constexpr (kTiled) {
        if (!mbar_wait_bounded(bar_a, 0)) s_fail = 1;
    }
    __syncthreads();
    if constexpr (kTiled) {
        if (s_fail) {
            if (tid == 0) {
                atomicAdd(fail, 1u);
                mbar_wait_bounded(bar_a, 0);
            }
            return;
        }
    }
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    // the tile origin, or the image itself when reading global records
    const int ox = kTiled ? x0 - r : 0, oy = kTiled ? y0 - r : 0;
    const int64_t stride = kTiled ? tw : prm.w;
    const int64_t plane = kTiled ? int64_t(tw) * th : np;
    const float4* S = kTiled ? T : rec;
    const int64_t ei = int64_t(y - oy) * stride + (x - ox);
    const float4 ci = S[B_COL * plane + ei], ni = S[B_NRM * plane + ei], ai = S[B_ALB * plane + ei];
    float g0 = 0.0f, g1 = 0.0f, g2 = 0.0f, gw = 0.0f;
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, cw = 0.0f;
    float j0 = 0.0f, j1 = 0.0f, j2 = 0.0f, jw = 0.0f;
    for (int dy = -r; dy <= r; ++dy) {
        const int cy = iclamps(y + dy, 0, prm.h - 1);  // joint_bilateral.cpp:60
        const int ddy = y - cy;
        const int64_t row = int64_t(cy - oy) * stride - ox;
#pragma unroll 4
        for (int dx = -r; dx <= r; ++dx) {
            const int cx = iclamps(x + dx, 0, prm.w - 1);
            const int ddx = x - cx;
            const int d = ddy * ddy + ddx * ddx;
            const int64_t e = row + cx;
            const float4 cj = S[B_COL * plane + e], nj = S[B_NRM * plane + e], aj = S[B_ALB * plane + e];
            const float r0 = ci.x - cj.x, r1 = ci.y - cj.y, r2 = ci.z - cj.z;
            const float dsc = (r0 * r0 + r1 * r1 + r2 * r2) * 0.5f;  // alpha = 0.5
            const float nv = acosf(fclamps(dot_lr(ni, nj), -1.0f, 1.0f));
            const float nv2 = nv * nv * 1.5f;                       // beta = 2 - alpha
            const float a0 = ai.x - aj.x, a1 = ai.y - aj.y, a2 = ai.z - aj.z;
            const float dsa = a0 * a0 + a1 * a1 + a2 * a2;
            const float wg = eg[d];
            const float ec = __fmaf_rn(-dsc, prm.kc, ep[d]);
            const float wc = __expf(ec);
            const float wj = __expf(__fmaf_rn(-dsa, prm.ka, __fmaf_rn(-nv2, prm.kn, ec)));
            g0 = __fmaf_rn(wg, cj.x, g0);
            g1 = __fmaf_rn(wg, cj.y, g1);
            g2 = __fmaf_rn(wg, cj.z, g2);
            gw += wg;
            c0 = __fmaf_rn(wc, cj.x, c0);
            c1 = __fmaf_rn(wc, cj.y, c1);
            c2 = __fmaf_rn(wc, cj.z, c2);
            cw += wc;
            j0 = __fmaf_rn(wj, cj.x, j0);
            j1 = __fmaf_rn(wj, cj.y, j1);
            j2 = __fmaf_rn(wj, cj.z, j2);
            jw += wj;
        }
    }
    const int64_t i = int64_t(y) * prm.w + x;
    gaussian[3 * i] = g0 / gw;
    gaussian[3 * i + 1] = g1 / gw;
    gaussian[3 * i + 2] = g2 / gw;
    bilateral[3 * i] = c0 / cw;
    bilateral[3 * i + 1] = c1 / cw;
    bilateral[3 * i + 2] = c2 / cw;
    joint[3 * i] = j0 / jw;
    joint[3 * i + 1] = j1 / jw;
    joint[3 * i + 2] = j2 / jw;
}

float inv_two_sq(float sigma) { return float(1.0 / (2.0 * double(sigma) * double(sigma))); }

}  // namespace

cudaError_t launch_atrous(const float* raw, const float* normal, const float* albedo, int w, int h, float sigma_c,
                          float sigma_n, float sigma_a, int iterations, float* buf_a, float* buf_b, float4* records,
                          float** result, cudaStream_t stream, uint64_t* launches) {
    const int64_t np = int64_t(w) * h;
    const dim3 block(32, 8);
    const dim3 grid((w + 31) / 32, (h + 7) / 8);
    float4* nrm = records;
    float4* alb = records ? records + np : nullptr;
    if (records && iterations > 0) {
        k_atrous_records<<<grid_for(np, 256), 256, 0, stream>>>(normal, albedo, np, nrm, alb);
        *launches += 1;
    }
    const float kc = inv_two_sq(sigma_c), kn = inv_two_sq(sigma_n), ka = inv_two_sq(sigma_a);
    const float* in = raw;
    float* out = buf_a;
    float* other = buf_b;
    *result = const_cast<float*>(raw);
    for (int it = 0; it < iterations; ++it) {
        if (records)
            k_atrous_pass<true><<<grid, block, 0, stream>>>(in, out, nrm, alb, nullptr, nullptr, w, h, 1 << it, kc, kn, ka);
        else
            k_atrous_pass<false><<<grid, block, 0, stream>>>(in, out, nullptr, nullptr, normal, albedo, w, h, 1 << it, kc,
                                                             kn, ka);
        *launches += 1;
        *result = out;
        in = out;
        float* t = out;
        out = other;
        other = t;
    }
    return cudaGetLastError();
}

uint64_t joint_bilateral_scratch_bytes(int w, int h) { return uint64_t(w) * h * B_COUNT * sizeof(float4) + 256; }

cudaError_t launch_joint_bilateral(const float* raw, const float* normal, const float* albedo, int w, int h,
                                   float sigma_c, float sigma_n, float sigma_p, float sigma_a, float* gaussian,
                                   float* bilateral, float* joint, void* scratch, cudaStream_t stream,
                                   uint64_t* launches) {
    const int64_t np = int64_t(w) * h;
    float4* rec = static_cast<float4*>(scratch);
    unsigned* fail = reinterpret_cast<unsigned*>(rec + B_COUNT * np);
    cudaError_t e = cudaMemsetAsync(fail, 0, sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    k_bilateral_records<<<grid_for(np, 256), 256, 0, stream>>>(raw, normal, albedo, np, rec);
    BilateralParams prm{};
    prm.w = w;
    prm.h = h;
    prm.r = std::max(1, int(std::ceil(3.0f * sigma_p)));  // joint_bilateral.cpp:43
    prm.kp = inv_two_sq(sigma_p);
    prm.kc = inv_two_sq(sigma_c);
    prm.kn = inv_two_sq(sigma_n);
    prm.ka = inv_two_sq(sigma_a);
    const dim3 block(kBx, kBy);
    const dim3 grid((w + kBx - 1) / kBx, (h + kBy - 1) / kBy);
    const size_t tables = size_t(2) * (2 * size_t(prm.r) * prm.r + 1) * sizeof(float);
    const bool tiled = prm.r <= 16;
    CUtensorMap map{};
    size_t smem = 128 + tables;
    if (tiled) {
        smem += size_t(kBx + 2 * prm.r) * (kBy + 2 * prm.r) * B_COUNT * sizeof(float4);
        e = encode_record_map(&map, rec, w, h, B_COUNT, kBx + 2 * prm.r, kBy + 2 * prm.r);
        if (e != cudaSuccess) return e;
    }
    if (smem > 48 * 1024) {
        e = tiled ? cudaFuncSetAttribute(k_joint_bilateral<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))
                  : cudaFuncSetAttribute(k_joint_bilateral<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem));
        if (e != cudaSuccess) return e;
    }
    if (tiled)
        k_joint_bilateral<true><<<grid, block, smem, stream>>>(rec, prm, gaussian, bilateral, joint, fail, map);
    else
        k_joint_bilateral<false><<<grid, block, smem, stream>>>(rec, prm, gaussian, bilateral, joint, fail, map);
    *launches += 2;
    return cudaGetLastError();
}

}  // namespace rpd
