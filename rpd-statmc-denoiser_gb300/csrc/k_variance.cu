// variance_denoise (main.cpp:1166-1268): Jacobi iterations of the gated neighbour mean
// with the upward-only update, ping-ponging two planes, then max with the raw variance.
// Single precision throughout, in the reference's order, so the result is bit-identical.
//
// The ping-pong planes carry the hit test in their sign: a pixel with a primary hit holds its
// variance (>= EPS_SMALL), a pixel without one the negated clamped variance, which the
// iterations copy unchanged (main.cpp:1198-1201) and the final max with the clamped raw
// variance turns back into the value the reference keeps. A block's halo tile is then the
// plane's box as it lies in HBM — the tensor copy's zero fill past the image edges reads as
// "no neighbour" like a pixel without a hit — so each iteration stages its tile with one
// tiled tensor copy (cp.async.bulk.tensor) instead of per-thread gathers, and the gate records
// (unit normal, depth) with a second one. Rows of the ping-pong planes are padded to 4 floats,
// the 16-byte row pitch tensor copies need.
#include "rpd_internal.h"
#include "device_math.cuh"
#include "tma.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ float pixel_variance(float m2, int n) { return (n > 1) ? m2 / float(n - 1) : 0.0f; }

inline int var_pitch(int w) { return (w + 3) & ~3; }

// The clamped variance (main.cpp:1182-1186), negated for a pixel without a primary hit; the
// pixel's gate record.
__global__ void k_var_init(PixelPlanes p, int w, int h, int pitch, float max_variance, float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(w) * h) return;
    float v = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(v)) v = 1e-8f;
    v = fclamps(v, 1e-8f, max_variance);
    const bool hit = p.hit_count[i] > 0;
    const int64_t y = i / w, x = i - y * w;
    curr[y * pitch + x] = hit ? v : -v;
    p.var_gate[i] = make_float4(p.f_normal[0][i], p.f_normal[1][i], p.f_normal[2][i], p.f_depth[i]);
}

struct VarParams {
    int w, h, radius, pitch;
    float normal_threshold, depth_threshold, compat_sigma, shrinkage_k;
};

// rpf::conservative_variance_update (core/stats.h:85-91)
__device__ __forceinline__ float conservative_variance_update(float value, float neighbor, float stabilizer) {
    const float blend = fclamps(fmaxs(0.0f, neighbor - value) / fmaxs(1e-8f, value + neighbor + stabilizer), 0.0f, 1.0f);
    return lerp_std(value, neighbor, blend);
}

constexpr int kVarTx = 32, kVarTy = 16;
constexpr float kGateBand = 1.0f / 1048576.0f;  // 2^-20
constexpr int kVarPad = 4;  // the variance box starts 4 floats left of the block (a 16-byte boundary)

// The depth gate relative_depth_delta(d_i, d_j) > threshold (main.cpp:266-268): fl(num / m)
// against the threshold, decided by the product threshold * m away from it and by the IEEE
// quotient near it.
__device__ __forceinline__ bool depth_far(float dabs_i, float di, float dj, float dthr) {
    float m = dabs_i;
    if (m < fabsf(dj)) m = fabsf(dj);
    if (m < 1e-8f) m = 1e-8f;
    const float num = fabsf(di - dj);
    const float tm = dthr * m;
    const bool d_hi = num > tm * (1.0f + kGateBand), d_lo = num < tm * (1.0f - kGateBand);
    if (tm >= 1e-30f && (d_hi || d_lo)) return d_hi;
    return num / m > dthr;
}

// |var_i - var_j| / max(EPS_SMALL, sqrt(var_i * var_j)) > compat_sigma (main.cpp:1228-1232),
// by a reciprocal square root away from the threshold and the IEEE quotient near it.
__device__ __forceinline__ bool incompatible(float var_i, float var_j, float sigma) {
    const float diff = fabsf(var_i - var_j);
    const float prod = var_i * var_j;
    const float approx = diff * rsqrtf(prod);
    if (fabsf(approx - sigma) > sigma * kGateBand && prod >= 1e-16f && prod < 1e36f) return approx > sigma;
    return diff / fmaxs(1e-8f, sqrtf(prod)) > sigma;
}

// One Jacobi iteration (main.cpp:1198-1249) with the radius fixed at compile time. A 32 x 16
// block's halo tile arrives by tensor copies: the variance box (the 4-float-aligned
// (32 + 8) x (16 + 2R) floats) and, unless MODE 2, the gate records' (32 + 2R) x (16 + 2R) box.
// The window is unrolled, every gate is evaluated as a predicate (the lanes of a warp stay
// converged; the quotient gates branch only within the bands of their thresholds), and the
// accepted neighbours are added in the reference's order; a rejected neighbour adds nothing, as
// the reference's `continue` does.
//
// The hit, normal and depth gates depend on the features only, which the iterations do not
// change. MODE 0 evaluates every gate; MODE 1 also writes each pixel's geometric-gate bits (one
// per neighbour, in window order) to var_mask; MODE 2 reads them and evaluates only the
// variance-compatibility gate of the neighbours they pass.
template <int R, int MODE>
__global__ void __launch_bounds__(kVarTx * kVarTy)
    k_var_smooth_r(PixelPlanes p, VarParams prm, float* dst, unsigned long long* timeouts,
                   const __grid_constant__ CUtensorMap gmap, const __grid_constant__ CUtensorMap vmap) {
    static_assert(R <= kVarPad, "the variance box covers a halo of at most 4 columns");
    static_assert(MODE == 0 || (2 * R + 1) * (2 * R + 1) - 1 <= 64, "the gate bits fit one word");
    constexpr int gw = kVarTx + 2 * R, vw = kVarTx + 2 * kVarPad, th = kVarTy + 2 * R;
    __shared__ __align__(128) float4 G[MODE == 2 ? 1 : gw * th];  // (unit normal, depth)
    __shared__ __align__(128) float V[vw * th];                   // the source plane's box
    __shared__ __align__(8) unsigned long long bar;
    __shared__ int s_fail;
    const int x0 = blockIdx.x * kVarTx, y0 = blockIdx.y * kVarTy;
    const int tid = threadIdx.y * kVarTx + threadIdx.x;
    const uint32_t bar_a = smem_addr(&bar);
    if (tid == 0) {
        mbar_init(bar_a, 1);
        s_fail = 0;
    }
    __syncthreads();
    if (tid == 0) {
        mbar_expect_tx(bar_a, uint32_t(vw * th * 4 + (MODE == 2 ? 0 : gw * th * 16)));
        tma_load_2d(smem_addr(V), &vmap, x0 - kVarPad, y0 - R, bar_a);
        if (MODE != 2) tma_load_3d(smem_addr(G), &gmap, 4 * (x0 - R), y0 - R, 0, bar_a);
    }
    if (!mbar_wait_bounded(bar_a, 0)) s_fail = 1;
    __syncthreads();
    if (s_fail) {  // report, and let the copies land (bounded) before the shared memory is released
        if (tid == 0) {
            atomicAdd(timeouts, 1ull);
            mbar_wait_bounded(bar_a, 0);
        }
        return;
    }
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t idx = int64_t(y) * prm.w + x;
    const int64_t pidx = int64_t(y) * prm.pitch + x;
    const int vi = (threadIdx.y + R) * vw + threadIdx.x + kVarPad;
    const float src_i = V[vi];
    if (!(src_i > 0.0f)) {  // no primary hit (hit_count == 0): copied unchanged
        dst[pidx] = src_i;
        return;
    }
    const float var_i = fmaxs(1e-8f, src_i);
    const float sigma = prm.compat_sigma;
    float weight_sum = 0.0f, weighted_sum = 0.0f;
    uint64_t gates = MODE == 2 ? p.var_mask[idx] : 0ull;
    float4 gi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int gi_e = (threadIdx.y + R) * gw + threadIdx.x + R;
    if (MODE != 2) gi = G[gi_e];
    const float dabs_i = fabsf(gi.w);
    int bit = 0;
#pragma unroll
    for (int dy = -R; dy <= R; ++dy) {
#pragma unroll
        for (int dx = -R; dx <= R; ++dx) {
            if (dx == 0 && dy == 0) continue;
            const float src_j = V[vi + dy * vw + dx];
            bool ok;
            if (MODE == 2) {
                ok = (gates >> bit) & 1ull;
            } else {
                // outside the image (zero fill) or no primary hit (negative)
                const float4 gj = G[gi_e + dy * gw + dx];
                ok = src_j > 0.0f && !(dot3(gi.x, gi.y, gi.z, gj.x, gj.y, gj.z) < prm.normal_threshold);
                ok = ok && !depth_far(dabs_i, gi.w, gj.w, prm.depth_threshold);
                if (MODE == 1 && ok) gates |= 1ull << bit;
            }
            ++bit;
            const float var_j = fmaxs(1e-8f, src_j);
            ok = ok && !incompatible(var_i, var_j, sigma);
            const float w_j = 1.0f / (1.0f + float(dx * dx + dy * dy));
            if (ok) {
                weighted_sum += w_j * var_j;
                weight_sum += w_j;
            }
        }
    }
    if (MODE == 1) p.var_mask[idx] = gates;
    float neighbor_mean = var_i;
    if (weight_sum > 1e-8f) neighbor_mean = weighted_sum / weight_sum;
    dst[pidx] = conservative_variance_update(var_i, neighbor_mean, prm.shrinkage_k);
}

// The same iteration for radii above 4 (the radius at run time): the halo is gathered by the
// threads into dynamic shared memory, the window loops at run time.
__global__ void __launch_bounds__(kVarTx * kVarTy) k_var_smooth(PixelPlanes p, VarParams prm, const float* src,
                                                                float* dst) {
    extern __shared__ float4 vsm[];
    const int r = prm.radius;
    const int tw = kVarTx + 2 * r, th = kVarTy + 2 * r, tn = tw * th;
    const int side = 2 * r + 1;
    float4* G = vsm;                                // (normal, depth)
    float* V = reinterpret_cast<float*>(vsm + tn);  // the source plane, 0 outside the image
    float* W = V + tn;                              // 1 / (1 + d^2)
    const int x0 = blockIdx.x * kVarTx, y0 = blockIdx.y * kVarTy;
    const int tid = threadIdx.y * kVarTx + threadIdx.x;
    for (int e = tid; e < side * side; e += kVarTx * kVarTy) {
        const int dx = e % side - r, dy = e / side - r;
        W[e] = 1.0f / (1.0f + float(dx * dx + dy * dy));
    }
    for (int e = tid; e < tn; e += kVarTx * kVarTy) {
        const int gx = x0 - r + e % tw, gy = y0 - r + e / tw;
        const bool inside = gx >= 0 && gx < prm.w && gy >= 0 && gy < prm.h;
        G[e] = inside ? p.var_gate[int64_t(gy) * prm.w + gx] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        V[e] = inside ? src[int64_t(gy) * prm.pitch + gx] : 0.0f;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t pidx = int64_t(y) * prm.pitch + x;
    const int ei = (threadIdx.y + r) * tw + threadIdx.x + r;
    const float src_i = V[ei];
    if (!(src_i > 0.0f)) {
        dst[pidx] = src_i;
        return;
    }
    const float4 gi = G[ei];
    const float var_i = fmaxs(1e-8f, src_i);
    const float dabs_i = fabsf(gi.w);
    float weight_sum = 0.0f, weighted_sum = 0.0f;
    for (int dy = -r; dy <= r; ++dy) {
        const int erow = ei + dy * tw;
        const float* wrow = W + (dy + r) * side + r;
        for (int dx = -r; dx <= r; ++dx) {
            if (dx == 0 && dy == 0) continue;
            const float src_j = V[erow + dx];
            if (!(src_j > 0.0f)) continue;  // outside the image or no primary hit
            const float4 gj = G[erow + dx];
            if (dot3(gi.x, gi.y, gi.z, gj.x, gj.y, gj.z) < prm.normal_threshold) continue;
            if (depth_far(dabs_i, gi.w, gj.w, prm.depth_threshold)) continue;
            const float var_j = fmaxs(1e-8f, src_j);
            if (incompatible(var_i, var_j, prm.compat_sigma)) continue;
            const float w_j = wrow[dx];
            weighted_sum += w_j * var_j;
            weight_sum += w_j;
        }
    }
    float neighbor_mean = var_i;
    if (weight_sum > 1e-8f) neighbor_mean = weighted_sum / weight_sum;
    dst[pidx] = conservative_variance_update(var_i, neighbor_mean, prm.shrinkage_k);
}

// Tensor maps of the gate records and the two ping-pong planes for halo radius R.
template <int R>
cudaError_t var_maps(Job& j, int pitch) {
    if (j.var_map_r == R) return cudaSuccess;
    CUtensorMap* m = reinterpret_cast<CUtensorMap*>(j.var_maps[0]);
    cudaError_t e = encode_record_map(m, j.p.var_gate, j.g.w, j.g.h, 1, kVarTx + 2 * R, kVarTy + 2 * R);
    if (e == cudaSuccess)
        e = encode_plane_map(reinterpret_cast<CUtensorMap*>(j.var_maps[1]), j.p.var_ping, j.g.w, j.g.h, pitch,
                             kVarTx + 2 * kVarPad, kVarTy + 2 * R);
    if (e == cudaSuccess)
        e = encode_plane_map(reinterpret_cast<CUtensorMap*>(j.var_maps[2]), j.p.var_pong, j.g.w, j.g.h, pitch,
                             kVarTx + 2 * kVarPad, kVarTy + 2 * R);
    if (e != cudaSuccess) return e;
    j.var_map_r = R;
    return cudaSuccess;
}

template <int R>
cudaError_t launch_smooth_r(Job& j, const VarParams& prm, float*& curr, float*& next, dim3 vgrid) {
    const cudaError_t e = var_maps<R>(j, prm.pitch);
    if (e != cudaSuccess) return e;
    CUtensorMap gmap, ping, pong;
    std::memcpy(&gmap, j.var_maps[0], sizeof(gmap));
    std::memcpy(&ping, j.var_maps[1], sizeof(ping));
    std::memcpy(&pong, j.var_maps[2], sizeof(pong));
    unsigned long long* timeouts = j.p.counters + RPD_COUNTER_DEVICE_WAIT_TIMEOUTS;
    const int iters = j.cfg.var_iterations;
    constexpr bool kMask = (2 * R + 1) * (2 * R + 1) - 1 <= 64;
    for (int it = 0; it < iters; ++it) {
        const CUtensorMap& vmap = curr == j.p.var_ping ? ping : pong;
        if (!kMask || iters == 1)
            k_var_smooth_r<R, 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, next, timeouts, gmap, vmap);
        else if (it == 0)
            k_var_smooth_r<R, kMask ? 1 : 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, next, timeouts,
                                                                                         gmap, vmap);
        else
            k_var_smooth_r<R, kMask ? 2 : 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, next, timeouts,
                                                                                         gmap, vmap);
        float* t = curr;
        curr = next;
        next = t;
    }
    return cudaGetLastError();
}

// max(iterated, clamped raw) (main.cpp:1252-1261); for a pixel without a hit the iterated plane
// holds the negated clamped raw variance, so the max is the clamped raw variance.
__global__ void k_var_final(PixelPlanes p, int w, int h, int pitch, float max_variance, const float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= int64_t(w) * h) return;
    float raw = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(raw)) raw = 1e-8f;
    raw = fclamps(raw, 1e-8f, max_variance);
    const int64_t y = i / w, x = i - y * w;
    p.variance_denoised[i] = fmaxs(curr[y * pitch + x], raw);
}

}  // namespace

cudaError_t launch_variance(Job& j) {
    KernelScope ks(j, RPD_KERNEL_VARIANCE);
    const int64_t np = j.g.np;
    const float max_variance = j.cfg.adaptive_sigma_max * j.cfg.adaptive_sigma_max;
    const int pitch = var_pitch(j.g.w);
    float* curr = j.p.var_ping;
    float* next = j.p.var_pong;
    k_var_init<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, j.g.w, j.g.h, pitch, max_variance, curr);
    VarParams prm{j.g.w, j.g.h, j.cfg.var_window_radius, pitch, j.cfg.var_normal_threshold, j.cfg.var_depth_threshold,
                  j.cfg.var_compat_sigma, j.cfg.var_shrinkage_k};
    const int r = prm.radius;
    const dim3 vgrid((j.g.w + kVarTx - 1) / kVarTx, (j.g.h + kVarTy - 1) / kVarTy);
    cudaError_t e = cudaSuccess;
    if (r >= 1 && r <= 4) {
        e = r == 1 ? launch_smooth_r<1>(j, prm, curr, next, vgrid)
          : r == 2 ? launch_smooth_r<2>(j, prm, curr, next, vgrid)
          : r == 3 ? launch_smooth_r<3>(j, prm, curr, next, vgrid)
                   : launch_smooth_r<4>(j, prm, curr, next, vgrid);
    } else {
        const size_t smem = size_t(kVarTx + 2 * r) * size_t(kVarTy + 2 * r) * (sizeof(float4) + sizeof(float)) +
                            size_t(2 * r + 1) * size_t(2 * r + 1) * sizeof(float);
        if (smem > size_t(200) * 1024) return cudaErrorInvalidValue;  // radius beyond the shared-memory tile
        e = cudaFuncSetAttribute(k_var_smooth, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        for (int it = 0; it < j.cfg.var_iterations && e == cudaSuccess; ++it) {
            k_var_smooth<<<vgrid, dim3(kVarTx, kVarTy), smem, j.stream>>>(j.p, prm, curr, next);
            float* t = curr;
            curr = next;
            next = t;
        }
    }
    if (e != cudaSuccess) return e;
    k_var_final<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, j.g.w, j.g.h, pitch, max_variance, curr);
    j.launches += 2 + j.cfg.var_iterations;
    return cudaGetLastError();
}

}  // namespace rpd
