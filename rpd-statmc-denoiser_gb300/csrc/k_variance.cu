// variance_denoise (main.cpp:1166-1268): Jacobi iterations of the gated neighbour mean
// with the upward-only update, ping-ponging two planes, then max with the raw variance.
// Single precision throughout, in the reference's order, so the result is bit-identical.
#include "rpd_internal.h"
#include "device_math.cuh"

namespace rpd {

namespace {

__device__ __forceinline__ float pixel_variance(float m2, int n) { return (n > 1) ? m2 / float(n - 1) : 0.0f; }

__global__ void k_var_init(PixelPlanes p, int64_t np, float max_variance, float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float v = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(v)) v = 1e-8f;
    curr[i] = fclamps(v, 1e-8f, max_variance);
}

struct VarParams {
    int w, h, radius;
    float normal_threshold, depth_threshold, compat_sigma, shrinkage_k;
};

// rpf::conservative_variance_update (core/stats.h:85-91)
__device__ __forceinline__ float conservative_variance_update(float value, float neighbor, float stabilizer) {
    const float blend = fclamps(fmaxs(0.0f, neighbor - value) / fmaxs(1e-8f, value + neighbor + stabilizer), 0.0f, 1.0f);
    return lerp_std(value, neighbor, blend);
}

// One Jacobi iteration (main.cpp:1198-1249). A 32 x 8 block stages its (32+2r) x (8+2r) halo
// in shared memory: (unit normal, depth) as float4 and the current variance, -1 for pixels
// outside the image or without a primary hit (the reference's bounds and hit_count tests). The
// per-neighbour
// float operations are the reference's, in its order; the two quotient gates are decided by a
// product or a reciprocal square root away from their thresholds and by the IEEE quotient near
// them, and the spatial weights 1 / (1 + d^2) come from a table.
constexpr int kVarTx = 32, kVarTy = 16;
constexpr float kGateBand = 1.0f / 1048576.0f;  // 2^-20

__global__ void __launch_bounds__(kVarTx * kVarTy) k_var_smooth(PixelPlanes p, VarParams prm, const float* src,
                                                                float* dst) {
    extern __shared__ float4 vsm[];
    const int r = prm.radius;
    const int tw = kVarTx + 2 * r, th = kVarTy + 2 * r, tn = tw * th;
    const int side = 2 * r + 1;
    float4* G = vsm;                                          // (normal, depth)
    float* V = reinterpret_cast<float*>(vsm + tn);            // max(EPS_SMALL, src)
    float* W = V + tn;                                        // 1 / (1 + d^2)
    const int x0 = blockIdx.x * kVarTx, y0 = blockIdx.y * kVarTy;
    const int tid = threadIdx.y * kVarTx + threadIdx.x;
    for (int e = tid; e < side * side; e += kVarTx * kVarTy) {
        const int dx = e % side - r, dy = e / side - r;
        W[e] = 1.0f / (1.0f + float(dx * dx + dy * dy));
    }
    for (int e = tid; e < tn; e += kVarTx * kVarTy) {
        const int gx = x0 - r + e % tw, gy = y0 - r + e / tw;
        const bool inside = gx >= 0 && gx < prm.w && gy >= 0 && gy < prm.h;
        const int64_t q = inside ? int64_t(gy) * prm.w + gx : 0;
        const bool hit = inside && p.hit_count[q] > 0;
        G[e] = hit ? make_float4(p.f_normal[0][q], p.f_normal[1][q], p.f_normal[2][q], p.f_depth[q])
                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        V[e] = hit ? fmaxs(1e-8f, src[q]) : -1.0f;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t idx = int64_t(y) * prm.w + x;
    if (p.hit_count[idx] == 0) {
        dst[idx] = src[idx];
        return;
    }
    const int ei = (threadIdx.y + r) * tw + threadIdx.x + r;
    const float4 gi = G[ei];
    const float var_i = V[ei];
    const float dabs_i = fabsf(gi.w);
    const float dthr = prm.depth_threshold;
    float weight_sum = 0.0f, weighted_sum = 0.0f;
    for (int dy = -r; dy <= r; ++dy) {
        const int erow = ei + dy * tw;
        const float* wrow = W + (dy + r) * side + r;
        for (int dx = -r; dx <= r; ++dx) {
            if (dx == 0 && dy == 0) continue;
            const float var_j = V[erow + dx];
            if (var_j < 0.0f) continue;  // outside the image or no primary hit
            const float4 gj = G[erow + dx];
            if (dot3(gi.x, gi.y, gi.z, gj.x, gj.y, gj.z) < prm.normal_threshold) continue;
            // relative_depth_delta(depth_i, depth_j) > threshold (main.cpp:266-268)
            float m = dabs_i;
            if (m < fabsf(gj.w)) m = fabsf(gj.w);
            if (m < 1e-8f) m = 1e-8f;
            const float num = fabsf(gi.w - gj.w);
            const float tm = dthr * m;
            bool far;
            if (!(tm >= 1e-30f)) far = num / m > dthr;
            else if (num > tm * (1.0f + kGateBand)) far = true;
            else if (num < tm * (1.0f - kGateBand)) far = false;
            else far = num / m > dthr;
            if (far) continue;
            // |var_i - var_j| / max(EPS_SMALL, sqrt(var_i * var_j)) > compat_sigma
            const float diff = fabsf(var_i - var_j);
            const float prod = var_i * var_j;
            const float approx = diff * rsqrtf(prod);
            bool incompatible;
            if (fabsf(approx - prm.compat_sigma) > prm.compat_sigma * kGateBand && prod >= 1e-16f && prod < 1e36f)
                incompatible = approx > prm.compat_sigma;
            else
                incompatible = diff / fmaxs(1e-8f, sqrtf(prod)) > prm.compat_sigma;
            if (incompatible) continue;
            const float w_j = wrow[dx];
            weighted_sum += w_j * var_j;
            weight_sum += w_j;
        }
    }
    float neighbor_mean = var_i;
    if (weight_sum > 1e-8f) neighbor_mean = weighted_sum / weight_sum;
    dst[idx] = conservative_variance_update(var_i, neighbor_mean, prm.shrinkage_k);
}

// The same iteration with the radius fixed at compile time: the window is unrolled, every
// gate of a neighbour is evaluated as a predicate (the lanes of a warp stay converged; the
// quotient gates branch only for the rare values within the band of their thresholds), and
// the accepted neighbours are added in the reference's order. A rejected neighbour adds
// nothing, exactly as the reference's `continue` does.
//
// The hit, normal and depth gates depend on the features only, which the iterations do not
// change. MODE 0 evaluates every gate; MODE 1 also writes each pixel's geometric-gate bits (one
// per neighbour, in window order) to var_mask; MODE 2 reads them and evaluates only the
// variance-compatibility gate of the neighbours they pass.
template <int R, int MODE>
__global__ void __launch_bounds__(kVarTx * kVarTy) k_var_smooth_r(PixelPlanes p, VarParams prm, const float* src,
                                                                  float* dst) {
    static_assert(MODE == 0 || (2 * R + 1) * (2 * R + 1) - 1 <= 64, "the gate bits fit one word");
    constexpr int tw = kVarTx + 2 * R, th = kVarTy + 2 * R, tn = tw * th;
    __shared__ float4 G[MODE == 2 ? 1 : tn];  // (normal, depth)
    __shared__ float V[tn];                   // max(EPS_SMALL, src), -1 outside the image or without a hit
    const int x0 = blockIdx.x * kVarTx, y0 = blockIdx.y * kVarTy;
    const int tid = threadIdx.y * kVarTx + threadIdx.x;
    for (int e = tid; e < tn; e += kVarTx * kVarTy) {
        const int gx = x0 - R + e % tw, gy = y0 - R + e / tw;
        const bool inside = gx >= 0 && gx < prm.w && gy >= 0 && gy < prm.h;
        const int64_t q = inside ? int64_t(gy) * prm.w + gx : 0;
        const bool hit = inside && p.hit_count[q] > 0;
        if (MODE != 2)
            G[e] = hit ? make_float4(p.f_normal[0][q], p.f_normal[1][q], p.f_normal[2][q], p.f_depth[q])
                       : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        V[e] = hit ? fmaxs(1e-8f, src[q]) : -1.0f;
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= prm.w || y >= prm.h) return;
    const int64_t idx = int64_t(y) * prm.w + x;
    const int ei = (threadIdx.y + R) * tw + threadIdx.x + R;
    const float var_i = V[ei];
    if (var_i < 0.0f) {  // no primary hit (hit_count == 0)
        dst[idx] = src[idx];
        return;
    }
    const float sigma = prm.compat_sigma;
    const float sigma_band = sigma * kGateBand;
    float weight_sum = 0.0f, weighted_sum = 0.0f;
    uint64_t gates = MODE == 2 ? p.var_mask[idx] : 0ull;
    float4 gi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (MODE != 2) gi = G[ei];
    const float dabs_i = fabsf(gi.w);
    const float dthr = prm.depth_threshold;
    const float nthr = prm.normal_threshold;
    int bit = 0;
#pragma unroll
    for (int dy = -R; dy <= R; ++dy) {
#pragma unroll
        for (int dx = -R; dx <= R; ++dx) {
            if (dx == 0 && dy == 0) continue;
            const int e = ei + dy * tw + dx;
            const float var_j = V[e];
            bool ok;
            if (MODE == 2) {
                ok = (gates >> bit) & 1ull;
            } else {
                const float4 gj = G[e];
                ok = var_j >= 0.0f && !(dot3(gi.x, gi.y, gi.z, gj.x, gj.y, gj.z) < nthr);
                // relative_depth_delta(depth_i, depth_j) > threshold (main.cpp:266-268)
                float m = dabs_i;
                if (m < fabsf(gj.w)) m = fabsf(gj.w);
                if (m < 1e-8f) m = 1e-8f;
                const float num = fabsf(gi.w - gj.w);
                const float tm = dthr * m;
                const bool d_hi = num > tm * (1.0f + kGateBand), d_lo = num < tm * (1.0f - kGateBand);
                bool far = d_hi;
                if (ok && !(tm >= 1e-30f && (d_hi || d_lo))) far = num / m > dthr;
                ok = ok && !far;
                if (MODE == 1 && ok) gates |= 1ull << bit;
            }
            ++bit;
            // |var_i - var_j| / max(EPS_SMALL, sqrt(var_i * var_j)) > compat_sigma
            const float diff = fabsf(var_i - var_j);
            const float prod = var_i * var_j;
            const float approx = diff * rsqrtf(prod);
            bool incompatible = approx > sigma;
            if (ok && !(fabsf(approx - sigma) > sigma_band && prod >= 1e-16f && prod < 1e36f))
                incompatible = diff / fmaxs(1e-8f, sqrtf(prod)) > sigma;
            ok = ok && !incompatible;
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
    dst[idx] = conservative_variance_update(var_i, neighbor_mean, prm.shrinkage_k);
}

template <int R>
cudaError_t launch_smooth_r(Job& j, const VarParams& prm, float*& curr, float*& next, dim3 vgrid) {
    const int iters = j.cfg.var_iterations;
    constexpr bool kMask = (2 * R + 1) * (2 * R + 1) - 1 <= 64;
    for (int it = 0; it < iters; ++it) {
        if (!kMask || iters == 1)
            k_var_smooth_r<R, 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, curr, next);
        else if (it == 0)
            k_var_smooth_r<R, kMask ? 1 : 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, curr, next);
        else
            k_var_smooth_r<R, kMask ? 2 : 0><<<vgrid, dim3(kVarTx, kVarTy), 0, j.stream>>>(j.p, prm, curr, next);
        float* t = curr;
        curr = next;
        next = t;
    }
    return cudaGetLastError();
}

__global__ void k_var_final(PixelPlanes p, int64_t np, float max_variance, const float* curr) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    float raw = pixel_variance(p.square_diff[i], p.n[i]);
    if (!isfinite(raw)) raw = 1e-8f;
    raw = fclamps(raw, 1e-8f, max_variance);
    p.variance_denoised[i] = fmaxs(curr[i], raw);
}

}  // namespace

cudaError_t launch_variance(Job& j) {
    KernelScope ks(j, RPD_KERNEL_VARIANCE);
    const int64_t np = j.g.np;
    const float max_variance = j.cfg.adaptive_sigma_max * j.cfg.adaptive_sigma_max;
    float* curr = j.p.var_ping;
    float* next = j.p.var_pong;
    k_var_init<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, max_variance, curr);
    VarParams prm{j.g.w, j.g.h, j.cfg.var_window_radius, j.cfg.var_normal_threshold, j.cfg.var_depth_threshold,
                  j.cfg.var_compat_sigma, j.cfg.var_shrinkage_k};
    const int r = prm.radius;
    const dim3 vgrid((j.g.w + kVarTx - 1) / kVarTx, (j.g.h + kVarTy - 1) / kVarTy);
    if (r >= 1 && r <= 4) {
        cudaError_t e = r == 1 ? launch_smooth_r<1>(j, prm, curr, next, vgrid)
                      : r == 2 ? launch_smooth_r<2>(j, prm, curr, next, vgrid)
                      : r == 3 ? launch_smooth_r<3>(j, prm, curr, next, vgrid)
                               : launch_smooth_r<4>(j, prm, curr, next, vgrid);
        if (e != cudaSuccess) return e;
        k_var_final<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, max_variance, curr);
        j.launches += 2 + j.cfg.var_iterations;
        return cudaGetLastError();
    }
    const size_t smem = size_t(kVarTx + 2 * r) * size_t(kVarTy + 2 * r) * (sizeof(float4) + sizeof(float)) +
                        size_t(2 * r + 1) * size_t(2 * r + 1) * sizeof(float);
    if (smem > size_t(200) * 1024) return cudaErrorInvalidValue;  // radius beyond the shared-memory tile
    cudaError_t e = cudaFuncSetAttribute(k_var_smooth, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    for (int it = 0; it < j.cfg.var_iterations; ++it) {
        k_var_smooth<<<vgrid, dim3(kVarTx, kVarTy), smem, j.stream>>>(j.p, prm, curr, next);
        float* t = curr;
        curr = next;
        next = t;
    }
    k_var_final<<<grid_for(np, 256), 256, 0, j.stream>>>(j.p, np, max_variance, curr);
    j.launches += 2 + j.cfg.var_iterations;
    return cudaGetLastError();
}

}  // namespace rpd
