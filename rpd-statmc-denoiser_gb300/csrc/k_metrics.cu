// Image-quality metrics on the GPU: what `eval_tools hdr-metrics <ref> <test>` reports
// (shared/tools/eval_tools.cpp:215-286 with compute_extended_metrics 121-213), in double
// precision like the reference, so a caller can score a denoised frame where it lies in HBM.
//
//   k_metrics_pixels   per pixel: |a-b|, (a-b)^2, a^2, the channel sums and the peaks of a and of
//                      log1p(max(0, luminance(a))); writes the two log-luminance planes. Each block
//                      reduces its grid-stride share; the block partials are summed in block order
//                      (deterministic, another order than the reference's sequential loop: the
//                      scalars agree to ~1e-14 relative).
//   k_metrics_rows     the 11-wide window sums (clipped at the image edges) of L_a, L_b, L_a^2,
//                      L_b^2 and L_a L_b along each row, a warp of threads sliding along 32-pixel
//                      segments (add the entering pixel, subtract the leaving one)
//   k_metrics_cols     the same down the columns over the row sums: each pixel's 11x11 box sums,
//                      from which its SSIM term (eval_tools.cpp:174-186); and per pixel the global
//                      SSIM's centred sums (232-270) and the log-gradient sums (194-210)
//   k_metrics_final    one block: the partials in block order and the formulas of the reference.
//
// The reference forms the box sums from integral images (differences of prefix sums); sliding
// sums give the same sums with less cancellation, within ~1e-12 of the reference's per-pixel
// terms.
#include <cmath>

#include "rpd_internal.h"

namespace rpd {

namespace {

constexpr int kMetricBlocks = 304;  // grid-stride blocks (2 per SM)
constexpr int kMetricThreads = 256;
constexpr int kSeg = 32;            // pixels per sliding segment
constexpr int kHalf = 5;            // the 11x11 window's half width

// per-block partial sums of pass 1
enum P1 { P1_SUM_SQ = 0, P1_SUM_ABS, P1_REF_E, P1_ERR_E, P1_MR0, P1_MR1, P1_MR2, P1_MT0, P1_MT1, P1_MT2, P1_N };
// per-block partial sums of pass 2
enum P2 { P2_VR0 = 0, P2_VR1, P2_VR2, P2_VT0, P2_VT1, P2_VT2, P2_CV0, P2_CV1, P2_CV2, P2_SSIM, P2_GERR, P2_GREF, P2_N };

struct Scalars {  // what pass 2 needs from pass 1
    double mean_ref[3], mean_tst[3], c1, c2;
};

__device__ __forceinline__ double dmax0(double a, double b) { return (a < b) ? b : a; }



template <int N>
__device__ void block_reduce(double (&v)[N], double* out) {
    __shared__ double sm[N][kMetricThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        double x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sm[k][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double s = 0.0;
        for (int wp = 0; wp < kMetricThreads / 32; ++wp) s += sm[threadIdx.x][wp];
        out[threadIdx.x] = s;
    }
}

__device__ void block_max2(double a, double b, double* out) {
    __shared__ double sm[2][kMetricThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a = dmax0(a, __shfl_down_sync(0xffffffffu, a, o));
        b = dmax0(b, __shfl_down_sync(0xffffffffu, b, o));
    }
    if (lane == 0) {
        sm[0][warp] = a;
        sm[1][warp] = b;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double m = 0.0;
        for (int wp = 0; wp < kMetricThreads / 32; ++wp) m = dmax0(m, sm[threadIdx.x][wp]);
        out[threadIdx.x] = m;
    }
}

__global__ void __launch_bounds__(kMetricThreads) k_metrics_pixels(Img3 ref, Img3 tst, int64_t np,
                                                                   double* __restrict__ lref, double* __restrict__ ltst,
                                                                   double* __restrict__ part, double* __restrict__ peaks) {
    double v[P1_N] = {};
    double peak = 0.0, log_peak = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < np; i += int64_t(gridDim.x) * blockDim.x) {
        double rl = 0.0, tl = 0.0;
        const double wgt[3] = {0.2126, 0.7152, 0.0722};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double a = ref.at(i, c), b = tst.at(i, c);
            const double d = a - b;
            v[P1_SUM_SQ] += d * d;
            v[P1_SUM_ABS] += fabs(d);
            v[P1_REF_E] += a * a;
            v[P1_ERR_E] += d * d;
            v[P1_MR0 + c] += a;
            v[P1_MT0 + c] += b;
            peak = dmax0(peak, fabs(a));
            rl += wgt[c] * a;
            tl += wgt[c] * b;
        }
        const double lr = log1p(dmax0(0.0, rl)), lt = log1p(dmax0(0.0, tl));
        lref[i] = lr;
        ltst[i] = lt;
        log_peak = dmax0(log_peak, lr);
    }
    block_reduce(v, part + size_t(blockIdx.x) * P1_N);
    block_max2(peak, log_peak, peaks + 2 * blockIdx.x);
}

__global__ void k_metrics_scalars(const double* __restrict__ part, const double* __restrict__ peaks, int64_t np,
                                  Scalars* out) {
    if (threadIdx.x != 0) return;
    double s[P1_N] = {};
    double peak = 0.0, log_peak = 0.0;
    for (int b = 0; b < kMetricBlocks; ++b) {
        for (int k = 0; k < P1_N; ++k) s[k] += part[b * P1_N + k];
        peak = dmax0(peak, peaks[2 * b]);
        log_peak = dmax0(log_peak, peaks[2 * b + 1]);
    }
    for (int c = 0; c < 3; ++c) {
        out->mean_ref[c] = s[P1_MR0 + c] / double(np);
        out->mean_tst[c] = s[P1_MT0 + c] / double(np);
    }
    log_peak = dmax0(1e-6, log_peak);
    out->c1 = pow(0.01 * log_peak, 2.0);
    out->c2 = pow(0.03 * log_peak, 2.0);
}

// Row window sums: R5[k][i] for k = L_a, L_b, L_a^2, L_b^2, L_a L_b.
__global__ void __launch_bounds__(kMetricThreads) k_metrics_rows(const double* __restrict__ lref,
                                                                 const double* __restrict__ ltst, int w, int h,
                                                                 double* __restrict__ rows) {
    const int segs = (w + kSeg - 1) / kSeg;
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= int64_t(segs) * h) return;
    const int y = int(t / segs), x0 = int(t % segs) * kSeg;
    const int64_t row = int64_t(y) * w;
    const int64_t np = int64_t(w) * h;
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int x = max(0, x0 - kHalf); x < min(w, x0 + kHalf + 1); ++x) {
        const double a = lref[row + x], b = ltst[row + x];
        s[0] += a;
        s[1] += b;
        s[2] += a * a;
        s[3] += b * b;
        s[4] += a * b;
    }
    const int x1 = min(w, x0 + kSeg);
    for (int x = x0; x < x1; ++x) {
        for (int k = 0; k < 5; ++k) rows[k * np + row + x] = s[k];
        const int in = x + kHalf + 1, out = x - kHalf;  // the window of x + 1 gains `in`, loses `out`
        if (in < w) {
            const double a = lref[row + in], b = ltst[row + in];
            s[0] += a;
            s[1] += b;
            s[2] += a * a;
            s[3] += b * b;
            s[4] += a * b;
        }
        if (out >= 0) {
            const double a = lref[row + out], b = ltst[row + out];
            s[0] -= a;
            s[1] -= b;
            s[2] -= a * a;
            s[3] -= b * b;
            s[4] -= a * b;
        }
    }
}

// Column window sums over the row sums, the SSIM term of each pixel, and the centred and
// gradient sums of its pixels; one thread per 32-row segment of a column.
__global__ void __launch_bounds__(kMetricThreads) k_metrics_cols(Img3 ref, Img3 tst,
                                                                 const double* __restrict__ lref,
                                                                 const double* __restrict__ ltst,
                                                                 const double* __restrict__ rows, int w, int h,
                                                                 const Scalars* __restrict__ sc,
                                                                 double* __restrict__ part) {
    double v[P2_N] = {};
    const int segs = (h + kSeg - 1) / kSeg;
    const int64_t np = int64_t(w) * h;
    const double c1 = sc->c1, c2 = sc->c2;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < int64_t(segs) * w;
         t += int64_t(gridDim.x) * blockDim.x) {
        const int x = int(t % w), y0 = int(t / w) * kSeg;
        double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int y = max(0, y0 - kHalf); y < min(h, y0 + kHalf + 1); ++y)
            for (int k = 0; k < 5; ++k) s[k] += rows[k * np + int64_t(y) * w + x];
        const int nx = min(w, x + kHalf + 1) - max(0, x - kHalf);
        const int y1 = min(h, y0 + kSeg);
        for (int y = y0; y < y1; ++y) {
            const int64_t i = int64_t(y) * w + x;
            const double n = double(nx * (min(h, y + kHalf + 1) - max(0, y - kHalf)));
            const double mr = s[0] / n, mt = s[1] / n;
            const double vr = dmax0(0.0, s[2] / n - mr * mr);
            const double vt = dmax0(0.0, s[3] / n - mt * mt);
            const double cv = s[4] / n - mr * mt;
            const double num = (2.0 * mr * mt + c1) * (2.0 * cv + c2);
            const double den = (mr * mr + mt * mt + c1) * (vr + vt + c2);
            v[P2_SSIM] += (den > 0.0) ? num / den : 1.0;
            // the global per-channel SSIM's centred sums
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double a = ref.at(i, c) - sc->mean_ref[c];
                const double b = tst.at(i, c) - sc->mean_tst[c];
                v[P2_VR0 + c] += a * a;
                v[P2_VT0 + c] += b * b;
                v[P2_CV0 + c] += a * b;
            }
            // forward differences of the log luminance
            if (x < w - 1 && y < h - 1) {
                const double rdx = lref[i + 1] - lref[i], rdy = lref[i + w] - lref[i];
                const double tdx = ltst[i + 1] - ltst[i], tdy = ltst[i + w] - ltst[i];
                v[P2_GERR] += (rdx - tdx) * (rdx - tdx) + (rdy - tdy) * (rdy - tdy);
                v[P2_GREF] += rdx * rdx + rdy * rdy;
            }
            const int in = y + kHalf + 1, out = y - kHalf;
            for (int k = 0; k < 5; ++k) {
                if (in < h) s[k] += rows[k * np + int64_t(in) * w + x];
                if (out >= 0) s[k] -= rows[k * np + int64_t(out) * w + x];
            }
        }
    }
    block_reduce(v, part + size_t(blockIdx.x) * P2_N);
}

__global__ void k_metrics_final(const double* __restrict__ p1, const double* __restrict__ peaks,
                                const double* __restrict__ p2, int64_t np, const Scalars* __restrict__ sc,
                                rpd_image_metrics* out) {
    if (threadIdx.x != 0) return;
    double s1[P1_N] = {}, s2[P2_N] = {};
    double peak = 0.0;
    for (int b = 0; b < kMetricBlocks; ++b) {
        for (int k = 0; k < P1_N; ++k) s1[k] += p1[b * P1_N + k];
        for (int k = 0; k < P2_N; ++k) s2[k] += p2[b * P2_N + k];
        peak = dmax0(peak, peaks[2 * b]);
    }
    if (peak <= 0.0) peak = 1.0;
    const double C1 = (0.01 * peak) * (0.01 * peak), C2 = (0.03 * peak) * (0.03 * peak);
    const double pixels = double(np);
    for (int c = 0; c < 3; ++c) {
        const double vr = s2[P2_VR0 + c] / pixels, vt = s2[P2_VT0 + c] / pixels, cv = s2[P2_CV0 + c] / pixels;
        const double mr = sc->mean_ref[c], mt = sc->mean_tst[c];
        const double num = (2.0 * mr * mt + C1) * (2.0 * cv + C2);
        const double den = (mr * mr + mt * mt + C1) * (vr + vt + C2);
        out->ssim[c] = (den > 0.0) ? num / den : 0.0;
    }
    out->ssim_mean = (out->ssim[0] + out->ssim[1] + out->ssim[2]) / 3.0;
    out->mae = s1[P1_SUM_ABS] / (pixels * 3.0);
    out->rmse = sqrt(s1[P1_SUM_SQ] / (pixels * 3.0));
    out->peak = peak;
    out->psnr = out->rmse > 0.0 ? 20.0 * log10(peak / out->rmse) : INFINITY;
    out->nrmse = sqrt(s1[P1_ERR_E] / dmax0(1e-18, s1[P1_REF_E]));
    out->log_ssim11 = s2[P2_SSIM] / pixels;
    out->log_gradient_nrmse = sqrt(s2[P2_GERR] / dmax0(1e-18, s2[P2_GREF]));
}

}  // namespace

uint64_t metrics_scratch_bytes(int w, int h) {
    const uint64_t np = uint64_t(w) * h;
    return np * 7 * sizeof(double) + kMetricBlocks * (P1_N + P2_N + 2) * sizeof(double) + sizeof(Scalars) + 256;
}

cudaError_t launch_metrics(const Img3& ref, const Img3& tst, int w, int h, void* scratch, rpd_image_metrics* d_out,
                           cudaStream_t stream) {
    const int64_t np = int64_t(w) * h;
    double* lref = static_cast<double*>(scratch);
    double* ltst = lref + np;
    double* rows = ltst + np;                   // 5 planes
    double* p1 = rows + 5 * np;
    double* peaks = p1 + kMetricBlocks * P1_N;
    double* p2 = peaks + 2 * kMetricBlocks;
    Scalars* sc = reinterpret_cast<Scalars*>(p2 + kMetricBlocks * P2_N);
    k_metrics_pixels<<<kMetricBlocks, kMetricThreads, 0, stream>>>(ref, tst, np, lref, ltst, p1, peaks);
    k_metrics_scalars<<<1, 32, 0, stream>>>(p1, peaks, np, sc);
    const int64_t row_threads = int64_t((w + kSeg - 1) / kSeg) * h;
    k_metrics_rows<<<grid_for(row_threads, kMetricThreads), kMetricThreads, 0, stream>>>(lref, ltst, w, h, rows);
    k_metrics_cols<<<kMetricBlocks, kMetricThreads, 0, stream>>>(ref, tst, lref, ltst, rows, w, h, sc, p2);
    k_metrics_final<<<1, 32, 0, stream>>>(p1, peaks, p2, np, sc, d_out);
    return cudaGetLastError();
}

}  // namespace rpd
