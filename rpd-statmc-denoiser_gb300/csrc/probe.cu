// FP32 issue-rate probe: the denominator of the window filters' roofline.
//
// Every thread of a grid that fills every SM (kBlocksPerSm blocks of kThreads per SM, 64
// resident warps) runs kChains independent chains of single-precision fused multiply-adds,
// so each warp scheduler always has an independent FFMA to issue. The count of FFMA lane
// instructions divided by the best CUDA-event time of `repeats` launches is the issue rate
// the FP32 pipes sustain at the clock the GPU runs at; nothing here changes a clock or power
// setting.
#include <cuda_runtime.h>

#include <string>

#include "rpd_internal.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;
constexpr int kIters = 16384;

__global__ void __launch_bounds__(kThreads) k_ffma_issue(float* sink, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = float(threadIdx.x + c) * 1e-3f;
    for (int i = 0; i < kIters; ++i) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = __fmaf_rn(x[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5f) sink[threadIdx.x] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int rpd_probe_fp32_issue(int device, int32_t repeats, double* per_second, double* ms) {
    using rpd::fail;
    if (!per_second || repeats <= 0) return fail(RPD_ERR_INVALID_ARGUMENT, "bad probe arguments");
    RPD_CUDA(cudaSetDevice(device));
    int sms = 0;
    RPD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    float* sink = nullptr;
    RPD_CUDA(cudaMalloc(&sink, kThreads * sizeof(float)));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float best = -1.0f;
    const unsigned blocks = unsigned(sms) * kBlocksPerSm;
    // one untimed launch first (module load, clocks leaving idle)
    for (int r = 0; r <= repeats && e == cudaSuccess; ++r) {
        e = cudaEventRecord(e0);
        if (e == cudaSuccess) {
            k_ffma_issue<<<blocks, kThreads>>>(sink, 0.999f, 1e-4f);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float t = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
        if (e == cudaSuccess && r > 0 && (best < 0.0f || t < best)) best = t;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return rpd::cuda_fail(e, "FP32 issue probe");
    const double lane_instr = double(blocks) * kThreads * double(kIters) * kChains;
    *per_second = lane_instr / (double(best) * 1e-3);
    if (ms) *ms = best;
    return RPD_OK;
}
