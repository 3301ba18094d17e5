// rpd_atrous_wavelet_noalloc: the a-trous wavelet filter with its ping-pong scratch in a
// fixed device array of this translation unit instead of memory allocated per call.
//
// Callers that may not allocate device memory while they run (a host loop that has
// reserved all of its HBM up front, a thread that must not stall on the device-wide
// synchronisation cudaFree performs, an embedder whose allocator forbids library-internal
// allocations) use this entry point: every buffer it touches is either the caller's or
// the array below, which the CUDA runtime reserves when this module is first loaded on a
// device.
//
// The scratch holds one interleaved RGB FP32 image of at most RPD_NOALLOC_MAX_PIXELS
// pixels (2048 x 2048 = 48 MiB). Each pass of the filter writes every pixel of its
// destination before the next pass reads it, so nothing in the scratch needs clearing.
// There is one scratch per device: calls that overlap on the same device (two streams,
// or two host threads) race on it. The first call on a device looks the scratch address
// up (cudaGetSymbolAddress, which also loads this module) and should happen before any
// stream capture the caller runs.
#include <mutex>
#include <string>

#include "rpd_internal.h"

namespace {

__device__ __align__(256) float g_atrous_scratch[size_t(RPD_NOALLOC_MAX_PIXELS) * 3];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float* g_scratch_ptr[kMaxDevices] = {};

// Looks up this device's scratch address once; `device` is the caller's current device.
int scratch_for(int device, float** out) {
    if (device < 0 || device >= kMaxDevices)
        return rpd::fail(RPD_ERR_NO_DEVICE, "device ordinal " + std::to_string(device) + " out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_atrous_scratch);
        if (e != cudaSuccess) return rpd::cuda_fail(e, "cudaGetSymbolAddress(g_atrous_scratch)");
        g_scratch_ptr[device] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[device];
    return RPD_OK;
}

bool overlaps(const float* a, const float* b, size_t n) { return a < b + n && b < a + n; }

}  // namespace

extern "C" int rpd_atrous_wavelet_noalloc(const float* raw, const float* normal, const float* albedo, int32_t width,
                                          int32_t height, float sigma_c, float sigma_n, float sigma_a,
                                          int32_t iterations, float* out, void* stream) {
    using rpd::fail;
    if (!raw || !normal || !albedo || !out || width <= 0 || height <= 0 || iterations < 0)
        return fail(RPD_ERR_INVALID_ARGUMENT, "bad a-trous arguments");
    const int64_t pixels = int64_t(width) * height;
    if (pixels > RPD_NOALLOC_MAX_PIXELS)
        return fail(RPD_ERR_INVALID_ARGUMENT, "image of " + std::to_string(pixels) +
                                                  " pixels exceeds the no-allocation scratch of " +
                                                  std::to_string(RPD_NOALLOC_MAX_PIXELS) + " pixels");
    const size_t n = size_t(pixels) * 3;
    if (overlaps(out, raw, n) || overlaps(out, normal, n) || overlaps(out, albedo, n))
        return fail(RPD_ERR_INVALID_ARGUMENT, "out must not overlap raw, normal or albedo");
    int device = -1;
    RPD_CUDA(cudaGetDevice(&device));
    float* scratch = nullptr;
    const int st = scratch_for(device, &scratch);
    if (st != RPD_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (iterations == 0) {
        RPD_CUDA(cudaMemcpyAsync(out, raw, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        return RPD_OK;
    }
    // passes alternate between the two buffers starting with the first, so an odd count
    // ends in the first and an even count in the second: put `out` where the last pass lands
    float* first = (iterations & 1) ? out : scratch;
    float* second = (iterations & 1) ? scratch : out;
    float* result = nullptr;
    uint64_t launches = 0;
    // no records scratch: the passes renormalise each tap's normal from the caller's buffer
    RPD_CUDA(rpd::launch_atrous(raw, normal, albedo, width, height, sigma_c, sigma_n, sigma_a, iterations, first,
                                second, nullptr, &result, s, &launches));
    if (result != out) return fail(RPD_ERR_STATE, "a-trous passes did not end in the output buffer");
    return RPD_OK;
}
