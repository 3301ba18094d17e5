// Host side of the halo-tile copies (tma.cuh): the tensor map of a record array.
#include "tma.cuh"

namespace rpd {

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver the runtime uses (no link against libcuda).
EncodeTiled encoder() {
    static const EncodeTiled fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<EncodeTiled>(f);
    }();
    return fn;
}

}  // namespace

cudaError_t encode_record_map(CUtensorMap* map, const void* base, int w, int h, int planes, int bw, int bh) {
    if (bw < 1 || bw > 64 || bh < 1 || bh > 256 || planes < 1 || planes > 256 || w < 1 || h < 1)
        return cudaErrorInvalidValue;
    const EncodeTiled fn = encoder();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t W = cuuint64_t(w), H = cuuint64_t(h);
    const cuuint64_t dims[3] = {4 * W, H, cuuint64_t(planes)};
    const cuuint64_t strides[2] = {16 * W, 16 * W * H};  // bytes between rows, between planes
    const cuuint32_t box[3] = {cuuint32_t(4 * bw), cuuint32_t(bh), cuuint32_t(planes)};
    const cuuint32_t estride[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, estride,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t encode_plane_map(CUtensorMap* map, const float* base, int w, int h, int pitch, int bw, int bh) {
    if (w < 1 || h < 1 || pitch < w || pitch % 4 || bw < 4 || bw > 256 || bw % 4 || bh < 1 || bh > 256)
        return cudaErrorInvalidValue;
    const EncodeTiled fn = encoder();
    if (!fn) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {cuuint64_t(w), cuuint64_t(h)};
    const cuuint64_t strides[1] = {cuuint64_t(pitch) * 4};
    const cuuint32_t box[2] = {cuuint32_t(bw), cuuint32_t(bh)};
    const cuuint32_t estride[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estride,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace rpd
