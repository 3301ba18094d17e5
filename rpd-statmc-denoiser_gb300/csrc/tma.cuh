// Halo tiles staged by the tensor memory accelerator: one tiled tensor copy
// (cp.async.bulk.tensor) moves a block's whole box of per-pixel float4 records from HBM into
// shared memory and completes on an mbarrier the block waits on, with a bound.
//
// The records form a 3-D float tensor (4 W, H, planes): a row of W float4 records, H rows per
// plane, the planes one after the other. A box of (4 bw, bh, planes) floats starting at pixel
// (x, y) covers bw x bh pixels of every plane; its start column 4 x is a multiple of 4 floats
// (16 bytes) for any x, negative or past the edge, and the copy fills what lies outside the
// image with zeros. Everything here stays on this GPU (no cluster multicast).
#pragma once

#include <cuda.h>  // CUtensorMap and its encoding enums; the encoder comes from the driver at run time
#include <cuda_runtime.h>

#include <cstdint>

namespace rpd {

// ~1 s at GB300 clocks: a copy that has not landed by then is reported, not waited on forever
constexpr long long kTileWaitCycles = 1ll << 31;

__device__ __forceinline__ uint32_t smem_addr(const void* ptr) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier phase with a bound; false when the bound ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kTileWaitCycles) return false;
    return true;
}

// One tiled tensor copy global -> shared of the box at (c0, c1, c2), completing on `bar`.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// One tiled tensor copy global -> shared of the 2-D box at (c0, c1), completing on `bar`.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
        : "memory");
}

// The box of records around pixel (x0, y0) - (r, r): bw x bh pixels of every plane, into
// shared memory at `dst` (128-byte aligned), with `bar` expecting its bytes. One thread calls it.
__device__ __forceinline__ void tile_load(float4* dst, const CUtensorMap* map, int x0, int y0, int r, int bw, int bh,
                                          int planes, uint32_t bar) {
    mbar_expect_tx(bar, uint32_t(bw * bh * planes) * 16u);
    tma_load_3d(smem_addr(dst), map, 4 * (x0 - r), y0 - r, 0, bar);
}

// Host: the tensor map of `planes` planes of w x h float4 records starting at `base`, for
// boxes of bw x bh pixels (bw <= 64, bh <= 256). Returns cudaErrorNotSupported when the
// driver has no tensor-map encoder, cudaErrorInvalidValue when it rejects the layout.
cudaError_t encode_record_map(CUtensorMap* map, const void* base, int w, int h, int planes, int bw, int bh);
// Host: the tensor map of one w x h float plane with rows `pitch` floats apart (pitch a multiple
// of 4, so rows start 16 bytes apart), for boxes of bw x bh floats (bw a multiple of 4, <= 256).
// Columns from w to the pitch lie outside the tensor: a box reading them gets zeros.
cudaError_t encode_plane_map(CUtensorMap* map, const float* base, int w, int h, int pitch, int bw, int bh);

}  // namespace rpd
