"""rpd_atrous_wavelet_noalloc: the a-trous filter with a fixed device scratch.

Collected last so that it also runs after every other GPU test in the same process. Two
calls in a row (different images, odd and even pass counts, so the scratch is reused with
the output landing in either ping-pong slot) are compared with rpd_atrous_wavelet, the
allocating entry point, which runs the same kernel.
"""
from __future__ import annotations

import numpy as np
import pytest

import rpd_gb300 as R

TOL = 1e-6  # same kernel, same inputs: the outputs agree to rounding


def _images(seed: int, h: int, w: int):
    rng = np.random.default_rng(seed)
    raw = rng.lognormal(-1.0, 0.8, size=(h, w, 3)).astype(np.float32)
    normal = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    albedo = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    return raw, normal, albedo


def _run_noalloc(ctx, stream, raw, normal, albedo, sigmas, iterations):
    h, w, _ = raw.shape
    bufs = [R.DeviceBuffer(ctx, raw.nbytes) for _ in range(4)]
    try:
        for b, a in zip(bufs, (raw, normal, albedo)):
            b.upload(a)
        R.atrous_noalloc(bufs[0], bufs[1], bufs[2], w, h, *sigmas, iterations, bufs[3], stream.cuda_stream)
        stream.synchronize()
        return bufs[3].download(np.empty_like(raw))
    finally:
        for b in bufs:
            b.free()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice(gpu_ctx):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    cases = [(11, 61, 97, (0.3, 0.2, 0.1), 5), (12, 128, 160, (0.5, 0.1, 0.2), 4)]
    for seed, h, w, sigmas, iterations in cases:
        raw, normal, albedo = _images(seed, h, w)
        want = gpu_ctx.atrous(raw, normal, albedo, *sigmas, iterations)
        got = _run_noalloc(gpu_ctx, stream, raw, normal, albedo, sigmas, iterations)
        err = np.max(np.abs(got.astype(np.float64) - want) / np.maximum(np.abs(want), 1e-3))
        assert err <= TOL, f"{h}x{w}, {iterations} passes: max relative error {err:.3e}"


@pytest.mark.gpu
def test_noalloc_zero_passes_copies_input(gpu_ctx):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    raw, normal, albedo = _images(13, 8, 24)
    got = _run_noalloc(gpu_ctx, stream, raw, normal, albedo, (0.3, 0.2, 0.1), 0)
    assert np.array_equal(got.view(np.uint32), raw.view(np.uint32))


@pytest.mark.gpu
def test_noalloc_rejects_images_beyond_the_scratch(gpu_ctx):
    buf = R.DeviceBuffer(gpu_ctx, 256)
    out = R.DeviceBuffer(gpu_ctx, 256)
    try:
        with pytest.raises(R.RpdError, match="exceeds the no-allocation scratch"):
            R.atrous_noalloc(buf, buf, buf, 2049, 2048, 0.3, 0.2, 0.1, 1, out)
    finally:
        buf.free()
        out.free()
