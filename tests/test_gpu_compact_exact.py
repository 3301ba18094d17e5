"""The statistics pass on compact planes computes exactly what it computes on FP32 planes holding
the decoded values: the compact samples are decoded on the host the way the kernel decodes them
(radiance = half^2, normal = max(q / 32767, -1), depth = half * depth_scale, u = q / 65536) and
pushed as FP32 planes into a second job; every statistics plane, the hit and sample counts and
the grid must carry the same bits. This pins the compact kernel's shortcuts to the reference's
operations: the exact roots sqrt(half^2) = half, the seven quotients by the sample count from
one reciprocal (Markstein's correction), and the random-dimension bins q >> 14 - on the
vector paths (4, 8, 16 and 64 samples per pixel), the scalar path (5) and per-pixel counts."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu

STATS = ("STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
         "STATS_SQRT_SQUARE_DIFF", "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM",
         "DEPTH_SUM", "GRID")


def decode(dev16: "R.DeviceSamples16") -> "R.HostSamples":
    """The kernel's decoding of every compact plane, on the host in float32."""
    def get(name):
        comps, dt, per = R.PLANES16[name]
        n = dev16.n_samples if per == "sample" else dev16.n_pixels
        return np.stack([b.download(np.zeros(n, dtype=dt)) for b in dev16.bufs[name]])
    names = {"sqrt_radiance": "radiance", "normal": "normal", "depth": "depth", "pixel_albedo": "pixel_albedo",
             "pixel_u": "pixel_u", "lens_u": "lens_u", "brdf_u": "brdf_u", "light_u": "light_u", "env_u": "env_u",
             "flags": "flags", "category": "category"}
    hs = R.HostSamples(dev16.n_samples, dev16.n_pixels, tuple(names[n] for n in dev16.bufs))
    f32 = np.float32
    for name in dev16.bufs:
        q = get(name)
        if name == "sqrt_radiance":
            h = q.view(np.float16).astype(f32)
            v = np.abs(h) * np.abs(h)
        elif name == "normal":
            v = np.maximum(q.astype(f32) * (f32(1.0) / f32(32767.0)), f32(-1.0))
        elif name == "depth":
            v = q.view(np.float16).astype(f32) * f32(dev16.depth_scale)
        elif name == "pixel_albedo":
            v = q.view(np.float16).astype(f32)
        elif name in ("flags", "category"):
            v = q
        else:
            v = q.astype(f32) * f32(1.0 / 65536.0)
        dst = hs.planes[names[name]]
        dst[...] = v.reshape(dst.shape)
    return hs


@pytest.mark.parametrize("spp", [4, 8, 16, 64, 5])
def test_compact_statistics_equal_the_decoded_fp32_ones(gpu_ctx, spp):
    w, h = 72, 40
    cfg = small_config(w, h)
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(R.synth_params(w, h, 31 + spp), 0, w * h, spp, dev)
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev, depth_scale=2.0)
    host = decode(dev16)
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    try:
        for job, s in ((a, host), (b, dev16)):
            job.begin_frame()
            job.push(s, 0, w * h, spp)
            job.end_pass()
        for f in STATS:
            assert_bitwise(a.read(f), b.read(f), f)
    finally:
        a.close()
        b.close()
        dev16.free()
        dev.free()


def test_compact_statistics_with_per_pixel_counts(gpu_ctx):
    w, h = 64, 48
    cfg = small_config(w, h)
    rng = np.random.default_rng(8)
    counts = rng.integers(0, 12, w * h).astype(np.int32)
    n = int(counts.sum())
    dev = R.DeviceSamples(gpu_ctx, n, w * h)
    gpu_ctx.synth_fill(R.synth_params(w, h, 44), 0, w * h, 0, dev, counts=counts, start_n=np.zeros(w * h, np.int32))
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
    host = decode(dev16)
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    try:
        for job, s in ((a, host), (b, dev16)):
            job.begin_frame()
            job.push(s, 0, w * h, 0, counts=counts)
            job.end_pass()
        for f in STATS:
            assert_bitwise(a.read(f), b.read(f), f)
    finally:
        a.close()
        b.close()
        dev16.free()
        dev.free()
