"""The precision form: compact per-sample storage (rpd_sample_soa16: binary16 sqrt-radiance,
snorm16 normals, binary16 depth, unorm16 random dimensions), decoded and accumulated in
single precision. Its error is measured against the same frame pushed as FP32 planes (the
path the oracle pins), as relMSE = mean((x - r)^2 / (r^2 + 1e-2)) over pixels and channels;
the bar is 1e-3. The random-dimension bins are the unquantised ones, so their weights match
exactly."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu

REL_MSE_BAR = 1e-3
RANDOM_DEPS = [R.DEP_NAMES.index(n) for n in ("brdf", "lens", "light_uv", "light_select", "rr")]


def rel_mse(x, r):
    x = x.astype(np.float64)
    r = r.astype(np.float64)
    return float(np.mean((x - r) ** 2 / (r * r + 1e-2)))


def run(job, samples, w, h, spp):
    job.begin_frame()
    job.push(samples, 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()


@pytest.mark.parametrize("w,h,spp,tile", [(96, 64, 8, 16), (61, 37, 4, 8), (40, 30, 5, 6)])
def test_compact_storage_against_fp32(gpu_ctx, w, h, spp, tile):
    cfg = small_config(w, h, rpf_tile_size=tile)
    p = R.synth_params(w, h, 23)
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(p, 0, w * h, spp, dev)
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev, depth_scale=4.0)
    assert dev16.nbytes < 0.55 * dev.nbytes
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    run(a, dev, w, h, spp)
    run(b, dev16, w, h, spp)
    for f in ("STATS_N", "HIT_COUNT", "SAMPLE_COUNT"):
        assert_bitwise(a.read(f), b.read(f), f)
    err = rel_mse(b.read("DENOISED"), a.read("DENOISED"))
    assert err <= REL_MSE_BAR, err
    ga, gb = a.read("GRID"), b.read("GRID")
    for d in RANDOM_DEPS:  # bin weights of the random dimensions: identical bins, identical weights
        np.testing.assert_array_equal(ga[:, d, :16], gb[:, d, :16])
    for j in (a, b):
        j.close()
    dev.free()
    dev16.free()


def test_compact_adaptive_pass(gpu_ctx):
    w, h, spp = 48, 40, 4
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1)
    p = R.synth_params(w, h, 29)
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(p, 0, w * h, spp, dev)
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    run(a, dev, w, h, spp)
    run(b, dev16, w, h, spp)
    ca, cb = a.compute_adaptive_sample_counts(), b.compute_adaptive_sample_counts()
    assert ca.sum() == cb.sum() == cfg.adaptive_spp * w * h
    # the importance follows the stabilised variance, which moves by the storage error
    assert float(np.abs(ca - cb).sum()) <= 0.05 * ca.sum()
    extra_n = int(cb.sum())
    ex = R.DeviceSamples(gpu_ctx, extra_n, w * h)
    gpu_ctx.synth_fill(p, 0, w * h, 0, ex, counts=cb, start_n=np.full(w * h, spp, np.int32))
    ex16 = R.DeviceSamples16.encode(gpu_ctx, ex)
    # the same extra samples into both jobs: compact planes with per-pixel counts (b) against FP32
    # planes with the same counts (a)
    counts_dev = R.DeviceBuffer(gpu_ctx, cb.nbytes)
    counts_dev.upload(cb)
    a.push(ex, 0, w * h, 0, counts=counts_dev)
    b.push(ex16, 0, w * h, 0, counts=cb)
    for j in (a, b):
        j.end_pass()
        j.recompute_sensitivity()
        j.statmc_denoise()
    assert np.all(np.isfinite(b.read("DENOISED")))
    assert int(b.read("SAMPLE_COUNT").sum()) == w * h * spp + extra_n
    assert_bitwise(a.read("SAMPLE_COUNT"), b.read("SAMPLE_COUNT"), "SAMPLE_COUNT")
    assert rel_mse(b.read("DENOISED"), a.read("DENOISED")) <= REL_MSE_BAR
    counts_dev.free()
    for j in (a, b):
        j.close()
    for d in (dev, dev16, ex, ex16):
        d.free()


def test_compact_rejects_exact_grid(gpu_ctx):
    w, h, spp = 16, 16, 4
    cfg = small_config(w, h)
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(R.synth_params(w, h, 3), 0, w * h, spp, dev)
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
    job = R.Job(gpu_ctx, cfg)
    job.set_exact(grid=True, window=False)
    job.begin_frame()
    with pytest.raises(R.RpdError, match="exact grid mode"):
        job.push(dev16, 0, w * h, spp)
    job.close()
    dev.free()
    dev16.free()


@pytest.mark.parametrize("w,h,spp", [(256, 256, 4), (320, 180, 16)])
def test_forms_against_the_fp64_oracle(gpu_ctx, w, h, spp):
    """The plain FP32 path and the compact form against the double-precision restatement
    (oracle/rpd_oracle64.c): relMSE with epsilon 1e-2."""
    from conftest import B

    cfg = small_config(w, h)
    p = R.synth_params(w, h, 1234)
    host = B.synth_fill(p, 0, w * h, spp, threads=8)
    ref = B.fp64_denoise(cfg, host, spp, threads=8)
    dev = R.DeviceSamples.from_host(gpu_ctx, host)
    dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    try:
        run(a, dev, w, h, spp)
        run(b, dev16, w, h, spp)
        e32 = rel_mse(a.read("DENOISED"), ref)
        e16 = rel_mse(b.read("DENOISED"), ref)
        assert e32 <= 1e-6, e32
        assert e16 <= REL_MSE_BAR, e16
    finally:
        a.close()
        b.close()
        dev.free()
        dev16.free()


@pytest.mark.parametrize("w,h,spp", [(256, 256, 16), (640, 360, 4)])
def test_served_sequence_against_the_fp64_oracle(gpu_ctx, w, h, spp):
    """The serving workload's request (3 adaptive passes of 4 extra samples per pixel on
    average, floor 1) in compact storage, as the serving loop runs it — base pass, then per
    adaptive pass variance_denoise, the adaptive counts and the extra samples drawn for them
    (ordinals from p << 16), then recompute_sensitivity and statmc_denoise — against the
    double-precision restatement fed the same samples: relMSE <= 1e-3 (epsilon 1e-2)."""
    from conftest import B

    cfg = small_config(w, h, adaptive_passes=3, adaptive_spp=4, adaptive_base_samples=1,
                       color_normal_threshold=0.6, color_depth_threshold=0.2, color_compat_alpha=0.01,
                       color_sigma_max=4.0, var_normal_threshold=0.6, var_compat_sigma=3.0, var_shrinkage_k=0.7,
                       adaptive_sigma_max=4.0)
    n = w * h
    p = R.synth_params(w, h, 777)
    job = R.Job(gpu_ctx, cfg)
    bufs = []
    pushes = []
    try:
        dev = R.DeviceSamples(gpu_ctx, n * spp, n)
        bufs.append(dev)
        gpu_ctx.synth_fill(p, 0, n, spp, dev)
        dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
        bufs.append(dev16)
        job.begin_frame()
        job.push(dev16, 0, n, spp)
        job.end_pass()
        pushes.append((B.synth_fill(p, 0, n, spp, threads=8), spp, None))
        for k in range(1, cfg.adaptive_passes + 1):
            job.variance_denoise()
            counts = job.compute_adaptive_sample_counts()
            start = np.full(n, k << 16, dtype=np.int32)
            ex = R.DeviceSamples(gpu_ctx, int(counts.sum()), n)
            bufs.append(ex)
            gpu_ctx.synth_fill(p, 0, n, 0, ex, counts=counts, start_n=start)
            ex16 = R.DeviceSamples16.encode(gpu_ctx, ex)
            bufs.append(ex16)
            job.push(ex16, 0, n, 0, counts=counts)
            job.end_pass()
            pushes.append((B.synth_fill(p, 0, n, 0, counts=counts, start_n=start, threads=8), 0, counts))
        job.recompute_sensitivity()
        job.statmc_denoise()
        ref = B.fp64_sequence(cfg, pushes, threads=8)
        err = rel_mse(job.read("DENOISED"), ref)
        assert err <= REL_MSE_BAR, err
    finally:
        job.close()
        for b in bufs:
            b.free()
