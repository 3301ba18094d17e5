"""The batched form: frames of uneven size and spp, one job each, captured into one CUDA graph
(rpd_batch) after the autotuner picked each frame class's launch shapes. Every frame's result
equals the same frame run alone with the same shapes (the graph replays the same kernels)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu

FRAMES = [(96, 64, 8), (64, 48, 4), (120, 72, 16), (64, 48, 4), (33, 29, 8)]


def test_batch_equals_frames_alone(gpu_ctx):
    jobs, planes, alone = [], [], []
    batch = R.Batch(gpu_ctx)
    try:
        for i, (w, h, spp) in enumerate(FRAMES):
            cfg = small_config(w, h, rpf_tile_size=16 if i % 2 == 0 else 8)
            dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
            gpu_ctx.synth_fill(R.synth_params(w, h, 100 + i), 0, w * h, spp, dev)
            dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
            dev.free()
            job = R.Job(gpu_ctx, cfg)
            job.autotune(dev16, spp)  # leaves the frame denoised with the chosen shapes
            alone.append({f: job.read(f) for f in ("DENOISED", "VARIANCE_DENOISED", "STATS_N", "GRID")})
            jobs.append(job)
            planes.append(dev16)
            batch.add(job, dev16, spp)
        assert jobs[1].get_tuning("grid_shape") == jobs[3].get_tuning("grid_shape")  # cached class
        for _ in range(3):
            batch.run()
        batch.sync()
        assert batch.last_ms() > 0.0
        assert batch.kernel_count() >= 10 * len(FRAMES)
        for job, ref in zip(jobs, alone):
            for f, v in ref.items():
                assert_bitwise(job.read(f), v, f)
    finally:
        batch.close()
        for j in jobs:
            j.close()
        for p in planes:
            p.free()


def test_batch_rejects_duplicate_job(gpu_ctx):
    w, h, spp = 32, 32, 4
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(R.synth_params(w, h, 7), 0, w * h, spp, dev)
    job = R.Job(gpu_ctx, small_config(w, h))
    batch = R.Batch(gpu_ctx)
    batch.add(job, dev, spp)
    with pytest.raises(R.RpdError, match="once"):
        batch.add(job, dev, spp)
    batch.close()
    job.close()
    dev.free()


def test_batched_frames_against_the_fp64_oracle(gpu_ctx):
    """Each frame of a batch (compact storage, autotuned shapes, one graph) against the
    double-precision restatement of the same frame (oracle/rpd_oracle64.c on the FP32 samples):
    relMSE = mean((x - r)^2 / (r^2 + 1e-2)) <= 1e-3, the precision form's bar."""
    from conftest import B

    frames = [(256, 256, 16), (160, 90, 4), (96, 64, 32)]
    jobs, planes, refs = [], [], []
    batch = R.Batch(gpu_ctx)
    try:
        for i, (w, h, spp) in enumerate(frames):
            cfg = small_config(w, h)
            p = R.synth_params(w, h, 500 + i)
            host = B.synth_fill(p, 0, w * h, spp, threads=8)
            refs.append(B.fp64_denoise(cfg, host, spp, threads=8).astype(np.float64))
            dev = R.DeviceSamples.from_host(gpu_ctx, host)
            dev16 = R.DeviceSamples16.encode(gpu_ctx, dev)
            dev.free()
            job = R.Job(gpu_ctx, cfg)
            job.autotune(dev16, spp)
            jobs.append(job)
            planes.append(dev16)
            batch.add(job, dev16, spp)
        batch.run()
        batch.sync()
        for job, r in zip(jobs, refs):
            x = job.read("DENOISED").astype(np.float64)
            err = float(np.mean((x - r) ** 2 / (r * r + 1e-2)))
            assert err <= 1e-3, err
    finally:
        batch.close()
        for j in jobs:
            j.close()
        for p in planes:
            p.free()
