"""rpd_job_push_samples_async / rpd_job_push_samples16_async: pushes of page-locked host planes
that return before their copies complete give the same bits as the synchronous host push, in one
band and in several, and with two jobs alternating as a frame stream drives them."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu

FIELDS = ["GRID", "STATS_MEAN", "DENOISED", "VARIANCE_DENOISED"]


class PinnedSamples(R.HostSamples):
    """A copy of host sample planes in page-locked memory (rpd_host_alloc)."""

    def __init__(self, src: "R.HostSamples"):
        super().__init__(src.n_samples, src.n_pixels, tuple(src.planes))
        self.bufs = []
        for name, arr in src.planes.items():
            buf = R.PinnedBuffer(max(1, arr.nbytes))
            view = buf.array(arr.dtype, arr.shape)
            view[...] = arr
            self.planes[name] = view
            self.bufs.append(buf)

    def free(self):
        for b in self.bufs:
            b.free()
        self.bufs = []


def denoise_async(job, samples, spp):
    job.begin_frame()
    job.push_async(samples, 0, job.cfg.image_width * job.cfg.image_height, spp)
    job.end_pass()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()
    job.sync()


@pytest.mark.parametrize("band_mb", [0, 1])
def test_async_host_push_matches_sync(gpu_ctx, band_mb):
    w, h, spp = 96, 64, 8
    cfg = small_config(w, h)
    host = B.synth_fill(R.synth_params(w, h, 29), 0, w * h, spp)
    pinned = PinnedSamples(host)
    g_sync = R.Job(gpu_ctx, cfg)
    g_async = R.Job(gpu_ctx, cfg)
    if band_mb:
        # bands of 1 MB on both: the push splits into several row bands (the grid's double-float
        # sums follow the bands, so both jobs use the same ones)
        g_sync.set_tuning("host_band_mb", band_mb)
        g_async.set_tuning("host_band_mb", band_mb)
    B.run_pipeline(g_sync, host, spp)
    denoise_async(g_async, pinned, spp)
    for f in FIELDS:
        assert_bitwise(g_async.read(f), g_sync.read(f), f)
    g_sync.close()
    g_async.close()
    pinned.free()


def test_async_host_push_alternating_jobs(gpu_ctx):
    """Two jobs, four frames from two sets of planes, each push enqueued before the other job's
    frame has finished: every frame matches its synchronous result."""
    w, h, spp = 64, 48, 4
    cfg = small_config(w, h)
    hosts = [B.synth_fill(R.synth_params(w, h, 31 + k), 0, w * h, spp) for k in range(2)]
    pinned = [PinnedSamples(hs) for hs in hosts]
    ref = []
    for hs in hosts:
        g = R.Job(gpu_ctx, cfg)
        B.run_pipeline(g, hs, spp)
        ref.append(g.read("DENOISED"))
        g.close()
    jobs = [R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)]
    for i in range(4):
        jb = jobs[i % 2]
        jb.sync()
        jb.begin_frame()
        jb.push_async(pinned[i % 2], 0, w * h, spp)
        jb.end_pass()
        jb.recompute_sensitivity()
        jb.statmc_denoise()
        jb.variance_denoise()
    for k, jb in enumerate(jobs):
        jb.sync()
        assert_bitwise(jb.read("DENOISED"), ref[k], f"job {k}")
        jb.close()
    for p in pinned:
        p.free()
