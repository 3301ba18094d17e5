"""The adaptive importance smoothing (main.cpp:1331-1368) with its double-precision products
and sums carried out in integer instructions (the default) against the same kernel on the
double-precision instructions (RPD_TUNE_SMOOTHING = 1): identical bits of the smoothed
importance and identical counts, on synthetic frames of several sizes and radii, including
frames whose features make the weights exact small fractions (ties in the sums)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu


def smoothed(gpu_ctx, cfg, samples, spp, fp64):
    job = R.Job(gpu_ctx, cfg)
    try:
        job.set_tuning("smoothing", 1 if fp64 else 0)
        job.begin_frame()
        job.push(samples, 0, cfg.image_width * cfg.image_height, spp)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
        counts = job.compute_adaptive_sample_counts()
        return job.read("ADAPTIVE_IMPORTANCE"), counts
    finally:
        job.close()


@pytest.mark.parametrize("w,h,radius,seed", [(48, 36, 1, 3), (160, 120, 1, 4), (160, 120, 2, 5), (97, 61, 3, 6),
                                             (640, 360, 1, 7)])
def test_integer_smoothing_equals_double_precision(gpu_ctx, w, h, radius, seed):
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, adaptive_importance_smoothing_radius=radius,
                       seed=seed)
    s = B.synth_fill(R.synth_params(w, h, seed), 0, w * h, 4, threads=4)
    imp0, c0 = smoothed(gpu_ctx, cfg, s, 4, fp64=False)
    imp1, c1 = smoothed(gpu_ctx, cfg, s, 4, fp64=True)
    assert_bitwise(imp0, imp1, "smoothed importance")
    np.testing.assert_array_equal(c0, c1)


def test_flat_features_make_exact_weights(gpu_ctx):
    """One normal and one depth everywhere: the normal and depth weights are exactly 1, so each
    neighbour weight is 1 / (1 + d^2) and the sums meet exact ties of the rounding."""
    w, h, spp = 64, 48, 4
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, adaptive_importance_smoothing_radius=2)
    s = B.synth_fill(R.synth_params(w, h, 9), 0, w * h, spp, threads=4)
    for ch, v in ((0, 0.0), (1, 0.0), (2, 1.0)):
        s.planes["normal"][ch][:] = v
    s.planes["depth"][:] = 2.0
    imp0, c0 = smoothed(gpu_ctx, cfg, s, spp, fp64=False)
    imp1, c1 = smoothed(gpu_ctx, cfg, s, spp, fp64=True)
    assert_bitwise(imp0, imp1, "smoothed importance")
    np.testing.assert_array_equal(c0, c1)
