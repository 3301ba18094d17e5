"""The fast StatMC window's guard bands and its per-block loops.

The window evaluates each neighbour's Welch compatibility in single precision and hands a
pixel to its slow pass (one warp per pixel) when one of its decisions — q against 25 and
against 2 ln 20, df against the t-table switch, the df denominator against 1e-8 — lies within
the guard band (the neighbour's q is then recomputed in double, the reference's operations in
its order), or its weight sum lies within the band of the 1.1 test (the whole pixel in double). On
the synthetic frames the default band (2^-15) is rarely entered, so these cases widen it
(RPD_TUNE_WINDOW_GUARD down to 2^0, where most decisions are recomputed) and check that the
result stays within the plain-form bar of the oracle for every width, and that the rechecks
did fire.

The cases also reach each of the kernel's loops: every df of a block below the table switch
(n - 1 <= 15), every df at or above 31 (n - 1 >= 31, the normal quantile), and mixed blocks
(samples dropped as non-finite make n vary), for both t tables and the normal-quantile alpha,
with radius 2 (the generic-radius kernel) and 3, 5 and 7 (the fixed-radius kernels).
"""
from __future__ import annotations

import pytest

from conftest import B, R, small_config
from test_gpu_parity import check_pipeline

pytestmark = pytest.mark.gpu

CASES = [
    # w, h, spp, radius, alpha, nan_rate
    (70, 41, 7, 5, 0.05, 0.0),
    (64, 48, 16, 3, 0.01, 0.0),
    (45, 30, 40, 7, 0.05, 0.0),
    (33, 20, 33, 2, 0.01, 0.02),
    (52, 37, 24, 5, 0.1, 0.01),
    (40, 36, 12, 7, 0.1, 0.0),
]


@pytest.mark.parametrize("guard", [15, 6, 2, 0])
@pytest.mark.parametrize("w,h,spp,radius,alpha,nan_rate", CASES)
def test_guard_band_width(gpu_ctx, w, h, spp, radius, alpha, nan_rate, guard):
    cfg = small_config(w, h, color_window_radius=radius, color_compat_alpha=alpha)
    p = R.synth_params(w, h, 5 + spp, miss_regions=3, nan_rate=nan_rate)
    s = B.synth_fill(p, 0, w * h, spp)
    g = R.Job(gpu_ctx, cfg)
    g.set_tuning("window_guard", guard)
    o = B.OracleJob(cfg, threads=1)
    for job in (g, o):
        B.run_pipeline(job, s, spp)
    counters = g.counters()
    check_pipeline(g, o, exact_grid=False)
    assert counters["device_wait_timeouts"] == 0
    assert counters["window_slow_pixels"] <= w * h, counters
    if guard == 0:
        # a band as wide as the decision points themselves: most neighbour decisions were
        # recomputed in double, on most pixels
        assert counters["window_pair_rechecks"] > (w * h) // 4, counters
        assert counters["window_slow_pixels"] > (w * h) // 4, counters
    g.close()
    o.close()
