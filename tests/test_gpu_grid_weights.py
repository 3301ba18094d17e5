"""The random-dimension grid pass picks 16-bit lane bin weights for a per-pixel-count push when the
push's largest count keeps every lane sum below 2^16. With counts in host memory the host knows
that count; with counts in device memory the offsets scan produces it on the device and both forms
are launched, each running only where it applies. Either way the grid is the same bits."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, small_config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("big", [0, 90, 300])
def test_count_push_device_counts_match_host_counts(gpu_ctx, big):
    # big 0: every count small (16-bit weights); 90: just above the largest count the 16-bit
    # weights allow at tile 16 (89); 300: far above it (32-bit weights)
    w, h = 64, 48
    n = w * h
    cfg = small_config(w, h)
    rng = np.random.default_rng(5 + big)
    counts = rng.integers(0, 7, n).astype(np.int32)
    if big:
        counts[n // 2 + 7] = big
    p = R.synth_params(w, h, 41)
    host = B.synth_fill(p, 0, n, 0, counts=counts)
    dev = R.DeviceSamples(gpu_ctx, int(counts.sum()), n)
    gpu_ctx.synth_fill(p, 0, n, 0, dev, counts=counts)
    dcounts = R.DeviceBuffer(gpu_ctx, counts.nbytes)
    dcounts.upload(counts)
    jobs = []
    for s, c in ((host, counts), (dev, dcounts)):
        g = R.Job(gpu_ctx, cfg)
        g.begin_frame()
        g.push(s, 0, n, 0, counts=c)
        g.end_pass()
        jobs.append(g)
    for f in ["GRID", "STATS_MEAN"]:
        assert_bitwise(jobs[1].read(f), jobs[0].read(f), f)
    for g in jobs:
        g.close()
    dcounts.free()
    dev.free()
