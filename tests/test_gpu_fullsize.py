"""Parity at the benchmark's own frame: 1920x1080, 16 spp, the seeded synthetic samples and
the denoise knobs bench.py times (cornell.yaml's stage knobs, rpf tile 16, colour radius 5,
variance radius 3, 2 variance iterations), fast mode, against the oracle restatement run on
every host core.

The fast StatMC window decides its gates exactly and evaluates the Welch compatibility in
single precision, recomputing in double every neighbour whose q lies within 2^-15 of a
decision point and every pixel whose weight sum lies within 2^-16 of the blend's 1.1 test.
The chance that some decision escapes a band grows with the pixel count, so this frame —
25x the pixels of the next largest parity case — is checked with the plain-form bars of
test_gpu_parity.py, and the test reports how many decisions the bands sent to double.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import bench
from conftest import B, R, max_rel_err
from test_gpu_parity import FLOOR, TOL, check_pipeline

pytestmark = pytest.mark.gpu


def test_bench_frame_matches_oracle(gpu_ctx):
    threads = os.cpu_count() or 1
    cfg = bench.workload_config(R)
    w, h, spp = bench.W, bench.H, bench.SPP
    assert (cfg.image_width, cfg.image_height) == (1920, 1080) and spp == 16
    samples = B.synth_fill(R.synth_params(w, h, bench.SEED), 0, w * h, spp, threads=threads)
    g = R.Job(gpu_ctx, cfg)
    o = B.OracleJob(cfg, threads=threads)
    try:
        for job in (g, o):
            B.run_pipeline(job, samples, spp)
        counters = g.counters()
        check_pipeline(g, o, exact_grid=False)
        errs = {f: max_rel_err(g.read(f), o.read(f), FLOOR) for f in ("DENOISED", "UNCERTAINTY", "ALPHA")}
        print(f"1920x1080x16: max relative errors {errs}, rechecks {counters}")
        assert all(e <= TOL for e in errs.values()), errs
        # the recheck counters are reported, not required: on this frame the Welch q of no
        # neighbour falls within the guard bands (the bands' own parity is shown on the cases
        # of test_gpu_window_rechecks.py, where they fire)
        assert counters["device_wait_timeouts"] == 0, counters
    finally:
        g.close()
        o.close()
