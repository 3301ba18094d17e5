"""The tracer-side emitter (rpd_emitter_*): per-sample records written row by row from several
host threads into page-locked ring buffers and streamed to the job band by band, against a
single push of the same samples, for a uniform first pass and an adaptive pass with the job's own
per-pixel counts (render_image_adaptive, main.cpp:1451-1538):
  * the pixel statistics and sums: bit for bit (each pixel's samples are accumulated in order);
  * the RPD grid: bit for bit in the exact grid mode (the reference's sequential order runs on
    across the bands); in the default double-float mode a node straddling two bands sums their
    contributions in another order, within the grid's bar (1e-9 of each dependency's largest sum);
  * the stage's outputs: within the plain-form bar (1e-4), bit for bit in the exact grid mode."""
from __future__ import annotations

import threading

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, max_rel_err, small_config
from test_gpu_parity import assert_grid_close

pytestmark = pytest.mark.gpu

STATS = ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN", "STATS_SQRT_SQUARE_DIFF",
         "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM", "DEPTH_SUM", "VARIANCE_DENOISED"]
OUTPUTS = ["DENOISED", "UNCERTAINTY", "ALPHA", "SENSITIVITY_CONFIDENCE"]


def compare(b, a, exact):
    for f in STATS:
        assert_bitwise(b.read(f), a.read(f), f)
    if exact:
        for f in ["GRID"] + OUTPUTS:
            assert_bitwise(b.read(f), a.read(f), f)
    else:
        assert_grid_close(b.read("GRID"), a.read("GRID"))
        for f in OUTPUTS:
            assert max_rel_err(b.read(f), a.read(f), 1e-3) <= 1e-4, f


def emit_pass(em, p, w, h, spp=0, counts=None, start=None, threads=4):
    """The render loop's rows from `threads` threads, handed out in increasing order."""
    em.begin_pass(spp, counts)
    rows = iter(range(h))
    lock = threading.Lock()
    errors = []

    def worker():
        try:
            while True:
                with lock:
                    y = next(rows, None)
                if y is None:
                    return
                c = None if counts is None else counts[y * w:(y + 1) * w]
                st = None if start is None else start[y * w:(y + 1) * w]
                em.write_row(y, B.synth_fill(p, y * w, w, spp, counts=c, start_n=st))
        except Exception as e:  # noqa: BLE001 (reported below)
            errors.append(e)

    ts = [threading.Thread(target=worker) for _ in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    em.end_pass()


@pytest.mark.parametrize("exact", [False, True], ids=["fast_grid", "exact_grid"])
@pytest.mark.parametrize("band_rows,slots", [(8, 2), (3, 4), (64, 2)])
def test_emitted_pass_equals_one_push(gpu_ctx, band_rows, slots, exact):
    w, h, spp = 96, 70, 8
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1)
    p = R.synth_params(w, h, 17, nan_rate=0.005, miss_regions=2)
    a, b = R.Job(gpu_ctx, cfg), R.Job(gpu_ctx, cfg)
    for j in (a, b):
        j.set_exact(grid=exact, window=False)
    em = R.Emitter(b, band_rows, slots, max_spp=48)
    try:
        a.begin_frame()
        a.push(B.synth_fill(p, 0, w * h, spp), 0, w * h, spp)
        a.end_pass()
        b.begin_frame()
        emit_pass(em, p, w, h, spp)
        for j in (a, b):
            j.recompute_sensitivity()
            j.statmc_denoise()
            j.variance_denoise()
        compare(b, a, exact)
        # an adaptive pass: the job's counts, samples drawn for them from ordinal spp on
        counts = a.compute_adaptive_sample_counts()
        if exact:
            assert np.array_equal(counts, b.compute_adaptive_sample_counts())
        else:
            b.compute_adaptive_sample_counts()  # the job's own counts may differ at a boundary; both trace `counts`
        start = np.full(w * h, spp, dtype=np.int32)
        a.push(B.synth_fill(p, 0, w * h, 0, counts=counts, start_n=start), 0, w * h, 0, counts=counts)
        a.end_pass()
        emit_pass(em, p, w, h, counts=counts, start=start)
        for j in (a, b):
            j.recompute_sensitivity()
            j.statmc_denoise()
            j.variance_denoise()
        compare(b, a, exact)
    finally:
        em.close()
        a.close()
        b.close()


def test_emitter_rejects_a_band_beyond_its_slots(gpu_ctx):
    w, h = 32, 16
    job = R.Job(gpu_ctx, small_config(w, h))
    em = R.Emitter(job, 4, 2, max_spp=4)
    try:
        job.begin_frame()
        with pytest.raises(R.RpdError, match="more than the emitter"):
            em.begin_pass(8)
        em.begin_pass(4)
        with pytest.raises(R.RpdError, match="not done"):
            em.end_pass()
    finally:
        em.close()
        job.close()
