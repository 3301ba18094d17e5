"""The parallel allocation of the adaptive counts (k_allocate.cu) against the oracle's
sequential allocation (main.cpp:1372-1438 restated in oracle/rpd_oracle.c): bit-identical
counts on importance maps built to stress each sequential chain — wide dynamic ranges that
cross many binades, values with few mantissa bits that produce rounding ties, heavy tails
that clip many pixels over several water-filling passes, zeros, constants and frames from
one chunk to a full 1080p frame. The one-thread kernel (RPD_TUNE_ALLOCATOR = 1) must agree
too, and the parallel kernel must report that it finished without handing over."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, small_config

pytestmark = pytest.mark.gpu


def importance_map(kind: str, n: int, rng: np.random.Generator) -> np.ndarray:
    if kind == "lognormal":
        return rng.lognormal(-1.0, 1.5, n).astype(np.float32)
    if kind == "ties":  # multiples of 2^-10: sums hit exact halves of the rounding grid
        return (rng.integers(0, 4096, n) / 1024.0).astype(np.float32)
    if kind == "binades":  # 1e-4 .. 1e4 across the frame
        return (10.0 ** rng.uniform(-4, 4, n)).astype(np.float32)
    if kind == "fireflies":  # 3 % of the pixels far above the rest: many clips, several passes
        v = rng.uniform(0.05, 0.2, n)
        hot = rng.random(n) < 0.03
        v[hot] *= rng.uniform(50, 500, hot.sum())
        return v.astype(np.float32)
    if kind == "zeros":
        v = rng.uniform(0.0, 1.0, n)
        v[rng.random(n) < 0.5] = 0.0
        return v.astype(np.float32)
    if kind == "constant":
        return np.full(n, 0.37, dtype=np.float32)
    if kind == "steps":  # long runs of equal values with jumps between them
        return np.repeat(rng.uniform(0.01, 3.0, n // 97 + 1), 97)[:n].astype(np.float32)
    raise ValueError(kind)


CASES = [
    # (w, h, kind, adaptive_spp, base, seed)
    (7, 5, "lognormal", 4, 1, 11),
    (64, 64, "ties", 4, 1, 12),
    (64, 64, "fireflies", 4, 0, 13),
    (300, 200, "lognormal", 4, 1, 14),
    (300, 200, "ties", 8, 2, 15),
    (300, 200, "binades", 4, 1, 16),
    (300, 200, "fireflies", 4, 1, 17),
    (300, 200, "zeros", 2, 0, 18),
    (300, 200, "constant", 4, 1, 19),
    (333, 211, "steps", 16, 3, 20),
    (1000, 700, "fireflies", 4, 1, 21),
    (1000, 700, "binades", 1, 0, 22),
    (1000, 700, "ties", 4, 1, 23),
]


@pytest.mark.parametrize("w,h,kind,spp,base,seed", CASES)
def test_parallel_allocation_matches_the_sequential_one(gpu_ctx, w, h, kind, spp, base, seed):
    rng = np.random.default_rng(seed)
    imp = importance_map(kind, w * h, rng)
    cfg = small_config(w, h, adaptive_spp=spp, adaptive_base_samples=base, seed=seed)
    want = B.port_allocate(imp, cfg)
    job = R.Job(gpu_ctx, cfg)
    try:
        got = job.adaptive_allocate(imp)
        st = job.allocator_stats()
        assert st["parallel_done"] == 1 and st["fallback"] == 0 and st["timeout"] == 0, st
        np.testing.assert_array_equal(got, want)
        assert int(got.sum()) <= spp * w * h
        job.set_tuning("allocator", 1)
        np.testing.assert_array_equal(job.adaptive_allocate(imp), want)
    finally:
        job.close()


def test_full_hd_allocation(gpu_ctx):
    w, h = 1920, 1080
    rng = np.random.default_rng(5)
    imp = importance_map("fireflies", w * h, rng) * importance_map("lognormal", w * h, rng)
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, seed=99)
    want = B.port_allocate(imp, cfg)
    job = R.Job(gpu_ctx, cfg)
    try:
        got = job.adaptive_allocate(imp)
        st = job.allocator_stats()
        assert st["parallel_done"] == 1 and st["fallback"] == 0, st
        assert st["passes"] >= 2  # the heavy tail needs more than one water-filling pass
        np.testing.assert_array_equal(got, want)
    finally:
        job.close()


@pytest.mark.parametrize("case", ["no_budget", "all_zero"])
def test_allocation_edge_cases(gpu_ctx, case):
    w, h = 96, 80
    imp = np.full(w * h, 0.5, dtype=np.float32) if case == "no_budget" else np.zeros(w * h, dtype=np.float32)
    base = 4 if case == "no_budget" else 1
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=base)
    job = R.Job(gpu_ctx, cfg)
    try:
        got = job.adaptive_allocate(imp)
        np.testing.assert_array_equal(got, np.full(w * h, base, dtype=np.int32))
        np.testing.assert_array_equal(got, B.port_allocate(imp, cfg))
    finally:
        job.close()


def test_negative_importance_goes_to_the_serial_kernel(gpu_ctx):
    """A map outside the method's assumptions (a negative value) is handed to the one-thread
    kernel, whose counts still equal the sequential ones."""
    w, h = 128, 96
    rng = np.random.default_rng(3)
    imp = rng.uniform(0.0, 1.0, w * h).astype(np.float32)
    imp[17] = -0.25
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1)
    job = R.Job(gpu_ctx, cfg)
    try:
        got = job.adaptive_allocate(imp)
        assert job.allocator_stats()["fallback"] == 1
        np.testing.assert_array_equal(got, B.port_allocate(imp, cfg))
    finally:
        job.close()


def test_pipeline_counts_match_the_oracle_with_both_allocators(gpu_ctx):
    """compute_adaptive_sample_counts end to end (importance from the frame's variances, the
    smoothing, the allocation) on a synthetic frame, parallel and serial."""
    w, h, spp = 160, 120, 8
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, adaptive_passes=1, seed=4321)
    params = R.synth_params(w, h, 77)
    host = B.synth_fill(params, 0, w * h, spp, threads=4)
    ref = B.OracleJob(cfg, threads=4)
    ref.begin_frame()
    ref.push(host, 0, w * h, spp)
    ref.end_pass()
    ref.recompute_sensitivity()
    ref.statmc_denoise()
    ref.variance_denoise()
    want = ref.compute_adaptive_sample_counts()
    ref.close()
    for allocator in (0, 1):
        job = R.Job(gpu_ctx, cfg)
        try:
            job.set_tuning("allocator", allocator)
            job.begin_frame()
            job.push(host, 0, w * h, spp)
            job.end_pass()
            job.recompute_sensitivity()
            job.statmc_denoise()
            job.variance_denoise()
            np.testing.assert_array_equal(job.compute_adaptive_sample_counts(), want)
        finally:
            job.close()


@pytest.mark.parametrize("blocks", [2, 7, 152])
@pytest.mark.parametrize("w,h,kind", [(300, 200, "ties"), (1000, 700, "fireflies"), (640, 360, "binades")])
def test_allocation_does_not_depend_on_the_launch_shape(gpu_ctx, blocks, w, h, kind):
    rng = np.random.default_rng(blocks * 1000 + w)
    imp = importance_map(kind, w * h, rng)
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, seed=blocks)
    job = R.Job(gpu_ctx, cfg)
    try:
        job.set_tuning("allocator", blocks)
        got = job.adaptive_allocate(imp)
        st = job.allocator_stats()
        assert st["parallel_done"] == 1 and st["fallback"] == 0, st
        np.testing.assert_array_equal(got, B.port_allocate(imp, cfg))
    finally:
        job.close()
