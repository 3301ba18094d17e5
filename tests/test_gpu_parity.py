"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same inputs.

Bars, per stage:
  * pixel statistics, features and the variance stabilisation: bit-exact in every mode
    (the kernels perform the reference's IEEE operations in its order);
  * the RPD grid: bit-exact in the exact mode (the reference's single-thread order, so the
    oracle runs with one thread), and within 1e-9 relative of each dependency's largest
    sum in the default double-float mode;
  * stages that call expf / exp (prior smoothing, the StatMC weights, importance
    smoothing, the filters) and the single-precision StatMC window: the plain-form
    tolerance, max per-pixel relative error <= 1e-4 with a 1e-3 floor on |reference|
    (`max_rel_err`);
  * adaptive sample counts: bit-exact when the importance map is bit-exact.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, max_rel_err, small_config

pytestmark = pytest.mark.gpu

TOL = 1e-4
FLOOR = 1e-3

EXACT_FIELDS = ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
                "STATS_SQRT_SQUARE_DIFF", "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM",
                "DEPTH_SUM", "GRID"]
NODE_FIELDS = [f for f in R.FIELDS if f.startswith("NODE_")]
CLOSE_PIXEL_FIELDS = ["SENSITIVITY_CONFIDENCE", "SENSITIVITY_GRADIENT", "DENOISED", "UNCERTAINTY", "ALPHA",
                      "VAR_TOTAL_DEBUG", "VAR_EFF_DEBUG", "VAR_RATIO_DEBUG"]


def run_both(gpu_ctx, cfg, samples, spp, threads=1, exact=False):
    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=exact, window=exact)
    o = B.OracleJob(cfg, threads=threads)
    for job in (g, o):
        B.run_pipeline(job, samples, spp)
    return g, o


def assert_grid_close(x, y, rel=1e-9):
    scale = np.max(np.abs(y), axis=2, keepdims=True)
    err = np.abs(x - y) - rel * scale
    assert np.all(err <= 0.0), f"grid differs by {np.max(np.abs(x - y) / np.maximum(scale, 1e-300)):.3e} relative"


def check_pipeline(g, o, exact_grid=True):
    for f in EXACT_FIELDS:
        if f == "GRID" and not exact_grid:
            assert_grid_close(g.read(f), o.read(f))
            continue
        assert_bitwise(g.read(f), o.read(f), f)
    for f in NODE_FIELDS:
        x, y = g.read(f), o.read(f)
        assert np.max(np.abs(x - y)) <= 1e-5, f
    for f in CLOSE_PIXEL_FIELDS:
        x, y = g.read(f), o.read(f)
        err = max_rel_err(x, y, FLOOR) if f != "SENSITIVITY_GRADIENT" else float(np.max(np.abs(x - y)))
        assert err <= TOL, (f, err)
    # the variance stabilisation is single precision without exp: bit-exact
    assert_bitwise(g.read("VARIANCE_DENOISED"), o.read("VARIANCE_DENOISED"), "VARIANCE_DENOISED")
    # the window's sqrt variance: the reference's double 3x3 average, bit-exact
    assert_bitwise(g.read("SQRT_VARIANCE_STABLE"), o.read("SQRT_VARIANCE_STABLE"), "SQRT_VARIANCE_STABLE")


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
@pytest.mark.parametrize("w,h,spp,tile", [(37, 23, 5, 16), (64, 48, 8, 16), (33, 17, 4, 6), (16, 16, 3, 1),
                                          (70, 41, 7, 8), (45, 30, 9, 4)])
def test_synthetic_pipeline(gpu_ctx, w, h, spp, tile, exact):
    cfg = small_config(w, h, rpf_tile_size=tile)
    p = R.synth_params(w, h, 11, miss_regions=4, nan_rate=0.005)
    s = B.synth_fill(p, 0, w * h, spp)
    g, o = run_both(gpu_ctx, cfg, s, spp, exact=exact)
    check_pipeline(g, o, exact_grid=exact)
    g.close()
    o.close()


def test_default_knobs_and_alpha(gpu_ctx):
    # RenderConfig defaults: tile 8, colour radius 7, alpha 0.05 (t table), variance radius 1
    w, h, spp = 40, 30, 6
    cfg = R.default_config(image_width=w, image_height=h, seed=5)
    s = B.synth_fill(R.synth_params(w, h, 3), 0, w * h, spp)
    g, o = run_both(gpu_ctx, cfg, s, spp)
    check_pipeline(g, o, exact_grid=False)
    # an alpha outside the two tables takes the normal-quantile branch
    cfg2 = cfg.replace(color_compat_alpha=0.2)
    for job in (g, o):
        job.set_config(cfg2)
        job.statmc_denoise()
    assert max_rel_err(g.read("DENOISED"), o.read("DENOISED"), FLOOR) <= TOL


def test_rpd_disabled_matches(gpu_ctx):
    w, h, spp = 32, 24, 4
    cfg = small_config(w, h, rpf_shrinkage_scale=0.0)
    s = B.synth_fill(R.synth_params(w, h, 9), 0, w * h, spp)
    g, o = run_both(gpu_ctx, cfg, s, spp)
    check_pipeline(g, o, exact_grid=False)
    assert not np.any(g.read("SENSITIVITY_GRADIENT"))


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_chunked_pushes_equal_single_push(gpu_ctx, exact):
    """Pushing a pass in row bands gives the same result as one push (in the exact mode the
    same bits: the grid keeps the reference's sequential order across pushes)."""
    w, h, spp = 30, 20, 4
    cfg = small_config(w, h, rpf_tile_size=8)
    s = B.synth_fill(R.synth_params(w, h, 21), 0, w * h, spp)
    g1 = R.Job(gpu_ctx, cfg)
    g1.set_exact(grid=exact, window=exact)
    B.run_pipeline(g1, s, spp)
    g2 = R.Job(gpu_ctx, cfg)
    g2.set_exact(grid=exact, window=exact)
    g2.begin_frame()
    offsets = np.arange(w * h + 1) * spp
    for p0, p1 in [(0, 7), (7, 133), (133, 400), (400, w * h)]:
        g2.push(s.slice_pixels(offsets, p0, p1), p0, p1 - p0, spp)
    g2.end_pass()
    g2.recompute_sensitivity()
    g2.statmc_denoise()
    g2.variance_denoise()
    for f in ["STATS_MEAN", "VARIANCE_DENOISED"]:
        assert_bitwise(g1.read(f), g2.read(f), f)
    if exact:
        for f in ["GRID", "DENOISED", "NODE_ALL"]:
            assert_bitwise(g1.read(f), g2.read(f), f)
    else:
        assert_grid_close(g2.read("GRID"), g1.read("GRID"), rel=1e-12)
        assert max_rel_err(g2.read("DENOISED"), g1.read("DENOISED"), FLOOR) <= 1e-6


def test_ragged_counts_and_empty_pixels(gpu_ctx):
    w, h = 25, 19
    rng = np.random.default_rng(4)
    counts = rng.integers(0, 9, size=w * h).astype(np.int32)
    counts[::7] = 0
    cfg = small_config(w, h)
    s = B.synth_fill(R.synth_params(w, h, 8, miss_regions=2), 0, w * h, 0, counts=counts)
    g = R.Job(gpu_ctx, cfg)
    o = B.OracleJob(cfg, threads=1)
    for job in (g, o):
        job.begin_frame()
        job.push(s, 0, w * h, 0, counts=counts)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
    check_pipeline(g, o, exact_grid=False)


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_single_pixel_and_thin_images(gpu_ctx, exact):
    for w, h in [(1, 1), (1, 9), (7, 1), (2, 3)]:
        cfg = small_config(w, h, color_window_radius=2, var_window_radius=1)
        s = B.synth_fill(R.synth_params(w, h, 2), 0, w * h, 3)
        g, o = run_both(gpu_ctx, cfg, s, 3, exact=exact)
        check_pipeline(g, o, exact_grid=exact)
        g.close()


def test_adaptive_counts_bit_exact(gpu_ctx):
    w, h, spp = 48, 36, 4
    for radius in (0, 1, 2):
        cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, adaptive_importance_smoothing_radius=radius,
                           seed=77)
        s = B.synth_fill(R.synth_params(w, h, 13), 0, w * h, spp)
        g, o = run_both(gpu_ctx, cfg, s, spp, exact=True)
        cg = g.compute_adaptive_sample_counts()
        co = o.compute_adaptive_sample_counts()
        imp_g, imp_o = g.read("ADAPTIVE_IMPORTANCE"), o.read("ADAPTIVE_IMPORTANCE")
        if radius == 0:
            assert_bitwise(imp_g, imp_o, "importance")
        if np.array_equal(imp_g.view(np.uint32), imp_o.view(np.uint32)):
            assert np.array_equal(cg, co)
        else:
            # importance differs only through expf rounding in the smoothing weights
            assert max_rel_err(imp_g, imp_o, 1e-6) <= 1e-5
            assert int(np.abs(cg - co).sum()) <= 4
        assert cg.sum() == co.sum() == cfg.adaptive_spp * w * h
        assert cg.min() >= cfg.adaptive_base_samples
        assert cg.max() <= cfg.adaptive_base_samples + max(4, 8 * cfg.adaptive_spp) + 1


def test_adaptive_passes_sequence(gpu_ctx):
    """render()'s adaptive loop (main.cpp:1547-1552) with synthetic extra samples."""
    w, h, spp = 32, 24, 2
    cfg = small_config(w, h, adaptive_spp=4, adaptive_base_samples=1, adaptive_passes=2,
                       adaptive_importance_smoothing_radius=0)
    p = R.synth_params(w, h, 31)
    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=True, window=True)
    o = B.OracleJob(cfg, threads=1)
    s0 = B.synth_fill(p, 0, w * h, spp)
    for job in (g, o):
        job.begin_frame()
        job.push(s0, 0, w * h, spp)
        job.end_pass()
        job.recompute_sensitivity()
    for _ in range(cfg.adaptive_passes):
        cs = []
        for job in (g, o):
            job.statmc_denoise()
            job.variance_denoise()
            cs.append(job.compute_adaptive_sample_counts())
        assert np.array_equal(cs[0], cs[1])
        n = o.read("STATS_N").ravel()
        extra = B.synth_fill(p, 0, w * h, 0, counts=cs[1], start_n=n)
        for job in (g, o):
            job.push(extra, 0, w * h, 0, counts=cs[1])
            job.end_pass()
            job.recompute_sensitivity()
    for job in (g, o):
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
        job.finalize()
    check_pipeline(g, o)


def test_filters(gpu_ctx):
    rng = np.random.default_rng(1)
    h, w = 37, 53
    raw = rng.lognormal(-1.0, 0.8, size=(h, w, 3)).astype(np.float32)
    normal = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    albedo = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    out_g = gpu_ctx.atrous(raw, normal, albedo, 0.3, 0.2, 0.1, 5)
    out_o = np.empty_like(raw)
    B.port().orc_atrous_wavelet(raw.ctypes.data, normal.ctypes.data, albedo.ctypes.data, w, h, 0.3, 0.2, 0.1, 5,
                                out_o.ctypes.data, 1)
    assert max_rel_err(out_g, out_o, FLOOR) <= TOL
    gs = gpu_ctx.joint_bilateral(raw, normal, albedo, 0.3, 0.2, 2.0, 0.1)
    os_ = [np.empty_like(raw) for _ in range(3)]
    B.port().orc_joint_bilateral(raw.ctypes.data, normal.ctypes.data, albedo.ctypes.data, w, h, 0.3, 0.2, 2.0, 0.1,
                                 *[o.ctypes.data for o in os_], 1)
    for a, b in zip(gs, os_):
        assert max_rel_err(a, b, FLOOR) <= TOL


def test_device_resident_push_matches_host_push(gpu_ctx):
    w, h, spp = 40, 24, 4
    cfg = small_config(w, h)
    p = R.synth_params(w, h, 17)
    host = B.synth_fill(p, 0, w * h, spp)
    dev = R.DeviceSamples(gpu_ctx, w * h * spp, w * h)
    gpu_ctx.synth_fill(p, 0, w * h, spp, dev)
    g1 = R.Job(gpu_ctx, cfg)
    g2 = R.Job(gpu_ctx, cfg)
    B.run_pipeline(g1, host, spp)
    B.run_pipeline(g2, dev, spp)
    for f in ["GRID", "STATS_MEAN", "DENOISED", "VARIANCE_DENOISED"]:
        assert_bitwise(g1.read(f), g2.read(f), f)
    dev.free()


def test_plain_256x256_4spp(gpu_ctx):
    """The plain method at the size of the 256x256 / 4 spp cornell_box case, on synthetic
    samples, default (fast) mode against the oracle."""
    w, h, spp = 256, 256, 4
    cfg = small_config(w, h)
    s = B.synth_fill(R.synth_params(w, h, 1234, miss_regions=3), 0, w * h, spp)
    g, o = run_both(gpu_ctx, cfg, s, spp, threads=1)
    check_pipeline(g, o, exact_grid=False)


@pytest.mark.parametrize("shape", [1, 2, 3, 4, 5, 6])
def test_grid_launch_shapes_agree(gpu_ctx, shape):
    """Every launch shape of the random-dimension grid pass gives the oracle's grid (the
    shapes change only the order of the double-float sums)."""
    w, h, spp = 50, 34, 6
    cfg = small_config(w, h, rpf_tile_size=8)
    s = B.synth_fill(R.synth_params(w, h, 5, miss_regions=2), 0, w * h, spp)
    g = R.Job(gpu_ctx, cfg)
    g.set_tuning("grid_shape", shape)
    assert g.get_tuning("grid_shape") == shape
    o = B.OracleJob(cfg, threads=1)
    for job in (g, o):
        B.run_pipeline(job, s, spp)
    check_pipeline(g, o, exact_grid=False)
    g.close()
    o.close()


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_non_finite_features(gpu_ctx, exact):
    """NaN normals, infinite and NaN depths and NaN albedo in some pixels: every gate
    treats them as the reference's float comparisons do."""
    w, h, spp = 36, 28, 4
    cfg = small_config(w, h, var_window_radius=2)
    s = B.synth_fill(R.synth_params(w, h, 19, miss_regions=2), 0, w * h, spp)
    rng = np.random.default_rng(3)
    pix = rng.choice(w * h, size=40, replace=False)
    for i, px in enumerate(pix):
        k = slice(px * spp, (px + 1) * spp)
        if i % 4 == 0:
            s.planes["normal"][0][k] = np.nan
        elif i % 4 == 1:
            s.planes["depth"][k] = np.inf
        elif i % 4 == 2:
            s.planes["depth"][k] = np.nan
        else:
            s.planes["pixel_albedo"][1][px] = np.nan
    g, o = run_both(gpu_ctx, cfg, s, spp, exact=exact)
    check_pipeline(g, o, exact_grid=exact)
    g.close()
    o.close()


@pytest.mark.parametrize("counts_mode", [False, True], ids=["uniform", "counts"])
def test_banded_host_push_equals_device_push(gpu_ctx, counts_mode):
    """A host push copied in several row bands (each band's copy overlapping the previous
    band's passes) gives exactly the result of one device-resident push."""
    w, h, spp = 80, 60, 8
    cfg = small_config(w, h, rpf_tile_size=8)
    p = R.synth_params(w, h, 41, miss_regions=2)
    counts = None
    if counts_mode:
        counts = np.random.default_rng(5).integers(0, 12, size=w * h).astype(np.int32)
        host = B.synth_fill(p, 0, w * h, 0, counts=counts)
    else:
        host = B.synth_fill(p, 0, w * h, spp)
    dev = R.DeviceSamples.from_host(gpu_ctx, host)
    a = R.Job(gpu_ctx, cfg)
    a.set_tuning("host_band_mb", 1)  # 2.4 MB of planes: two bands
    b = R.Job(gpu_ctx, cfg)
    for job, src in ((a, host), (b, dev)):
        job.begin_frame()
        job.push(src, 0, w * h, 0 if counts_mode else spp, counts=counts)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
    for f in ["STATS_MEAN", "STATS_N", "RADIANCE_SUM", "VARIANCE_DENOISED", "GRID", "DENOISED"]:
        if f == "GRID":
            assert_grid_close(a.read(f), b.read(f), rel=1e-12)
        elif f == "DENOISED":
            assert max_rel_err(a.read(f), b.read(f), FLOOR) <= 1e-6
        else:
            assert_bitwise(a.read(f), b.read(f), f)
    a.close()
    b.close()
    dev.free()


@pytest.mark.parametrize("modes", [(False, True, False), (True, False, False), (False, False, True)],
                         ids=["fast-exact-fast", "exact-fast-fast", "fast-fast-exact"])
def test_grid_modes_across_passes(gpu_ctx, modes):
    """Three passes of one frame whose grid mode changes between passes, the first pushed in two
    row bands: in the double-float mode the pushes add their pairs straight into the frame grid
    (or into the pass grid when an exact pass has left the frame grid in doubles), the exact mode
    adds into the pass grid and merges. The frame grid stays within 1e-9 of the oracle's, and the
    node fields within their bar."""
    w, h, spp = 40, 36, 4
    cfg = small_config(w, h, rpf_tile_size=8)
    p = R.synth_params(w, h, 23, miss_regions=3)
    passes = [B.synth_fill(p, 0, w * h, spp, start_n=np.full(w * h, q << 16, dtype=np.int32)) for q in range(3)]
    offsets = np.arange(w * h + 1, dtype=np.int64) * spp
    g = R.Job(gpu_ctx, cfg)
    o = B.OracleJob(cfg, threads=1)
    for job in (g, o):
        job.begin_frame()
        for q, s in enumerate(passes):
            if job is g:
                g.set_exact(grid=modes[q], window=False)
            if q == 0:
                mid = (h // 2) * w
                job.push(s.slice_pixels(offsets, 0, mid), 0, mid, spp)
                job.push(s.slice_pixels(offsets, mid, w * h), mid, w * h - mid, spp)
            else:
                job.push(s, 0, w * h, spp)
            job.end_pass()
        job.recompute_sensitivity()
    assert_grid_close(g.read("GRID"), o.read("GRID"))
    for f in NODE_FIELDS:
        assert np.max(np.abs(g.read(f) - o.read(f))) <= 1e-5, f
    for f in ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N"]:
        assert_bitwise(g.read(f), o.read(f), f)
    g.close()
    o.close()
