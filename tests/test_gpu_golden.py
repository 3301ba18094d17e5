"""GPU parity against the golden fixtures: the reference's own outputs, stored by
tests/golden/make_golden.py, so these checks need neither the oracle nor the reference on
the GPU machine.

Bars (the plain-form tolerances of test_gpu_parity.py):
  * pixel statistics, features, variance stabilisation: bit-exact;
  * the RPD grid: bit-exact in the exact mode, within 1e-9 of each dependency's largest sum
    in the double-float mode;
  * node sensitivities within 1e-5; exp-dependent pixel outputs within 1e-4 relative
    (floor 1e-3 on |reference|);
  * adaptive counts bit-exact when the importance map is, else sum-preserving and within 4
    samples in total (expf rounding in the importance smoothing).
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import B, R, assert_bitwise, golden_config, golden_samples, load_golden, max_rel_err, replay_adaptive

pytestmark = pytest.mark.gpu

TOL, FLOOR = 1e-4, 1e-3
EXACT = ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN", "STATS_SQRT_SQUARE_DIFF",
         "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM", "DEPTH_SUM", "VARIANCE_DENOISED"]
NODES = [f for f in R.FIELDS if f.startswith("NODE_")]
CLOSE = ["SENSITIVITY_CONFIDENCE", "DENOISED", "UNCERTAINTY", "ALPHA", "VAR_TOTAL_DEBUG", "VAR_EFF_DEBUG",
         "VAR_RATIO_DEBUG"]


def check_golden(job, a, exact):
    for f in EXACT:
        assert_bitwise(job.read(f), a["out_" + f], f)
    grid, ref = job.read("GRID"), a["out_GRID"]
    if exact:
        assert_bitwise(grid, ref, "GRID")
    else:
        scale = np.max(np.abs(ref), axis=2, keepdims=True)
        assert np.all(np.abs(grid - ref) <= 1e-9 * scale), "GRID"
    for f in NODES:
        assert np.max(np.abs(job.read(f) - a["out_" + f])) <= 1e-5, f
    for f in CLOSE:
        assert max_rel_err(job.read(f), a["out_" + f], FLOOR) <= TOL, f
    assert np.max(np.abs(job.read("SENSITIVITY_GRADIENT") - a["out_SENSITIVITY_GRADIENT"])) <= TOL


def check_counts(counts, importance, want_counts, want_importance):
    if np.array_equal(importance.view(np.uint32), want_importance.view(np.uint32)):
        assert np.array_equal(counts, want_counts)
    else:
        assert max_rel_err(importance, want_importance, 1e-6) <= 1e-5
        assert counts.sum() == want_counts.sum()
        assert int(np.abs(counts - want_counts).sum()) <= 4


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_cornell_golden(gpu_ctx, exact):
    meta, a = load_golden("cornell_48x48x4.npz")
    cfg = golden_config(meta)
    s = golden_samples(a, "s_", meta["planes"], cfg.image_width * cfg.image_height)
    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=exact, window=exact)
    B.run_pipeline(g, s, meta["spp"])
    check_golden(g, a, exact)
    counts = g.compute_adaptive_sample_counts()
    check_counts(counts, g.read("ADAPTIVE_IMPORTANCE"), a["counts"], a["out_ADAPTIVE_IMPORTANCE"])
    g.close()


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_cornell_256x256x4_golden(gpu_ctx, exact):
    """The plain-method cornell_box configuration at its own size: 256x256, 4 spp, seed 1234,
    samples traced by the reference, every stage output the reference's."""
    meta, a = load_golden("cornell_256x256x4.npz")
    cfg = golden_config(meta)
    assert (cfg.image_width, cfg.image_height, meta["spp"], cfg.seed) == (256, 256, 4, 1234)
    s = golden_samples(a, "s_", meta["planes"], cfg.image_width * cfg.image_height)
    for name, plane in s.planes.items():
        assert hashlib.sha256(np.ascontiguousarray(plane).tobytes()).hexdigest() == meta["sample_sha256"][name]
    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=exact, window=exact)
    B.run_pipeline(g, s, meta["spp"])
    check_golden(g, a, exact)
    g.close()


@pytest.mark.parametrize("exact", [True, False], ids=["exact", "fast"])
def test_cornell_adaptive_golden(gpu_ctx, exact):
    """render()'s adaptive loop with the reference's traced extra samples: each pass pushes
    the samples the reference drew for its own counts."""
    meta, a = load_golden("cornell_32x32_adaptive.npz")
    cfg = golden_config(meta)
    n = cfg.image_width * cfg.image_height

    def extra(p, counts):
        if p < 0:
            return golden_samples(a, "s_", meta["planes"], n), None
        return golden_samples(a, f"x{p}_", meta["planes"], n), a[f"counts{p}"]

    def on_counts(p, job, counts):
        check_counts(counts, job.read("ADAPTIVE_IMPORTANCE"), a[f"counts{p}"], a[f"importance{p}"])

    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=exact, window=exact)
    replay_adaptive(g, cfg, a, meta["spp"], extra, on_counts)
    check_golden(g, a, exact)
    g.close()


def test_synthetic_golden_with_device_generator(gpu_ctx):
    """Samples generated on the device match the pinned hashes, and the pipeline over them
    matches the reference's outputs."""
    meta, a = load_golden("synth_48x32x8.npz")
    cfg = golden_config(meta)
    n = cfg.image_width * cfg.image_height
    spp = meta["spp"]
    p = B.synth_from(meta["synth"])
    dev = R.DeviceSamples(gpu_ctx, n * spp, n)
    gpu_ctx.synth_fill(p, 0, n, spp, dev)
    for name, bufs in dev.bufs.items():
        comps, dt, per = R.PLANES[name]
        m = n * spp if per == "sample" else n
        host = np.stack([b.download(np.empty(m, dtype=dt)) for b in bufs]) if comps > 1 else \
            bufs[0].download(np.empty(m, dtype=dt))
        assert hashlib.sha256(host.tobytes()).hexdigest() == meta["sample_sha256"][name], name
    for exact in (True, False):
        g = R.Job(gpu_ctx, cfg)
        g.set_exact(grid=exact, window=exact)
        B.run_pipeline(g, dev, spp)
        check_golden(g, a, exact)
        g.close()
    dev.free()


def test_synthetic_adaptive_golden(gpu_ctx):
    meta, a = load_golden("synth_32x24_adaptive.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    p = B.synth_from(meta["synth"])
    state = {}

    def extra(q, counts):
        if q < 0:
            return B.synth_fill(p, 0, w * h, meta["spp"]), None
        # the extra samples the reference drew for its counts of this pass
        want = a[f"counts{q}"]
        return B.synth_fill(p, 0, w * h, 0, counts=want, start_n=state["n"]), want

    def on_counts(q, job, counts):
        check_counts(counts, job.read("ADAPTIVE_IMPORTANCE"), a[f"counts{q}"], a[f"importance{q}"])
        state["n"] = job.read("STATS_N").ravel()

    g = R.Job(gpu_ctx, cfg)
    g.set_exact(grid=True, window=True)
    replay_adaptive(g, cfg, a, meta["spp"], extra, on_counts)
    check_golden(g, a, True)
    g.close()


def test_filters_golden(gpu_ctx):
    meta, a = load_golden("filters_37x53.npz")
    out = gpu_ctx.atrous(a["raw"], a["normal"], a["albedo"], *meta["atrous"])
    assert max_rel_err(out, a["atrous"], FLOOR) <= TOL
    for got, name in zip(gpu_ctx.joint_bilateral(a["raw"], a["normal"], a["albedo"], *meta["joint"]),
                         ("gaussian", "bilateral", "joint")):
        assert max_rel_err(got, a[name], FLOOR) <= TOL, name
