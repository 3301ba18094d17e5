"""The oracle pinned to the reference (CPU only).

  * the reference's own unit tests (path_tracer/tests/stats_test.cpp, config_test.cpp),
    compiled from its sources against the shims, pass;
  * the C restatement (oracle/rpd_oracle.c) reproduces every golden fixture bit for bit —
    the fixtures are the reference's own outputs (tests/golden/make_golden.py);
  * where the reference harness is built (oracle/_ref), the restatement also matches the
    live reference on seeded cases the fixtures do not cover.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import (B, GOLDEN, ROOT, R, assert_bitwise, golden_config, golden_samples, load_golden, replay_adaptive,
                      small_config)

REF_DIR = B.HERE / "_ref"
needs_ref = pytest.mark.skipif(not B.have_ref(), reason="reference harness (oracle/_ref) not built on this machine")

STAGE_FIELDS = ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
                "STATS_SQRT_SQUARE_DIFF", "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM",
                "DEPTH_SUM", "GRID"] + [f for f in R.FIELDS if f.startswith("NODE_")] + [
                "SENSITIVITY_CONFIDENCE", "SENSITIVITY_GRADIENT", "DENOISED", "UNCERTAINTY", "ALPHA",
                "VAR_TOTAL_DEBUG", "VAR_EFF_DEBUG", "VAR_RATIO_DEBUG", "VARIANCE_DENOISED"]


def assert_all_fields(job, arrays, prefix="out_"):
    for f in STAGE_FIELDS:
        assert_bitwise(job.read(f), arrays[prefix + f], f)


# ---- the reference's own unit tests ------------------------------------------------------

@needs_ref
@pytest.mark.parametrize("binary", ["stats_test", "config_test"])
def test_reference_unit_tests_pass(binary):
    exe = REF_DIR / binary
    if not exe.exists():
        pytest.skip(f"{binary} not built")
    args = [str(exe)]
    if binary == "config_test":
        # the test parses every YAML of the reference's config folder (its CTest argument)
        cfg_dir = Path(os.environ.get("REF_ROOT", ROOT.parent / "reference")) / "path_tracer" / "config"
        if not cfg_dir.is_dir():
            pytest.skip("reference config folder not present")
        args.append(str(cfg_dir))
    r = subprocess.run(args, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


# ---- restatement vs golden fixtures ------------------------------------------------------

def test_port_cornell_golden():
    meta, a = load_golden("cornell_48x48x4.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    s = golden_samples(a, "s_", meta["planes"], w * h)
    o = B.OracleJob(cfg, threads=1)
    B.run_pipeline(o, s, meta["spp"])
    assert_all_fields(o, a)
    assert np.array_equal(o.compute_adaptive_sample_counts(), a["counts"])
    assert_bitwise(o.read("ADAPTIVE_IMPORTANCE"), a["out_ADAPTIVE_IMPORTANCE"], "importance")
    o.close()


def test_port_cornell_256x256x4_golden():
    """The plain-method cornell_box configuration at its own size (256x256, 4 spp)."""
    meta, a = load_golden("cornell_256x256x4.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    s = golden_samples(a, "s_", meta["planes"], w * h)
    o = B.OracleJob(cfg, threads=1)
    B.run_pipeline(o, s, meta["spp"])
    assert_all_fields(o, a)
    o.close()


def test_port_cornell_adaptive_golden():
    meta, a = load_golden("cornell_32x32_adaptive.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    planes = meta["planes"]

    def extra(p, counts):
        if p < 0:
            return golden_samples(a, "s_", planes, w * h), None
        return golden_samples(a, f"x{p}_", planes, w * h), a[f"counts{p}"]

    def on_counts(p, job, counts):
        assert np.array_equal(counts, a[f"counts{p}"]), f"pass {p} counts"
        assert_bitwise(job.read("ADAPTIVE_IMPORTANCE"), a[f"importance{p}"], f"pass {p} importance")

    o = B.OracleJob(cfg, threads=1)
    replay_adaptive(o, cfg, a, meta["spp"], extra, on_counts)
    assert_all_fields(o, a)
    o.close()


def test_port_synthetic_golden_and_generator_pin():
    meta, a = load_golden("synth_48x32x8.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    s = B.synth_fill(B.synth_from(meta["synth"]), 0, w * h, meta["spp"])
    for k, v in s.planes.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == meta["sample_sha256"][k], k
    o = B.OracleJob(cfg, threads=1)
    B.run_pipeline(o, s, meta["spp"])
    assert_all_fields(o, a)
    assert np.array_equal(o.compute_adaptive_sample_counts(), a["counts"])
    o.close()


def test_port_synthetic_adaptive_golden():
    meta, a = load_golden("synth_32x24_adaptive.npz")
    cfg = golden_config(meta)
    w, h = cfg.image_width, cfg.image_height
    p = B.synth_from(meta["synth"])
    state = {}

    def extra(q, counts):
        if q < 0:
            return B.synth_fill(p, 0, w * h, meta["spp"]), None
        return B.synth_fill(p, 0, w * h, 0, counts=counts, start_n=state["job"].read("STATS_N").ravel()), counts

    def on_counts(q, job, counts):
        assert np.array_equal(counts, a[f"counts{q}"]), f"pass {q} counts"

    o = B.OracleJob(cfg, threads=1)
    state["job"] = o
    replay_adaptive(o, cfg, a, meta["spp"], extra, on_counts)
    assert_all_fields(o, a)
    o.close()


def test_port_filters_golden():
    meta, a = load_golden("filters_37x53.npz")
    out = B.port_atrous(a["raw"], a["normal"], a["albedo"], *meta["atrous"])
    assert_bitwise(out, a["atrous"], "atrous")
    for got, name in zip(B.port_joint_bilateral(a["raw"], a["normal"], a["albedo"], *meta["joint"]),
                         ("gaussian", "bilateral", "joint")):
        assert_bitwise(got, a[name], name)


def test_port_threads_do_not_change_results():
    """The restatement's row-block threading keeps every output of one thread."""
    meta, a = load_golden("cornell_48x48x4.npz")
    cfg = golden_config(meta)
    s = golden_samples(a, "s_", meta["planes"], cfg.image_width * cfg.image_height)
    o = B.OracleJob(cfg, threads=4)
    B.run_pipeline(o, s, meta["spp"])
    for f in STAGE_FIELDS:
        if f == "GRID" or f.startswith("NODE_"):
            continue  # per-thread grids are merged in thread order, as the reference merges them
        assert_bitwise(o.read(f), a["out_" + f], f)
    o.close()


def test_port_validation_messages():
    g = json.loads((GOLDEN / "config_messages.json").read_text())
    base = B.config_from(g["base"])
    assert B.port().orc_config_validate(B.C.byref(base), None, 0) == 0
    for row in g["invalid"]:
        cfg = base.replace(**{row["field"]: row["value"]})
        msg = B.C.create_string_buffer(256)
        st = B.port().orc_config_validate(B.C.byref(cfg), msg, 256)
        assert st == 1, row
        assert msg.value.decode() == row["message"], row


# ---- restatement vs the live reference -----------------------------------------------------

@needs_ref
@pytest.mark.parametrize("w,h,spp,tile,seed", [(37, 23, 5, 16, 3), (33, 17, 4, 6, 4), (16, 16, 3, 1, 5),
                                               (45, 30, 9, 4, 6), (1, 7, 2, 16, 7)])
def test_port_matches_live_reference(w, h, spp, tile, seed):
    cfg = small_config(w, h, rpf_tile_size=tile, adaptive_spp=3, adaptive_base_samples=1)
    s = B.synth_fill(R.synth_params(w, h, seed, miss_regions=3, nan_rate=0.01), 0, w * h, spp)
    o = B.OracleJob(cfg, threads=1)
    r = B.RefJob(cfg, threads=1)
    for job in (o, r):
        B.run_pipeline(job, s, spp)
    for f in STAGE_FIELDS:
        assert_bitwise(o.read(f), r.read(f), f)
    assert np.array_equal(o.compute_adaptive_sample_counts(), r.compute_adaptive_sample_counts())
    o.close()
    r.close()


@needs_ref
def test_port_matches_live_reference_ragged_counts():
    w, h = 25, 19
    rng = np.random.default_rng(4)
    counts = rng.integers(0, 9, size=w * h).astype(np.int32)
    counts[::7] = 0
    cfg = small_config(w, h)
    s = B.synth_fill(R.synth_params(w, h, 8, miss_regions=2), 0, w * h, 0, counts=counts)
    o = B.OracleJob(cfg, threads=1)
    r = B.RefJob(cfg, threads=1)
    for job in (o, r):
        job.begin_frame()
        job.push(s, 0, w * h, 0, counts=counts)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
    for f in STAGE_FIELDS:
        assert_bitwise(o.read(f), r.read(f), f)
    o.close()
    r.close()


@needs_ref
def test_port_filters_match_live_reference():
    rng = np.random.default_rng(9)
    h, w = 21, 30
    raw = rng.lognormal(-0.5, 1.0, size=(h, w, 3)).astype(np.float32)
    normal = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    albedo = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    assert_bitwise(B.port_atrous(raw, normal, albedo, 0.5, 0.3, 0.2, 3),
                   B.ref_atrous(raw, normal, albedo, 0.5, 0.3, 0.2, 3), "atrous")
    for x, y in zip(B.port_joint_bilateral(raw, normal, albedo, 0.4, 0.3, 1.0, 0.2),
                    B.ref_joint_bilateral(raw, normal, albedo, 0.4, 0.3, 1.0, 0.2)):
        assert_bitwise(x, y, "joint")


def test_fp64_restatement_stays_close_to_the_float_one():
    """oracle/rpd_oracle64.c (the stage's single-precision quantities in double) against the
    float restatement on a synthetic frame: the same method, so the two agree to rounding."""
    w, h, spp = 64, 48, 8
    cfg = R.default_config(image_width=w, image_height=h, rpf_tile_size=16, color_window_radius=5,
                           var_window_radius=3, var_iterations=2, seed=1234)
    s = B.synth_fill(R.synth_params(w, h, 77), 0, w * h, spp, threads=2)
    d64 = B.fp64_denoise(cfg, s, spp, threads=2).astype(np.float64)
    j = B.OracleJob(cfg, threads=2)
    j.begin_frame()
    j.push(s, 0, w * h, spp)
    j.end_pass()
    j.recompute_sensitivity()
    j.statmc_denoise()
    j.variance_denoise()
    d32 = j.read("DENOISED").astype(np.float64)
    j.close()
    assert np.all(np.isfinite(d64))
    assert float(np.mean((d32 - d64) ** 2 / (d64 ** 2 + 1e-2))) <= 1e-9



# ---- evaluation metrics (shared/tools/eval_tools.cpp) -------------------------------------

PRINTED = {"mae": 1e-10, "rmse": 1e-10, "peak": 1e-10, "psnr": 1e-5}  # %.12g and %.6g in the report


def assert_metrics_match(got: dict, want: dict, extended_exact: bool) -> None:
    for k in ("nrmse", "log_ssim11", "log_gradient_nrmse"):
        if extended_exact:
            assert got[k] == want[k], (k, got[k], want[k])
        else:
            assert got[k] == pytest.approx(want[k], rel=1e-9, abs=1e-12), k
    for k, rel in PRINTED.items():
        if np.isinf(want[k]):
            assert np.isinf(got[k]), k
        else:
            assert got[k] == pytest.approx(want[k], rel=rel, abs=1e-12), k
    for c in range(3):
        assert abs(got["ssim"][c] - want["ssim"][c]) <= 5e-5  # printed with 4 decimals
    assert abs(got["ssim_mean"] - want["ssim_mean"]) <= 5e-5


def test_port_metrics_golden():
    meta, a = load_golden("eval_metrics.npz")
    for name, want in meta["metrics"].items():
        got = B.port_hdr_metrics(a[f"{name}_ref"], a[f"{name}_tst"])
        assert_metrics_match(got, want, extended_exact=True)


def test_port_metrics_self_test_properties():
    """eval_tools self-test (eval_tools.cpp:317-338): identical images give NRMSE 0,
    LogSSIM11 1 and LogGradNRMSE 0; one changed value moves all three."""
    meta, a = load_golden("eval_metrics.npz")
    same = B.port_hdr_metrics(a["identical_ref"], a["identical_tst"])
    assert same["nrmse"] <= 1e-12 and abs(same["log_ssim11"] - 1.0) <= 1e-12 and same["log_gradient_nrmse"] <= 1e-12
    diff = B.port_hdr_metrics(a["selftest_ref"], a["selftest_tst"])
    assert diff["nrmse"] > 0.0 and diff["log_ssim11"] < 1.0 and diff["log_gradient_nrmse"] > 0.0


@needs_ref
def test_port_metrics_match_live_reference():
    rng = np.random.default_rng(41)
    for (h, w) in [(17, 13), (64, 96), (5, 300)]:
        a = rng.lognormal(-0.5, 1.0, (h, w, 3)).astype(np.float32)
        b = (a + rng.normal(0, 0.05, a.shape)).astype(np.float32)
        assert_metrics_match(B.port_hdr_metrics(a, b), B.ref_hdr_metrics(a, b), extended_exact=True)
