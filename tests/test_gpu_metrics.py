"""Evaluation metrics on the GPU (rpd_hdr_metrics, rpd_job_hdr_metrics) against the reference's
eval_tools hdr-metrics: the golden fixture's reference values, and the oracle restatement (pinned
bit for bit to the reference's compute_extended_metrics) on larger images. The GPU sums in another
order than the reference's sequential loops, so the scalars agree to a relative 1e-9, not to the
bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import B, R, load_golden, small_config
from test_oracle import assert_metrics_match

pytestmark = pytest.mark.gpu


def test_metrics_golden(gpu_ctx):
    meta, a = load_golden("eval_metrics.npz")
    for name, want in meta["metrics"].items():
        got = gpu_ctx.hdr_metrics(a[f"{name}_ref"], a[f"{name}_tst"])
        assert_metrics_match(got, want, extended_exact=False)


def test_metrics_self_test_properties(gpu_ctx):
    meta, a = load_golden("eval_metrics.npz")
    same = gpu_ctx.hdr_metrics(a["identical_ref"], a["identical_tst"])
    assert same["nrmse"] == 0.0 and same["log_gradient_nrmse"] == 0.0
    assert abs(same["log_ssim11"] - 1.0) <= 1e-12 and np.isinf(same["psnr"])
    diff = gpu_ctx.hdr_metrics(a["selftest_ref"], a["selftest_tst"])
    assert diff["nrmse"] > 0.0 and diff["log_ssim11"] < 1.0 and diff["log_gradient_nrmse"] > 0.0


@pytest.mark.parametrize("h,w", [(1080, 1920), (7, 300), (300, 7), (1, 1), (33, 65)])
def test_metrics_against_the_oracle(gpu_ctx, h, w):
    rng = np.random.default_rng(h * 1000 + w)
    a = rng.lognormal(-0.5, 1.0, (h, w, 3)).astype(np.float32)
    b = (a + rng.normal(0, 0.05, a.shape)).astype(np.float32)
    assert_metrics_match(gpu_ctx.hdr_metrics(a, b), B.port_hdr_metrics(a, b), extended_exact=False)


def test_job_metrics_score_the_denoised_frame(gpu_ctx):
    """A job's denoised image scored in place equals the metrics of the image read back."""
    w, h, spp = 96, 64, 8
    cfg = small_config(w, h)
    job = R.Job(gpu_ctx, cfg)
    B.run_pipeline(job, B.synth_fill(R.synth_params(w, h, 5), 0, w * h, spp), spp)
    ref = B.synth_fill(R.synth_params(w, h, 5), 0, w * h, 64)
    conv = R.Job(gpu_ctx, cfg)
    B.run_pipeline(conv, ref, 64)
    target = conv.read("DENOISED")
    inline = job.hdr_metrics(target)
    readback = gpu_ctx.hdr_metrics(target, job.read("DENOISED"))
    for k in ("mae", "rmse", "nrmse", "log_ssim11", "log_gradient_nrmse"):
        assert inline[k] == pytest.approx(readback[k], rel=1e-12), k
    assert 0.0 < inline["nrmse"] < 1.0
    job.close()
    conv.close()
