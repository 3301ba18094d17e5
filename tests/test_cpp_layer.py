"""The header-only C++ layer (include/rpd_statmc.hpp): a render() clone that keeps the
reference's stage-function names compiles and links against librpd_gb300.so here, and on a
GPU its whole frame matches the oracle's render() sequence on the same samples (and the same
sequence driven through the Python binding)."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, B, R, max_rel_err

SRC = ROOT / "tests" / "cpp" / "render_clone.cpp"
BUILD = ROOT / "tests" / "cpp" / "_build"


def build_clone() -> str:
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    BUILD.mkdir(exist_ok=True)
    exe = BUILD / "render_clone"
    lib_dir = R.LIB_PATH.parent
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o",
           str(exe), f"-L{lib_dir}", "-lrpd_gb300", f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return str(exe)


def test_clone_compiles_and_links():
    if not R.LIB_PATH.exists():
        pytest.skip("librpd_gb300.so not built")
    build_clone()


@pytest.mark.gpu
def test_clone_matches_oracle(gpu_ctx, tmp_path):
    """The clone's whole frame (two adaptive passes) against the oracle running render()'s
    sequence on the same samples: each pass's counts as the oracle allocates them (bit-exact
    where the importance maps agree to the bit, else the same total and within 4 samples), then
    the final denoised image within the plain-form bar."""
    exe = build_clone()
    w, h, spp, passes = 48, 32, 4, 2
    out = tmp_path / "clone.bin"
    r = subprocess.run([exe, str(w), str(h), str(spp), str(passes), str(out)], capture_output=True, text=True,
                       timeout=120, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    raw = out.read_bytes()
    np_ = w * h
    counts = np.frombuffer(raw[:passes * np_ * 4], dtype=np.int32).reshape(passes, np_)
    denoised = np.frombuffer(raw[passes * np_ * 4:], dtype=np.float32).reshape(h, w, 3)
    cfg = R.default_config(image_width=w, image_height=h, rpf_tile_size=16, color_window_radius=5,
                           color_normal_threshold=0.6, color_depth_threshold=0.2, color_compat_alpha=0.01,
                           color_sigma_max=4.0, var_window_radius=3, var_normal_threshold=0.6, var_compat_sigma=3.0,
                           var_shrinkage_k=0.7, var_iterations=2, adaptive_base_samples=1, adaptive_spp=4,
                           adaptive_sigma_max=4.0, adaptive_passes=passes, seed=1234)
    p = R.synth_params(w, h, 1234)
    o = B.OracleJob(cfg, threads=1)
    o.begin_frame()
    o.push(B.synth_fill(p, 0, np_, spp), 0, np_, spp)
    o.end_pass()
    o.recompute_sensitivity()
    n = np.full(np_, spp, dtype=np.int32)
    for k in range(passes):
        o.statmc_denoise()
        o.variance_denoise()
        want = o.compute_adaptive_sample_counts()
        got = counts[k]
        assert int(got.sum()) == int(want.sum())
        assert int(np.abs(got - want).sum()) <= 4, int(np.abs(got - want).sum())
        # the clone's samples of this pass (drawn for its counts)
        o.push(B.synth_fill(p, 0, np_, 0, counts=got, start_n=n), 0, np_, 0, counts=got)
        o.end_pass()
        n = n + got
        o.recompute_sensitivity()
    o.recompute_sensitivity()
    o.statmc_denoise()
    o.variance_denoise()
    o.finalize()
    assert max_rel_err(denoised, o.read("DENOISED"), 1e-3) <= 1e-4
    o.close()


@pytest.mark.gpu
def test_clone_matches_python_sequence(gpu_ctx):
    exe = build_clone()
    w, h, spp, passes = 48, 32, 4, 2
    r = subprocess.run([exe, str(w), str(h), str(spp), str(passes)], capture_output=True, text=True, timeout=120,
                       env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    fields = dict(zip(r.stdout.split()[0::2], r.stdout.split()[1::2]))
    cfg = R.default_config(image_width=w, image_height=h, rpf_tile_size=16, color_window_radius=5,
                           color_normal_threshold=0.6, color_depth_threshold=0.2, color_compat_alpha=0.01,
                           color_sigma_max=4.0, var_window_radius=3, var_normal_threshold=0.6, var_compat_sigma=3.0,
                           var_shrinkage_k=0.7, var_iterations=2, adaptive_base_samples=1, adaptive_spp=4,
                           adaptive_sigma_max=4.0, adaptive_passes=passes, seed=1234)
    p = R.synth_params(w, h, 1234)
    job = R.Job(gpu_ctx, cfg)
    job.begin_frame()
    job.push(B.synth_fill(p, 0, w * h, spp), 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    n = np.full(w * h, spp, dtype=np.int32)
    total = 0
    for _ in range(passes):
        job.statmc_denoise()
        job.variance_denoise()
        counts = job.compute_adaptive_sample_counts()
        total += int(counts.sum())
        job.push(B.synth_fill(p, 0, w * h, 0, counts=counts, start_n=n), 0, w * h, 0, counts=counts)
        job.end_pass()
        n = n + counts
        job.recompute_sensitivity()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()
    job.finalize()
    mean = float(job.read("DENOISED").astype(np.float64).mean())
    assert int(fields["adaptive_total"]) == total
    assert abs(float(fields["denoised_mean"]) - mean) <= 1e-6 * abs(mean)
    job.close()
