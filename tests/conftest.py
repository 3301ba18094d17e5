"""Shared test set-up: markers, import paths and the three implementations.

`gpu`   the product (librpd_gb300.so on an sm_103 GPU) — only in tests marked gpu.
`port`  the C restatement oracle (oracle/_build/librpd_oracle.so), on every machine.
`ref`   the reference's own sources compiled against the shims (oracle/_ref), only where
        the reference checkout was present when it was built.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "rpd-statmc-denoiser_gb300"))

import rpd_gb300 as R  # noqa: E402
from oracle import binding as B  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU and the built librpd_gb300.so")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def gpu_ctx():
    ctx = R.Context(0, 0)
    yield ctx
    ctx.close()


def fbits(a: np.ndarray) -> np.ndarray:
    """Bit pattern view for exact float comparisons. Every NaN maps to one pattern: NaN
    payloads and signs are not part of the contract (x86 propagates an operand's payload where
    the GPU returns its canonical NaN)."""
    if a.dtype == np.float32:
        b = a.view(np.uint32).copy()
        b[np.isnan(a)] = 0x7FC00000
        return b
    if a.dtype == np.float64:
        b = a.view(np.uint64).copy()
        b[np.isnan(a)] = 0x7FF8000000000000
        return b
    return a


def assert_bitwise(x: np.ndarray, y: np.ndarray, name: str = "") -> None:
    if not np.array_equal(fbits(x), fbits(y)):
        diff = np.abs(x.astype(np.float64) - y.astype(np.float64))
        n = int(np.count_nonzero(fbits(x) != fbits(y)))
        raise AssertionError(f"{name}: {n} values differ, max abs diff {np.nanmax(diff):.3e}")


def max_rel_err(x: np.ndarray, ref: np.ndarray, floor: float) -> float:
    """max |x - ref| / max(|ref|, floor), the per-pixel relative error of the plain-form
    parity bar; `floor` keeps near-black pixels from dividing by ~0."""
    x = x.astype(np.float64)
    ref = ref.astype(np.float64)
    return float(np.max(np.abs(x - ref) / np.maximum(np.abs(ref), floor)))


def small_config(w: int, h: int, **kw) -> R.Config:
    """The plain-method knobs of the 256x256 cornell_box case (rpf tile 16, colour radius 5,
    variance radius 3, 2 variance iterations) at another size."""
    base = dict(image_width=w, image_height=h, rpf_tile_size=16, color_window_radius=5, var_window_radius=3,
                var_iterations=2, seed=1234)
    base.update(kw)
    return R.default_config(**base)


# ---- golden fixtures (tests/golden/make_golden.py) ----------------------------------------

def load_golden(name: str):
    """(meta dict, arrays dict) of one fixture."""
    import json

    with np.load(GOLDEN / name) as z:
        arrays = {k: z[k] for k in z.files}
    return json.loads(str(arrays.pop("meta"))), arrays


def golden_samples(arrays: dict, prefix: str, planes: list[str], n_pixels: int) -> "R.HostSamples":
    """HostSamples rebuilt from the planes stored under `prefix`."""
    hs = R.HostSamples.__new__(R.HostSamples)
    hs.planes = {p: np.ascontiguousarray(arrays[prefix + p]) for p in planes}
    hs.n_samples = int(hs.planes["flags"].shape[-1])
    hs.n_pixels = n_pixels
    return hs


def golden_config(meta: dict) -> "R.Config":
    return B.config_from(meta["config"])


def replay_adaptive(job, cfg, arrays: dict, spp: int, extra_for_pass, on_counts=None) -> None:
    """render()'s adaptive sequence (main.cpp:1543-1559 minus the final radiance swap): the
    base pass, then per adaptive pass denoise, variance, counts, the pass's extra samples
    (`extra_for_pass(p, counts)` returns HostSamples and the counts they were drawn with),
    sensitivity; then the final sensitivity, denoise, variance and finalize."""
    w, h = cfg.image_width, cfg.image_height
    s0 = extra_for_pass(-1, None)[0]
    job.begin_frame()
    job.push(s0, 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    for p in range(cfg.adaptive_passes):
        job.statmc_denoise()
        job.variance_denoise()
        counts = job.compute_adaptive_sample_counts()
        if on_counts:
            on_counts(p, job, counts)
        extra, used = extra_for_pass(p, counts)
        job.push(extra, 0, w * h, 0, counts=used)
        job.end_pass()
        job.recompute_sensitivity()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()
    job.finalize()
