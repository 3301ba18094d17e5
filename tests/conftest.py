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
    """Bit pattern view for exact float comparisons."""
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
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
