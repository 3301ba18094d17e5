"""The C ABI without a GPU: the library loads, exports every function include/*.h declares,
and its host-side logic (validation, names, status strings, no-device errors) behaves."""
from __future__ import annotations

import ctypes as C
import json
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, B, R

HEADERS = sorted((ROOT / "include").glob("*.h"))
# a declaration at file scope: return type, rpd_ name, '(' ... ');' (the RPD_HD helpers of
# rpd_synth.h are header-only and have bodies)
DECL = re.compile(r"^(?!static|inline|typedef|#|RPD_HD|return)[A-Za-z_][\w \*]*?\b(rpd_\w+)\s*\(([^;{]*?)\)\s*;",
                  re.M | re.S)


def declared_functions() -> set[str]:
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(m.group(1) for m in DECL.finditer(text))
    return names


def test_headers_declare_the_binding_table():
    decl = declared_functions()
    assert "rpd_statmc_denoise" in decl and "rpd_job_push_samples" in decl
    assert decl == set(R.exported_symbols()), sorted(decl ^ set(R.exported_symbols()))


def test_library_exports_every_declared_function():
    lib = C.CDLL(str(R.LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_validation_messages_match_the_reference():
    g = json.loads((GOLDEN / "config_messages.json").read_text())
    base = B.config_from(g["base"])
    st, msg = R.validate(base)
    assert st == R.OK, msg
    for row in g["invalid"]:
        st, msg = R.validate(base.replace(**{row["field"]: row["value"]}))
        assert st == 1 and msg == row["message"], (row, st, msg)


def test_defaults_are_the_reference_defaults():
    """rpd_config_defaults gives RenderConfig's defaults (core/config.h:27-48); the golden
    base config is cornell.yaml over them, so every key cornell.yaml leaves out agrees."""
    cfg = R.Config()
    R.lib().rpd_config_defaults(C.byref(cfg))
    d = B.config_dict(cfg)
    base = json.loads((GOLDEN / "config_messages.json").read_text())["base"]
    for key in ("rpf_tile_size", "rpf_shrinkage_scale", "rpf_confidence_samples", "color_window_radius",
                "var_depth_threshold", "adaptive_importance_smoothing_radius", "debug_statmc_outputs"):
        assert d[key] == base[key], key
    assert B.config_dict(R.default_config()) == d


def test_status_and_kernel_names():
    for code in range(9):
        assert R.lib().rpd_status_string(code)
    names = [R.lib().rpd_kernel_name(k).decode() for k in range(len(R.KERNELS))]
    assert names == R.KERNELS


def test_no_device_is_an_error_not_a_crash():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = R.lib().rpd_ctx_create(0, 0, C.byref(h))
    assert st == 8 and not h.value  # RPD_ERR_NO_DEVICE
    assert R.lib().rpd_last_error()


def test_noalloc_rejects_before_touching_a_device():
    with pytest.raises(R.RpdError, match="exceeds the no-allocation scratch"):
        R.lib().rpd_atrous_wavelet_noalloc  # the symbol exists
        R.check(R.lib().rpd_atrous_wavelet_noalloc(1, 1, 1, 4096, 4096, 0.3, 0.2, 0.1, 1, 1 << 40, None))


def test_footprint_grows_with_the_frame():
    small = R.lib().rpd_job_footprint(C.byref(R.default_config(image_width=64, image_height=64)))
    big = R.lib().rpd_job_footprint(C.byref(R.default_config(image_width=1920, image_height=1080)))
    assert 0 < small < big
    # per-pixel planes dominate: at least the 24 B/pixel of required outputs
    assert big >= 1920 * 1080 * 24


def test_synthetic_generator_host_matches_pinned_hashes():
    """include/rpd_synth.h evaluated on the host reproduces the pinned planes (the GPU test
    checks the device evaluation against the same hashes)."""
    import hashlib

    with np.load(GOLDEN / "synth_48x32x8.npz") as z:
        meta = json.loads(str(z["meta"]))
    p = B.synth_from(meta["synth"])
    s = B.synth_fill(p, 0, p.width * p.height, meta["spp"], threads=3)
    for k, v in s.planes.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == meta["sample_sha256"][k], k
