"""Generate the golden fixtures in this folder from the reference itself.

Every output stored here comes from the reference's own code, compiled from its checkout
by `make -C oracle ref` against the shims in oracle/ref_shim and loaded through
oracle/binding.py:

  * `RefJob`: path_tracer/main.cpp's accumulate_sample / accumulate_rpf_sample_to_grid /
    merge_rpf_grids_into / recompute_sensitivity / statmc_denoise / variance_denoise /
    compute_adaptive_sample_counts / FrameBuffers::finalize on the process globals;
  * `trace_cornell`: the reference's own cornell_box tracer recording each camera sample
    (the per-sample buffers of the 256x256 4-spp cornell configuration, at smaller sizes);
  * `ref_render_cornell`: the reference's render() loop end to end, used here to check that
    the replayed adaptive sequence is the one render() performs;
  * `ref_atrous` / `ref_joint_bilateral`: denoising/atrous_wavelet.cpp and
    joint_bilateral.cpp filter() on in-memory images;
  * `ref_hdr_metrics`: shared/tools/eval_tools.cpp (its hdr-metrics command and
    compute_extended_metrics) on in-memory images;
  * `ref_parse_yaml`: core/config.h parse_render_config, for the validation messages.

Fixtures (numpy .npz, compressed; `meta` is a JSON string):

  cornell_48x48x4.npz         reference-traced samples + every stage output + counts
  cornell_256x256x4.npz       the plain-method cornell_box configuration at its full size
                              (256x256, 4 spp, seed 1234, adaptive_passes 0): reference-traced
                              samples and every stage output
  cornell_32x32_adaptive.npz  base + per-pass extra samples (traced with the reference's
                              counts), per-pass counts, final outputs (adaptive_passes 2)
  synth_48x32x8.npz           outputs for the synthetic generator (samples regenerated from
                              `meta.synth`; a SHA-256 of each plane pins the generator)
  synth_32x24_adaptive.npz    the adaptive sequence with synthetic extra samples
  filters_37x53.npz           filter inputs and the reference filter outputs
  outputs_48x48.npz           every image output_buffers writes for the 48x48 cornell frame
                              (HDR floats, tonemapped PNG bytes) and the tonemapping curves
  eval_metrics.npz            image pairs and the reference's eval_tools hdr-metrics of each
                              (compute_extended_metrics in full precision, the printed report)
  config_messages.json        (field, value, message) of the reference's validation

    REF_ROOT=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
from oracle import binding as B  # noqa: E402

R = B.R
# the reference checkout: REF_ROOT, else a checkout named "reference" beside this repository
REF_ROOT = Path(os.environ.get("REF_ROOT", ROOT.parent / "reference"))
YAML = REF_ROOT / "path_tracer" / "config" / "cornell.yaml"

# Fields compared by the tests (EXPANDED_* are the caches behind the sensitivity maps; the
# maps themselves are stored).
STAGE_FIELDS = ["STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
                "STATS_SQRT_SQUARE_DIFF", "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM",
                "DEPTH_SUM", "GRID"] + [f for f in R.FIELDS if f.startswith("NODE_")] + [
                "SENSITIVITY_CONFIDENCE", "SENSITIVITY_GRADIENT", "DENOISED", "UNCERTAINTY", "ALPHA",
                "VAR_TOTAL_DEBUG", "VAR_EFF_DEBUG", "VAR_RATIO_DEBUG", "VARIANCE_DENOISED"]

# the stage knobs of the 256x256 cornell configuration: cornell.yaml plus tile 16, colour
# window 5, variance window 3, 2 variance iterations, seed 1234
CORNELL_KNOBS = dict(rpf_tile_size=16, color_window_radius=5, var_window_radius=3, var_iterations=2, seed=1234)


def sample_hashes(s: R.HostSamples) -> dict:
    return {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() for k, v in s.planes.items()}


def put_samples(out: dict, prefix: str, s: R.HostSamples) -> None:
    for k, v in s.planes.items():
        out[f"{prefix}{k}"] = v


def put_fields(out: dict, job, prefix: str = "out_") -> None:
    for f in STAGE_FIELDS:
        out[prefix + f] = job.read(f)


def save(name: str, meta: dict, arrays: dict) -> None:
    np.savez_compressed(HERE / name, meta=np.array(json.dumps(meta, sort_keys=True)), **arrays)
    print(f"{name}: {(HERE / name).stat().st_size / 1024:.0f} KiB")


def cornell_single() -> None:
    w = h = 48
    spp = 4
    cfg = B.ref_parse_yaml(str(YAML)).replace(image_width=w, image_height=h, adaptive_passes=0,
                                               adaptive_spp=4, adaptive_base_samples=1, **CORNELL_KNOBS)
    s = B.trace_cornell(str(YAML), w, h, spp, cfg.seed)
    job = B.RefJob(cfg, threads=1)
    B.run_pipeline(job, s, spp)
    arrays = {}
    put_samples(arrays, "s_", s)
    put_fields(arrays, job)
    arrays["counts"] = job.compute_adaptive_sample_counts()
    arrays["out_ADAPTIVE_IMPORTANCE"] = job.read("ADAPTIVE_IMPORTANCE")
    job.close()
    save("cornell_48x48x4.npz", {"config": B.config_dict(cfg), "spp": spp, "planes": list(s.planes)}, arrays)


def cornell_full() -> None:
    """The 256x256 4-spp cornell_box configuration itself (one frame, no adaptive pass)."""
    w = h = 256
    spp = 4
    cfg = B.ref_parse_yaml(str(YAML)).replace(image_width=w, image_height=h, adaptive_passes=0,
                                               adaptive_spp=4, adaptive_base_samples=1, **CORNELL_KNOBS)
    s = B.trace_cornell(str(YAML), w, h, spp, cfg.seed)
    job = B.RefJob(cfg, threads=1)  # the single-thread grid order, which the exact grid mode reproduces
    B.run_pipeline(job, s, spp)
    arrays = {}
    # lens and environment samples are never valid in this scene (zero planes): not stored
    planes = [k for k, v in s.planes.items() if np.any(v)]
    for k in planes:
        arrays["s_" + k] = s.planes[k]
    put_fields(arrays, job)
    job.close()
    save("cornell_256x256x4.npz", {"config": B.config_dict(cfg), "spp": spp, "planes": planes,
                                   "sample_sha256": sample_hashes(s)}, arrays)


def cornell_adaptive() -> None:
    w = h = 32
    spp = 4
    cfg = B.ref_parse_yaml(str(YAML)).replace(image_width=w, image_height=h, adaptive_passes=2, adaptive_spp=4,
                                               adaptive_base_samples=2, **{**CORNELL_KNOBS, "seed": 99})
    arrays = {}
    job = B.RefJob(cfg, threads=1)
    job.begin_frame()
    s0 = B.trace_cornell(str(YAML), w, h, spp, cfg.seed)
    put_samples(arrays, "s_", s0)
    job.push(s0, 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    for p in range(cfg.adaptive_passes):
        job.statmc_denoise()
        job.variance_denoise()
        counts = job.compute_adaptive_sample_counts()
        n = job.read("STATS_N").ravel()
        extra = B.trace_cornell(str(YAML), w, h, 0, cfg.seed, start_n=n, counts=counts)
        arrays[f"counts{p}"] = counts
        arrays[f"importance{p}"] = job.read("ADAPTIVE_IMPORTANCE")
        put_samples(arrays, f"x{p}_", extra)
        job.push(extra, 0, w * h, 0, counts=counts)
        job.end_pass()
        job.recompute_sensitivity()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()
    job.finalize()
    put_fields(arrays, job)
    # render() ends by moving the denoised image into buffers.radiance (main.cpp:1558-1559)
    replay = {f: arrays["out_" + f] for f in ("DENOISED", "VARIANCE_DENOISED", "STATS_N", "GRID")}
    replay["RADIANCE_SUM"] = arrays["out_DENOISED"]
    job.close()
    # the replay must be render()'s own sequence: run render() itself and compare
    B.ref().ref_render_cornell(str(YAML).encode(), B.C.byref(cfg), spp, 1)
    direct = B.RefJob.__new__(B.RefJob)
    direct.cfg, direct.threads = cfg, 1
    for f, v in replay.items():
        d = direct.read(f)
        assert np.array_equal(d.view(np.uint8), v.view(np.uint8)), f"replay differs from render() in {f}"
    save("cornell_32x32_adaptive.npz", {"config": B.config_dict(cfg), "spp": spp, "planes": list(s0.planes)},
         arrays)


def synth_config(w: int, h: int, **kw) -> R.Config:
    return R.default_config(image_width=w, image_height=h, rpf_tile_size=16, color_window_radius=5,
                            var_window_radius=3, var_iterations=2, seed=1234, adaptive_spp=4,
                            adaptive_base_samples=1, **kw)


def synth_single() -> None:
    w, h, spp = 48, 32, 8
    cfg = synth_config(w, h)
    p = R.synth_params(w, h, 7, miss_regions=3, nan_rate=0.01)
    s = B.synth_fill(p, 0, w * h, spp)
    job = B.RefJob(cfg, threads=1)
    B.run_pipeline(job, s, spp)
    arrays = {}
    put_fields(arrays, job)
    arrays["counts"] = job.compute_adaptive_sample_counts()
    arrays["out_ADAPTIVE_IMPORTANCE"] = job.read("ADAPTIVE_IMPORTANCE")
    job.close()
    save("synth_48x32x8.npz", {"config": B.config_dict(cfg), "spp": spp, "synth": B.synth_dict(p),
                               "sample_sha256": sample_hashes(s)}, arrays)


def synth_adaptive() -> None:
    w, h, spp = 32, 24, 2
    cfg = synth_config(w, h, adaptive_passes=2, adaptive_importance_smoothing_radius=1)
    p = R.synth_params(w, h, 31)
    arrays = {}
    job = B.RefJob(cfg, threads=1)
    job.begin_frame()
    s0 = B.synth_fill(p, 0, w * h, spp)
    job.push(s0, 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    for q in range(cfg.adaptive_passes):
        job.statmc_denoise()
        job.variance_denoise()
        counts = job.compute_adaptive_sample_counts()
        arrays[f"counts{q}"] = counts
        arrays[f"importance{q}"] = job.read("ADAPTIVE_IMPORTANCE")
        n = job.read("STATS_N").ravel()
        extra = B.synth_fill(p, 0, w * h, 0, counts=counts, start_n=n)
        job.push(extra, 0, w * h, 0, counts=counts)
        job.end_pass()
        job.recompute_sensitivity()
    job.recompute_sensitivity()
    job.statmc_denoise()
    job.variance_denoise()
    job.finalize()
    put_fields(arrays, job)
    job.close()
    save("synth_32x24_adaptive.npz", {"config": B.config_dict(cfg), "spp": spp, "synth": B.synth_dict(p)}, arrays)


def filters() -> None:
    rng = np.random.default_rng(1)
    h, w = 37, 53
    raw = rng.lognormal(-1.0, 0.8, size=(h, w, 3)).astype(np.float32)
    normal = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    albedo = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    atrous = (0.3, 0.2, 0.1, 5)
    joint = (0.3, 0.2, 2.0, 0.1)
    a = B.ref_atrous(raw, normal, albedo, *atrous)
    g, b, j = B.ref_joint_bilateral(raw, normal, albedo, *joint)
    save("filters_37x53.npz", {"atrous": atrous, "joint": joint},
         dict(raw=raw, normal=normal, albedo=albedo, atrous=a, gaussian=g, bilateral=b, joint=j))


def outputs() -> None:
    """output_buffers of the 48x48 cornell frame (agx preset) as the reference writes it, and its
    tonemapping curves (every preset) on a spread of HDR values."""
    w = h = 48
    spp = 4
    cfg = B.ref_parse_yaml(str(YAML)).replace(image_width=w, image_height=h, adaptive_passes=0,
                                               adaptive_spp=4, adaptive_base_samples=1, **CORNELL_KNOBS)
    s = B.trace_cornell(str(YAML), w, h, spp, cfg.seed)
    job = B.RefJob(cfg, threads=1)
    B.run_pipeline(job, s, spp)
    job.compute_adaptive_sample_counts()  # fills adaptive_importance
    job.finalize()
    files = B.ref_outputs("out", 0)
    job.close()
    arrays = {}
    for name, arr in files.items():
        arrays["f_" + name.replace(".", "__")] = arr
    put_samples(arrays, "s_", s)
    rng = np.random.default_rng(21)
    vals = np.concatenate([rng.lognormal(-1.5, 2.0, (3000, 3)), rng.uniform(0, 1, (800, 3)),
                           np.array([[0, 0, 0], [1e-9, 0, 0], [1e4, 1e4, 1e4], [1, 1, 1], [0.5, 0.25, 0.125]])]
                          ).astype(np.float32)
    arrays["tonemap_in"] = vals
    for t in range(4):
        arrays[f"tonemap_{t}"] = B.ref_tonemap(vals, t)
    save("outputs_48x48.npz", {"config": B.config_dict(cfg), "spp": spp, "planes": list(s.planes), "prefix": "out",
                               "files": sorted(files)}, arrays)


def metrics() -> None:
    """eval_tools hdr-metrics of image pairs: the reference's compute_extended_metrics (full
    precision) and its printed report, with the images."""
    rng = np.random.default_rng(9)
    pairs = {}
    ref = rng.lognormal(-1.0, 0.8, size=(29, 37, 3)).astype(np.float32)
    pairs["noisy"] = (ref, (ref * rng.lognormal(0.0, 0.1, ref.shape)).astype(np.float32))
    ramp = np.add.outer(np.arange(16), np.arange(16)).astype(np.float32)[..., None] + 1.0
    ramp = np.repeat(ramp / 32.0, 3, axis=2).astype(np.float32)
    changed = ramp.copy()
    changed[8, 8, 0] += 0.25  # the reference's self-test pair (eval_tools.cpp:317-338)
    pairs["selftest"] = (ramp, changed)
    pairs["identical"] = (ramp, ramp.copy())
    dark = rng.uniform(-0.05, 0.2, size=(23, 41, 3)).astype(np.float32)  # negative luminance clamps to 0
    pairs["dark"] = (dark, (dark + rng.normal(0, 0.02, dark.shape)).astype(np.float32))
    arrays, meta = {}, {}
    for name, (a, b) in pairs.items():
        arrays[f"{name}_ref"], arrays[f"{name}_tst"] = a, b
        r = B.ref_hdr_metrics(a, b)
        meta[name] = {k: v for k, v in r.items() if k != "text"}
    save("eval_metrics.npz", {"metrics": meta}, arrays)


# (field, invalid value) pairs for the stage knobs core/config.h:116-195 validates
INVALID = [
    ("image_width", 0), ("image_height", -3), ("rpf_tile_size", 0), ("color_window_radius", 0),
    ("color_normal_threshold", 0.0), ("color_normal_threshold", 1.5), ("color_depth_threshold", -0.1),
    ("color_compat_alpha", 0.0), ("color_compat_alpha", 1.0), ("color_sigma_max", 0.0),
    ("var_window_radius", 0), ("var_normal_threshold", 0.0), ("var_depth_threshold", -1.0),
    ("var_compat_sigma", 0.0), ("var_shrinkage_k", -2.0), ("adaptive_base_samples", -1),
    ("adaptive_spp", -1), ("adaptive_base_samples", 9), ("adaptive_sigma_max", 0.0), ("adaptive_passes", -1),
    ("adaptive_importance_smoothing_radius", -1), ("var_iterations", 0), ("rpf_shrinkage_scale", -0.5),
    ("rpf_confidence_samples", 0.0),
]


def config_messages() -> None:
    base = YAML.read_text().splitlines()
    rows = []
    with tempfile.TemporaryDirectory() as td:
        for field, value in INVALID:
            lines = [ln for ln in base if not ln.startswith(field + ":")]
            lines.append(f"{field}: {value}")
            path = Path(td) / "c.yaml"
            path.write_text("\n".join(lines) + "\n")
            try:
                B.ref_parse_yaml(str(path))
            except ValueError as e:
                rows.append({"field": field, "value": value, "message": str(e)})
                continue
            raise AssertionError(f"the reference accepted {field}={value}")
    base_cfg = B.config_dict(B.ref_parse_yaml(str(YAML)))
    (HERE / "config_messages.json").write_text(json.dumps({"base": base_cfg, "invalid": rows}, indent=1) + "\n")
    print(f"config_messages.json: {len(rows)} rows")


if __name__ == "__main__":
    if not B.have_ref():
        sys.exit("oracle/_ref is not built: run `make -C oracle ref REF_ROOT=<reference checkout>` first")
    cornell_single()
    cornell_full()
    cornell_adaptive()
    synth_single()
    synth_adaptive()
    filters()
    metrics()
    outputs()
    config_messages()
