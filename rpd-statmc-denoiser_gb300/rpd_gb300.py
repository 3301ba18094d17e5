"""ctypes binding of the GB300 denoise-stage C ABI (include/rpd_gb300.h).

The product is the shared library librpd_gb300.so; this module is the thin Python view
the tests and bench.py use. Loading fails loudly when the library has not been built:
there is no Python or CPU fallback for any stage.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "librpd_gb300.so"

# ---- enums (include/rpd_gb300.h) ---------------------------------------------------------

OK = 0
STATUS = {0: "ok", 1: "invalid config", 2: "invalid argument", 3: "out of memory", 4: "over budget",
          5: "cuda error", 6: "timeout", 7: "state", 8: "no device"}
MEM_HOST, MEM_DEVICE = 0, 1

FIELDS = [
    "DENOISED", "UNCERTAINTY", "ALPHA", "VAR_TOTAL_DEBUG", "VAR_EFF_DEBUG", "VAR_RATIO_DEBUG",
    "VARIANCE_DENOISED", "ADAPTIVE_IMPORTANCE", "SENSITIVITY_CONFIDENCE", "SENSITIVITY_GRADIENT",
    "HIT_COUNT", "SAMPLE_COUNT", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM", "DEPTH_SUM",
    "STATS_MEAN", "STATS_SQUARE_DIFF", "STATS_N", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
    "STATS_SQRT_SQUARE_DIFF",
    "NODE_ALL", "NODE_ALL_CONF", "NODE_PIXEL", "NODE_PIXEL_CONF", "NODE_BRDF", "NODE_BRDF_CONF",
    "NODE_LENS", "NODE_LENS_CONF", "NODE_LIGHT", "NODE_LIGHT_CONF", "NODE_LIGHT_UV", "NODE_LIGHT_UV_CONF",
    "NODE_LIGHT_SELECT", "NODE_LIGHT_SELECT_CONF", "NODE_ENVIRONMENT", "NODE_ENVIRONMENT_CONF",
    "NODE_RR", "NODE_RR_CONF",
    "GRID",
    "EXPANDED_ALL", "EXPANDED_PIXEL", "EXPANDED_BRDF", "EXPANDED_LENS", "EXPANDED_LIGHT",
    "EXPANDED_LIGHT_UV", "EXPANDED_LIGHT_SELECT", "EXPANDED_ENVIRONMENT", "EXPANDED_RR",
    "ADAPTIVE_COUNTS", "SQRT_VARIANCE_STABLE",
]
FIELD = {name: i for i, name in enumerate(FIELDS)}
RGB_FIELDS = {"DENOISED", "RADIANCE_SUM", "NORMAL_SUM", "ALBEDO_SUM", "STATS_COLOR_MEAN", "STATS_SQRT_MEAN",
              "STATS_SQRT_SQUARE_DIFF", "SQRT_VARIANCE_STABLE"}
INT_FIELDS = {"HIT_COUNT", "SAMPLE_COUNT", "STATS_N", "ADAPTIVE_COUNTS"}
STAGES = ["ACCUMULATE", "SENSITIVITY", "STATMC", "VARIANCE", "ADAPTIVE"]
KERNELS = ["offsets", "accumulate_pixels", "grid", "grid_random", "merge", "features", "node_stats", "node_combine", "sens_pixels",
           "rpd_cache", "sqrt_variance", "statmc_window", "variance", "adaptive", "other", "synth"]
STAGE = {name: i for i, name in enumerate(STAGES)}

HIT, PIXEL_VALID, LENS_VALID, BRDF_VALID, LIGHT_VALID, LIGHT_SELECT_VALID, ENV_VALID, RR_VALID = (
    0x01, 0x02, 0x04, 0x08, 0x10, 0x20, 0x40, 0x80)
LIGHT_INDEX_MASK, RR_SURVIVED = 0x0F, 0x10
GRID_DEPS, GRID_STRIDE = 13, 36
DEP_NAMES = ["pixel", "brdf", "screen_brdf", "lens", "screen_lens", "light_uv", "screen_light_uv",
             "environment", "screen_environment", "light_select", "screen_light_select", "rr", "screen_rr"]


class Config(C.Structure):
    """rpd_config: the RenderConfig fields the stage reads (path_tracer/core/config.h:15-49)."""
    _fields_ = [
        ("image_width", C.c_int32), ("image_height", C.c_int32), ("rpf_tile_size", C.c_int32),
        ("rpf_shrinkage_scale", C.c_float), ("rpf_confidence_samples", C.c_float),
        ("color_window_radius", C.c_int32), ("color_normal_threshold", C.c_float),
        ("color_depth_threshold", C.c_float), ("color_compat_alpha", C.c_float), ("color_sigma_max", C.c_float),
        ("var_window_radius", C.c_int32), ("var_normal_threshold", C.c_float), ("var_depth_threshold", C.c_float),
        ("var_compat_sigma", C.c_float), ("var_shrinkage_k", C.c_float), ("var_iterations", C.c_int32),
        ("adaptive_base_samples", C.c_int32), ("adaptive_spp", C.c_int32), ("adaptive_sigma_max", C.c_float),
        ("adaptive_passes", C.c_int32), ("adaptive_importance_smoothing_radius", C.c_int32),
        ("debug_statmc_outputs", C.c_int32), ("seed", C.c_uint32),
    ]

    def replace(self, **kw) -> "Config":
        c = Config()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(Config))
        for k, v in kw.items():
            if not hasattr(c, k):
                raise KeyError(k)
            setattr(c, k, v)
        return c

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def default_config(**kw) -> Config:
    """RenderConfig defaults (core/config.h:27-48) with overrides."""
    c = Config()
    c.rpf_tile_size = 8
    c.rpf_shrinkage_scale = 1.0
    c.rpf_confidence_samples = 128.0
    c.color_window_radius = 7
    c.color_normal_threshold = 0.5
    c.color_depth_threshold = 0.25
    c.color_compat_alpha = 0.05
    c.color_sigma_max = 6.0
    c.var_window_radius = 1
    c.var_normal_threshold = 0.5
    c.var_depth_threshold = 0.25
    c.var_compat_sigma = 30.0
    c.var_shrinkage_k = 1e-3
    c.var_iterations = 2
    c.adaptive_base_samples = 0
    c.adaptive_spp = 0
    c.adaptive_sigma_max = 3.0
    c.adaptive_passes = 1
    c.adaptive_importance_smoothing_radius = 1
    c.debug_statmc_outputs = 0
    c.seed = 0
    return c.replace(**kw) if kw else c


class SampleSoA(C.Structure):
    """rpd_sample_soa (all planes as raw pointers)."""
    _fields_ = [
        ("radiance", C.c_void_p * 3), ("normal", C.c_void_p * 3), ("depth", C.c_void_p),
        ("albedo", C.c_void_p * 3), ("pixel_albedo", C.c_void_p * 3), ("pixel_u", C.c_void_p * 2),
        ("lens_u", C.c_void_p * 2), ("brdf_u", C.c_void_p * 2), ("light_u", C.c_void_p * 2),
        ("env_u", C.c_void_p * 2), ("flags", C.c_void_p), ("category", C.c_void_p),
    ]


class SampleSoA16(C.Structure):
    """rpd_sample_soa16: the compact per-sample record (precision form)."""
    _fields_ = [
        ("sqrt_radiance", C.c_void_p * 3), ("normal", C.c_void_p * 3), ("depth", C.c_void_p),
        ("pixel_albedo", C.c_void_p * 3), ("pixel_u", C.c_void_p * 2), ("lens_u", C.c_void_p * 2),
        ("brdf_u", C.c_void_p * 2), ("light_u", C.c_void_p * 2), ("env_u", C.c_void_p * 2),
        ("flags", C.c_void_p), ("category", C.c_void_p), ("depth_scale", C.c_float),
    ]


class ImageMetrics(C.Structure):
    """rpd_image_metrics: what `eval_tools hdr-metrics` reports (shared/tools/eval_tools.cpp)."""
    _fields_ = [("mae", C.c_double), ("rmse", C.c_double), ("psnr", C.c_double), ("peak", C.c_double),
                ("ssim", C.c_double * 3), ("ssim_mean", C.c_double), ("nrmse", C.c_double),
                ("log_ssim11", C.c_double), ("log_gradient_nrmse", C.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "ssim"}
        d["ssim"] = list(self.ssim)
        return d


class SynthParams(C.Structure):
    """rpd_synth_params (include/rpd_synth.h)."""
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("seed", C.c_uint32), ("regions", C.c_int32),
        ("dependent_regions", C.c_int32), ("mu_min", C.c_float), ("mu_max", C.c_float), ("sigma", C.c_float),
        ("slope", C.c_float), ("firefly_rate", C.c_float), ("firefly_scale", C.c_float), ("lights", C.c_int32),
        ("miss_regions", C.c_int32), ("nan_rate", C.c_float),
    ]


class ServerConfig(C.Structure):
    """rpd_server_config."""
    _fields_ = [("knobs", Config), ("hbm_budget_bytes", C.c_uint64), ("max_inflight", C.c_int32),
                ("storage", C.c_int32), ("profile", C.c_int32), ("allocator_blocks", C.c_int32)]


class Request(C.Structure):
    """rpd_request."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("seed", C.c_uint32),
                ("denoised_out", C.c_void_p), ("out_where", C.c_int32), ("tag", C.c_uint64)]


class Completion(C.Structure):
    """rpd_completion."""
    _fields_ = [("id", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("spp", C.c_int32), ("samples", C.c_int64), ("submit_ms", C.c_double),
                ("admit_ms", C.c_double), ("done_ms", C.c_double)]


class ServerStats(C.Structure):
    """rpd_server_stats."""
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64), ("queued", C.c_int64),
                ("inflight", C.c_int64), ("bytes_reserved", C.c_uint64), ("bytes_peak", C.c_uint64),
                ("bytes_budget", C.c_uint64), ("jobs_cached", C.c_int64), ("now_ms", C.c_double),
                ("launches", C.c_int64), ("jobs_created", C.c_int64), ("jobs_destroyed", C.c_int64),
                ("scratch_grown", C.c_int64)]


STORAGE = {"fp32": 0, "fp16": 1}


def synth_params(width: int, height: int, seed: int, **kw) -> SynthParams:
    """Defaults of the full-size synthetic workload (rpd_synth_defaults)."""
    p = SynthParams(width=width, height=height, seed=seed, regions=48, dependent_regions=24, mu_min=-2.0,
                    mu_max=1.0, sigma=0.8, slope=0.5, firefly_rate=0.001, firefly_scale=100.0, lights=4,
                    miss_regions=0, nan_rate=0.0)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


# Sample planes: name -> (components, dtype, per) where per is "sample" or "pixel".
PLANES = {
    "radiance": (3, np.float32, "sample"), "normal": (3, np.float32, "sample"), "depth": (1, np.float32, "sample"),
    "albedo": (3, np.float32, "sample"), "pixel_albedo": (3, np.float32, "pixel"),
    "pixel_u": (2, np.float32, "sample"), "lens_u": (2, np.float32, "sample"), "brdf_u": (2, np.float32, "sample"),
    "light_u": (2, np.float32, "sample"), "env_u": (2, np.float32, "sample"), "flags": (1, np.uint8, "sample"),
    "category": (1, np.uint8, "sample"),
}


class HostSamples:
    """Per-sample planes in host memory (numpy), for pixels [first, first+count)."""

    def __init__(self, n_samples: int, n_pixels: int, planes: tuple[str, ...] | None = None):
        self.n_samples = int(n_samples)
        self.n_pixels = int(n_pixels)
        planes = planes or ("radiance", "normal", "depth", "pixel_albedo", "pixel_u", "lens_u", "brdf_u",
                            "light_u", "flags", "category")
        self.planes: dict[str, np.ndarray] = {}
        for name in planes:
            comps, dt, per = PLANES[name]
            n = self.n_samples if per == "sample" else self.n_pixels
            self.planes[name] = np.zeros((comps, n) if comps > 1 else (n,), dtype=dt)

    def soa(self) -> SampleSoA:
        s = SampleSoA()
        for name, arr in self.planes.items():
            comps = PLANES[name][0]
            if comps == 1:
                setattr(s, name, arr.ctypes.data)
            else:
                field = getattr(s, name)
                for c in range(comps):
                    field[c] = arr[c].ctypes.data
        return s

    def slice_pixels(self, offsets: np.ndarray, p0: int, p1: int) -> "HostSamples":
        """Samples of pixels [p0, p1) given per-pixel offsets (len n_pixels+1)."""
        k0, k1 = int(offsets[p0]), int(offsets[p1])
        out = HostSamples.__new__(HostSamples)
        out.n_samples, out.n_pixels = k1 - k0, p1 - p0
        out.planes = {}
        for name, arr in self.planes.items():
            per = PLANES[name][2]
            a, b = (k0, k1) if per == "sample" else (p0, p1)
            out.planes[name] = np.ascontiguousarray(arr[..., a:b])
        return out

    def concat(self, other: "HostSamples") -> "HostSamples":
        out = HostSamples.__new__(HostSamples)
        out.n_samples = self.n_samples + other.n_samples
        out.n_pixels = self.n_pixels + other.n_pixels
        out.planes = {k: np.concatenate([v, other.planes[k]], axis=-1) for k, v in self.planes.items()}
        return out

    @property
    def nbytes(self) -> int:
        return sum(a.nbytes for a in self.planes.values())


class RpdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    """Load librpd_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RpdError(8, f"{LIB_PATH} is missing; run __graft_entry__.build() first")
    L = C.CDLL(str(LIB_PATH))
    vp, i32, i64, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_float
    sig = {
        "rpd_config_defaults": (None, [C.POINTER(Config)]),
        "rpd_config_validate": (C.c_int, [C.POINTER(Config), C.c_char_p, C.c_size_t]),
        "rpd_ctx_create": (C.c_int, [C.c_int, u64, C.POINTER(vp)]),
        "rpd_ctx_destroy": (None, [vp]),
        "rpd_job_footprint": (u64, [C.POINTER(Config)]),
        "rpd_ctx_bytes_in_use": (u64, [vp]),
        "rpd_job_create": (C.c_int, [vp, C.POINTER(Config), C.POINTER(vp)]),
        "rpd_job_destroy": (None, [vp]),
        "rpd_job_set_config": (C.c_int, [vp, C.POINTER(Config)]),
        "rpd_job_set_exact": (C.c_int, [vp, C.c_int]),
        "rpd_job_set_tuning": (C.c_int, [vp, C.c_int, C.c_int]),
        "rpd_job_get_tuning": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int)]),
        "rpd_job_allocator_stats": (C.c_int, [vp, C.POINTER(C.c_int32)]),
        "rpd_adaptive_allocate": (C.c_int, [vp, vp, C.c_int, vp, C.c_int]),
        "rpd_job_allocator_timeline": (C.c_int, [vp, C.POINTER(C.c_uint64), i32, C.POINTER(i32)]),
        "rpd_job_begin_frame": (C.c_int, [vp]),
        "rpd_job_push_samples": (C.c_int, [vp, C.POINTER(SampleSoA), i64, i64, i32, vp, C.c_int]),
        "rpd_job_push_samples16": (C.c_int, [vp, C.POINTER(SampleSoA16), i64, i64, i32, vp, C.c_int]),
        "rpd_job_push_samples_async": (C.c_int, [vp, C.POINTER(SampleSoA), i64, i64, i32, vp]),
        "rpd_job_push_samples16_async": (C.c_int, [vp, C.POINTER(SampleSoA16), i64, i64, i32, vp]),
        "rpd_encode_samples16": (C.c_int, [vp, C.POINTER(SampleSoA), i64, i64, C.POINTER(SampleSoA16)]),
        "rpd_job_autotune": (C.c_int, [vp, C.POINTER(SampleSoA), C.POINTER(SampleSoA16), i32]),
        "rpd_batch_create": (C.c_int, [vp, C.POINTER(vp)]),
        "rpd_batch_add": (C.c_int, [vp, vp, C.POINTER(SampleSoA), C.POINTER(SampleSoA16), i32]),
        "rpd_batch_run": (C.c_int, [vp]),
        "rpd_batch_sync": (C.c_int, [vp]),
        "rpd_batch_last_ms": (C.c_int, [vp, C.POINTER(C.c_float)]),
        "rpd_batch_kernel_count": (u64, [vp]),
        "rpd_batch_set_lanes": (C.c_int, [vp, C.c_int]),
        "rpd_batch_destroy": (None, [vp]),
        "rpd_job_end_pass": (C.c_int, [vp]),
        "rpd_recompute_sensitivity": (C.c_int, [vp]),
        "rpd_statmc_denoise": (C.c_int, [vp]),
        "rpd_variance_denoise": (C.c_int, [vp]),
        "rpd_compute_adaptive_sample_counts": (C.c_int, [vp, vp, C.c_int]),
        "rpd_finalize": (C.c_int, [vp]),
        "rpd_job_read": (C.c_int, [vp, C.c_int, vp, C.c_size_t, C.c_int]),
        "rpd_job_read_async": (C.c_int, [vp, C.c_int, vp, C.c_size_t, C.c_int]),
        "rpd_field_bytes": (u64, [vp, C.c_int]),
        "rpd_job_sync": (C.c_int, [vp]),
        "rpd_job_stage_ms": (f32, [vp, C.c_int]),
        "rpd_job_launch_count": (u64, [vp]),
        "rpd_job_set_profiling": (C.c_int, [vp, C.c_int]),
        "rpd_job_kernel_time": (C.c_int, [vp, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
        "rpd_job_reset_kernel_times": (C.c_int, [vp]),
        "rpd_kernel_name": (C.c_char_p, [C.c_int]),
        "rpd_job_mark": (C.c_int, [vp, C.c_int]),
        "rpd_job_mark_elapsed": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]),
        "rpd_atrous_wavelet": (C.c_int, [vp, vp, vp, vp, i32, i32, f32, f32, f32, i32, vp, C.c_int]),
        "rpd_joint_bilateral": (C.c_int, [vp, vp, vp, vp, i32, i32, f32, f32, f32, f32, vp, vp, vp, C.c_int]),
        "rpd_atrous_wavelet_noalloc": (C.c_int, [vp, vp, vp, i32, i32, f32, f32, f32, i32, vp, vp]),
        "rpd_device_alloc": (C.c_int, [vp, u64, C.POINTER(vp)]),
        "rpd_device_free": (C.c_int, [vp, vp]),
        "rpd_host_alloc": (C.c_int, [u64, C.POINTER(vp)]),
        "rpd_host_free": (C.c_int, [vp]),
        "rpd_memcpy": (C.c_int, [vp, vp, vp, u64, C.c_int]),
        "rpd_synth_fill": (C.c_int, [vp, C.POINTER(SynthParams), i64, i64, i32, vp, vp, C.POINTER(SampleSoA),
                                     C.c_int]),
        "rpd_server_config_defaults": (None, [C.POINTER(ServerConfig)]),
        "rpd_server_create": (C.c_int, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "rpd_server_submit": (C.c_int, [vp, C.POINTER(Request), C.POINTER(C.c_uint64)]),
        "rpd_server_poll": (C.c_int, [vp, C.POINTER(Completion), i32, C.POINTER(i32)]),
        "rpd_server_drain": (C.c_int, [vp, i32]),
        "rpd_server_cancel": (C.c_int, [vp, u64]),
        "rpd_server_get_stats": (C.c_int, [vp, C.POINTER(ServerStats)]),
        "rpd_server_kernel_times": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
        "rpd_server_destroy": (None, [vp]),
        "rpd_job_counters": (C.c_int, [vp, C.POINTER(C.c_uint64), i32]),
        "rpd_hdr_metrics": (C.c_int, [vp, vp, vp, i32, i32, C.c_int, C.POINTER(ImageMetrics)]),
        "rpd_write_hdr": (C.c_int, [vp, vp, i32, i32, C.c_int, C.c_char_p]),
        "rpd_emitter_create": (C.c_int, [vp, i32, i32, i32, C.POINTER(vp)]),
        "rpd_emitter_begin_pass": (C.c_int, [vp, i32, vp]),
        "rpd_emitter_row": (C.c_int, [vp, i32, C.POINTER(SampleSoA), C.POINTER(C.POINTER(C.c_int64))]),
        "rpd_emitter_row_done": (C.c_int, [vp, i32]),
        "rpd_emitter_end_pass": (C.c_int, [vp]),
        "rpd_emitter_destroy": (None, [vp]),
        "rpd_write_png": (C.c_int, [vp, vp, i32, i32, C.c_int, C.c_int, C.c_char_p]),
        "rpd_job_write_outputs": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_int]),
        "rpd_job_hdr_metrics": (C.c_int, [vp, vp, C.c_int, C.POINTER(ImageMetrics)]),
        "rpd_probe_fp32_issue": (C.c_int, [C.c_int, i32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "rpd_last_error": (C.c_char_p, []),
        "rpd_status_string": (C.c_char_p, [C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names declared in include/rpd_gb300.h that the library must export."""
    return ["rpd_config_defaults", "rpd_config_validate", "rpd_ctx_create", "rpd_ctx_destroy", "rpd_job_footprint",
            "rpd_ctx_bytes_in_use", "rpd_job_create", "rpd_job_destroy", "rpd_job_set_config", "rpd_job_set_exact",
            "rpd_job_set_tuning", "rpd_job_get_tuning", "rpd_job_allocator_stats", "rpd_adaptive_allocate", "rpd_job_allocator_timeline",
            "rpd_server_config_defaults", "rpd_server_create", "rpd_server_submit", "rpd_server_poll",
            "rpd_server_drain", "rpd_server_cancel", "rpd_server_get_stats", "rpd_server_kernel_times",
            "rpd_server_destroy",
            "rpd_job_begin_frame", "rpd_job_push_samples", "rpd_job_push_samples16", "rpd_job_push_samples_async",
            "rpd_job_push_samples16_async", "rpd_encode_samples16",
            "rpd_job_autotune", "rpd_batch_create", "rpd_batch_add", "rpd_batch_run", "rpd_batch_sync",
            "rpd_batch_last_ms", "rpd_batch_kernel_count", "rpd_batch_set_lanes", "rpd_batch_destroy", "rpd_job_end_pass", "rpd_recompute_sensitivity",
            "rpd_statmc_denoise", "rpd_variance_denoise", "rpd_compute_adaptive_sample_counts", "rpd_finalize",
            "rpd_job_read", "rpd_job_read_async", "rpd_field_bytes", "rpd_job_sync", "rpd_job_stage_ms", "rpd_job_launch_count",
            "rpd_job_set_profiling", "rpd_job_kernel_time", "rpd_job_reset_kernel_times", "rpd_kernel_name",
            "rpd_job_mark", "rpd_job_mark_elapsed",
            "rpd_atrous_wavelet", "rpd_joint_bilateral", "rpd_atrous_wavelet_noalloc", "rpd_device_alloc", "rpd_device_free", "rpd_host_alloc",
            "rpd_host_free", "rpd_memcpy", "rpd_synth_fill", "rpd_last_error", "rpd_status_string",
            "rpd_job_counters", "rpd_probe_fp32_issue", "rpd_hdr_metrics", "rpd_job_hdr_metrics",
            "rpd_write_hdr", "rpd_write_png", "rpd_job_write_outputs", "rpd_emitter_create",
            "rpd_emitter_begin_pass", "rpd_emitter_row", "rpd_emitter_row_done", "rpd_emitter_end_pass",
            "rpd_emitter_destroy"]


def check(status: int) -> None:
    if status != OK:
        raise RpdError(status, lib().rpd_last_error().decode(errors="replace"))


def validate(cfg: Config) -> tuple[int, str]:
    buf = C.create_string_buffer(256)
    st = lib().rpd_config_validate(C.byref(cfg), buf, 256)
    return st, buf.value.decode()


def node_dims(cfg: Config) -> tuple[int, int]:
    step = max(1, cfg.rpf_tile_size // 2)
    nx = max(2, (cfg.image_width + step - 1) // step + 1)
    ny = max(2, (cfg.image_height + step - 1) // step + 1)
    return nx, ny


def field_shape(cfg: Config, name: str) -> tuple[tuple[int, ...], type]:
    w, h = cfg.image_width, cfg.image_height
    nx, ny = node_dims(cfg)
    if name == "GRID":
        return (ny * nx, GRID_DEPS, GRID_STRIDE), np.float64
    if name.startswith("NODE_"):
        return (ny, nx), np.float32
    dt = np.int32 if name in INT_FIELDS else np.float32
    if name in RGB_FIELDS:
        return (h, w, 3), dt
    return (h, w), dt


class DeviceBuffer:
    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        check(lib().rpd_device_alloc(ctx.handle, self.nbytes, C.byref(p)))
        self.ptr = p.value

    def free(self) -> None:
        if self.ptr:
            check(lib().rpd_device_free(self.ctx.handle, self.ptr))
            self.ptr = None

    def upload(self, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        check(lib().rpd_memcpy(self.ctx.handle, self.ptr, a.ctypes.data, a.nbytes, 0))

    def download(self, arr: np.ndarray) -> np.ndarray:
        assert arr.flags.c_contiguous and arr.nbytes <= self.nbytes
        check(lib().rpd_memcpy(self.ctx.handle, arr.ctypes.data, self.ptr, arr.nbytes, 1))
        return arr


class DeviceSamples:
    """Per-sample planes in HBM (one device buffer per plane component)."""

    def __init__(self, ctx: "Context", n_samples: int, n_pixels: int, planes: tuple[str, ...] | None = None):
        self.ctx = ctx
        self.n_samples, self.n_pixels = int(n_samples), int(n_pixels)
        planes = planes or ("radiance", "normal", "depth", "pixel_albedo", "pixel_u", "lens_u", "brdf_u", "light_u",
                            "flags", "category")
        self.bufs: dict[str, list[DeviceBuffer]] = {}
        for name in planes:
            comps, dt, per = PLANES[name]
            n = self.n_samples if per == "sample" else self.n_pixels
            self.bufs[name] = [DeviceBuffer(ctx, max(1, n) * np.dtype(dt).itemsize) for _ in range(comps)]

    @classmethod
    def from_host(cls, ctx: "Context", host: HostSamples) -> "DeviceSamples":
        d = cls(ctx, host.n_samples, host.n_pixels, tuple(host.planes))
        for name, arr in host.planes.items():
            comps = PLANES[name][0]
            for c in range(comps):
                d.bufs[name][c].upload(arr[c] if comps > 1 else arr)
        return d

    def soa(self) -> SampleSoA:
        s = SampleSoA()
        for name, bl in self.bufs.items():
            if len(bl) == 1 and PLANES[name][0] == 1:
                setattr(s, name, bl[0].ptr)
            else:
                field = getattr(s, name)
                for c, b in enumerate(bl):
                    field[c] = b.ptr
        return s

    @property
    def nbytes(self) -> int:
        total = 0
        for name in self.bufs:
            comps, dt, per = PLANES[name]
            n = self.n_samples if per == "sample" else self.n_pixels
            total += comps * n * np.dtype(dt).itemsize
        return total

    def free(self) -> None:
        for bl in self.bufs.values():
            for b in bl:
                b.free()
        self.bufs = {}


# Compact planes: name -> (components, dtype, per)
PLANES16 = {
    "sqrt_radiance": (3, np.uint16, "sample"), "normal": (3, np.int16, "sample"), "depth": (1, np.uint16, "sample"),
    "pixel_albedo": (3, np.uint16, "pixel"), "pixel_u": (2, np.uint16, "sample"), "lens_u": (2, np.uint16, "sample"),
    "brdf_u": (2, np.uint16, "sample"), "light_u": (2, np.uint16, "sample"), "env_u": (2, np.uint16, "sample"),
    "flags": (1, np.uint8, "sample"), "category": (1, np.uint8, "sample"),
}
# the compact planes that carry a given rpd_sample_soa plane
FROM32 = {"radiance": "sqrt_radiance", "normal": "normal", "depth": "depth", "pixel_albedo": "pixel_albedo",
          "pixel_u": "pixel_u", "lens_u": "lens_u", "brdf_u": "brdf_u", "light_u": "light_u", "env_u": "env_u",
          "flags": "flags", "category": "category"}


class DeviceSamples16:
    """rpd_sample_soa16 planes in HBM (the precision form's storage)."""

    def __init__(self, ctx: "Context", n_samples: int, n_pixels: int, planes: tuple[str, ...], depth_scale=1.0):
        self.ctx = ctx
        self.n_samples, self.n_pixels = int(n_samples), int(n_pixels)
        self.depth_scale = float(depth_scale)
        self.bufs: dict[str, list[DeviceBuffer]] = {}
        for name in planes:
            comps, dt, per = PLANES16[name]
            n = self.n_samples if per == "sample" else self.n_pixels
            self.bufs[name] = [DeviceBuffer(ctx, max(1, n) * np.dtype(dt).itemsize) for _ in range(comps)]

    @classmethod
    def encode(cls, ctx: "Context", dev: "DeviceSamples", depth_scale: float = 1.0) -> "DeviceSamples16":
        """rpd_encode_samples16 of device-resident FP32 planes; flags/category are copied."""
        planes = tuple(FROM32[n] for n in dev.bufs if n in FROM32)
        out = cls(ctx, dev.n_samples, dev.n_pixels, planes, depth_scale)
        check(lib().rpd_encode_samples16(ctx.handle, C.byref(dev.soa()), dev.n_samples, dev.n_pixels,
                                         C.byref(out.soa())))
        for name in ("flags", "category"):
            if name in dev.bufs:
                src, dst = dev.bufs[name][0], out.bufs[name][0]
                check(lib().rpd_memcpy(ctx.handle, dst.ptr, src.ptr, dev.n_samples, 2))
        return out

    def soa(self) -> SampleSoA16:
        s = SampleSoA16()
        for name, bl in self.bufs.items():
            if PLANES16[name][0] == 1:
                setattr(s, name, bl[0].ptr)
            else:
                field = getattr(s, name)
                for c, b in enumerate(bl):
                    field[c] = b.ptr
        s.depth_scale = self.depth_scale
        return s

    @property
    def nbytes(self) -> int:
        total = 0
        for name in self.bufs:
            comps, dt, per = PLANES16[name]
            n = self.n_samples if per == "sample" else self.n_pixels
            total += comps * n * np.dtype(dt).itemsize
        return total

    def free(self) -> None:
        for bl in self.bufs.values():
            for b in bl:
                b.free()
        self.bufs = {}


class Context:
    """rpd_ctx: one GPU and the HBM budget jobs are admitted against."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        h = C.c_void_p()
        check(lib().rpd_ctx_create(device, budget_bytes, C.byref(h)))
        self.handle = h.value

    def close(self) -> None:
        if self.handle:
            lib().rpd_ctx_destroy(self.handle)
            self.handle = None

    def bytes_in_use(self) -> int:
        return int(lib().rpd_ctx_bytes_in_use(self.handle))

    def synth_fill(self, params: SynthParams, first: int, count: int, spp: int, out, counts=None, start_n=None):
        """Fill HostSamples or DeviceSamples with synthetic samples."""
        where = MEM_DEVICE if isinstance(out, DeviceSamples) else MEM_HOST
        s = out.soa()
        cp = counts.ctypes.data if isinstance(counts, np.ndarray) else (counts.ptr if counts is not None else None)
        sp = start_n.ctypes.data if isinstance(start_n, np.ndarray) else (start_n.ptr if start_n is not None else None)
        check(lib().rpd_synth_fill(self.handle, C.byref(params), first, count, spp, cp, sp, C.byref(s), where))

    def atrous(self, raw, normal, albedo, sigma_c, sigma_n, sigma_a, iterations):
        h, w, _ = raw.shape
        out = np.empty_like(raw, dtype=np.float32)
        args = [np.ascontiguousarray(a, dtype=np.float32) for a in (raw, normal, albedo)]
        check(lib().rpd_atrous_wavelet(self.handle, *[a.ctypes.data for a in args], w, h, sigma_c, sigma_n, sigma_a,
                                       iterations, out.ctypes.data, MEM_HOST))
        return out

    def hdr_metrics(self, reference: np.ndarray, test: np.ndarray) -> dict:
        """rpd_hdr_metrics of two (H, W, 3) float images in host memory."""
        h, w, _ = reference.shape
        a = np.ascontiguousarray(reference, dtype=np.float32)
        b = np.ascontiguousarray(test, dtype=np.float32)
        m = ImageMetrics()
        check(lib().rpd_hdr_metrics(self.handle, a.ctypes.data, b.ctypes.data, w, h, MEM_HOST, C.byref(m)))
        return m.as_dict()

    def joint_bilateral(self, raw, normal, albedo, sigma_c, sigma_n, sigma_p, sigma_a):
        h, w, _ = raw.shape
        outs = [np.empty((h, w, 3), dtype=np.float32) for _ in range(3)]
        args = [np.ascontiguousarray(a, dtype=np.float32) for a in (raw, normal, albedo)]
        check(lib().rpd_joint_bilateral(self.handle, *[a.ctypes.data for a in args], w, h, sigma_c, sigma_n, sigma_p,
                                        sigma_a, *[o.ctypes.data for o in outs], MEM_HOST))
        return tuple(outs)


NOALLOC_MAX_PIXELS = 4194304  # RPD_NOALLOC_MAX_PIXELS


def atrous_noalloc(raw: "DeviceBuffer", normal: "DeviceBuffer", albedo: "DeviceBuffer", w: int, h: int,
                   sigma_c: float, sigma_n: float, sigma_a: float, iterations: int, out: "DeviceBuffer",
                   stream: int = 0) -> None:
    """rpd_atrous_wavelet_noalloc on device buffers; asynchronous on `stream` (0: default)."""
    check(lib().rpd_atrous_wavelet_noalloc(raw.ptr, normal.ptr, albedo.ptr, w, h, sigma_c, sigma_n, sigma_a,
                                           iterations, out.ptr, stream or None))


def _frame_args(samples):
    if isinstance(samples, DeviceSamples16):
        return None, C.byref(samples.soa())
    return C.byref(samples.soa()), None


class Batch:
    """rpd_batch: frames of several jobs captured into one CUDA graph."""

    def __init__(self, ctx: "Context"):
        h = C.c_void_p()
        check(lib().rpd_batch_create(ctx.handle, C.byref(h)))
        self.handle = h.value
        self.keep = []

    def add(self, job: "Job", samples, spp: int) -> None:
        s32, s16 = _frame_args(samples)
        self.keep.append(samples)
        check(lib().rpd_batch_add(self.handle, job.handle, s32, s16, spp))

    def run(self) -> None:
        check(lib().rpd_batch_run(self.handle))

    def sync(self) -> None:
        check(lib().rpd_batch_sync(self.handle))

    def last_ms(self) -> float:
        v = C.c_float()
        check(lib().rpd_batch_last_ms(self.handle, C.byref(v)))
        return float(v.value)

    def kernel_count(self) -> int:
        return int(lib().rpd_batch_kernel_count(self.handle))

    def set_lanes(self, lanes: int) -> None:
        check(lib().rpd_batch_set_lanes(self.handle, int(lanes)))

    def close(self) -> None:
        if self.handle:
            lib().rpd_batch_destroy(self.handle)
            self.handle = None


class Job:
    """rpd_job: one frame's state in HBM and the reference's stage entry points."""

    def __init__(self, ctx: Context, cfg: Config):
        self.ctx = ctx
        self.cfg = cfg
        h = C.c_void_p()
        check(lib().rpd_job_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value

    def close(self) -> None:
        if self.handle:
            lib().rpd_job_destroy(self.handle)
            self.handle = None

    def set_config(self, cfg: Config) -> None:
        check(lib().rpd_job_set_config(self.handle, C.byref(cfg)))
        self.cfg = cfg.replace(image_width=self.cfg.image_width, image_height=self.cfg.image_height,
                               rpf_tile_size=self.cfg.rpf_tile_size)

    def set_exact(self, grid: bool = False, window: bool = False) -> None:
        check(lib().rpd_job_set_exact(self.handle, (1 if grid else 0) | (2 if window else 0)))

    TUNING = {"grid_shape": 0, "host_band_mb": 1, "statmc_rows": 2, "allocator": 3, "smoothing": 4, "window_guard": 5}

    def autotune(self, samples, spp: int) -> None:
        """rpd_job_autotune on device-resident planes (leaves the frame denoised)."""
        s32, s16 = _frame_args(samples)
        check(lib().rpd_job_autotune(self.handle, s32, s16, spp))

    def set_tuning(self, knob: str, value: int) -> None:
        check(lib().rpd_job_set_tuning(self.handle, self.TUNING[knob], int(value)))

    def get_tuning(self, knob: str) -> int:
        v = C.c_int()
        check(lib().rpd_job_get_tuning(self.handle, self.TUNING[knob], C.byref(v)))
        return v.value

    def adaptive_allocate(self, importance: np.ndarray) -> np.ndarray:
        """rpd_adaptive_allocate on a host importance map; returns the counts."""
        imp = np.ascontiguousarray(importance, dtype=np.float32).ravel()
        out = np.empty(self.cfg.image_width * self.cfg.image_height, dtype=np.int32)
        if imp.size != out.size:
            raise ValueError("importance map size does not match the frame")
        check(lib().rpd_adaptive_allocate(self.handle, imp.ctypes.data, MEM_HOST, out.ctypes.data, MEM_HOST))
        return out

    def allocator_timeline(self) -> list[float]:
        """Microseconds from the last parallel allocation's launch to each of its barriers."""
        buf = (C.c_uint64 * 96)()
        n = C.c_int32()
        check(lib().rpd_job_allocator_timeline(self.handle, buf, 96, C.byref(n)))
        return [buf[i] / 1e3 for i in range(n.value)]

    def allocator_stats(self) -> dict:
        """Outcome of the last adaptive allocation (rpd_job_allocator_stats)."""
        out = (C.c_int32 * 7)()
        check(lib().rpd_job_allocator_stats(self.handle, out))
        keys = ("parallel_done", "fallback", "timeout", "passes", "rounds", "exact_chunks", "reason")
        return dict(zip(keys, (int(v) for v in out)))

    def begin_frame(self) -> None:
        check(lib().rpd_job_begin_frame(self.handle))

    def push(self, samples, first: int, count: int, spp: int = 0, counts=None) -> None:
        if isinstance(samples, DeviceSamples16):
            return self.push16(samples, first, count, spp, counts)
        where = MEM_DEVICE if isinstance(samples, DeviceSamples) else MEM_HOST
        s = samples.soa()
        if counts is None:
            cp = None
        elif isinstance(counts, np.ndarray):
            counts = np.ascontiguousarray(counts, dtype=np.int32)
            cp = counts.ctypes.data
        else:
            cp = counts.ptr
        check(lib().rpd_job_push_samples(self.handle, C.byref(s), first, count, spp, cp, where))

    def push_async(self, samples, first: int, count: int, spp: int = 0, counts_ptr=None) -> None:
        """rpd_job_push_samples_async (or its compact form, by the type of samples.soa()) of
        page-locked host planes (rpd_host_alloc memory, as are the counts at counts_ptr if given):
        the copies run after the call returns, so the planes must stay unchanged until sync()."""
        s = samples.soa()
        if isinstance(s, SampleSoA16):
            check(lib().rpd_job_push_samples16_async(self.handle, C.byref(s), first, count, spp, counts_ptr))
        else:
            check(lib().rpd_job_push_samples_async(self.handle, C.byref(s), first, count, spp, counts_ptr))

    def push16(self, samples, first: int, count: int, spp: int = 0, counts=None, where: int = MEM_DEVICE) -> None:
        """rpd_job_push_samples16 of compact planes (device-resident unless `where` says host)."""
        if where == MEM_HOST:
            cp = None if counts is None else np.ascontiguousarray(counts, dtype=np.int32)
            check(lib().rpd_job_push_samples16(self.handle, C.byref(samples.soa()), first, count, spp,
                                               None if cp is None else cp.ctypes.data, MEM_HOST))
            return
        if counts is None:
            cp = None
        elif isinstance(counts, np.ndarray):
            counts = np.ascontiguousarray(counts, dtype=np.int32)
            cp = counts.ctypes.data
        else:
            cp = counts.ptr
        if isinstance(counts, np.ndarray):
            # device planes with host counts: stage the counts on the device
            buf = DeviceBuffer(self.ctx, max(1, counts.nbytes))
            buf.upload(counts)
            try:
                check(lib().rpd_job_push_samples16(self.handle, C.byref(samples.soa()), first, count, spp, buf.ptr,
                                                   MEM_DEVICE))
                self.sync()
            finally:
                buf.free()
            return
        check(lib().rpd_job_push_samples16(self.handle, C.byref(samples.soa()), first, count, spp, cp, MEM_DEVICE))

    def end_pass(self) -> None:
        check(lib().rpd_job_end_pass(self.handle))

    def recompute_sensitivity(self) -> None:
        check(lib().rpd_recompute_sensitivity(self.handle))

    def statmc_denoise(self) -> None:
        check(lib().rpd_statmc_denoise(self.handle))

    def variance_denoise(self) -> None:
        check(lib().rpd_variance_denoise(self.handle))

    def compute_adaptive_sample_counts(self) -> np.ndarray:
        out = np.empty(self.cfg.image_width * self.cfg.image_height, dtype=np.int32)
        check(lib().rpd_compute_adaptive_sample_counts(self.handle, out.ctypes.data, MEM_HOST))
        return out

    def finalize(self) -> None:
        check(lib().rpd_finalize(self.handle))

    def sync(self) -> None:
        check(lib().rpd_job_sync(self.handle))

    def read(self, name: str) -> np.ndarray:
        shape, dt = field_shape(self.cfg, name)
        out = np.empty(shape, dtype=dt)
        check(lib().rpd_job_read(self.handle, FIELD[name], out.ctypes.data, out.nbytes, MEM_HOST))
        return out

    def stage_ms(self, stage: str) -> float:
        return float(lib().rpd_job_stage_ms(self.handle, STAGE[stage]))

    def launches(self) -> int:
        return int(lib().rpd_job_launch_count(self.handle))

    def mark(self, slot: int) -> None:
        check(lib().rpd_job_mark(self.handle, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        check(lib().rpd_job_mark_elapsed(self.handle, a, b, C.byref(ms)))
        return float(ms.value)

    def set_profiling(self, on: bool) -> None:
        check(lib().rpd_job_set_profiling(self.handle, 1 if on else 0))

    def reset_kernel_times(self) -> None:
        check(lib().rpd_job_reset_kernel_times(self.handle))

    def kernel_times(self) -> dict[str, tuple[float, int]]:
        """{kernel family: (total ms, launches)} since the last reset."""
        out = {}
        for i, name in enumerate(KERNELS):
            ms, n = C.c_double(), C.c_uint64()
            check(lib().rpd_job_kernel_time(self.handle, i, C.byref(ms), C.byref(n)))
            out[name] = (ms.value, n.value)
        return out

    def hdr_metrics(self, reference: np.ndarray) -> dict:
        """rpd_job_hdr_metrics: the job's denoised image against a (H, W, 3) host reference."""
        a = np.ascontiguousarray(reference, dtype=np.float32)
        m = ImageMetrics()
        check(lib().rpd_job_hdr_metrics(self.handle, a.ctypes.data, MEM_HOST, C.byref(m)))
        return m.as_dict()

    def counters(self) -> dict[str, int]:
        """The job's device counters (rpd_counter): the StatMC window's double-precision
        rechecks and slow-pass pixels of the last statmc_denoise, and the device waits that
        gave up."""
        out = (C.c_uint64 * 8)()
        check(lib().rpd_job_counters(self.handle, out, 8))
        return {"window_pair_rechecks": int(out[0]), "window_pixel_rechecks": int(out[1]),
                "device_wait_timeouts": int(out[2]), "window_slow_pixels": int(out[3])}


class Server:
    """rpd_server: the serving loop (continuous batching of denoise requests)."""

    def __init__(self, ctx: Context, knobs: Config, budget_bytes: int = 0, max_inflight: int = 16,
                 storage: str = "fp16", profile: bool = False, allocator_blocks: int = 0):
        cfg = ServerConfig()
        lib().rpd_server_config_defaults(C.byref(cfg))
        cfg.knobs = knobs
        cfg.hbm_budget_bytes = budget_bytes
        cfg.max_inflight = max_inflight
        cfg.storage = STORAGE[storage]
        cfg.profile = 1 if profile else 0
        cfg.allocator_blocks = allocator_blocks
        h = C.c_void_p()
        check(lib().rpd_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value

    def submit(self, width: int, height: int, spp: int, seed: int, out=None, tag: int = 0) -> int:
        """Queue a request; `out` is a pinned host or device buffer of width*height*3 floats
        (a DeviceBuffer, or an integer address of pinned memory), or None."""
        r = Request()
        r.width, r.height, r.spp, r.seed, r.tag = width, height, spp, seed & 0xFFFFFFFF, tag
        if isinstance(out, DeviceBuffer):
            r.denoised_out, r.out_where = out.ptr, MEM_DEVICE
        elif out is not None:
            r.denoised_out, r.out_where = int(out), MEM_HOST
        rid = C.c_uint64()
        check(lib().rpd_server_submit(self.handle, C.byref(r), C.byref(rid)))
        return rid.value

    def poll(self, max_n: int = 256) -> list[dict]:
        buf = (Completion * max_n)()
        n = C.c_int32()
        check(lib().rpd_server_poll(self.handle, buf, max_n, C.byref(n)))
        keys = [f for f, _ in Completion._fields_]
        return [{k: getattr(buf[i], k) for k in keys} for i in range(n.value)]

    def drain(self, timeout_ms: int = -1) -> None:
        check(lib().rpd_server_drain(self.handle, timeout_ms))

    def cancel(self, rid: int) -> None:
        check(lib().rpd_server_cancel(self.handle, rid))

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().rpd_server_get_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def kernel_times(self) -> dict[str, tuple[float, int]]:
        """{kernel family: (summed ms, launches)} over finished requests (profile=True)."""
        ms = (C.c_double * len(KERNELS))()
        n = (C.c_uint64 * len(KERNELS))()
        check(lib().rpd_server_kernel_times(self.handle, ms, n))
        return {name: (ms[i], int(n[i])) for i, name in enumerate(KERNELS)}

    def close(self) -> None:
        if self.handle:
            lib().rpd_server_destroy(self.handle)
            self.handle = None



# The planes the serving loop generates per sample (plus the per-pixel albedo).
SERVED_PLANES = ("radiance", "normal", "depth", "pixel_albedo", "pixel_u", "lens_u", "brdf_u", "light_u", "flags",
                 "category")


def plain_request(ctx: Context, knobs: Config, width: int, height: int, spp: int, seed: int,
                  job: "Job | None" = None, skip_dead: bool = False) -> tuple[np.ndarray, int]:
    """One synthetic request through the plain per-frame drop-in: render()'s call sequence
    (path_tracer/main.cpp:1543-1564) on one job from the host, FP32 planes generated on the
    device with the same ordinals the serving loop draws (first pass 0..spp-1, adaptive pass p
    from p << 16), the adaptive counts read back to the host as compute_adaptive_sample_counts
    returns them. Returns the denoised image (H, W, 3) and the samples denoised.

    skip_dead: leave out the calls whose results nothing reads before they are overwritten —
    the adaptive passes' statmc_denoise and recompute_sensitivity and the final variance_denoise —
    as the serving loop does (the denoised image is the same bits)."""
    cfg = knobs.replace(image_width=width, image_height=height)
    n = width * height
    passes = cfg.adaptive_passes if cfg.adaptive_spp > 0 else 0
    own = job is None
    if own:
        job = Job(ctx, cfg)
    dev = DeviceSamples(ctx, n * max(spp, cfg.adaptive_spp if passes else 0, 1), n, planes=SERVED_PLANES)
    counts_dev = DeviceBuffer(ctx, n * 4)
    start_dev = DeviceBuffer(ctx, n * 4)
    try:
        params = synth_params(width, height, seed)
        samples = n * spp
        ctx.synth_fill(params, 0, n, spp, dev)
        job.begin_frame()
        job.push(dev, 0, n, spp)
        job.end_pass()
        job.recompute_sensitivity()
        for p in range(1, passes + 1):
            if not skip_dead:
                job.statmc_denoise()
            job.variance_denoise()
            counts = job.compute_adaptive_sample_counts()
            samples += int(counts.sum())
            counts_dev.upload(counts)
            start_dev.upload(np.full(n, p << 16, dtype=np.int32))
            ctx.synth_fill(params, 0, n, 0, dev, counts=counts_dev, start_n=start_dev)
            job.push(dev, 0, n, 0, counts=counts_dev)
            job.end_pass()
            if not skip_dead:
                job.recompute_sensitivity()
        job.recompute_sensitivity()
        job.statmc_denoise()
        if not skip_dead:
            job.variance_denoise()
        job.finalize()
        return job.read("DENOISED"), samples
    finally:
        dev.free()
        counts_dev.free()
        start_dev.free()
        if own:
            job.close()


class Emitter:
    """rpd_emitter: a tracer's per-sample records streamed to a job band by band."""

    PLANES = {"radiance": 3, "normal": 3, "albedo": 3, "pixel_u": 2, "lens_u": 2, "brdf_u": 2, "light_u": 2,
              "env_u": 2}

    def __init__(self, job: "Job", band_rows: int, ring_slots: int, max_spp: int):
        self.job = job
        self.handle = C.c_void_p()
        check(lib().rpd_emitter_create(job.handle, band_rows, ring_slots, max_spp, C.byref(self.handle)))

    def close(self) -> None:
        if self.handle:
            lib().rpd_emitter_destroy(self.handle)
            self.handle = C.c_void_p()

    def begin_pass(self, spp: int = 0, counts: np.ndarray | None = None) -> None:
        self._counts = None if counts is None else np.ascontiguousarray(counts, dtype=np.int32)
        check(lib().rpd_emitter_begin_pass(self.handle, spp, None if self._counts is None else self._counts.ctypes.data))

    def write_row(self, y: int, samples: "HostSamples") -> None:
        """Row y's samples (all pixels of the row, pixel-major) copied into the ring."""
        soa = SampleSoA()
        offs = C.POINTER(C.c_int64)()
        check(lib().rpd_emitter_row(self.handle, y, C.byref(soa), C.byref(offs)))
        n = samples.n_samples
        planes = dict(samples.planes)
        if "albedo" not in planes and "pixel_albedo" in planes:
            # a pixel's albedo for each of its samples (the record carries albedo per sample)
            w = samples.n_pixels
            counts = np.diff(np.array([offs[x] - offs[0] for x in range(w + 1)], dtype=np.int64))
            planes["albedo"] = np.stack([np.repeat(planes["pixel_albedo"][c], counts) for c in range(3)])
        for name, comps in self.PLANES.items():
            src = planes.get(name)
            dst = getattr(soa, name)
            for c in range(comps):
                if src is None:
                    C.memset(dst[c], 0, 4 * n)
                else:
                    C.memmove(dst[c], np.ascontiguousarray(src[c], dtype=np.float32).ctypes.data, 4 * n)
        for name in ("depth", "flags", "category"):
            src = np.ascontiguousarray(samples.planes[name])
            C.memmove(getattr(soa, name), src.ctypes.data, src.nbytes)
        check(lib().rpd_emitter_row_done(self.handle, y))

    def end_pass(self) -> None:
        check(lib().rpd_emitter_end_pass(self.handle))


def probe_fp32_issue(device: int = 0, repeats: int = 5) -> dict:
    """FP32 lane instructions per second the device issues (rpd_probe_fp32_issue)."""
    rate, ms = C.c_double(), C.c_double()
    check(lib().rpd_probe_fp32_issue(device, repeats, C.byref(rate), C.byref(ms)))
    return {"per_second": rate.value, "ms": ms.value}


class PinnedBuffer:
    """Page-locked host memory (rpd_host_alloc) viewed as a numpy array."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        check(lib().rpd_host_alloc(int(nbytes), C.byref(p)))
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def array(self, dtype=np.float32, shape=None) -> np.ndarray:
        n = self.nbytes // np.dtype(dtype).itemsize
        buf = (C.c_char * self.nbytes).from_address(self.ptr)
        a = np.frombuffer(buf, dtype=dtype, count=n)
        return a.reshape(shape) if shape is not None else a

    def free(self) -> None:
        if self.ptr:
            lib().rpd_host_free(self.ptr)
            self.ptr = None
