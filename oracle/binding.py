"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

Two CPU implementations of the denoise stage with the same call sequence as the product
(include/rpd_gb300.h):

  OracleJob  the C restatement in oracle/rpd_oracle.c (built on every machine by
             `make -C oracle port`, loaded from oracle/_build/librpd_oracle.so)
  RefJob     the reference's own sources compiled against oracle/ref_shim
             (`make -C oracle ref`, oracle/_ref/librpdref.so; only where the reference
             checkout exists). Its state is the reference's process globals, so only one
             RefJob is live at a time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT / "rpd-statmc-denoiser_gb300"))
import rpd_gb300 as R  # noqa: E402  (structure definitions only; the CUDA library is not loaded)

PORT_LIB = HERE / "_build" / "librpd_oracle.so"
REF_LIB = HERE / "_ref" / "librpdref.so"

_port = None
_ref = None


def build_port() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE), "port"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return PORT_LIB


def port() -> C.CDLL:
    global _port
    if _port is not None:
        return _port
    if not PORT_LIB.exists():
        build_port()
    L = C.CDLL(str(PORT_LIB))
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    sig = {
        "orc_config_validate": (C.c_int, [C.POINTER(R.Config), C.c_char_p, C.c_size_t]),
        "orc_job_create": (vp, [C.POINTER(R.Config)]),
        "orc_job_destroy": (None, [vp]),
        "orc_set_threads": (None, [vp, C.c_int]),
        "orc_job_set_config": (C.c_int, [vp, C.POINTER(R.Config)]),
        "orc_job_begin_frame": (C.c_int, [vp]),
        "orc_job_push_samples": (C.c_int, [vp, C.POINTER(R.SampleSoA), i64, i64, i32, vp]),
        "orc_job_end_pass": (C.c_int, [vp]),
        "orc_recompute_sensitivity": (C.c_int, [vp]),
        "orc_statmc_denoise": (C.c_int, [vp]),
        "orc_variance_denoise": (C.c_int, [vp]),
        "orc_compute_adaptive_sample_counts": (C.c_int, [vp, vp]),
        "orc_allocate_counts_map": (None, [vp, i64, C.POINTER(R.Config), vp]),
        "orc_finalize": (C.c_int, [vp]),
        "orc_job_read": (C.c_int, [vp, C.c_int, vp, C.c_size_t]),
        "orc_stage_ms": (C.c_double, [vp, C.c_int]),
        "orc_atrous_wavelet": (C.c_int, [vp, vp, vp, i32, i32, f32, f32, f32, i32, vp, C.c_int]),
        "orc_joint_bilateral": (C.c_int, [vp, vp, vp, i32, i32, f32, f32, f32, f32, vp, vp, vp, C.c_int]),
        "orc_synth_fill": (i64, [C.POINTER(R.SynthParams), i64, i64, i32, vp, vp, C.POINTER(R.SampleSoA), C.c_int]),
        "orc_hdr_metrics": (C.c_int, [vp, vp, i32, i32, C.POINTER(R.ImageMetrics)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _port = L
    return L


_port64 = None
PORT64_LIB = HERE / "_build" / "librpd_oracle64.so"


def port64() -> C.CDLL:
    """The double-precision form of the restatement (oracle/rpd_oracle64.c)."""
    global _port64
    if _port64 is not None:
        return _port64
    if not PORT64_LIB.exists():
        build_port()
    L = C.CDLL(str(PORT64_LIB))
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    sig = {
        "orc_job_create": (vp, [C.POINTER(R.Config)]),
        "orc_job_destroy": (None, [vp]),
        "orc_set_threads": (None, [vp, C.c_int]),
        "orc_job_begin_frame": (C.c_int, [vp]),
        "orc_job_push_samples": (C.c_int, [vp, C.POINTER(R.SampleSoA), i64, i64, i32, vp]),
        "orc_job_end_pass": (C.c_int, [vp]),
        "orc_recompute_sensitivity": (C.c_int, [vp]),
        "orc_statmc_denoise": (C.c_int, [vp]),
        "orc_variance_denoise": (C.c_int, [vp]),
        "orc_finalize": (C.c_int, [vp]),
        "orc64_read": (C.c_int, [vp, C.c_int, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _port64 = L
    return L


def fp64_denoise(cfg: R.Config, samples: "R.HostSamples", spp: int, threads: int = 0) -> np.ndarray:
    """The plain method (accumulate, sensitivity, StatMC, variance) on one frame in the
    double-precision restatement; returns DENOISED (H, W, 3) as float."""
    L = port64()
    h = L.orc_job_create(C.byref(cfg))
    if not h:
        raise ValueError("invalid config")
    try:
        L.orc_set_threads(h, threads)
        L.orc_job_begin_frame(h)
        soa = samples.soa()
        n = cfg.image_width * cfg.image_height
        assert L.orc_job_push_samples(h, C.byref(soa), 0, n, spp, None) == 0
        L.orc_job_end_pass(h)
        L.orc_recompute_sensitivity(h)
        L.orc_statmc_denoise(h)
        L.orc_variance_denoise(h)
        out = np.empty((cfg.image_height, cfg.image_width, 3), dtype=np.float32)
        assert L.orc64_read(h, R.FIELD["DENOISED"], out.ctypes.data) == 0
        return out
    finally:
        L.orc_job_destroy(h)


def fp64_sequence(cfg: R.Config, pushes, threads: int = 0) -> np.ndarray:
    """render()'s adaptive sequence without its unread calls, in the double-precision
    restatement: pushes = [(HostSamples, spp, counts or None), ...], the first the base pass and
    each later one an adaptive pass's extra samples; recompute_sensitivity and statmc_denoise
    after the last pass. Returns DENOISED (H, W, 3) as float."""
    L = port64()
    h = L.orc_job_create(C.byref(cfg))
    if not h:
        raise ValueError("invalid config")
    n = cfg.image_width * cfg.image_height
    try:
        L.orc_set_threads(h, threads)
        L.orc_job_begin_frame(h)
        for samples, spp, counts in pushes:
            soa = samples.soa()
            c, cp = _counts_ptr(counts)
            assert L.orc_job_push_samples(h, C.byref(soa), 0, n, spp, cp) == 0
            L.orc_job_end_pass(h)
        L.orc_recompute_sensitivity(h)
        L.orc_statmc_denoise(h)
        out = np.empty((cfg.image_height, cfg.image_width, 3), dtype=np.float32)
        assert L.orc64_read(h, R.FIELD["DENOISED"], out.ctypes.data) == 0
        return out
    finally:
        L.orc_job_destroy(h)


def port_hdr_metrics(ref: np.ndarray, tst: np.ndarray) -> dict:
    """The restatement of eval_tools hdr-metrics on two (H, W, 3) float images."""
    h, w, _ = ref.shape
    a = np.ascontiguousarray(ref, dtype=np.float32)
    b = np.ascontiguousarray(tst, dtype=np.float32)
    m = R.ImageMetrics()
    assert port().orc_hdr_metrics(a.ctypes.data, b.ctypes.data, w, h, C.byref(m)) == 0
    return m.as_dict()


_ref_eval = None


def ref_eval() -> C.CDLL:
    """The reference's shared/tools/eval_tools.cpp (oracle/_ref/libref_eval.so)."""
    global _ref_eval
    if _ref_eval is None:
        L = C.CDLL(str(HERE / "_ref" / "libref_eval.so"))
        L.ref_extended_metrics.restype = None
        L.ref_extended_metrics.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.ref_hdr_metrics_text.restype = C.c_int
        L.ref_hdr_metrics_text.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_int]
        _ref_eval = L
    return _ref_eval


def ref_hdr_metrics(ref: np.ndarray, tst: np.ndarray) -> dict:
    """The reference's own metrics: compute_extended_metrics called directly (full double
    precision) and the printed report of `eval_tools hdr-metrics` parsed (MAE, RMSE, peak and
    PSNR to 12 and 6 significant digits, SSIM to 4 decimals)."""
    import re

    h, w, _ = ref.shape
    a = np.ascontiguousarray(ref, dtype=np.float32)
    b = np.ascontiguousarray(tst, dtype=np.float32)
    ext = np.zeros(3)
    L = ref_eval()
    L.ref_extended_metrics(a.ctypes.data, b.ctypes.data, w, h, ext.ctypes.data)
    buf = C.create_string_buffer(4096)
    assert L.ref_hdr_metrics_text(a.ctypes.data, b.ctypes.data, w, h, buf, 4096) == 0
    text = buf.value.decode()
    num = r"([-+0-9.eEinfa]+)"
    m = re.search(rf"MAE: {num}\s+RMSE: {num}\s+PSNR \(reference peak={num}\): {num} dB", text)
    s = re.search(rf"R={num} G={num} B={num}\s+mean={num}", text)
    return {"nrmse": ext[0], "log_ssim11": ext[1], "log_gradient_nrmse": ext[2],
            "mae": float(m.group(1)), "rmse": float(m.group(2)), "peak": float(m.group(3)), "psnr": float(m.group(4)),
            "ssim": [float(s.group(k)) for k in (1, 2, 3)], "ssim_mean": float(s.group(4)), "text": text}


def ref_outputs(prefix: str, tonemap: int, swap: bool = True) -> dict:
    """output_buffers of the reference's current frame (after ref_finalize): {file name: HDR
    floats (h, w, 3) or PNG bytes (h, w, 3) uint8}."""
    L = ref()
    L.ref_output_buffers.restype = C.c_int
    L.ref_output_buffers.argtypes = [C.c_char_p, C.c_int, C.c_int]
    L.ref_output_names.restype = C.c_int
    L.ref_output_names.argtypes = [C.c_char_p, C.c_size_t]
    L.ref_output_image.restype = C.c_int
    L.ref_output_image.argtypes = [C.c_char_p, C.c_int, C.c_void_p, C.c_size_t, C.POINTER(C.c_int32),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    assert L.ref_output_buffers(prefix.encode(), tonemap, 1 if swap else 0) == 0
    buf = C.create_string_buffer(1 << 16)
    assert L.ref_output_names(buf, 1 << 16) >= 0
    out = {}
    for name in buf.value.decode().split("\n"):
        if not name:
            continue
        png = name.startswith("png:")
        key = name[4:] if png else name
        w, h, comp = C.c_int32(), C.c_int32(), C.c_int32()
        data = np.empty(1 << 24, dtype=np.uint8)
        assert L.ref_output_image(key.encode(), 1 if png else 0, data.ctypes.data, data.nbytes, C.byref(w), C.byref(h),
                                  C.byref(comp)) == 0
        n = w.value * h.value * comp.value
        arr = data[:n].copy() if png else data[:4 * n].view(np.float32).copy()
        out[key] = arr.reshape(h.value, w.value, comp.value)
    return out


def ref_tonemap(rgb: np.ndarray, tonemap: int) -> np.ndarray:
    """Image::save_with_tonemapping's bytes for (n, 3) float values."""
    L = ref()
    L.ref_tonemap.restype = C.c_int
    L.ref_tonemap.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    a = np.ascontiguousarray(rgb, dtype=np.float32)
    out = np.empty(a.shape, dtype=np.uint8)
    assert L.ref_tonemap(a.ctypes.data, len(a), tonemap, out.ctypes.data) == 0
    return out


def have_ref() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is not None:
        return _ref
    if not REF_LIB.exists():
        raise RuntimeError(f"{REF_LIB} is not built (needs the reference checkout; make -C oracle ref)")
    L = C.CDLL(str(REF_LIB))
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    sig = {
        "ref_max_threads": (C.c_int, []),
        "ref_parse_yaml": (C.c_int, [C.c_char_p, C.POINTER(R.Config), C.c_char_p, C.c_size_t]),
        "ref_trace_cornell": (i64, [C.c_char_p, i32, i32, i32, C.c_uint32, vp, vp, C.POINTER(R.SampleSoA), i64]),
        "ref_begin_frame": (C.c_int, [C.POINTER(R.Config)]),
        "ref_set_config": (C.c_int, [C.POINTER(R.Config)]),
        "ref_push_samples": (C.c_int, [C.POINTER(R.SampleSoA), i64, i64, i32, vp, C.c_int]),
        "ref_end_pass": (C.c_int, [C.c_int]),
        "ref_recompute_sensitivity": (C.c_int, [C.c_int]),
        "ref_statmc_denoise": (C.c_int, [C.c_int]),
        "ref_variance_denoise": (C.c_int, [C.c_int]),
        "ref_compute_adaptive_sample_counts": (C.c_int, [vp, C.c_int]),
        "ref_finalize": (C.c_int, [C.c_int]),
        "ref_stage_ms": (C.c_double, [C.c_int]),
        "ref_read": (C.c_int, [C.c_int, vp, C.c_size_t]),
        "ref_render_cornell": (C.c_int, [C.c_char_p, C.POINTER(R.Config), i32, C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _ref = L
    return L


_ref_filters = None


def ref_filters() -> tuple[C.CDLL, C.CDLL]:
    """The reference's own denoising/atrous_wavelet.cpp and joint_bilateral.cpp filter()
    functions on in-memory images (oracle/ref/ref_filters.cpp)."""
    global _ref_filters
    if _ref_filters is None:
        A = C.CDLL(str(HERE / "_ref" / "libref_atrous.so"))
        J = C.CDLL(str(HERE / "_ref" / "libref_joint.so"))
        A.ref_atrous.restype = C.c_int
        A.ref_atrous.argtypes = [C.c_void_p] * 3 + [C.c_int] * 2 + [C.c_float] * 3 + [C.c_int, C.c_void_p]
        J.ref_joint_bilateral.restype = C.c_int
        J.ref_joint_bilateral.argtypes = [C.c_void_p] * 3 + [C.c_int] * 2 + [C.c_float] * 4 + [C.c_void_p] * 3
        _ref_filters = (A, J)
    return _ref_filters


def ref_atrous(raw, normal, albedo, sigma_c, sigma_n, sigma_a, iterations) -> np.ndarray:
    h, w, _ = raw.shape
    out = np.empty((h, w, 3), dtype=np.float32)
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (raw, normal, albedo)]
    rc = ref_filters()[0].ref_atrous(*[x.ctypes.data for x in a], w, h, sigma_c, sigma_n, sigma_a, iterations,
                                     out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"reference a-trous filter failed ({rc})")
    return out


def ref_joint_bilateral(raw, normal, albedo, sigma_c, sigma_n, sigma_p, sigma_a):
    h, w, _ = raw.shape
    outs = [np.empty((h, w, 3), dtype=np.float32) for _ in range(3)]
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (raw, normal, albedo)]
    rc = ref_filters()[1].ref_joint_bilateral(*[x.ctypes.data for x in a], w, h, sigma_c, sigma_n, sigma_p, sigma_a,
                                              *[o.ctypes.data for o in outs])
    if rc != 0:
        raise RuntimeError(f"reference joint-bilateral filter failed ({rc})")
    return tuple(outs)


def port_allocate(importance: np.ndarray, cfg) -> np.ndarray:
    """The allocation of compute_adaptive_sample_counts (main.cpp:1372-1438) on a given final
    importance map, in the reference's order."""
    imp = np.ascontiguousarray(importance, dtype=np.float32).ravel()
    counts = np.empty(imp.size, dtype=np.int32)
    port().orc_allocate_counts_map(imp.ctypes.data, imp.size, C.byref(cfg), counts.ctypes.data)
    return counts


def port_atrous(raw, normal, albedo, sigma_c, sigma_n, sigma_a, iterations, threads: int = 1) -> np.ndarray:
    h, w, _ = raw.shape
    out = np.empty((h, w, 3), dtype=np.float32)
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (raw, normal, albedo)]
    port().orc_atrous_wavelet(*[x.ctypes.data for x in a], w, h, sigma_c, sigma_n, sigma_a, iterations,
                              out.ctypes.data, threads)
    return out


def port_joint_bilateral(raw, normal, albedo, sigma_c, sigma_n, sigma_p, sigma_a, threads: int = 1):
    h, w, _ = raw.shape
    outs = [np.empty((h, w, 3), dtype=np.float32) for _ in range(3)]
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (raw, normal, albedo)]
    port().orc_joint_bilateral(*[x.ctypes.data for x in a], w, h, sigma_c, sigma_n, sigma_p, sigma_a,
                               *[o.ctypes.data for o in outs], threads)
    return tuple(outs)


def config_dict(cfg: R.Config) -> dict:
    return {name: getattr(cfg, name) for name, _ in R.Config._fields_}


def config_from(d: dict) -> R.Config:
    return R.default_config(**d)


def synth_dict(p: R.SynthParams) -> dict:
    return {name: getattr(p, name) for name, _ in R.SynthParams._fields_}


def synth_from(d: dict) -> R.SynthParams:
    p = R.SynthParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _counts_ptr(counts):
    if counts is None:
        return None, None
    c = np.ascontiguousarray(counts, dtype=np.int32)
    return c, c.ctypes.data


def synth_fill(params: R.SynthParams, first: int, count: int, spp: int, counts=None, start_n=None,
               threads: int = 0, planes=None) -> R.HostSamples:
    """Synthetic samples on the host (include/rpd_synth.h through oracle/synth_host.c)."""
    c, cp = _counts_ptr(counts)
    s0, sp = _counts_ptr(start_n)
    total = int(c.sum()) if c is not None else count * spp
    hs = R.HostSamples(total, count, planes)
    soa = hs.soa()
    n = port().orc_synth_fill(C.byref(params), first, count, spp, cp, sp, C.byref(soa), threads)
    assert n == total
    return hs


class OracleJob:
    """The C restatement (oracle/rpd_oracle.c) behind the product's call sequence."""

    def __init__(self, cfg: R.Config, threads: int = 0):
        self.cfg = cfg
        self.handle = port().orc_job_create(C.byref(cfg))
        if not self.handle:
            raise ValueError("invalid config")
        port().orc_set_threads(self.handle, threads)

    def close(self):
        if self.handle:
            port().orc_job_destroy(self.handle)
            self.handle = None

    def set_threads(self, threads: int):
        port().orc_set_threads(self.handle, threads)

    def set_config(self, cfg: R.Config):
        assert port().orc_job_set_config(self.handle, C.byref(cfg)) == 0
        self.cfg = cfg.replace(image_width=self.cfg.image_width, image_height=self.cfg.image_height,
                               rpf_tile_size=self.cfg.rpf_tile_size)

    def begin_frame(self):
        port().orc_job_begin_frame(self.handle)

    def push(self, samples: R.HostSamples, first: int, count: int, spp: int = 0, counts=None):
        c, cp = _counts_ptr(counts)
        soa = samples.soa()
        assert port().orc_job_push_samples(self.handle, C.byref(soa), first, count, spp, cp) == 0

    def end_pass(self):
        port().orc_job_end_pass(self.handle)

    def recompute_sensitivity(self):
        port().orc_recompute_sensitivity(self.handle)

    def statmc_denoise(self):
        port().orc_statmc_denoise(self.handle)

    def variance_denoise(self):
        port().orc_variance_denoise(self.handle)

    def compute_adaptive_sample_counts(self) -> np.ndarray:
        out = np.empty(self.cfg.image_width * self.cfg.image_height, dtype=np.int32)
        port().orc_compute_adaptive_sample_counts(self.handle, out.ctypes.data)
        return out

    def finalize(self):
        port().orc_finalize(self.handle)

    def read(self, name: str) -> np.ndarray:
        shape, dt = R.field_shape(self.cfg, name)
        out = np.empty(shape, dtype=dt)
        assert port().orc_job_read(self.handle, R.FIELD[name], out.ctypes.data, out.nbytes) == 0, name
        return out

    def stage_ms(self, stage: str) -> float:
        return float(port().orc_stage_ms(self.handle, R.STAGE[stage]))


class RefJob:
    """The reference's own code (compiled in oracle/_ref) behind the same call sequence."""

    def __init__(self, cfg: R.Config, threads: int = 1):
        self.cfg = cfg
        self.threads = threads
        ref().ref_begin_frame(C.byref(cfg))

    def close(self):
        pass

    def set_config(self, cfg: R.Config):
        ref().ref_set_config(C.byref(cfg))
        self.cfg = cfg.replace(image_width=self.cfg.image_width, image_height=self.cfg.image_height,
                               rpf_tile_size=self.cfg.rpf_tile_size)

    def begin_frame(self):
        ref().ref_begin_frame(C.byref(self.cfg))

    def push(self, samples: R.HostSamples, first: int, count: int, spp: int = 0, counts=None):
        c, cp = _counts_ptr(counts)
        soa = samples.soa()
        assert ref().ref_push_samples(C.byref(soa), first, count, spp, cp, self.threads) == 0

    def end_pass(self):
        ref().ref_end_pass(self.threads)

    def recompute_sensitivity(self):
        ref().ref_recompute_sensitivity(self.threads)

    def statmc_denoise(self):
        ref().ref_statmc_denoise(self.threads)

    def variance_denoise(self):
        ref().ref_variance_denoise(self.threads)

    def compute_adaptive_sample_counts(self) -> np.ndarray:
        out = np.empty(self.cfg.image_width * self.cfg.image_height, dtype=np.int32)
        ref().ref_compute_adaptive_sample_counts(out.ctypes.data, self.threads)
        return out

    def finalize(self):
        ref().ref_finalize(self.threads)

    def read(self, name: str) -> np.ndarray:
        shape, dt = R.field_shape(self.cfg, name)
        out = np.empty(shape, dtype=dt)
        assert ref().ref_read(R.FIELD[name], out.ctypes.data, out.nbytes) == 0, name
        return out

    def stage_ms(self, stage: str) -> float:
        return float(ref().ref_stage_ms(R.STAGE[stage]))


CORNELL_PLANES = ("radiance", "normal", "depth", "albedo", "pixel_u", "lens_u", "brdf_u", "light_u", "env_u",
                  "flags", "category")


def trace_cornell(yaml_path: str, w: int, h: int, spp: int, seed: int, start_n=None, counts=None) -> R.HostSamples:
    """Camera samples of the reference's cornell_box scene, traced by the reference."""
    s0, sp = _counts_ptr(start_n)
    c, cp = _counts_ptr(counts)
    total = int(c.sum()) if c is not None else w * h * spp
    hs = R.HostSamples(total, w * h, CORNELL_PLANES)
    soa = hs.soa()
    n = ref().ref_trace_cornell(yaml_path.encode(), w, h, spp, seed, sp, cp, C.byref(soa), total)
    assert n == total, (n, total)
    return hs


def ref_parse_yaml(path: str) -> R.Config:
    cfg = R.Config()
    msg = C.create_string_buffer(256)
    if ref().ref_parse_yaml(path.encode(), C.byref(cfg), msg, 256) != 0:
        raise ValueError(msg.value.decode())
    return cfg


def run_pipeline(job, samples: R.HostSamples, spp: int, statmc: bool = True, variance: bool = True) -> None:
    """The non-adaptive StatMC sequence of render() (main.cpp:1543-1557) minus finalize:
    one pass of samples, recompute_sensitivity, statmc_denoise, variance_denoise."""
    w, h = job.cfg.image_width, job.cfg.image_height
    job.begin_frame()
    job.push(samples, 0, w * h, spp)
    job.end_pass()
    job.recompute_sensitivity()
    if statmc:
        job.statmc_denoise()
    if variance:
        job.variance_denoise()
