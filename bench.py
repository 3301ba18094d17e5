"""Benchmark of the GB300 StatMC / RPD denoise stage.

Workload (one step = one frame of the plain method): 1920x1080, 16 samples per pixel of
seeded synthetic per-sample buffers (include/rpd_synth.h: 48 Voronoi regions, log-normal
radiance, 24 regions dependent on two random dims, 0.1% fireflies x100), denoise knobs of
the reference's cornell_box configuration (path_tracer/config/cornell.yaml) with rpf tile
16, colour window radius 5, variance radius 3, 2 variance iterations and no adaptive pass.
A step runs the stage as render() does for a frame: accumulate the samples (statistics,
features, RPD grid), recompute_sensitivity, statmc_denoise, variance_denoise.

  value  Msamples/s with the samples already resident in HBM (2.06 GB of FP32 planes per
         frame, larger than the 129 MB L2, so no flush is needed between steps).
  e2e    the same through the C ABI from pinned host buffers: every step copies the frame's
         sample planes host->HBM and reads the denoised image back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

`--impl reference` times the reference CPU implementation of the stage on this host's cores
(the C restatement in oracle/, since the reference checkout does not exist on the GPU host)
on a 1920x270 band of the same workload per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "rpd-statmc-denoiser_gb300"))

W, H, SPP, SEED = 1920, 1080, 16, 1234
# The headline metric: `value` is the plain form's throughput; the line's `served` object holds
# the served stream's throughput and p50/p99 latency against the plain per-frame drop-in
METRIC = "denoised Msamples/s at 1080p 16spp, plain vs served; p50/p99 ms @\u22641e-3 relMSE"
UNIT = "Msamples/s"


def workload_config(R, w=None, h=None):
    # path_tracer/config/cornell.yaml stage knobs + the plain-method overrides
    return R.default_config(
        image_width=W if w is None else w, image_height=H if h is None else h, rpf_tile_size=16, color_window_radius=5, color_normal_threshold=0.6,
        color_depth_threshold=0.2, color_compat_alpha=0.01, color_sigma_max=4.0, var_window_radius=3,
        var_normal_threshold=0.6, var_compat_sigma=3.0, var_shrinkage_k=0.7, var_iterations=2, adaptive_spp=4,
        adaptive_base_samples=2, adaptive_sigma_max=4.0, adaptive_passes=0, seed=SEED)


def config_json(R, cfg, extra=None):
    plane_gb = W * H * SPP * 62 / 1e9
    d = {"workload": f"plain method, {W}x{H}, {SPP} spp, synthetic per-sample FP32 buffers (seed {SEED})",
         "width": cfg.image_width, "height": cfg.image_height, "spp": SPP, "rpf_tile_size": cfg.rpf_tile_size,
         "color_window_radius": cfg.color_window_radius, "var_window_radius": cfg.var_window_radius,
         "var_iterations": cfg.var_iterations, "adaptive_passes": 0,
         "l2": f"inputs larger than L2 ({plane_gb:.2f} GB of sample planes per step vs 129 MB L2)"
               if plane_gb > 0.129 else "inputs smaller than L2: not a bench configuration",
         "parallelism": "replicas"}
    if extra:
        d.update(extra)
    return d


# Algorithmic bytes each kernel family must move for one frame (per launch of that family
# in a frame), from the plane sizes. Statistics pass: per sample 62 B of FP32 planes read
# (radiance 12, normal 12, depth 4, pixel/lens/brdf/light uv 32, flags 1, category 1) and 8 B
# written for the grid pass (luminance, packed key); per pixel 12 B of albedo read, 88 B of
# statistics and sums read and written (176 B) and 24 B of pattern sums written. Grid pass:
# per sample the 8 B the statistics pass wrote; per node 3744 B of grid read and written.
# StatMC window: per pixel the 96 B of packed neighbour records (read once; the halos of
# neighbouring tiles come from L2) and 20 B of outputs.
def algorithmic_bytes(kernel: str, np_: int, nn: int, n: int) -> float:
    if kernel == "accumulate_pixels":
        return 70.0 * n + (12.0 + 176.0 + 24.0) * np_
    if kernel == "grid":
        return 8.0 * n + 24.0 * np_ + 2.0 * 3744.0 * nn
    if kernel == "grid_random":
        return 8.0 * n + 2.0 * 3744.0 * nn
    if kernel == "statmc_window":
        return (96.0 + 20.0) * np_
    if kernel == "merge":
        return 3.0 * 3744.0 * nn
    if kernel == "variance":
        return np_ * (4 * 2 + 2 * (4 + 4 + 12 + 4 + 4 + 4) + 4 * 3)
    if kernel == "node_stats":
        return 3744.0 * nn + 4.0 * 34 * nn
    return 0.0


# FP32-equivalent operations per neighbour visit of the StatMC window, counted from the
# reference's loop body (main.cpp:1032-1096): gates ~15, Welch per channel ~12 (x3), RPD
# relaxation and weight ~10, weighted accumulation ~12. One frame visits W*H*(2r+1)^2
# neighbours. Fixed here once; the roofline's achieved rate for the window uses it.
WINDOW_OPS_PER_VISIT = 75


def window_visits(w: int, h: int, r: int) -> int:
    return w * h * (2 * r + 1) ** 2


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return world, rank, local, dist
    return 1, 0, 0, None


def max_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(dist, world: int, samples_per_rank: int, elapsed_ms: float, steps: int):
    """(ms per step, Msamples/s) of N replicas that each processed samples_per_rank samples per
    step: the slowest rank's time, every rank's samples."""
    ms_per_step = max_over_ranks(dist, elapsed_ms) / steps
    return ms_per_step, world * samples_per_rank / (ms_per_step * 1e-3) / 1e6


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_gpu(args):
    import rpd_gb300 as R

    world, rank, local, dist = dist_setup()
    cfg = workload_config(R)
    np_ = W * H
    n = np_ * SPP
    nx, ny = R.node_dims(cfg)
    nn = nx * ny
    ctx = R.Context(local, 0)
    params = R.synth_params(W, H, SEED + rank)
    dev = R.DeviceSamples(ctx, n, np_)
    ctx.synth_fill(params, 0, np_, SPP, dev)
    samples = dev
    quality = None
    if args.precision == "fp16":
        # the precision form: the same frame in compact storage; its error against the FP32 push
        samples = R.DeviceSamples16.encode(ctx, dev, depth_scale=1.0)
        quality = compact_quality(R, ctx, cfg, dev, samples)
    job = R.Job(ctx, cfg)
    if args.grid_shape:
        job.set_tuning("grid_shape", args.grid_shape)

    def step(samples):
        job.begin_frame()
        if getattr(samples, "compact_host", False):
            job.push16(samples, 0, np_, SPP, where=R.MEM_HOST)
        else:
            job.push(samples, 0, np_, SPP)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()

    for _ in range(args.warmup):
        step(samples)
    job.sync()
    # the FP32 issue rate of this GPU at its present clock: the window's roofline denominator
    fp32_peak = R.probe_fp32_issue(local, 5)
    # device-resident timed region
    job.set_profiling(True)
    job.reset_kernel_times()
    launches0 = job.launches()
    barrier(dist)
    job.sync()
    with ClockSampler(local) as clocks:
        job.mark(0)
        for _ in range(args.steps):
            step(samples)
        job.mark(1)
        elapsed = job.elapsed_ms(0, 1)
    launches = job.launches() - launches0
    ktimes = job.kernel_times()
    job.set_profiling(False)
    ms_per_step, value = replica_throughput(dist, world, n, elapsed, args.steps)

    # end-to-end through the C ABI from pinned host buffers: every step pushes the frame's
    # planes from host memory (copied to HBM inside the push) and reads the denoised image back.
    # Two jobs alternate, as a caller streaming frames would use them: while one job's push
    # copies frame i+1 (the host->device link runs at ~210 GB/s on this machine), the other
    # job's stages of frame i run on the GPU.
    e2e = None
    if not args.no_e2e:
        host = pinned_host_copy(R, ctx, samples)
        # one page-locked result buffer per job: a job's result is read back asynchronously while
        # the other job's push copies the next frame (the link carries both directions at once)
        outs = [R.PinnedBuffer(np_ * 12), R.PinnedBuffer(np_ * 12)]
        jobs = [job, R.Job(ctx, cfg)]
        if args.grid_shape:
            jobs[1].set_tuning("grid_shape", args.grid_shape)

        def start(jb):
            jb.begin_frame()
            if getattr(host, "compact_host", False):
                # compact planes (1.07 GB per frame): the GPU work, not the link, is the bound, and a
                # push that returns after its copies keeps the two jobs' stages apart (measured
                # faster than the asynchronous push here)
                jb.push16(host, 0, np_, SPP, where=R.MEM_HOST)
            else:
                # FP32 planes (2.08 GB per frame, link-bound): the push returns once its copies are
                # enqueued, so the next frame's copies queue behind them while this frame's stages run
                jb.push_async(host, 0, np_, SPP)
            jb.end_pass()
            jb.recompute_sensitivity()
            jb.statmc_denoise()
            jb.variance_denoise()

        def finish(k):
            R.check(R.lib().rpd_job_read_async(jobs[k].handle, R.FIELD["DENOISED"], outs[k].ptr, outs[k].nbytes,
                                               R.MEM_HOST))

        for i in range(max(2, args.warmup)):
            start(jobs[i % 2])
            finish(i % 2)
            jobs[i % 2].sync()
        barrier(dist)
        t0 = time.perf_counter()
        for i in range(args.steps):
            k = i % 2
            jobs[k].sync()  # this job's previous frame is copied in and its result is in host memory
            start(jobs[k])
            finish(k)
        for jb in jobs:
            jb.sync()
        wall_ms = (time.perf_counter() - t0) * 1e3
        e2e_ms = max_over_ranks(dist, wall_ms)
        e2e = {"value": round(world * n / (e2e_ms / args.steps * 1e-3) / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": int(outs[0].nbytes),
               "ms_per_step": round(e2e_ms / args.steps, 3),
               "pipeline": "two jobs alternating: frame i+1's host->device copy overlaps frame i's stages and "
                           "the asynchronous read-back of frame i-1's denoised image (FP32 planes: asynchronous "
                           "host pushes, so frame i+1's copy is enqueued while frame i's is on the link)"}
        jobs[1].close()
        host.free()
        for o in outs:
            o.free()

    # roofline of the dominant kernel (per-launch CUDA-event time on the job stream)
    peaks = measured_peaks()
    dominant = max(ktimes, key=lambda k: ktimes[k][0])
    roofline = kernel_roofline(dominant, ktimes[dominant], args.steps, cfg, np_, nn, n, peaks, fp32_peak)
    others = {k: kernel_roofline(k, ktimes[k], args.steps, cfg, np_, nn, n, peaks, fp32_peak)
              for k in ("statmc_window", "accumulate_pixels", "grid_random") if k != dominant and ktimes[k][1]}
    # the whole frame against HBM: the sample planes read once plus the required per-pixel
    # outputs (denoised RGB, uncertainty, alpha, variance_denoised) and the albedo input
    frame_bytes = 62.0 * n + (24.0 + 12.0) * np_
    frame_gbs = frame_bytes / (ms_per_step * 1e-3) / 1e9
    roofline["frame"] = {"bytes_per_step": frame_bytes, "achieved": round(frame_gbs, 1), "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": round(frame_gbs / peaks["hbm_gbs"], 4),
                         "floor_ms": round(frame_bytes / (peaks["hbm_gbs"] * 1e9) * 1e3, 4)}
    roofline["other_kernels"] = others
    kernels_ms = {k: round(v[0] / args.steps, 4) for k, v in ktimes.items() if v[1]}
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": config_json(R, cfg),
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks.summary(), "roofline": roofline,
        "kernels_ms_per_step": kernels_ms,
        "storage": "fp16/snorm16/unorm16 per-sample planes (32 B/sample), fp32 accumulation"
                   if args.precision == "fp16" else "fp32 per-sample planes (62 B/sample)",
    }
    if quality is not None:
        out["quality"] = quality
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, steps=3)
    job.close()
    if samples is not dev:
        samples.free()
    dev.free()
    if args.precision == "fp32" and (W, H, SPP) == (1920, 1080, 16):
        out["filters"] = filters_leg(R, ctx)
    if not args.no_served and args.precision == "fp32" and (W, H, SPP) == (1920, 1080, 16):
        # the served half of the metric (plain vs served; p50/p99 latency)
        out["served"] = served_summary(R, ctx, args, rank, dist, args.served_requests)
    ctx.close()
    if rank == 0:
        print(json.dumps(out))


def filters_leg(R, ctx, w=1920, h=1080, reps=10):
    """The standalone post-filters on a w x h frame in device memory, through their C ABI
    calls (each call synchronises; its scratch comes from the stream-ordered pool): a-trous with
    its 5 default passes and sigmas (denoising/atrous_wavelet.cpp:229) and the joint bilateral
    with sigma_p 2 (a 13x13 window). Mean host wall time per call after 2 warm-up calls."""
    rng = np.random.default_rng(5)
    imgs = [rng.lognormal(-1.0, 0.8, (h, w, 3)).astype(np.float32), rng.uniform(0, 1, (h, w, 3)).astype(np.float32),
            rng.uniform(0, 1, (h, w, 3)).astype(np.float32)]
    bufs = [R.DeviceBuffer(ctx, imgs[0].nbytes) for _ in range(6)]
    try:
        for b, a in zip(bufs, imgs):
            b.upload(a)
        L = R.lib()

        def atrous():
            R.check(L.rpd_atrous_wavelet(ctx.handle, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, w, h, 0.3, 0.2, 0.1, 5,
                                         bufs[3].ptr, R.MEM_DEVICE))

        def joint():
            R.check(L.rpd_joint_bilateral(ctx.handle, bufs[0].ptr, bufs[1].ptr, bufs[2].ptr, w, h, 0.3, 0.2, 2.0, 0.1,
                                          bufs[3].ptr, bufs[4].ptr, bufs[5].ptr, R.MEM_DEVICE))
        out = {"frame": f"{w}x{h}, device memory, host wall time per synchronous call"}
        for name, fn in (("atrous_5_passes_ms", atrous), ("joint_bilateral_r6_ms", joint)):
            for _ in range(2):
                fn()
            t = time.perf_counter()
            for _ in range(reps):
                fn()
            out[name] = round((time.perf_counter() - t) * 1e3 / reps, 4)
        return out
    finally:
        for b in bufs:
            b.free()


def pinned_host_copy(R, ctx, dev):
    """Copy device sample planes into page-locked host planes (for the end-to-end leg)."""
    import ctypes as C

    compact = isinstance(dev, R.DeviceSamples16)

    class PinnedSamples:
        compact_host = compact

        def __init__(self):
            self.ptrs = []
            self.planes = {}
            self.nbytes = 0
            for name, bl in dev.bufs.items():
                arrs = []
                for b in bl:
                    p = C.c_void_p()
                    R.check(R.lib().rpd_host_alloc(b.nbytes, C.byref(p)))
                    self.ptrs.append(p.value)
                    R.check(R.lib().rpd_memcpy(ctx.handle, p.value, b.ptr, b.nbytes, 1))
                    arrs.append(p.value)
                    self.nbytes += b.nbytes
                self.planes[name] = arrs

        def soa(self):
            s = R.SampleSoA16() if compact else R.SampleSoA()
            if compact:
                s.depth_scale = dev.depth_scale
            table = R.PLANES16 if compact else R.PLANES
            for name, arrs in self.planes.items():
                if len(arrs) == 1 and table[name][0] == 1:
                    setattr(s, name, arrs[0])
                else:
                    f = getattr(s, name)
                    for c, p in enumerate(arrs):
                        f[c] = p
            return s

        def free(self):
            for p in self.ptrs:
                R.lib().rpd_host_free(p)
            self.ptrs = []

    return PinnedSamples()


def compact_quality(R, ctx, cfg, dev, dev16):
    """relMSE = mean((x - r)^2 / (r^2 + 1e-2)) and max relative error of the compact-storage
    frame against the same frame pushed as FP32 planes."""
    out = []
    for samples in (dev, dev16):
        job = R.Job(ctx, cfg)
        job.begin_frame()
        job.push(samples, 0, W * H, SPP)
        job.end_pass()
        job.recompute_sensitivity()
        job.statmc_denoise()
        job.variance_denoise()
        out.append(job.read("DENOISED").astype(np.float64))
        job.close()
    r, x = out
    return {"reference": "the same frame pushed as FP32 planes (the oracle-pinned path)",
            "rel_mse": float(np.mean((x - r) ** 2 / (r * r + 1e-2))),
            "max_rel_err": float(np.max(np.abs(x - r) / np.maximum(np.abs(r), 1e-3)))}


# DRAM bytes per pixel per launch (dram__bytes_read.sum + dram__bytes_write.sum) from the ncu
# captures summarised in profiles/, for the kernels whose traffic grows with the pixel count
NCU_TRAFFIC_PER_PIXEL = {
    # k_statmc_tma<5>, one launch at 960x540x16 (--set full): 49.88 MB read + 1.95 MB written
    "statmc_window": ((49.877504e6 + 1.950208e6) / (960 * 540), "ncu at 960x540x16, per pixel, scaled by the pixels"),
}


def kernel_roofline(kernel, times, steps, cfg, np_, nn, n, peaks, fp32_peak):
    """Roofline of one kernel family: achieved = algorithmic work per launch / average launch
    time. The StatMC window is bound by FP32 issue (its neighbour decisions), the rest by HBM."""
    total_ms, launches = times
    per_launch_ms = total_ms / max(1, launches)
    launches_per_frame = max(1, launches // steps)
    alg = algorithmic_bytes(kernel, np_, nn, n) / launches_per_frame
    gbs = alg / (per_launch_ms * 1e-3) / 1e9 if alg else None
    traffic = NCU_TRAFFIC_PER_PIXEL.get(kernel)
    hbm = {"achieved": round(gbs, 1) if gbs else None, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": round(gbs / peaks["hbm_gbs"], 4) if gbs else None, "peak_source": peaks["source"],
           "algorithmic_bytes_per_launch": alg,
           "traffic": round(traffic[0] * np_) if traffic else None,
           "traffic_source": traffic[1] if traffic else None}
    out = {"kernel": kernel, "ms_per_launch": round(per_launch_ms, 4)}
    if kernel == "statmc_window" and fp32_peak:
        visits = window_visits(cfg.image_width, cfg.image_height, cfg.color_window_radius)
        ops = WINDOW_OPS_PER_VISIT * visits
        achieved = ops / (per_launch_ms * 1e-3) / 1e9
        peak = fp32_peak["per_second"] / 1e9
        out.update({"bound": "fp32_issue", "achieved": round(achieved, 1), "peak": round(peak, 1),
                    "unit": "Gop/s (FP32 lane operations)", "frac": round(achieved / peak, 4),
                    "traffic": hbm["traffic"],
                    "ops_per_launch": ops, "ops_per_visit": WINDOW_OPS_PER_VISIT, "visits_per_launch": visits,
                    "peak_source": "measured here: rpd_probe_fp32_issue (independent FFMA chains on every SM, "
                                   f"CUDA events, best of 5: {fp32_peak['ms']:.3f} ms)",
                    "hbm": hbm})
    else:
        out.update({"bound": "hbm", "achieved": hbm["achieved"], "peak": hbm["peak"], "unit": "GB/s",
                    "frac": hbm["frac"], "traffic": hbm["traffic"], "traffic_source": hbm["traffic_source"],
                    "peak_source": hbm["peak_source"], "algorithmic_bytes_per_launch": alg})
    return out


def measured_peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        d = json.loads(path.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json)"}
    return {"hbm_gbs": 6800.0, "source": "fallback 6.8 TB/s"}


def cpu_baseline(args, steps=1, warmup=0):
    """The reference CPU path (the C restatement in oracle/) on this host's cores, on a
    band of a quarter of the frame's rows (1920x270 at 1080p) of the same workload."""
    import rpd_gb300 as R
    from oracle import binding as B

    threads = os.cpu_count() or 1
    band_h = H // 4
    cfg = workload_config(R, W, band_h)
    params = R.synth_params(W, band_h, SEED)
    samples = B.synth_fill(params, 0, W * band_h, SPP, threads=threads)
    job = B.OracleJob(cfg, threads=threads)
    for _ in range(warmup):
        B.run_pipeline(job, samples, SPP)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        B.run_pipeline(job, samples, SPP)
        times.append(time.perf_counter() - t0)
    job.close()
    sec = sum(times) / len(times)
    return {"value": round(W * band_h * SPP / sec / 1e6, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{W}x{band_h} band, {SPP} spp ({W * band_h * SPP} samples) per step, {len(times)} step(s), "
                      f"{sec:.2f} s per step"}


SIZES = [(256, 256), (640, 360), (1280, 720), (1920, 1080), (2048, 1152)]
SPPS = [4, 8, 16, 32, 64]


def mixed_frames(count: int, seed: int):
    """The mixed-size job stream: sizes and spp drawn uniformly from the stated sets."""
    rng = np.random.default_rng(seed)
    return [(*SIZES[int(rng.integers(len(SIZES)))], SPPS[int(rng.integers(len(SPPS)))]) for _ in range(count)]


def run_batched(args):
    """The batched form: 48 frames of uneven size and spp in compact storage, each job's launch
    shapes chosen by the autotuner, the whole batch captured into one CUDA graph and launched
    once per step; against the plain drop-in on the same frames (FP32 planes, default shapes,
    one frame after another)."""
    import rpd_gb300 as R

    world, rank, local, dist = dist_setup()
    ctx = R.Context(local, 0)
    frames = mixed_frames(args.frames, SEED + rank)
    batch = R.Batch(ctx)
    batch.set_lanes(args.lanes)
    jobs, planes = [], []
    plain_ms = 0.0
    plain_e2e_ms = 0.0
    rel = []
    total = 0
    for i, (w, h, spp) in enumerate(frames):
        cfg = workload_config(R, w, h)
        dev = R.DeviceSamples(ctx, w * h * spp, w * h)
        ctx.synth_fill(R.synth_params(w, h, SEED + 17 * i), 0, w * h, spp, dev)
        # the plain drop-in on this frame: FP32 planes, default shapes, one frame at a time;
        # inputs resident, and end to end from pinned host planes (copy in, denoised image out)
        plain = R.Job(ctx, cfg)
        for rep in range(2):
            plain.mark(0)
            plain.begin_frame()
            plain.push(dev, 0, w * h, spp)
            plain.end_pass()
            plain.recompute_sensitivity()
            plain.statmc_denoise()
            plain.variance_denoise()
            plain.mark(1)
            ms = plain.elapsed_ms(0, 1)
        plain_ms += ms
        ref = plain.read("DENOISED").astype(np.float64)
        host = pinned_host_copy(R, ctx, dev)
        out_img = np.empty((h, w, 3), dtype=np.float32)
        t0 = time.perf_counter()
        plain.begin_frame()
        plain.push(host, 0, w * h, spp)
        plain.end_pass()
        plain.recompute_sensitivity()
        plain.statmc_denoise()
        plain.variance_denoise()
        R.check(R.lib().rpd_job_read(plain.handle, R.FIELD["DENOISED"], out_img.ctypes.data, out_img.nbytes,
                                     R.MEM_HOST))
        plain_e2e_ms += (time.perf_counter() - t0) * 1e3
        host.free()
        plain.close()
        dev16 = R.DeviceSamples16.encode(ctx, dev)
        dev.free()
        job = R.Job(ctx, cfg)
        job.autotune(dev16, spp)
        x = job.read("DENOISED").astype(np.float64)
        rel.append(float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2))))
        batch.add(job, dev16, spp)
        jobs.append(job)
        planes.append(dev16)
        total += w * h * spp
    batch.run()  # direct run + capture + first launch
    batch.sync()
    for _ in range(args.warmup):
        batch.run()
    batch.sync()
    barrier(dist)
    with ClockSampler(local) as clocks:
        times = []
        for _ in range(args.steps):
            batch.run()
            times.append(batch.last_ms())
    ms = max_over_ranks(dist, sum(times) / len(times))
    value = world * total / (ms * 1e-3) / 1e6
    plain_value = total / (plain_ms * 1e-3) / 1e6
    plain_e2e_value = total / (plain_e2e_ms * 1e-3) / 1e6
    out = {"metric": "denoised Msamples/s, 48 uneven frames (batched graph, fp16 storage)" if args.frames == 48
           else f"denoised Msamples/s, {args.frames} uneven frames (batched graph, fp16 storage)",
           "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": f"{args.frames} frames, sizes from {SIZES}, spp from {SPPS} (seed {SEED})",
                      "samples_per_step": total, "frames": [list(f) for f in frames],
                      "tuned_shapes": sorted({(j.get_tuning("grid_shape"), j.get_tuning("statmc_rows")) for j in jobs}),
                      "lanes": args.lanes,
                      "parallelism": "replicas"},
           "plain": {"value": round(plain_value, 3), "ms_per_step": round(plain_ms, 4),
                     "form": "one frame after another, FP32 planes, default shapes, inputs resident"},
           "plain_e2e": {"value": round(plain_e2e_value, 3), "ms_per_step": round(plain_e2e_ms, 4),
                         "form": "the drop-in call sequence per frame from pinned host FP32 planes, "
                                 "denoised image read back"},
           "speedup_vs_plain": round(value / plain_value, 3),
           "speedup_vs_plain_e2e": round(value / plain_e2e_value, 3),
           "quality": {"reference": "the plain FP32 frames", "rel_mse_mean": float(np.mean(rel)),
                       "rel_mse_max": float(np.max(rel))},
           "gpu_launches": 1, "graph_kernel_nodes": batch.kernel_count(), "clocks": clocks.summary()}
    batch.close()
    for j in jobs:
        j.close()
    for p in planes:
        p.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(out))


def serving_knobs(R):
    """The serving workload's stage knobs: the plain method's, with three adaptive passes of 4
    extra samples per pixel on average and a floor of 1."""
    return workload_config(R, 1, 1).replace(adaptive_passes=3, adaptive_spp=4, adaptive_base_samples=1)


def request_stream(count: int, rate: float, seed: int):
    """A Poisson stream: (arrival s, width, height, spp, seed) with sizes and spp drawn as in the
    mixed-size job stream."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        w, h = SIZES[int(rng.integers(len(SIZES)))]
        out.append((float(t[i]), w, h, SPPS[int(rng.integers(len(SPPS)))], seed + 7919 * (i + 1)))
    return out


def served_stream(R, ctx, args, rank, dist, n_req, storage):
    """A Poisson stream of n_req requests (sizes and spp of the mixed stream, three adaptive
    passes each, extra samples generated on the device) submitted to rpd_server in real time;
    the server admits them against the HBM budget and overlaps them on the GPU. Returns the
    throughput, latencies and server statistics."""
    import threading

    knobs = serving_knobs(R)
    world = 1 if dist is None else dist.get_world_size()
    stream = request_stream(n_req, args.rate, SEED + 1000 * rank)
    srv = R.Server(ctx, knobs, budget_bytes=args.budget_gb << 30, max_inflight=args.inflight, storage=storage,
                   allocator_blocks=args.alloc_blocks)
    # warm-up: a few requests of every size (creates the cached jobs, fills the buffer pool)
    for k in range(max(1, args.warmup)):
        for (w, h) in SIZES:
            srv.submit(w, h, SPPS[k % len(SPPS)], 17 + k, tag=0)
    srv.drain(600000)
    srv.poll(4096)
    st0 = srv.stats()
    barrier(dist)

    def submitter(t0):  # the arrival process, in real time, from a host thread
        for (t, w, h, spp, seed) in stream:
            delay = t0 + t - time.perf_counter()
            if delay > 0.002:
                time.sleep(delay - 0.001)
            while time.perf_counter() < t0 + t:
                pass
            srv.submit(w, h, spp, seed, tag=seed)

    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        t0 = time.perf_counter()
        th = threading.Thread(target=submitter, args=(t0,))
        th.start()
        th.join()
        srv.drain(3600000)
    done = [c for c in srv.poll(n_req + 16) if c["tag"] != 0]
    st1 = srv.stats()
    srv.close()
    assert len(done) == n_req and all(c["status"] == 0 for c in done), "serving run incomplete"
    first = min(c["submit_ms"] for c in done)
    last = max(c["done_ms"] for c in done)
    wall_s = max_over_ranks(dist, (last - first) * 1e-3)
    samples = sum(c["samples"] for c in done)
    lat = np.array([c["done_ms"] - c["submit_ms"] for c in done])
    queue_ms = np.array([c["admit_ms"] - c["submit_ms"] for c in done])
    return {"value": world * samples / wall_s / 1e6, "samples": samples, "wall_s": wall_s, "stream": stream,
            "done": done, "stats": st1, "launches": int(st1["launches"] - st0["launches"]),
            "jobs": {k: int(st1[k] - st0[k]) for k in ("jobs_created", "jobs_destroyed", "scratch_grown")},
            "clocks": clocks.summary(),
            "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3), "p99": round(float(np.percentile(lat, 99)), 3),
                           "mean": round(float(lat.mean()), 3), "max": round(float(lat.max()), 3),
                           "queue_p50": round(float(np.percentile(queue_ms, 50)), 3),
                           "queue_p99": round(float(np.percentile(queue_ms, 99)), 3)}}


def plain_prefix(R, ctx, stream, n_plain, skip_dead=False):
    """The plain per-frame drop-in on a prefix of the stream, one request after another (jobs
    cached per size, as a caller of the drop-in would keep them): Msamples/s. skip_dead: without
    the calls whose results the sequence overwrites unread (what the serving loop leaves out)."""
    knobs = serving_knobs(R)
    jobs = {}
    samples = 0
    for (_, w, h, spp, seed) in stream[:2]:
        R.plain_request(ctx, knobs, w, h, spp, seed, skip_dead=skip_dead)  # warm-up
    t = time.perf_counter()
    for (_, w, h, spp, seed) in stream[:n_plain]:
        if (w, h) not in jobs:
            jobs[(w, h)] = R.Job(ctx, knobs.replace(image_width=w, image_height=h))
        _, ns = R.plain_request(ctx, knobs, w, h, spp, seed, job=jobs[(w, h)], skip_dead=skip_dead)
        samples += ns
    t = time.perf_counter() - t
    for j in jobs.values():
        j.close()
    return {"value": samples / t / 1e6, "requests": n_plain, "samples": samples, "s": round(t, 3)}


def served_quality(R, ctx, args, stream, storage):
    """The served result of the stream's first small requests against the plain FP32 drop-in on
    the same request, and both against the plain method at 1024 spp (converged)."""
    knobs = serving_knobs(R)

    def relmse(x, ref):
        return float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2)))
    picks = [r for r in stream if r[1] * r[2] <= 640 * 360][:4]
    qsrv = R.Server(ctx, knobs, budget_bytes=args.budget_gb << 30, max_inflight=4, storage=storage)
    bufs = []
    for (_, w, h, spp, seed) in picks:
        b = R.PinnedBuffer(w * h * 12)
        bufs.append(b)
        qsrv.submit(w, h, spp, seed, out=b.ptr, tag=seed)
    qsrv.drain(600000)
    qsrv.close()
    q_plain, q_served_conv, q_plain_conv = [], [], []
    for (_, w, h, spp, seed), b in zip(picks, bufs):
        plain_img, _ = R.plain_request(ctx, knobs, w, h, spp, seed)
        conv_img, _ = R.plain_request(ctx, knobs.replace(adaptive_passes=0), w, h, 1024, seed)
        x = b.array(np.float32, (h, w, 3)).astype(np.float64)
        p_ = plain_img.astype(np.float64)
        y = conv_img.astype(np.float64)
        q_plain.append(relmse(x, p_))
        q_served_conv.append(relmse(x, y))
        q_plain_conv.append(relmse(p_, y))
        b.free()
    return {"requests": [list(r[1:4]) for r in picks], "rel_mse_eps": 1e-2,
            "vs_plain_fp32": {"mean": float(np.mean(q_plain)), "max": float(np.max(q_plain))},
            "served_vs_converged": float(np.mean(q_served_conv)),
            "plain_vs_converged": float(np.mean(q_plain_conv)),
            "note": "with adaptive passes the compact storage also moves the adaptive counts a little (the "
                    "systematic residual sampling follows a running sum), so some pixels draw one sample more or "
                    "less than in the FP32 run; converged = the plain FP32 method at 1024 spp; the error of the "
                    "compact form against the FP64 oracle is a test (tests/test_gpu_precision.py)"}


def served_summary(R, ctx, args, rank, dist, n_req, breakdown=True):
    """The served half of the metric: the FP16-storage stream's Msamples/s and p50/p99 latency
    against the plain per-frame drop-in on a prefix of the same stream, and how the ratio splits
    into its parts (each measured): the dead calls the serving loop leaves out (the plain drop-in
    without them), the overlap of requests on the device (the served stream with FP32 storage),
    and the compact storage (FP16 against FP32 served)."""
    fp16 = served_stream(R, ctx, args, rank, dist, n_req, "fp16")
    stream = fp16["stream"]
    n_plain = min(n_req, args.plain_requests)
    plain = plain_prefix(R, ctx, stream, n_plain)
    out = {"metric": f"denoised Msamples/s, served stream ({n_req} requests, Poisson {args.rate:g} req/s, "
                     "3 adaptive passes, fp16 storage) vs the plain per-frame drop-in",
           "value": round(fp16["value"], 3), "unit": UNIT, "requests": n_req, "samples": fp16["samples"],
           "wall_s": round(fp16["wall_s"], 4), "latency_ms": fp16["latency_ms"],
           "p50_ms": fp16["latency_ms"]["p50"], "p99_ms": fp16["latency_ms"]["p99"],
           "plain": {**{k: (round(v, 3) if isinstance(v, float) else v) for k, v in plain.items()},
                     "form": "render()'s call sequence per request from the host, FP32 planes generated on the "
                             "device, adaptive counts read back, one request after another"},
           "vs_plain": round(fp16["value"] / plain["value"], 3),
           "gpu_launches": fp16["launches"], "clocks": fp16["clocks"],
           "server": {"bytes_peak": fp16["stats"]["bytes_peak"], "bytes_budget": fp16["stats"]["bytes_budget"],
                      "jobs_cached": fp16["stats"]["jobs_cached"], "hbm_budget_gb": args.budget_gb,
                      "max_inflight": args.inflight, "during_stream": fp16["jobs"]}}
    if breakdown:
        no_dead = plain_prefix(R, ctx, stream, n_plain, skip_dead=True)
        fp32 = served_stream(R, ctx, args, rank, dist, n_req, "fp32")
        out["breakdown"] = {
            "plain": round(plain["value"], 3),
            "plain_without_dead_calls": round(no_dead["value"], 3),
            "served_fp32": round(fp32["value"], 3),
            "served_fp16": round(fp16["value"], 3),
            "dead_call_elimination": round(no_dead["value"] / plain["value"], 3),
            "overlap_and_continuous_batching": round(fp32["value"] / no_dead["value"], 3),
            "fp16_storage": round(fp16["value"] / fp32["value"], 3),
            "served_fp32_latency_ms": fp32["latency_ms"],
            "note": "the factors multiply to vs_plain; each is the ratio of two measured runs of the same stream "
                    "(the plain legs on its first requests)"}
    out["quality"] = served_quality(R, ctx, args, stream, "fp16")
    return out


def run_serving(args):
    """The serving form alone: the served stream of --steps requests and its comparison with
    the plain per-frame drop-in (served_summary)."""
    import rpd_gb300 as R

    world, rank, local, dist = dist_setup()
    ctx = R.Context(local, 0)
    out = served_summary(R, ctx, args, rank, dist, args.steps, breakdown=not args.no_breakdown)
    out.update({"n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "ms_per_step": round(out["wall_s"] * 1e3 / args.steps, 4),
                "config": {"workload": f"{args.steps} requests, Poisson arrivals at {args.rate:g}/s, sizes from "
                                       f"{SIZES}, spp from {SPPS}, adaptive_passes 3, adaptive_spp 4, base samples "
                                       f"1; samples of every pass generated on the device (seed {SEED})",
                           "step": "one request", "l2": "sample planes of every request larger than L2 except the "
                                                        "256x256 ones", "parallelism": "replicas"},
                "e2e": {"value": out["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": int(np.mean([w * h * 12 for (_, w, h, _, _) in
                                                           request_stream(args.steps, args.rate, SEED + 1000 * rank)])),
                        "form": "submit to denoised image in host memory; the per-sample input is generated on the "
                                "device from each request's seed, so nothing crosses host->device"}})
    ctx.close()
    if rank == 0:
        print(json.dumps(out))


def run_request(args):
    """One request of the serving workload at --width x --height x --spp with --passes adaptive
    passes (a small case for profiling captures): through the plain drop-in sequence, or with
    --served through rpd_server (compact storage, --storage) alone on the GPU; prints the samples
    it denoised."""
    import rpd_gb300 as R

    ctx = R.Context(0, 0)
    knobs = serving_knobs(R).replace(adaptive_passes=args.passes)
    if args.served:
        srv = R.Server(ctx, knobs, budget_bytes=args.budget_gb << 30, max_inflight=1, storage=args.storage)
        srv.submit(args.width, args.height, args.spp, SEED)
        srv.drain(600000)
        done = srv.poll(4)
        srv.close()
        assert len(done) == 1 and done[0]["status"] == 0, done
        samples = done[0]["samples"]
        counters = None
    else:
        job = R.Job(ctx, knobs.replace(image_width=args.width, image_height=args.height))
        _, samples = R.plain_request(ctx, knobs, args.width, args.height, args.spp, SEED, job=job)
        counters = job.counters()  # the last statmc_denoise's slow-pass pixels and rechecks
        job.close()
    ctx.close()
    print(json.dumps({"form": "request", "served": bool(args.served), "width": args.width, "height": args.height,
                      "spp": args.spp, "adaptive_passes": args.passes, "samples": samples,
                      "window_counters": counters}))


def run_reference(args):
    world, rank, _, dist = dist_setup()
    if rank != 0:
        return
    import rpd_gb300 as R

    cb = cpu_baseline(args, steps=args.steps, warmup=min(args.warmup, 1))
    cfg = workload_config(R)
    out = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": min(args.warmup, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32+f64", "data": "synthetic", "impl": "reference",
           "config": config_json(R, cfg, {"sample": cb["sample"]}), "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def launch_replicas(n: int, argv: list[str]) -> int:
    """Run this bench as n replica processes (torch.distributed.run, rendezvous on 127.0.0.1);
    returns their exit status."""
    import socket

    with socket.socket() as sock:
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()), *argv]
    return subprocess.call(cmd)


def main():
    global W, H, SPP, METRIC
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    # a smaller frame of the same workload, for profiling captures (the bench line is 1080p16)
    ap.add_argument("--width", type=int, default=W)
    ap.add_argument("--height", type=int, default=H)
    ap.add_argument("--spp", type=int, default=SPP)
    ap.add_argument("--grid-shape", type=int, default=0, help="random-dimension grid launch shape 1..6 (0: default)")
    ap.add_argument("--precision", choices=["fp32", "fp16"], default="fp32",
                    help="fp16: the precision form (compact per-sample storage, single-precision accumulation)")
    ap.add_argument("--form", choices=["plain", "batched", "serving", "request", "filters"], default="plain",
                    help="batched: uneven frames in one graph-captured launch (fp16 storage, autotuned shapes); "
                         "serving: a Poisson stream of requests through rpd_server (--steps requests)")
    ap.add_argument("--frames", type=int, default=48, help="frames of the batched form")
    ap.add_argument("--lanes", type=int, default=4, help="concurrent frame chains of the batched form")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: arrivals per second")
    ap.add_argument("--budget-gb", type=int, default=120, help="serving: HBM admission budget")
    ap.add_argument("--inflight", type=int, default=32, help="serving: requests on the GPU at once")
    ap.add_argument("--storage", choices=["fp16", "fp32"], default="fp16", help="serving: sample storage")
    ap.add_argument("--served", action="store_true", help="request form: through rpd_server instead of the plain drop-in")
    ap.add_argument("--alloc-blocks", type=int, default=0,
                    help="serving: blocks of each request's parallel adaptive allocation (0: half the SMs)")
    ap.add_argument("--plain-requests", type=int, default=200, help="serving: stream prefix run through the plain drop-in")
    ap.add_argument("--passes", type=int, default=1, help="request: adaptive passes of the profiled request")
    ap.add_argument("--no-served", action="store_true", help="plain form: leave out the served stream")
    ap.add_argument("--served-requests", type=int, default=2000, help="plain form: requests of the served stream")
    ap.add_argument("--no-breakdown", action="store_true", help="serving: leave out the ratio's breakdown runs")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one replica process per GPU, as the driver launches it: rerun this command under
        # torch.distributed.run (rank r uses GPU r; rank 0 prints the line)
        sys.exit(launch_replicas(args.gpus, sys.argv[1:]))
    if "WORLD_SIZE" in os.environ and int(os.environ["WORLD_SIZE"]) != args.gpus:
        sys.exit(f"--gpus {args.gpus} does not match WORLD_SIZE={os.environ['WORLD_SIZE']}")
    if (args.width, args.height, args.spp) != (W, H, SPP):
        W, H, SPP = args.width, args.height, args.spp
        METRIC = f"denoised Msamples/s at {W}x{H} {SPP}spp (plain)"
    if args.precision == "fp16":
        METRIC = METRIC.replace("(plain)", "(fp16 storage)").replace(", plain vs served", " (fp16 storage), plain")
    if args.impl == "reference":
        run_reference(args)
    elif args.form == "batched":
        run_batched(args)
    elif args.form == "serving":
        run_serving(args)
    elif args.form == "request":
        run_request(args)
    elif args.form == "filters":
        import rpd_gb300 as R

        ctx = R.Context(0, 0)
        print(json.dumps(filters_leg(R, ctx, W, H, reps=max(1, args.steps))))
        ctx.close()
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
