"""Speed of the oracle restatement against the reference's own code (TEST INFRASTRUCTURE).

bench.py's reference arm times oracle/rpd_oracle.c on the GPU machine, where the reference
checkout (and so oracle/_ref) does not exist. This script times both implementations of the
stage on the same workload and the same host cores wherever oracle/_ref is built, so the
arm's speed can be compared with the reference's own: the bench's 1920x270 band of the
1920x1080 16-spp synthetic frame, with bench.py's knobs, accumulate + recompute_sensitivity +
statmc_denoise + variance_denoise per step, all host cores, best and mean of `--steps`.

    python oracle/compare_speed.py [--steps 5]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402
from oracle import binding as B  # noqa: E402

R = B.R


def timed(job, samples, spp, steps):
    B.run_pipeline(job, samples, spp)  # warm-up
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        B.run_pipeline(job, samples, spp)
        times.append(time.perf_counter() - t0)
    return times


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=5)
    args = ap.parse_args()
    if not B.have_ref():
        sys.exit("oracle/_ref is not built (make -C oracle ref needs the reference checkout)")
    threads = os.cpu_count() or 1
    w, band = bench.W, bench.H // 4
    cfg = bench.workload_config(R, w, band)
    samples = B.synth_fill(R.synth_params(w, band, bench.SEED), 0, w * band, bench.SPP, threads=threads)
    out = {"band": f"{w}x{band}, {bench.SPP} spp", "threads": threads}
    for name, job in (("port", B.OracleJob(cfg, threads=threads)), ("reference", B.RefJob(cfg, threads=threads))):
        t = timed(job, samples, bench.SPP, args.steps)
        job.close()
        out[name] = {"best_s": min(t), "mean_s": sum(t) / len(t),
                     "msamples_per_s": w * band * bench.SPP / (sum(t) / len(t)) / 1e6}
    out["port_over_reference_speed"] = out["port"]["msamples_per_s"] / out["reference"]["msamples_per_s"]
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
