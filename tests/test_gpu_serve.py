"""The serving form (rpd_server, serve.cu): requests of uneven size and spp with three adaptive
passes each, admitted against an HBM budget and overlapped on the GPU. Each result is the same
alone and in the mix; with FP32 storage it is the plain per-frame drop-in's result (the same
samples through render()'s call sequence from the host); admission refuses what cannot fit and
never holds more than the budget; a queued request can be cancelled."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import R, assert_bitwise, max_rel_err, small_config

pytestmark = pytest.mark.gpu

KNOBS = dict(adaptive_passes=3, adaptive_spp=4, adaptive_base_samples=1, seed=1234)
MIX = [(96, 64, 8, 11), (64, 48, 4, 12), (160, 90, 16, 13), (33, 29, 32, 14), (128, 72, 4, 15),
       (96, 64, 8, 16), (200, 120, 8, 17), (48, 48, 64, 18), (64, 48, 16, 19), (120, 80, 4, 20)]


def knobs():
    return small_config(1, 1, **KNOBS)


def run(ctx, requests, storage="fp16", max_inflight=8, budget=0):
    """Serve `requests` [(w, h, spp, seed)], all submitted at once; returns {seed: (image, completion)}."""
    srv = R.Server(ctx, knobs(), budget_bytes=budget, max_inflight=max_inflight, storage=storage)
    bufs = {}
    try:
        for (w, h, spp, seed) in requests:
            b = R.PinnedBuffer(w * h * 12)
            bufs[seed] = b
            srv.submit(w, h, spp, seed, out=b.ptr, tag=seed)
        srv.drain(120000)
        done = {c["tag"]: c for c in srv.poll(1024)}
        stats = srv.stats()
        out = {}
        for (w, h, spp, seed) in requests:
            c = done[seed]
            assert c["status"] == 0, c
            out[seed] = (bufs[seed].array(np.float32, (h, w, 3)).copy(), c)
        return out, stats
    finally:
        srv.close()
        for b in bufs.values():
            b.free()


@pytest.mark.parametrize("storage", ["fp16", "fp32"])
def test_each_result_is_the_same_alone_and_in_the_mix(gpu_ctx, storage):
    mixed, stats = run(gpu_ctx, MIX, storage=storage, max_inflight=8)
    assert stats["completed"] == len(MIX) and stats["inflight"] == 0 and stats["queued"] == 0
    for req in (MIX[2], MIX[3], MIX[6]):
        alone, _ = run(gpu_ctx, [req], storage=storage, max_inflight=1)
        assert_bitwise(mixed[req[3]][0], alone[req[3]][0], f"request {req}")


def test_fp32_serving_equals_the_plain_drop_in(gpu_ctx):
    reqs = [MIX[0], MIX[3], MIX[6]]
    served, _ = run(gpu_ctx, reqs, storage="fp32")
    for (w, h, spp, seed) in reqs:
        img, samples = R.plain_request(gpu_ctx, knobs(), w, h, spp, seed)
        assert served[seed][1]["samples"] == samples
        assert_bitwise(served[seed][0], img, f"request {(w, h, spp, seed)}")


def test_fp16_serving_stays_close_to_the_plain_drop_in(gpu_ctx):
    """Without adaptive passes the compact storage moves the result by the rounding of its
    planes only. With them, that rounding also moves the adaptive counts a little (the
    systematic residual sampling follows a running sum), so some pixels draw one extra sample
    more or less: a Monte Carlo-sized difference, bounded loosely here and reported by the
    bench against a converged image."""
    (w, h, spp, seed) = MIX[6]
    no_adaptive = small_config(1, 1, **dict(KNOBS, adaptive_passes=0))
    srv = R.Server(gpu_ctx, no_adaptive, max_inflight=1, storage="fp16")
    buf = R.PinnedBuffer(w * h * 12)
    try:
        srv.submit(w, h, spp, seed, out=buf.ptr)
        srv.drain(60000)
        got = buf.array(np.float32, (h, w, 3)).astype(np.float64)
    finally:
        srv.close()
        buf.free()
    img, _ = R.plain_request(gpu_ctx, no_adaptive, w, h, spp, seed)
    ref = img.astype(np.float64)
    assert float(np.mean((got - ref) ** 2 / (ref ** 2 + 1e-2))) <= 1e-6
    served, _ = run(gpu_ctx, [MIX[6]], storage="fp16")
    img, _ = R.plain_request(gpu_ctx, knobs(), w, h, spp, seed)
    ref = img.astype(np.float64)
    assert float(np.mean((served[seed][0] - ref) ** 2 / (ref ** 2 + 1e-2))) <= 1e-2


def test_sample_counts_of_the_adaptive_passes(gpu_ctx):
    out, _ = run(gpu_ctx, MIX[:4])
    for (w, h, spp, seed) in MIX[:4]:
        c = out[seed][1]
        assert c["samples"] <= (spp + 3 * 4) * w * h
        assert c["samples"] >= spp * w * h + 3 * (w * h)  # at least the per-pixel floor of each pass
        assert c["done_ms"] >= c["admit_ms"] >= c["submit_ms"]


def test_admission_keeps_to_the_budget(gpu_ctx):
    # a budget of a few of these small requests: some wait for memory, none exceeds it
    srv = R.Server(gpu_ctx, knobs(), budget_bytes=96 << 20, max_inflight=8)
    try:
        for (w, h, spp, seed) in MIX:
            srv.submit(w, h, spp, seed, tag=seed)
        srv.drain(120000)
        st = srv.stats()
        assert st["completed"] == len(MIX)
        assert 0 < st["bytes_peak"] <= st["bytes_budget"]
        assert all(c["status"] == 0 for c in srv.poll(64))
    finally:
        srv.close()
    tight = R.Server(gpu_ctx, knobs(), budget_bytes=64 << 20, max_inflight=8)
    try:
        with pytest.raises(R.RpdError, match="budget"):
            tight.submit(2048, 1152, 64, 1)
        assert tight.stats()["rejected"] == 1
    finally:
        tight.close()


def test_cancel_a_queued_request(gpu_ctx):
    srv = R.Server(gpu_ctx, knobs(), max_inflight=1)
    try:
        ids = [srv.submit(w, h, spp, seed, tag=seed) for (w, h, spp, seed) in MIX[:4]]
        srv.cancel(ids[-1])
        srv.drain(120000)
        done = {c["id"]: c for c in srv.poll(64)}
        assert done[ids[-1]]["status"] == 9  # RPD_ERR_CANCELLED
        assert all(done[i]["status"] == 0 for i in ids[:-1])
        with pytest.raises(R.RpdError):
            srv.cancel(ids[0])  # finished: nothing queued under this id
    finally:
        srv.close()


def test_bad_requests_are_refused_on_submit(gpu_ctx):
    srv = R.Server(gpu_ctx, knobs(), max_inflight=2)
    try:
        with pytest.raises(R.RpdError, match="positive"):
            srv.submit(0, 10, 4, 1)
        with pytest.raises(R.RpdError, match="positive"):
            srv.submit(10, 10, 70000, 1)
        assert srv.stats()["submitted"] == 0
    finally:
        srv.close()
