"""The output writers (rpd_job_write_outputs, rpd_write_hdr, rpd_write_png) against the files the
reference's output_buffers writes (tests/golden/outputs_48x48.npz, captured from the reference
through the stb shim: the float data of every HDR write and the bytes of every PNG write).

The files written here are decoded by a reader in this module — PNG chunks with their CRCs and
the zlib stream, Radiance headers with flat or run-length scanlines — and compared:
  * HDR: the decoded RGBE value of each component within one mantissa step (max component / 128)
    of the reference's float (plus the stage's 1e-4 relative bar for the denoised products);
    a negative component (RGBE has no sign) decodes to 0;
  * PNG: tonemapped bytes within one step of the reference's (log2 / pow are CUDA's).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np
import pytest

from conftest import B, R, golden_config, golden_samples, load_golden

pytestmark = pytest.mark.gpu


def read_png(path) -> np.ndarray:
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", None, None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert zlib.crc32(kind + body) & 0xffffffff == crc, kind
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 2)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 3 * w + 1)
    assert np.all(raw[:, 0] == 0)  # filter type 0 on every row
    return raw[:, 1:].reshape(h, w, 3)


def read_hdr(path) -> np.ndarray:
    data = open(path, "rb").read()
    assert data.startswith(b"#?RADIANCE\n")
    header_end = data.index(b"\n\n") + 2
    assert b"FORMAT=32-bit_rle_rgbe" in data[:header_end]
    line_end = data.index(b"\n", header_end)
    _, h, _, w = data[header_end:line_end].split()
    h, w = int(h), int(w)
    pos = line_end + 1
    out = np.zeros((h, w, 4), dtype=np.uint8)
    for y in range(h):
        if 8 <= w < 32768:
            assert tuple(data[pos:pos + 4]) == (2, 2, w >> 8, w & 255)
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    if n > 128:
                        out[y, x:x + n - 128, c] = data[pos + 1]
                        x += n - 128
                        pos += 2
                    else:
                        out[y, x:x + n, c] = np.frombuffer(data[pos + 1:pos + 1 + n], dtype=np.uint8)
                        x += n
                        pos += 1 + n
                assert x == w
        else:
            out[y] = np.frombuffer(data[pos:pos + 4 * w], dtype=np.uint8).reshape(w, 4)
            pos += 4 * w
    assert pos == len(data)
    e = out[..., 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)  # (mantissa + 0.5) 2^(e-128) / 256
    return np.where(e[..., None] > 0, (out[..., :3] + 0.5) * scale[..., None], 0.0)


def assert_hdr_close(got, ref, rel=0.0):
    ref = ref.astype(np.float64)
    m = np.max(np.maximum(ref, 0.0), axis=2, keepdims=True)
    want = np.maximum(ref, 0.0)
    tol = m / 128.0 + rel * np.abs(ref) + 1e-30
    assert np.all(np.abs(got - want) <= tol), float(np.max(np.abs(got - want) - tol))


def test_tonemap_curves(gpu_ctx, tmp_path):
    meta, a = load_golden("outputs_48x48.npz")
    vals = a["tonemap_in"]
    img = vals.reshape(1, -1, 3)
    for t in range(4):
        path = tmp_path / f"t{t}.png"
        R.check(R.lib().rpd_write_png(gpu_ctx.handle, img.ctypes.data, img.shape[1], 1, R.MEM_HOST, t,
                                      str(path).encode()))
        got = read_png(path).reshape(-1, 3).astype(np.int32)
        want = a[f"tonemap_{t}"].astype(np.int32)
        diff = np.abs(got - want)
        assert diff.max() <= 1, (t, int(diff.max()))
        assert np.mean(diff == 0) >= 0.99, (t, float(np.mean(diff == 0)))


@pytest.mark.parametrize("w,h", [(5, 3), (48, 7), (300, 2)])
def test_hdr_round_trip(gpu_ctx, tmp_path, w, h):
    """Flat scanlines (width below 8) and run-length ones; zeros, tiny and large values."""
    rng = np.random.default_rng(w * h)
    img = rng.lognormal(-1.0, 3.0, (h, w, 3)).astype(np.float32)
    img[0, 0] = 0.0
    img[-1, -1] = [1e-35, 2.0, 0.0]
    img[:, :2] = img[:, :1]  # runs
    path = tmp_path / "x.hdr"
    R.check(R.lib().rpd_write_hdr(gpu_ctx.handle, img.ctypes.data, w, h, R.MEM_HOST, str(path).encode()))
    assert_hdr_close(read_hdr(path), img)


def test_job_outputs_match_the_reference(gpu_ctx, tmp_path):
    meta, a = load_golden("outputs_48x48.npz")
    cfg = golden_config(meta)
    n = cfg.image_width * cfg.image_height
    s = golden_samples(a, "s_", meta["planes"], n)
    job = R.Job(gpu_ctx, cfg)
    B.run_pipeline(job, s, meta["spp"])
    job.compute_adaptive_sample_counts()
    job.finalize()
    prefix = str(tmp_path / meta["prefix"])
    R.check(R.lib().rpd_job_write_outputs(job.handle, prefix.encode(), 0, 1))
    job.close()
    written = {p.name for p in tmp_path.iterdir()}
    assert written == set(meta["files"]) - {"out_worldpos.hdr"}, sorted(written ^ set(meta["files"]))
    # the products that pass through exp (the denoised image, its PNG, the sensitivity maps and
    # the StatMC outputs) carry the stage's 1e-4 bar; the rest are bit-exact before encoding
    close = {"out.hdr", "out_uncertainty.hdr", "out_alpha.hdr", "out_sensitivity_confidence.hdr",
             "out_sensitivity_gradient.hdr", "out_adaptive_importance.hdr", "out_var_ratio.hdr"}
    for name in sorted(written):
        ref = a["f_" + name.replace(".", "__")]
        if name.endswith(".png"):
            diff = np.abs(read_png(tmp_path / name).astype(np.int32) - ref.astype(np.int32))
            assert diff.max() <= 1, (name, int(diff.max()))
        else:
            rel = 1e-4 if (name in close or name.startswith("out_sensitivity")) else 0.0
            assert_hdr_close(read_hdr(tmp_path / name), ref, rel)
