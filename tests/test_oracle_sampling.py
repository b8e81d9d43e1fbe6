"""Extension-profile texturing in the oracle (no GPU): the sRGB tables against the transfer
function, and LOD selection, bilinear / trilinear filtering, address modes and sRGB decode against
an independent float64 model of the sampling rules, on screen-aligned quads whose LOD is known
in closed form; sRGB-target encoding of a clear colour.

The oracle computes in binary32 and the model in float64, so outputs may differ by one unorm8
step where a value lies next to a truncation boundary; the GPU tests hold the kernels to the
oracle bit for bit."""

import math
import os
import re
import struct

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "wgpu-cpu_gb300", "csrc", "srgb_tables.h")


def eotf(c):
    c = np.asarray(c, dtype=np.float64)
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


def f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def parse_table(name: str) -> np.ndarray:
    text = open(HEADER).read()
    body = re.search(name + r"\[256\] = \{(.*?)\};", text, re.S).group(1)
    vals = [v.strip().rstrip("f") for v in body.replace("\n", " ").split(",") if v.strip()]
    return np.array([float.fromhex(v) if "0x" in v else float(v) for v in vals])


def test_srgb_tables_match_the_transfer_function():
    dec = parse_table("kSrgbToLinear")
    thr = parse_table("kSrgbEncodeThreshold")
    assert dec.size == 256 and thr.size == 256
    for k in range(256):
        assert dec[k] == f32(float(eotf(k / 255.0)))
    for k in range(1, 256):
        assert thr[k] == f32(float(eotf((k - 0.5) / 255.0)))
    assert np.all(np.diff(thr[1:]) > 0)


# ---------------------------------------------------------------- float64 model of the rules
def wrap(i, n, mode):
    if mode == W.AddressMode.REPEAT:
        return np.mod(i, n)
    if mode == W.AddressMode.MIRROR_REPEAT:
        t = np.mod(i, 2 * n)
        return np.where(t < n, t, 2 * n - 1 - t)
    return np.clip(i, 0, n - 1)


def decoded(img, srgb):
    f = img.astype(np.float64) / 255.0
    if srgb:
        f[..., :3] = eotf(f[..., :3])
    return f


def sample_level(dimg, u, v, linear, mode):
    h, w = dimg.shape[:2]
    if not linear:
        x = wrap(np.floor(u * w).astype(np.int64), w, mode)
        y = wrap(np.floor(v * h).astype(np.int64), h, mode)
        return dimg[y, x]
    xs, ys = u * w - 0.5, v * h - 0.5
    xf, yf = np.floor(xs), np.floor(ys)
    fx, fy = (xs - xf)[:, None], (ys - yf)[:, None]
    x0, y0 = xf.astype(np.int64), yf.astype(np.int64)
    x1, y1 = wrap(x0 + 1, w, mode), wrap(y0 + 1, h, mode)
    x0, y0 = wrap(x0, w, mode), wrap(y0, h, mode)
    top = dimg[y0, x0] + (dimg[y0, x1] - dimg[y0, x0]) * fx
    bot = dimg[y1, x0] + (dimg[y1, x1] - dimg[y1, x0]) * fx
    return top + (bot - top) * fy


def sample_model(levels, srgb, u, v, lod, mode, mag, min_, mip):
    d = [decoded(im, srgb) for im in levels]
    last = len(levels) - 1
    if lod <= 0:
        return sample_level(d[0], u, v, mag == W.FilterMode.LINEAR, mode)
    lin = min_ == W.FilterMode.LINEAR
    if mip != W.FilterMode.LINEAR:
        return sample_level(d[min(last, int(math.ceil(lod + 0.5)) - 1)], u, v, lin, mode)
    lc = min(lod, float(last))
    l0 = int(math.floor(lc))
    f = lc - l0
    c0 = sample_level(d[l0], u, v, lin, mode)
    if f == 0 or l0 >= last:
        return c0
    return c0 + (sample_level(d[l0 + 1], u, v, lin, mode) - c0) * f


def unorm8_trunc(x):
    return np.clip(np.floor(np.clip(x * 255.0, 0.0, 255.0)), 0, 255).astype(np.int64)


@pytest.fixture(scope="module")
def orc_ext():
    return oracle_device.device(profile=W.Profile.EXTENSION, threads=8)


@pytest.fixture(scope="module")
def levels():
    return wl.mip_chain(wl.checker_noise_texture(256, 7))


@pytest.mark.parametrize("side,uv_scale,srgb,mode,mag,min_,mip", [
    (64, 1.0, False, W.AddressMode.REPEAT, 1, 1, 1),            # LOD 2 exactly: level 2 alone
    (48, 1.0, True, W.AddressMode.REPEAT, 1, 1, 1),             # LOD 2.415: levels 2 and 3 blended
    (32, 2.0, False, W.AddressMode.MIRROR_REPEAT, 1, 1, 1),     # LOD 4, mirrored second period
    (101, 1.37, True, W.AddressMode.CLAMP_TO_EDGE, 1, 0, 1),    # nearest within levels, linear across
    (90, 1.3, False, W.AddressMode.REPEAT, 1, 1, 0),            # LOD 1.89: nearest mip = level 2
    (512, 1.0, False, W.AddressMode.REPEAT, 1, 1, 1),           # LOD -1: magnified, bilinear level 0
    (383, 1.0, True, W.AddressMode.REPEAT, 0, 1, 1),            # LOD -0.58: magnified, nearest level 0
])
# (sizes and uv scales keep nearest-filter texel boundaries off exact binary values, where the
# float64 model and the binary32 oracle could legitimately pick neighbouring texels)
def test_oracle_sampling_matches_model(orc_ext, levels, side, uv_scale, srgb, mode, mag, min_, mip):
    W_, H_ = 600, 560
    x0, y0 = 17, 9
    out, n = scenes.textured_quad(orc_ext, W_, H_, x0, y0, side, levels, uv_scale=uv_scale, srgb_texture=srgb,
                                  address=mode, mag=mag, min_=min_, mip=mip)
    assert n > side * side
    lod = math.log2(256.0 * uv_scale / side)
    ys, xs = np.mgrid[y0:y0 + side, x0:x0 + side]
    u = (xs.ravel() - x0) / side * uv_scale
    v = (ys.ravel() - y0) / side * uv_scale
    want = unorm8_trunc(sample_model(levels, srgb, u, v, lod, mode, mag, min_, mip))
    got = out[y0:y0 + side, x0:x0 + side].reshape(-1, 4).astype(np.int64)
    diff = np.abs(got - want)
    assert diff.max() <= 1, f"max diff {diff.max()} at {np.unravel_index(diff.argmax(), diff.shape)}"
    assert (diff == 0).mean() > 0.9  # exact half-texel averages sit on truncation boundaries


def test_oracle_srgb_target_encodes_clear(orc_ext):
    """Rgba8UnormSrgb targets in the extension profile store sRGB-encoded colour (RGB rounded to the
    nearest unorm8 of the encoded value, alpha rounded); the parity profile keeps truncation."""
    vals = [0.0, 0.002, 0.0031308, 0.01, 0.18, 0.2140, 0.5, 0.73, 0.999, 1.0]
    for c in vals:
        clear = (c, min(1.0, c * 0.5), min(1.0, c + 0.1), 0.37)
        for prof in (W.Profile.EXTENSION, W.Profile.PARITY):
            dev = orc_ext if prof == W.Profile.EXTENSION else oracle_device.device()
            tex = dev.create_texture(4, 4, W.TextureFormat.RGBA8_UNORM_SRGB)
            enc = dev.create_command_encoder()
            rp = enc.begin_render_pass([W.RenderPassColorAttachment(tex, clear)], None)
            rp.end()
            dev.poll(True, dev.queue.submit([enc.finish()]))
            px = dev.read_texture(tex)[0, 0].astype(np.int64)
            lin = np.array([f32(x) for x in clear], np.float64)
            if prof == W.Profile.EXTENSION:
                e = np.where(lin[:3] <= 0.0031308, lin[:3] * 12.92, 1.055 * lin[:3] ** (1 / 2.4) - 0.055)
                want = list(np.floor(e * 255.0 + 0.5).astype(np.int64)) + [int(np.rint(lin[3] * 255.0))]
            else:
                want = list(unorm8_trunc(lin))
            assert list(px) == want, (prof, clear, px, want)
