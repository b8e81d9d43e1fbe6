"""Host-side pieces of bench.py that decide what its line reports, checked without a GPU: the
clock summary (the median SM clock under load and the throttle reasons that reject a run) and
the byte model behind the roofline's `achieved` (target pixels, depth per covered fragment,
colour / blend / texel bytes per fragment-stage run)."""

import types

import pytest

import bench
from wgpu_gb300 import api as W


def sampler_with(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s


def row(sm, mx=2070, hw="Not Active", hw_thermal="Not Active", sw_thermal="Not Active", power_cap="Not Active"):
    return f"0, {sm}, {mx}, 900.00, 0x0000000000000000, {hw}, {hw_thermal}, {sw_thermal}, {power_cap}"


def test_clock_summary_median_and_reasons():
    s = sampler_with([row(2070), row(1900), row(2070, power_cap="Active"), row(2055)]).summary()
    assert s["sm_mhz"] == pytest.approx((2055 + 2070) / 2) and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 4


def test_clock_summary_reports_thermal_and_hw_slowdown():
    s = sampler_with([row(1500, hw="Active"), row(1500, sw_thermal="Active"), row(1500, hw_thermal="Active")]).summary()
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_summary_skips_malformed_lines_and_reports_unsampled():
    assert sampler_with(["", "garbage", "0, [N/A], 2070, 1, 0, a, b, c, d"]).summary() == {
        "sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
    s = sampler_with(["garbage", row(2000)]).summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 2000.0


def tex(w, h, fmt):
    return types.SimpleNamespace(width=w, height=h, format=fmt)


def stats(covered, fs, tex_runs):
    return types.SimpleNamespace(fragments_shaded=covered, fs_invocations=fs, texture_fs_invocations=tex_runs)


def test_byte_model_depth_tested_textured_passes():
    wk = types.SimpleNamespace(blend_bytes=0, texel_bytes=4)
    scene = types.SimpleNamespace(passes=[(tex(100, 50, W.TextureFormat.RGBA8_UNORM), tex(100, 50, 9), []),
                                          (tex(10, 10, W.TextureFormat.RGBA8_UNORM), tex(10, 10, 9), [])])
    b = bench.algorithmic_bytes(wk, scene, stats(covered=7000, fs=4000, tex_runs=1500))
    pixels = (100 * 50 + 10 * 10) * (4 + 4)  # colour + depth written once
    assert b["target_pixels"] == pixels
    assert b["total"] == pixels + 7000 * 8 + 4000 * 4 + 1500 * 4


def test_byte_model_blended_float_target_without_depth():
    wk = types.SimpleNamespace(blend_bytes=8, texel_bytes=0)
    scene = types.SimpleNamespace(color=tex(64, 32, W.TextureFormat.RGBA16_FLOAT), depth=None)
    b = bench.algorithmic_bytes(wk, scene, stats(covered=5000, fs=5000, tex_runs=0))
    # no depth bytes; every blended fragment reads and writes its 8-byte Rgba16Float texel
    assert b["total"] == 64 * 32 * 8 + 5000 * (8 + 8)


def test_measured_peak_comes_from_the_measured_file():
    peak, source = bench.measured_peak_hbm()
    assert peak > 1000 and source in ("measured", "fallback")
