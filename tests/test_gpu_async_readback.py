"""GPU: asynchronous texture readback (gbr_queue_read_textures, wgpu's copy_texture_to_buffer +
map_async) in a pipelined frame loop.  Every frame changes its uniforms; frame k + 1 is enqueued
while frame k's readback runs, and the worker plans it past the queued writes and readback.  Each
frame must read back exactly the bytes of rendering it alone with a blocking readback."""

import numpy as np
import pytest

from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

W_, H_ = 512, 512


def frame_matrices(n=6):
    return [wl.mvp_bytes(wl.camera_mvp(W_, H_, model=wl.random_rotation(np.random.default_rng(100 + k))))
            for k in range(n)]


def blocking_frames(mats):
    dev = W.Device()
    try:
        s = wl.scene_colored_sphere(dev, W_, H_)
        ub = s.uploads[2][0]
        out = []
        for m in mats:
            dev.queue.write_buffer(ub, 0, np.frombuffer(m, np.uint8))
            s.render()
            out.append(dev.read_texture(s.color).copy())
        return out
    finally:
        dev.close()


def test_pipelined_frames_read_back_their_own_targets():
    mats = frame_matrices()
    ref = blocking_frames(mats)
    assert not np.array_equal(ref[0], ref[1])  # the frames differ
    dev = W.Device()
    try:
        s = wl.scene_colored_sphere(dev, W_, H_)
        ub = s.uploads[2][0]
        enc = dev.create_command_encoder()
        s.record(enc)
        cmd = enc.finish()
        outs = [np.full((H_, W_, 4), 0xCD, np.uint8) for _ in mats]
        idx = []
        for m, o in zip(mats, outs):
            dev.queue.write_buffer(ub, 0, np.frombuffer(m, np.uint8))
            dev.queue.submit([cmd])
            idx.append(dev.read_textures_into_async([(s.color, 0, o.ctypes.data, o.nbytes)]))
        assert all(b > a for a, b in zip(idx, idx[1:]))
        dev.poll(True, idx[-1])
        for k, (o, r) in enumerate(zip(outs, ref)):
            assert np.array_equal(o, r), f"frame {k}: {int((o != r).any(-1).sum())} pixels differ"
        for i in idx:  # every readback index completed without error
            dev.poll(True, i)
    finally:
        dev.close()


def test_async_readback_validates_at_the_call():
    dev = W.Device()
    try:
        t = dev.create_texture(64, 64, W.TextureFormat.RGBA8_UNORM)
        small = np.empty(64 * 64 * 4 - 1, np.uint8)
        with pytest.raises(W.GbrError):
            dev.read_textures_into_async([(t, 0, small.ctypes.data, small.nbytes)])
        ok = np.empty(64 * 64 * 4, np.uint8)
        i = dev.read_textures_into_async([(t, 0, ok.ctypes.data, ok.nbytes)])
        dev.poll(True, i)
    finally:
        dev.close()


def test_double_buffered_frames_read_back_their_own_targets():
    """Two target sets alternate (as a swapchain's images): frame k + 1 renders into the other set
    while frame k's readback runs on the copy engines, and frame k + 2 (the first set again) waits
    for frame k's readback before it overwrites those targets."""
    mats = frame_matrices(8)
    ref = blocking_frames(mats)
    dev = W.Device()
    try:
        s = wl.scene_colored_sphere(dev, W_, H_)
        sb = wl.with_new_targets(s)
        ub = s.uploads[2][0]
        cmds = []
        for sc in (s, sb):
            enc = dev.create_command_encoder()
            sc.record(enc)
            cmds.append(enc.finish())
        outs = [np.full((H_, W_, 4), 0xCD, np.uint8) for _ in mats]
        idx = []
        for k, (m, o) in enumerate(zip(mats, outs)):
            dev.queue.write_buffer(ub, 0, np.frombuffer(m, np.uint8))
            dev.queue.submit([cmds[k % 2]])
            tgt = (s, sb)[k % 2].color
            idx.append(dev.read_textures_into_async([(tgt, 0, o.ctypes.data, o.nbytes)]))
        dev.poll(True, idx[-1])
        for k, (o, r) in enumerate(zip(outs, ref)):
            assert np.array_equal(o, r), f"frame {k}: {int((o != r).any(-1).sum())} pixels differ"
    finally:
        dev.close()


def test_texture_write_waits_for_the_readback_in_flight():
    """A write_texture queued behind an asynchronous readback of the same texture must not land
    before the readback has copied the texture out."""
    dev = W.Device()
    try:
        t = dev.create_texture(1024, 1024, W.TextureFormat.RGBA8_UNORM)
        a = np.random.default_rng(1).integers(0, 256, (1024, 1024, 4), dtype=np.uint8)
        b = np.random.default_rng(2).integers(0, 256, (1024, 1024, 4), dtype=np.uint8)
        dev.queue.write_texture(t, a)
        got = np.empty_like(a)
        i = dev.read_textures_into_async([(t, 0, got.ctypes.data, got.nbytes)])
        dev.queue.write_texture(t, b)
        dev.poll(True, i)
        assert np.array_equal(got, a)
        assert np.array_equal(dev.read_texture(t), b)
    finally:
        dev.close()
