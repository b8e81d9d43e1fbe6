"""Buffer ranges whose end does not fit in 64 bits are rejected, never wrapped.

An offset of 2^64 - 4 with a size of 8 wraps to an end of 4, which a check written as
`offset + size > buffer_size` accepts; the reference converts every range with try_into and slices
its Vec<u8> (buffer.rs, device.rs:332-344), so such a range panics there.  Every entry point that
takes a buffer range (write_buffer, write_buffers, buffer reads, buffer-to-buffer and
buffer/texture copies, clear_buffer, index and vertex buffer slices, bind group buffer entries,
write_texture layouts) must return GBR_ERR_VALIDATION instead.  The same cases run through the
oracle on the CPU and through libgbr on the GPU.
"""

import ctypes

import numpy as np
import pytest

import oracle_device
from wgpu_gb300 import _abi as A
from wgpu_gb300 import api as W

HUGE = (1 << 64) - 4  # a multiple of 4 (and of every texel size used here): only the range is wrong


def _devices():
    return [pytest.param("oracle", id="oracle"), pytest.param("gpu", id="gpu", marks=pytest.mark.gpu)]


@pytest.fixture(params=_devices())
def dev(request):
    if request.param == "oracle":
        d = oracle_device.device(profile=W.Profile.EXTENSION)
    else:
        d = W.Device(profile=W.Profile.EXTENSION)
    yield d
    d.close()


def _expect_validation(dev, fn):
    try:
        idx = fn()
        if idx is not None:  # a submission: the error may surface when it executes
            dev.poll(True, idx)
    except W.GbrError as e:
        assert e.status == A.ERR_VALIDATION, str(e)
        return
    pytest.fail("the wrapped range was accepted")


def test_write_buffer(dev):
    buf = dev.create_buffer(64)
    data = np.arange(8, dtype=np.uint8)
    st = dev.lib.queue_write_buffer(dev.handle, buf.handle, HUGE, data.ctypes.data, 8)
    assert st == A.ERR_VALIDATION, dev.lib.error_text()


def test_write_buffers(dev):
    if dev.lib.queue_write_buffers is None:
        pytest.skip("this library has no batched write entry point")
    buf = dev.create_buffer(64)
    data = np.arange(8, dtype=np.uint8)
    arr = (A.BufferWrite * 2)(A.BufferWrite(buf.handle, 0, data.ctypes.data, 8),
                              A.BufferWrite(buf.handle, HUGE, data.ctypes.data, 8))
    st = dev.lib.queue_write_buffers(dev.handle, 2, ctypes.cast(arr, ctypes.c_void_p))
    assert st == A.ERR_VALIDATION, dev.lib.error_text()


def test_buffer_read(dev):
    buf = dev.create_buffer(64)
    out = np.zeros(8, np.uint8)
    st = dev.lib.buffer_read(dev.handle, buf.handle, HUGE, out.ctypes.data, 8)
    assert st == A.ERR_VALIDATION, dev.lib.error_text()


def test_copy_buffer_to_buffer(dev):
    a, b = dev.create_buffer(64), dev.create_buffer(64)
    for so, do in ((HUGE, 0), (0, HUGE)):
        enc = dev.create_command_encoder()
        enc.copy_buffer_to_buffer(a, so, b, do, 8)
        _expect_validation(dev, lambda: dev.queue.submit([enc.finish()]))


def test_clear_buffer(dev):
    buf = dev.create_buffer(64)
    enc = dev.create_command_encoder()
    enc.clear_buffer(buf, HUGE, 8)
    _expect_validation(dev, lambda: dev.queue.submit([enc.finish()]))


def test_copy_buffer_texture_layout(dev):
    buf = dev.create_buffer(4096)
    tex = dev.create_texture(4, 4, W.TextureFormat.RGBA8_UNORM)
    for op in ("to_texture", "to_buffer"):
        enc = dev.create_command_encoder()
        if op == "to_texture":
            enc.copy_buffer_to_texture(buf, HUGE, 256, 4, tex, (4, 4, 1))
        else:
            enc.copy_texture_to_buffer(tex, buf, HUGE, 256, 4, (4, 4, 1))
        _expect_validation(dev, lambda: dev.queue.submit([enc.finish()]))


def test_write_texture_layout(dev):
    tex = dev.create_texture(4, 4, W.TextureFormat.RGBA8_UNORM)
    data = np.zeros(64, np.uint8)
    with pytest.raises(W.GbrError) as ei:
        dev.queue.write_texture(tex, data, offset=HUGE)
    assert ei.value.status == A.ERR_VALIDATION


@pytest.mark.parametrize("which", ["index", "vertex"])
def test_index_and_vertex_slices(dev, which):
    buf = dev.create_buffer(64)
    target = dev.create_texture(8, 8, W.TextureFormat.RGBA8_UNORM)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(target, "clear")])
    if which == "index":
        rp.set_index_buffer(buf, W.IndexFormat.UINT32, HUGE, 8)
    else:
        rp.set_vertex_buffer(0, buf, HUGE, 8)
    rp.end()
    _expect_validation(dev, lambda: dev.queue.submit([enc.finish()]))


def test_bind_group_buffer_entry(dev):
    buf = dev.create_buffer(64)
    with pytest.raises(W.GbrError) as ei:
        dev.create_bind_group([W.BindGroupEntry(0, buf, HUGE, 8)])
    assert ei.value.status == A.ERR_VALIDATION
