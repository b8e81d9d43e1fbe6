"""Encoder copies and clears in the oracle (no GPU).  The reference leaves them todo!
(command.rs:37-115): the parity profile rejects each one; the extension profile gives WebGPU's
results, checked here against numpy slicing of the initial data."""

import numpy as np
import pytest

import oracle_device
import scenes
from wgpu_gb300 import _abi as A
from wgpu_gb300 import api as W


def test_copies_follow_webgpu_semantics():
    dev = oracle_device.device(profile=W.Profile.EXTENSION)
    r = scenes.copy_scenario(dev)
    a = r["a"]
    want_b = np.zeros(4096, np.uint8)
    want_b[512:1536] = a[256:1280]
    want_b[:64] = 0
    assert np.array_equal(r["B"], want_b)
    # buffer -> T1 mip 0 layer 1: 16 x 8 texels from A with 256-byte rows
    t1 = [lv.copy() for lv in r["t1_init"]]
    block = np.stack([a[y * 256: y * 256 + 64].reshape(16, 4) for y in range(8)])
    t1[0][1, 3:11, 5:21] = block
    for m in range(3):
        assert np.array_equal(r["T1"][m], t1[m]), m
    # T1 mip 1 layer 0 (2, 1) 10 x 6 -> T2 mip 1 layer 1 (20, 10); T2 mip 2 cleared
    t2 = [lv.copy() for lv in r["t2_init"]]
    t2[1][1, 10:16, 20:30] = t1[1][0, 1:7, 2:12]
    t2[2][:] = 0
    for m in range(3):
        assert np.array_equal(r["T2"][m], t2[m]), m
    # T1 mip 0 layer 1 (5, 3) -> C with 256-byte rows
    want_c = np.zeros(4096, np.uint8)
    for y in range(8):
        want_c[y * 256: y * 256 + 64] = t1[0][1, 3 + y, 5:21].reshape(-1)
    assert np.array_equal(r["C"], want_c)
    # the copy between the passes saw the first frame; the target then holds the red clear
    assert (r["X"] == np.array([255, 0, 0, 255], np.uint8)).all()
    assert r["Y"].any() and not np.array_equal(r["Y"], r["X"])


@pytest.mark.parametrize("op", ["b2b", "b2t", "t2b", "t2t", "clear_b", "clear_t"])
def test_parity_profile_rejects_copies(op):
    dev = oracle_device.device()
    ba = dev.create_buffer_init(np.zeros(1024, np.uint8))
    bb = dev.create_buffer_init(np.zeros(1024, np.uint8))
    T = dev.create_texture(8, 8, W.TextureFormat.RGBA8_UNORM)
    U = dev.create_texture(8, 8, W.TextureFormat.RGBA8_UNORM)
    enc = dev.create_command_encoder()
    {"b2b": lambda: enc.copy_buffer_to_buffer(ba, 0, bb, 0, 64),
     "b2t": lambda: enc.copy_buffer_to_texture(ba, 0, 256, 1, T, (8, 1, 1)),
     "t2b": lambda: enc.copy_texture_to_buffer(T, ba, 0, 256, 1, (8, 1, 1)),
     "t2t": lambda: enc.copy_texture_to_texture(T, U, (8, 8, 1)),
     "clear_b": lambda: enc.clear_buffer(ba),
     "clear_t": lambda: enc.clear_texture(T)}[op]()
    with pytest.raises(W.GbrError) as e:
        dev.queue.submit([enc.finish()])
    assert e.value.status == A.ERR_UNSUPPORTED
    assert "todo" in e.value.message


def test_write_buffers_falls_back_to_single_writes():
    """Queue.write_buffers on a library without gbr_queue_write_buffers (the oracle) issues one
    write_buffer per entry, in order."""
    import ctypes

    dev = oracle_device.device(profile=W.Profile.EXTENSION)
    assert dev.lib.queue_write_buffers is None
    buf = dev.create_buffer_init(np.zeros(256, np.uint8))
    items = [(buf, 0, np.full(100, 1, np.uint8)), (buf, 50, np.full(100, 2, np.uint8)), (buf, 200, np.arange(56, dtype=np.uint8))]
    dev.queue.write_buffers(items)
    out = np.empty(256, np.uint8)
    assert dev.lib.buffer_read(dev.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes) == 0
    want = np.zeros(256, np.uint8)
    for _, off, data in items:
        want[off:off + data.size] = data
    assert np.array_equal(out, want)


def test_prepared_writes_accept_any_buffer():
    """PreparedWrites takes bytes, bytearrays, memoryviews and non-contiguous arrays (copied to a
    contiguous array it keeps), and contiguous arrays by reference: the bytes written are the
    array's contents at each write_buffers call."""
    import ctypes

    dev = oracle_device.device(profile=W.Profile.EXTENSION)
    buf = dev.create_buffer_init(np.zeros(64, np.uint8))
    live = np.zeros(8, np.uint8)
    strided = np.arange(32, dtype=np.uint8)[::2]  # not contiguous
    items = [(buf, 0, b"\x01\x02\x03\x04"), (buf, 4, bytearray(b"\x05\x06")), (buf, 8, memoryview(b"\x07" * 4)),
             (buf, 16, strided), (buf, 40, live), (buf, 60, b"")]
    prepared = W.PreparedWrites(items)
    live[:] = 9  # after preparing: the contiguous array is read when written
    dev.queue.write_buffers(prepared)
    out = np.empty(64, np.uint8)
    assert dev.lib.buffer_read(dev.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes) == 0
    want = np.zeros(64, np.uint8)
    want[0:4] = [1, 2, 3, 4]
    want[4:6] = [5, 6]
    want[8:12] = 7
    want[16:32] = strided
    want[40:48] = 9
    assert np.array_equal(out, want)


def test_buffer_init_from_strided_array():
    """create_buffer_init and write_buffer take a non-contiguous array's elements in order."""
    import ctypes

    dev = oracle_device.device(profile=W.Profile.EXTENSION)
    src = np.arange(40, dtype=np.float32).reshape(8, 5)[:, 1:4]  # 8 x 3, not contiguous
    buf = dev.create_buffer_init(src)
    assert buf.size == src.nbytes
    out = np.empty(src.size, np.float32)
    assert dev.lib.buffer_read(dev.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes) == 0
    assert np.array_equal(out, src.reshape(-1))
    dev.queue.write_buffer(buf, 0, src[::-1])
    assert dev.lib.buffer_read(dev.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes) == 0
    assert np.array_equal(out, src[::-1].reshape(-1))
