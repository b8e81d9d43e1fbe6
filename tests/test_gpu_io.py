"""Host <-> device transfers through the C ABI on the GPU: writes are captured at call time and
applied in queue order (device staging), batched texture reads return the bytes single reads do."""

import numpy as np
import pytest

import scenes
from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    d = W.Device()
    yield d
    d.close()


def test_write_after_submit_keeps_queue_order(gpu):
    """A vertex buffer overwritten right after a submission that reads it: the submission still
    sees the old bytes, the next one the new bytes, exactly as rendering each alone."""
    s = wl.scene_colored_sphere(gpu, 256, 256)
    vb_obj, vdata = s.uploads[0]
    enc = gpu.create_command_encoder()
    s.record(enc)
    first = gpu.queue.submit([enc.finish()])
    moved = np.array(vdata, copy=True).reshape(-1, 6)
    moved[:, :3] *= 0.5  # a smaller sphere
    gpu.queue.write_buffer(vb_obj, 0, moved)
    gpu.poll(True, first)
    img_old = gpu.read_texture(s.color)
    second = s.render()
    img_new = gpu.read_texture(s.color)
    assert gpu.submission_stats(first).fragments_shaded > gpu.submission_stats(second).fragments_shaded

    ref = W.Device()
    try:
        r_old = scenes.render_scene(ref, wl.scene_colored_sphere, width=256, height=256)[0]
        s2 = wl.scene_colored_sphere(ref, 256, 256)
        ref.queue.write_buffer(s2.uploads[0][0], 0, moved)
        s2.render()
        r_new = ref.read_texture(s2.color)
    finally:
        ref.close()
    assert np.array_equal(img_old, r_old)
    assert np.array_equal(img_new, r_new)


def test_buffer_write_read_round_trip(gpu):
    rng = np.random.default_rng(3)
    data = rng.integers(0, 256, 1 << 20, dtype=np.uint8)
    buf = gpu.create_buffer_init(np.zeros(1 << 20, np.uint8))
    gpu.queue.write_buffer(buf, 4096, data[: (1 << 20) - 4096])
    out = np.empty(1 << 20, np.uint8)
    import ctypes

    st = gpu.lib.buffer_read(gpu.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
    assert st == 0, gpu.lib.error_text()
    assert not out[:4096].any()
    assert np.array_equal(out[4096:], data[: (1 << 20) - 4096])


def test_batched_texture_reads_equal_single_reads(gpu):
    ms = wl.scene_batched(gpu, n_targets=6, n_draws=12, seed=9, tri_hi=5000, side_hi=512)
    ms.render()
    targets = [p[0] for p in ms.passes]
    many = gpu.read_textures(targets)
    for t, img in zip(targets, many):
        assert np.array_equal(img, gpu.read_texture(t))
    assert gpu.lib.textures_read is not None


def test_many_small_writes_apply_in_order(gpu):
    """Hundreds of small writes (odd sizes and offsets, some overlapping earlier ones) queued
    back to back, as per-draw uniform updates are: the buffers end up exactly as writing them one
    by one on the host would leave them."""
    import ctypes

    rng = np.random.default_rng(17)
    sizes = [4096, 1000, 64 * 1024, 77]
    bufs = [gpu.create_buffer_init(np.zeros(n, np.uint8)) for n in sizes]
    mirror = [np.zeros(n, np.uint8) for n in sizes]
    for _ in range(600):
        b = int(rng.integers(0, len(sizes)))
        n = int(rng.integers(1, min(300, sizes[b]) + 1))
        off = int(rng.integers(0, sizes[b] - n + 1))
        data = rng.integers(0, 256, n, dtype=np.uint8)
        gpu.queue.write_buffer(bufs[b], off, data)
        mirror[b][off:off + n] = data
    for buf, want in zip(bufs, mirror):
        out = np.empty(want.size, np.uint8)
        st = gpu.lib.buffer_read(gpu.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
        assert st == 0, gpu.lib.error_text()
        assert np.array_equal(out, want)


def test_batched_writes_equal_single_writes(gpu):
    """gbr_queue_write_buffers: the writes land in array order (a later entry overlapping an
    earlier one wins), small and large (device-staged) entries alike, and an invalid entry
    queues none of the batch."""
    import ctypes

    rng = np.random.default_rng(23)
    big = gpu.create_buffer_init(np.zeros(3 << 20, np.uint8))
    small = gpu.create_buffer_init(np.zeros(4096, np.uint8))
    want_big, want_small = np.zeros(3 << 20, np.uint8), np.zeros(4096, np.uint8)
    items = []
    for k in range(40):
        if k % 10 == 0:
            n, off = 1 << 20, int(rng.integers(0, 2 << 20))
            buf, want = big, want_big
        else:
            n = int(rng.integers(1, 600))
            off = int(rng.integers(0, 4096 - n + 1))
            buf, want = small, want_small
        data = rng.integers(0, 256, n, dtype=np.uint8)
        items.append((buf, off, data))
        want[off:off + n] = data
    prepared = W.PreparedWrites(items)
    gpu.queue.write_buffers(prepared)
    for buf, want in ((big, want_big), (small, want_small)):
        out = np.empty(want.size, np.uint8)
        st = gpu.lib.buffer_read(gpu.handle, buf.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
        assert st == 0, gpu.lib.error_text()
        assert np.array_equal(out, want)
    # the prepared list reads its arrays at each call: change them and write again
    for _, off, data in prepared.items:
        data[:] = 7
    gpu.queue.write_buffers(prepared)
    out = np.empty(4096, np.uint8)
    gpu.lib.buffer_read(gpu.handle, small.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
    touched = np.zeros(4096, bool)
    for buf, off, data in items:
        if buf is small:
            touched[off:off + data.size] = True
    assert (out[touched] == 7).all() and np.array_equal(out[~touched], want_small[~touched])
    # an out-of-range entry: an error, and the valid entry before it is not applied either
    before = out.copy()
    bad = [(small, 0, np.full(16, 9, np.uint8)), (small, 4090, np.zeros(16, np.uint8))]
    with pytest.raises(W.GbrError):
        gpu.queue.write_buffers(bad)
    gpu.lib.buffer_read(gpu.handle, small.handle, 0, out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
    assert np.array_equal(out, before)
    assert gpu.lib.queue_write_buffers is not None


def test_texture_reads_into_pinned_memory(gpu):
    """Batched reads into pinned host memory (written by the copy kernel), into pinned memory at an
    unaligned offset and into pageable memory (both copied by cudaMemcpyAsync) all return the
    bytes of single reads."""
    import torch

    ms = wl.scene_batched(gpu, n_targets=5, n_draws=10, seed=4, tri_hi=4000, side_hi=300)
    ms.render()
    targets = [p[0] for p in ms.passes]
    want = [gpu.read_texture(t) for t in targets]
    sizes = [w.nbytes for w in want]
    pinned = [torch.zeros(n + 16, dtype=torch.uint8).pin_memory() for n in sizes]
    pageable = [np.zeros(n, np.uint8) for n in sizes]
    items = []
    for k, t in enumerate(targets):
        if k % 3 == 0:
            items.append((t, 0, pinned[k].data_ptr(), sizes[k]))           # aligned pinned: kernel
        elif k % 3 == 1:
            items.append((t, 0, pinned[k].data_ptr() + 4, sizes[k]))       # unaligned pinned: copy
        else:
            items.append((t, 0, pageable[k].ctypes.data, sizes[k]))        # pageable: copy
    gpu.read_textures_into(items)
    for k, w in enumerate(want):
        if k % 3 == 2:
            got = pageable[k]
        else:
            off = 0 if k % 3 == 0 else 4
            got = pinned[k].numpy()[off:off + sizes[k]]
            assert not pinned[k].numpy()[off + sizes[k]:].any()  # nothing past the destination
        assert np.array_equal(got, w.reshape(-1)), k
