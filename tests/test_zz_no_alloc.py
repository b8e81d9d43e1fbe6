"""The allocation-free entry point (gbr_render_triangles_noalloc) against the device/queue path
and the oracle.

gbr_render_triangles_noalloc is for callers that cannot allocate device memory: it renders into
buffers the caller already owns and takes its scratch space from a fixed array inside the
library.  Here it is called through the C ABI twice in a row, with different triangles, targets
and raster state, and each result must be bit-exact (the same tolerance as every other parity
test: none) to what the ordinary submit path renders from the same inputs and to what the CPU
oracle renders.  The second call also shows that what the first call left in the shared scratch
array does not leak into it.  The other tests cover what the header promises at the edges: a
call with no triangles only clears, a colour target loaded without a depth target keeps its
contents under the new triangles, and a call that runs out of scratch returns
GBR_ERR_OUT_OF_MEMORY with the targets left exactly as they were.
"""

import ctypes

import numpy as np
import pytest

import oracle_device
from wgpu_gb300 import _abi as A
from wgpu_gb300 import api as W

pytestmark = pytest.mark.gpu


class NoallocState(ctypes.Structure):
    _fields_ = [("cull_mode", ctypes.c_uint32), ("front_face", ctypes.c_uint32), ("depth_compare", ctypes.c_uint32),
                ("depth_write_enabled", ctypes.c_uint32), ("color_load_op", ctypes.c_uint32),
                ("depth_load_op", ctypes.c_uint32), ("clear_color", ctypes.c_float * 4),
                ("clear_depth", ctypes.c_float), ("_pad", ctypes.c_uint32)]


def triangles(n, seed):
    rng = np.random.default_rng(seed)
    nv = 3 * n
    w = rng.uniform(0.3, 2.0, nv)
    pos = np.stack([rng.uniform(-1.6, 1.6, nv) * w, rng.uniform(-1.6, 1.6, nv) * w,
                    rng.uniform(-0.2, 1.2, nv) * w, w], 1).astype(np.float32)
    col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
    return pos, col


def render_with_queue(dev, pos, col, width, height, cull, depth_compare, clear, depth_clear):
    """The existing entry points: buffers, a clip_passthrough pipeline, one render pass."""
    vb_pos = dev.create_buffer_init(pos)
    vb_col = dev.create_buffer_init(col)
    sm = dev.create_shader_module(native="clip_passthrough")
    ds = W.DepthStencilState(True, depth_compare) if depth_compare else None
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
             W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=cull), ds, sm,
        [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    depth = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT) if depth_compare else None
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, clear)],
                               W.RenderPassDepthStencilAttachment(depth, depth_clear) if depth else None)
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, vb_pos)
    rp.set_vertex_buffer(1, vb_col)
    rp.draw(range(0, len(pos)))
    rp.end()
    dev.poll(True, dev.queue.submit([enc.finish()]))
    return dev.read_texture(color), (dev.read_texture(depth).view(np.float32)[..., 0] if depth else None)


def call_noalloc(lib, pos, col, d_color, d_depth, width, height, cull, depth_compare, clear, depth_clear,
                 color_load=W.LoadOp.CLEAR, depth_load=W.LoadOp.CLEAR):
    """One call of the allocation-free entry point into caller-owned torch buffers; returns its
    status.  `pos` / `col` are device tensors (or None with no triangles)."""
    import torch

    st = NoallocState()
    st.cull_mode = cull
    st.front_face = W.FrontFace.CCW
    st.depth_compare = depth_compare or 0
    st.depth_write_enabled = 1
    st.color_load_op = color_load
    st.depth_load_op = depth_load
    for k in range(4):
        st.clear_color[k] = clear[k]
    st.clear_depth = depth_clear
    torch.cuda.synchronize()
    n = (pos.shape[0] // 3) if pos is not None else 0
    return lib.gbr_render_triangles_noalloc(
        ctypes.c_void_p(pos.data_ptr() if pos is not None else 0), ctypes.c_void_p(col.data_ptr() if col is not None else 0),
        ctypes.c_uint32(n), ctypes.c_void_p(d_color.data_ptr()),
        ctypes.c_void_p(d_depth.data_ptr() if d_depth is not None else 0),
        ctypes.c_uint32(width), ctypes.c_uint32(height), ctypes.byref(st),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def render_noalloc(lib, pos, col, width, height, cull, depth_compare, clear, depth_clear):
    """The allocation-free entry point; the caller (here: torch) owns every device buffer."""
    import torch

    d_pos = torch.from_numpy(pos).cuda()
    d_col = torch.from_numpy(col).cuda()
    d_color = torch.zeros(height * width * 4, dtype=torch.uint8, device="cuda")
    d_depth = torch.zeros(height * width, dtype=torch.float32, device="cuda") if depth_compare else None
    status = call_noalloc(lib, d_pos, d_col, d_color, d_depth, width, height, cull, depth_compare, clear, depth_clear)
    assert status == 0, W.gpu_lib().error_text()
    color = d_color.cpu().numpy().reshape(height, width, 4)
    depth = d_depth.cpu().numpy().reshape(height, width) if d_depth is not None else None
    return color, depth


def _lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.init()
    lib = W.gpu_lib().cdll
    lib.gbr_render_triangles_noalloc.restype = ctypes.c_int32
    return lib


def test_noalloc_matches_queue_path_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    torch.cuda.init()
    dev = W.Device()
    lib = dev.lib.cdll
    lib.gbr_render_triangles_noalloc.restype = ctypes.c_int32
    cases = [
        dict(n=600, seed=31, width=200, height=150, cull=W.Face.NONE, depth_compare=W.CompareFunction.LESS,
             clear=(0.1, 0.2, 0.3, 1.0), depth_clear=0.75),
        dict(n=250, seed=32, width=97, height=61, cull=W.Face.BACK, depth_compare=None,
             clear=(0.0, 0.0, 0.0, 1.0), depth_clear=1.0),
    ]
    orc = oracle_device.device()
    try:
        for c in cases:  # two calls in a row through the allocation-free entry point
            pos, col = triangles(c["n"], c["seed"])
            args = (pos, col, c["width"], c["height"], c["cull"], c["depth_compare"], c["clear"], c["depth_clear"])
            ref_color, ref_depth = render_with_queue(dev, *args)
            orc_color, orc_depth = render_with_queue(orc, *args)
            got_color, got_depth = render_noalloc(lib, *args)
            assert np.array_equal(got_color, ref_color), f"colour differs in {int((got_color != ref_color).any(-1).sum())} px"
            assert np.array_equal(got_color, orc_color), f"colour differs from the oracle in {int((got_color != orc_color).any(-1).sum())} px"
            if ref_depth is not None:
                assert np.array_equal(got_depth.view(np.uint32), ref_depth.view(np.uint32))
                assert np.array_equal(got_depth.view(np.uint32), orc_depth.view(np.uint32))
            assert ref_color[..., :3].any()
    finally:
        dev.close()
        orc.close()


def test_noalloc_zero_triangles_only_clears():
    import torch

    lib = _lib()
    w, h = 37, 23
    d_color = torch.full((h * w * 4,), 7, dtype=torch.uint8, device="cuda")
    d_depth = torch.full((h * w,), 0.25, dtype=torch.float32, device="cuda")
    clear = (0.5, 0.25, 1.0, 0.75)
    st = call_noalloc(lib, None, None, d_color, d_depth, w, h, W.Face.NONE, W.CompareFunction.LESS, clear, 0.625)
    assert st == 0, W.gpu_lib().error_text()
    # the clear is encoded as the reference encodes it: (v * 255) truncated to unorm8
    want = np.array([int(np.float32(v) * np.float32(255.0)) for v in clear], np.uint8)
    assert (d_color.cpu().numpy().reshape(h, w, 4) == want).all()
    assert (d_depth.cpu().numpy() == np.float32(0.625)).all()


def test_noalloc_load_color_without_depth():
    """Color load op LOAD with no depth target: the second call draws over the first call's
    pixels; the result equals one render pass of both triangle sets in order (oracle)."""
    import torch

    lib = _lib()
    w, h = 120, 90
    p1, c1 = triangles(80, 41)
    p2, c2 = triangles(60, 42)
    d_color = torch.zeros(h * w * 4, dtype=torch.uint8, device="cuda")
    clear = (0.2, 0.4, 0.6, 1.0)
    for k, (p, c) in enumerate(((p1, c1), (p2, c2))):
        st = call_noalloc(lib, torch.from_numpy(p).cuda(), torch.from_numpy(c).cuda(), d_color, None, w, h,
                          W.Face.NONE, None, clear, 1.0, color_load=W.LoadOp.CLEAR if k == 0 else W.LoadOp.LOAD)
        assert st == 0, W.gpu_lib().error_text()
    got = d_color.cpu().numpy().reshape(h, w, 4)
    orc = oracle_device.device()
    try:
        both_p, both_c = np.concatenate([p1, p2]), np.concatenate([c1, c2])
        want, _ = render_with_queue(orc, both_p, both_c, w, h, W.Face.NONE, None, clear, 1.0)
    finally:
        orc.close()
    assert np.array_equal(got, want), f"{int((got != want).any(-1).sum())} px differ"


def _overflow_case(kind):
    """Triangles that exceed one scratch limit: full-screen triangles on a 2048x2048 target touch
    every 16x16 tile (300 x 16,384 triangle/tile pairs > GBR_NOALLOC_MAX_BIN_ENTRIES), or
    triangles straddling the left and right clip planes (each clips into at least two pieces, so
    9,000 of them need more than GBR_NOALLOC_MAX_CLIPPED extra sub-triangles)."""
    if kind == "bins":
        n = 300
        tri = np.array([[-1.0, -1.0, 0.5, 1.0], [3.0, -1.0, 0.5, 1.0], [-1.0, 3.0, 0.5, 1.0]], np.float32)
        return np.tile(tri, (n, 1)), 2048, 2048, "GBR_NOALLOC_MAX_BIN_ENTRIES"
    n = 9000
    tri = np.array([[-3.0, -0.5, 0.5, 1.0], [3.0, -0.4, 0.5, 1.0], [0.0, 0.5, 0.5, 1.0]], np.float32)
    return np.tile(tri, (n, 1)), 64, 64, "GBR_NOALLOC_MAX_CLIPPED"


@pytest.mark.parametrize("kind", ["bins", "clipped"])
def test_noalloc_overflow_leaves_targets_unchanged(kind):
    import torch

    lib = _lib()
    pos, w, h, limit = _overflow_case(kind)
    col = np.ones((len(pos), 4), np.float32)
    d_color = torch.full((h * w * 4,), 0x5A, dtype=torch.uint8, device="cuda")
    d_depth = torch.full((h * w,), 0.125, dtype=torch.float32, device="cuda")
    st = call_noalloc(lib, torch.from_numpy(pos).cuda(), torch.from_numpy(col).cuda(), d_color, d_depth, w, h,
                      W.Face.NONE, W.CompareFunction.LESS, (1.0, 0.0, 0.0, 1.0), 1.0)
    assert st == A.ERR_OUT_OF_MEMORY, W.gpu_lib().error_text()
    assert limit in W.gpu_lib().error_text()
    torch.cuda.synchronize()
    assert (d_color == 0x5A).all().item(), "the colour target was written"
    assert (d_depth == 0.125).all().item(), "the depth target was written"
    # the scratch array is usable again: a small call right after renders bit-exact
    small = triangles(50, 43)
    got, _ = render_noalloc(lib, *small, 64, 48, W.Face.NONE, None, (0, 0, 0, 1), 1.0)
    orc = oracle_device.device()
    try:
        want, _ = render_with_queue(orc, *small, 64, 48, W.Face.NONE, None, (0, 0, 0, 1), 1.0)
    finally:
        orc.close()
    assert np.array_equal(got, want)


def test_noalloc_rejects_unknown_load_op():
    import torch

    lib = _lib()
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    st = call_noalloc(lib, None, None, buf, None, 4, 4, W.Face.NONE, None, (0, 0, 0, 1), 1.0, color_load=7)
    assert st == A.ERR_INVALID_ARGUMENT
    assert "load op" in W.gpu_lib().error_text()


def test_noalloc_rejects_oversized_requests():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = W.gpu_lib().cdll
    st = NoallocState()
    buf = torch.zeros(16, dtype=torch.uint8, device="cuda")
    status = lib.gbr_render_triangles_noalloc(None, None, ctypes.c_uint32(0), ctypes.c_void_p(buf.data_ptr()), None,
                                              ctypes.c_uint32(4096), ctypes.c_uint32(16), ctypes.byref(st), None)
    assert status == A.ERR_OUT_OF_MEMORY
    assert "GBR_NOALLOC_MAX_DIM" in W.gpu_lib().error_text()
