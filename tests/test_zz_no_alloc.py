"""The allocation-free entry point (gbr_render_triangles_noalloc) against the device/queue path.

gbr_render_triangles_noalloc is for callers that cannot allocate device memory: it renders into
buffers the caller already owns and takes its scratch space from a fixed array inside the
library.  Here it is called through the C ABI twice in a row, with different triangles, targets
and raster state, and each result must be bit-exact (the same tolerance as every other parity
test: none) to what the ordinary submit path renders from the same inputs.  The second call
also shows that what the first call left in the shared scratch array does not leak into it.
"""

import ctypes

import numpy as np
import pytest

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


def render_noalloc(lib, pos, col, width, height, cull, depth_compare, clear, depth_clear):
    """The allocation-free entry point; the caller (here: torch) owns every device buffer."""
    import torch

    d_pos = torch.from_numpy(pos).cuda()
    d_col = torch.from_numpy(col).cuda()
    d_color = torch.zeros(height * width * 4, dtype=torch.uint8, device="cuda")
    d_depth = torch.zeros(height * width, dtype=torch.float32, device="cuda") if depth_compare else None
    st = NoallocState()
    st.cull_mode = cull
    st.front_face = W.FrontFace.CCW
    st.depth_compare = depth_compare or 0
    st.depth_write_enabled = 1
    st.color_load_op = W.LoadOp.CLEAR
    st.depth_load_op = W.LoadOp.CLEAR
    for k in range(4):
        st.clear_color[k] = clear[k]
    st.clear_depth = depth_clear
    torch.cuda.synchronize()
    status = lib.gbr_render_triangles_noalloc(
        ctypes.c_void_p(d_pos.data_ptr()), ctypes.c_void_p(d_col.data_ptr()), ctypes.c_uint32(len(pos) // 3),
        ctypes.c_void_p(d_color.data_ptr()), ctypes.c_void_p(d_depth.data_ptr() if d_depth is not None else 0),
        ctypes.c_uint32(width), ctypes.c_uint32(height), ctypes.byref(st),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert status == 0, W.gpu_lib().error_text()
    color = d_color.cpu().numpy().reshape(height, width, 4)
    depth = d_depth.cpu().numpy().reshape(height, width) if d_depth is not None else None
    return color, depth


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
    try:
        for c in cases:  # two calls in a row through the allocation-free entry point
            pos, col = triangles(c["n"], c["seed"])
            args = (pos, col, c["width"], c["height"], c["cull"], c["depth_compare"], c["clear"], c["depth_clear"])
            ref_color, ref_depth = render_with_queue(dev, *args)
            got_color, got_depth = render_noalloc(lib, *args)
            assert np.array_equal(got_color, ref_color), f"colour differs in {int((got_color != ref_color).any(-1).sum())} px"
            if ref_depth is not None:
                assert np.array_equal(got_depth.view(np.uint32), ref_depth.view(np.uint32))
            assert ref_color[..., :3].any()
    finally:
        dev.close()


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
