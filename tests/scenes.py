"""Extra seeded scenes for the parity tests (built through the public API, any device)."""

import numpy as np

from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl


def random_clip_triangles(dev, n_tris, width, height, seed, topology=W.PrimitiveTopology.TRIANGLE_LIST,
                          index_format=None, depth=None, cull=W.Face.NONE, front_face=W.FrontFace.CCW,
                          depth_write=True, spread=1.6, w_range=(0.3, 2.0), z_range=(-0.3, 1.3),
                          clear=(0.1, 0.2, 0.3, 1.0), color_format=W.TextureFormat.RGBA8_UNORM,
                          instances=1, base_vertex=0, scissor=None, viewport=None, blend=None, depth_clear=0.75):
    """Random triangles given directly in clip space (clip_passthrough program): they cross
    every clip plane, so the clipper, the sub-triangle order and degenerate spans all get hit."""
    rng = np.random.default_rng(seed)
    nv = n_tris * 3 if topology == W.PrimitiveTopology.TRIANGLE_LIST else n_tris + 2
    w = rng.uniform(*w_range, nv)
    pos = np.stack([rng.uniform(-spread, spread, nv) * w, rng.uniform(-spread, spread, nv) * w,
                    rng.uniform(*z_range, nv) * w, w], 1).astype(np.float32)
    col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
    pad = np.zeros((max(0, base_vertex), 4), np.float32)
    vb_pos = dev.create_buffer_init(np.concatenate([pad, pos]))
    vb_col = dev.create_buffer_init(np.concatenate([pad, col]))
    idx = None
    if index_format is not None:
        perm = np.arange(nv)
        if index_format == W.IndexFormat.UINT16:
            idx = dev.create_buffer_init(perm.astype(np.uint16))
        else:
            idx = dev.create_buffer_init(perm.astype(np.uint32))
    sm = dev.create_shader_module(native="clip_passthrough")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
             W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])],
        W.PrimitiveState(topology, front_face=front_face, cull_mode=cull),
        W.DepthStencilState(depth_write, depth) if depth is not None else None, sm,
        [W.ColorTargetState(color_format, blend)])
    color = dev.create_texture(width, height, color_format)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT) if depth is not None else None
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, clear)],
                               W.RenderPassDepthStencilAttachment(dtex, depth_clear) if dtex is not None else None)
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, vb_pos)
    rp.set_vertex_buffer(1, vb_col)
    if viewport is not None:
        rp.set_viewport(*viewport)
    if scissor is not None:
        rp.set_scissor_rect(*scissor)
    if idx is not None:
        rp.set_index_buffer(idx, index_format)
        rp.draw_indexed(range(0, nv), base_vertex, range(0, instances))
    else:
        rp.draw(range(base_vertex, base_vertex + nv), range(0, instances))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    out = dev.read_texture(color)
    d = dev.read_texture(dtex) if dtex is not None else None
    return out, d, dev.submission_stats(sub).fragments_shaded


def render_scene(dev, builder, **kw):
    s = builder(dev, **kw)
    idx = s.render()
    color = dev.read_texture(s.color)
    depth = dev.read_texture(s.depth) if s.depth is not None else None
    return color, depth, dev.submission_stats(idx).fragments_shaded
