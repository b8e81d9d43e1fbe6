"""Extra seeded scenes for the parity tests (built through the public API, any device)."""

import numpy as np

from wgpu_gb300 import api as W
from wgpu_gb300 import workloads as wl


def random_clip_triangles(dev, n_tris, width, height, seed, topology=W.PrimitiveTopology.TRIANGLE_LIST,
                          index_format=None, depth=None, cull=W.Face.NONE, front_face=W.FrontFace.CCW,
                          depth_write=True, spread=1.6, w_range=(0.3, 2.0), z_range=(-0.3, 1.3),
                          clear=(0.1, 0.2, 0.3, 1.0), color_format=W.TextureFormat.RGBA8_UNORM,
                          instances=1, base_vertex=0, scissor=None, viewport=None, blend=None, depth_clear=0.75,
                          program="clip_passthrough", stats=None):
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
    sm = dev.create_shader_module(native=program)
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
    if stats is not None:
        stats.append(dev.submission_stats(sub))
    return out, d, dev.submission_stats(sub).fragments_shaded


def render_scene(dev, builder, **kw):
    s = builder(dev, **kw)
    idx = s.render()
    color = dev.read_texture(s.color)
    depth = dev.read_texture(s.depth) if s.depth is not None else None
    return color, depth, dev.submission_stats(idx).fragments_shaded


def restart_strips(dev, n_indices, width, height, seed, index_format=W.IndexFormat.UINT32, instances=1,
                   depth=W.CompareFunction.LESS, cull=W.Face.NONE, sep_prob=0.08):
    """Triangle strips with primitive restart: a random index stream over random clip-space
    vertices with separator indices (0xFFFF / 0xFFFFFFFF) at random positions — back to back,
    first and last included — so runs of every length occur, short ones producing nothing."""
    rng = np.random.default_rng(seed)
    nv = 256
    w = rng.uniform(0.4, 2.0, nv)
    pos = np.stack([rng.uniform(-1.3, 1.3, nv) * w, rng.uniform(-1.3, 1.3, nv) * w,
                    rng.uniform(0.0, 1.0, nv) * w, w], 1).astype(np.float32)
    col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
    sep = 0xFFFF if index_format == W.IndexFormat.UINT16 else 0xFFFFFFFF
    idx = rng.integers(0, nv, n_indices).astype(np.int64)
    mask = rng.random(n_indices) < sep_prob
    mask[0] = True
    mask[-1] = True
    mask[n_indices // 2: n_indices // 2 + 3] = True
    idx[mask] = sep
    vb_pos = dev.create_buffer_init(pos)
    vb_col = dev.create_buffer_init(col)
    ib = dev.create_buffer_init(idx.astype(np.uint16 if index_format == W.IndexFormat.UINT16 else np.uint32))
    sm = dev.create_shader_module(native="clip_passthrough")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
             W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_STRIP, strip_index_format=index_format, cull_mode=cull),
        W.DepthStencilState(True, depth), sm, [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.0, 0.0, 0.0, 1.0))],
                               W.RenderPassDepthStencilAttachment(dtex, 1.0))
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, vb_pos)
    rp.set_vertex_buffer(1, vb_col)
    rp.set_index_buffer(ib, index_format)
    rp.draw_indexed(range(0, n_indices), 0, range(0, instances))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    return dev.read_texture(color), dev.read_texture(dtex), dev.submission_stats(sub).fragments_shaded


def lines_points(dev, topology, n, width, height, seed, index_format=None, restart=False, instances=1,
                 depth=W.CompareFunction.LESS_EQUAL, scissor=None, clear=(0.0, 0.0, 0.0, 1.0),
                 program="clip_passthrough", depth_write=True):
    """Lines or points given in clip space (clip_passthrough program), crossing the clip planes:
    line lists / strips (optionally indexed, with separator indices) and point lists."""
    rng = np.random.default_rng(seed)
    nv = n
    w = rng.uniform(0.4, 2.0, nv)
    pos = np.stack([rng.uniform(-1.4, 1.4, nv) * w, rng.uniform(-1.4, 1.4, nv) * w,
                    rng.uniform(-0.2, 1.2, nv) * w, w], 1).astype(np.float32)
    col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
    vb_pos = dev.create_buffer_init(pos)
    vb_col = dev.create_buffer_init(col)
    sm = dev.create_shader_module(native=program)
    sif = index_format if restart else W.IndexFormat.NONE
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
             W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])],
        W.PrimitiveState(topology, strip_index_format=sif), W.DepthStencilState(depth_write, depth), sm,
        [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, clear)], W.RenderPassDepthStencilAttachment(dtex, 1.0))
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, vb_pos)
    rp.set_vertex_buffer(1, vb_col)
    if scissor is not None:
        rp.set_scissor_rect(*scissor)
    if index_format is not None:
        idx = rng.permutation(nv).astype(np.int64)
        if restart:
            sep = 0xFFFF if index_format == W.IndexFormat.UINT16 else 0xFFFFFFFF
            m = rng.random(nv) < 0.1
            m[3:5] = True
            idx[m] = sep
        ib = dev.create_buffer_init(idx.astype(np.uint16 if index_format == W.IndexFormat.UINT16 else np.uint32))
        rp.set_index_buffer(ib, index_format)
        rp.draw_indexed(range(0, nv), 0, range(0, instances))
    else:
        rp.draw(range(0, nv), range(0, instances))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    return dev.read_texture(color), dev.read_texture(dtex), dev.submission_stats(sub).fragments_shaded


def mixed_pass(dev, width, height, seed):
    """One pass: random triangles, then lines over them, then points, then more triangles, into the
    same colour + depth target (draw order across topologies)."""
    rng = np.random.default_rng(seed)
    sm = dev.create_shader_module(native="clip_passthrough")
    layouts = [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
               W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])]
    ds = W.DepthStencilState(True, W.CompareFunction.LESS_EQUAL)
    pls = {t: dev.create_render_pipeline(sm, layouts, W.PrimitiveState(t), ds, sm,
                                         [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
           for t in (W.PrimitiveTopology.TRIANGLE_LIST, W.PrimitiveTopology.LINE_LIST, W.PrimitiveTopology.POINT_LIST)}
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.2, 0.1, 0.0, 1.0))],
                               W.RenderPassDepthStencilAttachment(dtex, 1.0))
    keep = []
    for topo, nv in [(W.PrimitiveTopology.TRIANGLE_LIST, 300), (W.PrimitiveTopology.LINE_LIST, 400),
                     (W.PrimitiveTopology.POINT_LIST, 500), (W.PrimitiveTopology.TRIANGLE_LIST, 150)]:
        w = rng.uniform(0.5, 1.5, nv)
        pos = np.stack([rng.uniform(-1.2, 1.2, nv) * w, rng.uniform(-1.2, 1.2, nv) * w,
                        rng.uniform(0.0, 1.0, nv) * w, w], 1).astype(np.float32)
        col = rng.uniform(0, 1, (nv, 4)).astype(np.float32)
        vp, vc = dev.create_buffer_init(pos), dev.create_buffer_init(col)
        keep += [vp, vc]
        rp.set_pipeline(pls[topo])
        rp.set_vertex_buffer(0, vp)
        rp.set_vertex_buffer(1, vc)
        rp.draw(range(0, nv))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    return dev.read_texture(color), dev.read_texture(dtex), dev.submission_stats(sub).fragments_shaded


def textured_quad(dev, width, height, x0, y0, side, tex_levels, uv_scale=1.0, srgb_texture=False,
                  color_format=W.TextureFormat.RGBA8_UNORM, address=W.AddressMode.REPEAT,
                  mag=W.FilterMode.LINEAR, min_=W.FilterMode.LINEAR, mip=W.FilterMode.LINEAR,
                  lod_min=0.0, lod_max=32.0, clear=(0.0, 0.0, 0.0, 0.0)):
    """A screen-aligned quad over pixels [x0, x0 + side] x [y0, y0 + side] textured with uv from 0
    to uv_scale through mesh_tex_lambert, identity MVP, normal and light both +z (Lambert factor
    exactly 1, so every covered pixel shows the texture sample itself).  tex_levels: RGBA8 mip
    images, level 0 first.  Returns (colour bytes, fragments shaded)."""
    def ndc(px, py):
        return 2.0 * px / width - 1.0, 1.0 - 2.0 * py / height
    corners = [(x0, y0, 0.0, 0.0), (x0 + side, y0, uv_scale, 0.0), (x0 + side, y0 + side, uv_scale, uv_scale),
               (x0, y0 + side, 0.0, uv_scale)]
    vdata = np.array([[*ndc(px, py), 0.5, 0.0, 0.0, 1.0, u, v] for px, py, u, v in corners], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    vb = dev.create_buffer_init(vdata)
    ib = dev.create_buffer_init(idx)
    ub = dev.create_buffer_init(np.concatenate([np.eye(4, dtype=np.float32).ravel(),
                                                np.array([0.0, 0.0, 1.0, 0.0], np.float32)]))
    tfmt = W.TextureFormat.RGBA8_UNORM_SRGB if srgb_texture else W.TextureFormat.RGBA8_UNORM
    ts = tex_levels[0].shape[0]
    tex = dev.create_texture(ts, ts, tfmt, mip_level_count=len(tex_levels))
    for m, im in enumerate(tex_levels):
        if m == 0 or dev.profile == W.Profile.EXTENSION:
            dev.queue.write_texture(tex, im, mip_level=m)
    samp = dev.create_sampler(address, address, address, mag, min_, mip, lod_min, lod_max)
    sm = dev.create_shader_module(native="mesh_tex_lambert")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(32, [W.VertexAttribute(W.VertexFormat.FLOAT32X3, 0, 0),
                                       W.VertexAttribute(W.VertexFormat.FLOAT32X3, 12, 1),
                                       W.VertexAttribute(W.VertexFormat.FLOAT32X2, 24, 2)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.NONE), None, sm,
        [W.ColorTargetState(color_format)])
    g0 = dev.create_bind_group([W.BindGroupEntry(0, ub)])
    g1 = dev.create_bind_group([W.BindGroupEntry(0, tex), W.BindGroupEntry(1, samp)])
    color = dev.create_texture(width, height, color_format)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, clear)], None)
    rp.set_pipeline(pl)
    rp.set_bind_group(0, g0)
    rp.set_bind_group(1, g1)
    rp.set_vertex_buffer(0, vb)
    rp.set_index_buffer(ib, W.IndexFormat.UINT32)
    rp.draw_indexed(range(0, 6), 0, range(0, 1))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    return dev.read_texture(color), dev.submission_stats(sub).fragments_shaded


def coverage_counts(dev, width, height, tris_px):
    """Triangles given in framebuffer pixel coordinates (tris_px: (n, 3, 2)), drawn with colour
    (1, 0, 0, 1) and additive blending (One/One) into an Rgba16Float target: each texel's red
    channel counts the fragments that landed on it (exact in f16 for small counts).  Extension
    profile.  Returns (counts (height, width) int array, fragments shaded)."""
    t = np.asarray(tris_px, np.float64).reshape(-1, 2)
    ndc = np.stack([2.0 * t[:, 0] / width - 1.0, 1.0 - 2.0 * t[:, 1] / height], 1)
    pos = np.concatenate([ndc, np.full((len(t), 1), 0.5), np.ones((len(t), 1))], 1).astype(np.float32)
    col = np.tile(np.array([1.0, 0.0, 0.0, 1.0], np.float32), (len(t), 1))
    vb_pos = dev.create_buffer_init(pos)
    vb_col = dev.create_buffer_init(col)
    add = W.BlendComponent(W.BlendFactor.ONE, W.BlendFactor.ONE)
    sm = dev.create_shader_module(native="clip_passthrough")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 0)]),
             W.VertexBufferLayout(16, [W.VertexAttribute(W.VertexFormat.FLOAT32X4, 0, 1)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.NONE), None, sm,
        [W.ColorTargetState(W.TextureFormat.RGBA16_FLOAT, W.BlendState(add, add))])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA16_FLOAT)
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.0, 0.0, 0.0, 0.0))], None)
    rp.set_pipeline(pl)
    rp.set_vertex_buffer(0, vb_pos)
    rp.set_vertex_buffer(1, vb_col)
    rp.draw(range(0, len(t)), range(0, 1))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    img = dev.read_texture(color).view(np.float16).astype(np.float32)
    return img[..., 0].astype(np.int64), dev.submission_stats(sub).fragments_shaded


def copy_scenario(dev, seed=5):
    """Encoder copies and clears (extension profile) between and around render passes.  Returns
    the initial data and every resource the commands touched, read back:
      A (4096 B) -> B: copy A[256:1280] to B[512:1536], clear B[0:64];
      A -> T1 mip 0 layer 1 at (5, 3), 16 x 8 texels, 256-byte rows;
      T1 mip 1 layer 0 (2, 1) 10 x 6 -> T2 mip 1 layer 1 (20, 10); clear T2 mip 2, all layers;
      T1 mip 0 layer 1 (5, 3) 16 x 8 -> C at 0, 256-byte rows;
      render a sphere into X, copy X to Y, render X again cleared to red (Y keeps the first frame)."""
    rng = np.random.default_rng(seed)
    a_data = rng.integers(0, 256, 4096, dtype=np.uint8)
    A = dev.create_buffer_init(a_data)
    B = dev.create_buffer_init(np.zeros(4096, np.uint8))
    C = dev.create_buffer_init(np.zeros(4096, np.uint8))
    f = W.TextureFormat.RGBA8_UNORM
    t1_levels = [rng.integers(0, 256, (2, 32 >> m, 64 >> m, 4), dtype=np.uint8) for m in range(3)]
    t2_levels = [rng.integers(0, 256, (2, 32 >> m, 64 >> m, 4), dtype=np.uint8) for m in range(3)]
    T1 = dev.create_texture(64, 32, f, mip_level_count=3, layers=2)
    T2 = dev.create_texture(64, 32, f, mip_level_count=3, layers=2)
    for m in range(3):
        dev.queue.write_texture(T1, t1_levels[m], mip_level=m)
        dev.queue.write_texture(T2, t2_levels[m], mip_level=m)
    enc = dev.create_command_encoder()
    enc.copy_buffer_to_buffer(A, 256, B, 512, 1024)
    enc.clear_buffer(B, 0, 64)
    enc.copy_buffer_to_texture(A, 0, 256, 8, T1, (16, 8, 1), mip_level=0, origin=(5, 3, 1))
    enc.copy_texture_to_texture(T1, T2, (10, 6, 1), source_mip=1, source_origin=(2, 1, 0), destination_mip=1,
                                destination_origin=(20, 10, 1))
    enc.clear_texture(T2, base_mip_level=2)
    enc.copy_texture_to_buffer(T1, C, 0, 256, 8, (16, 8, 1), mip_level=0, origin=(5, 3, 1))
    dev.poll(True, dev.queue.submit([enc.finish()]))

    s = wl.scene_colored_sphere(dev, 64, 64)
    Y = dev.create_texture(64, 64, W.TextureFormat.RGBA8_UNORM)
    enc = dev.create_command_encoder()
    s.record(enc)
    enc.copy_texture_to_texture(s.color, Y, (64, 64, 1))
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(s.color, (1.0, 0.0, 0.0, 1.0))], None)
    rp.end()
    dev.poll(True, dev.queue.submit([enc.finish()]))
    return {
        "a": a_data, "t1_init": t1_levels, "t2_init": t2_levels,
        "B": np.frombuffer(B.read(), np.uint8), "C": np.frombuffer(C.read(), np.uint8),
        "T1": [dev.read_texture(T1, m) for m in range(3)], "T2": [dev.read_texture(T2, m) for m in range(3)],
        "X": dev.read_texture(s.color), "Y": dev.read_texture(Y),
    }


def perspective_sphere(dev, width, height, seed=9, level=3, eye=1.25, near=0.45, depth=W.CompareFunction.LESS):
    """A vertex-coloured icosphere seen from close by with perspective-correct interpolation
    (mesh_color_perspective, extension profile): the near plane cuts through the sphere, so
    clipped triangles interpolate with the clip barycentrics and 1/w of the unclipped vertices."""
    v, f = wl.icosphere(level)
    rng = np.random.default_rng(seed)
    col = rng.random((len(v), 3))
    vdata = np.concatenate([v, col], 1).astype(np.float32)
    vb = dev.create_buffer_init(vdata)
    ib = dev.create_buffer_init(f.ravel())
    mvp = wl.camera_mvp(width, height, eye=(0.3, 0.2, eye), near=near)
    ub = dev.create_buffer_init(wl.mvp_bytes(mvp))
    sm = dev.create_shader_module(native="mesh_color_perspective")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(24, [W.VertexAttribute(W.VertexFormat.FLOAT32X3, 0, 0),
                                       W.VertexAttribute(W.VertexFormat.FLOAT32X3, 12, 1)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.NONE),
        W.DepthStencilState(True, depth) if depth is not None else None, sm,
        [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    bg = dev.create_bind_group([W.BindGroupEntry(0, ub)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    dtex = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT) if depth is not None else None
    enc = dev.create_command_encoder()
    rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.0, 0.0, 0.0, 1.0))],
                               W.RenderPassDepthStencilAttachment(dtex, 1.0) if dtex is not None else None)
    rp.set_pipeline(pl)
    rp.set_bind_group(0, bg)
    rp.set_vertex_buffer(0, vb)
    rp.set_index_buffer(ib, W.IndexFormat.UINT32)
    rp.draw_indexed(range(0, f.size))
    rp.end()
    sub = dev.queue.submit([enc.finish()])
    dev.poll(True, sub)
    st = dev.submission_stats(sub)
    return (dev.read_texture(color), dev.read_texture(dtex) if dtex is not None else None, st.fragments_shaded), st
