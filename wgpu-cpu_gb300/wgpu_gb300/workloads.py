"""Seeded synthetic workloads for the render-pass path: meshes, textures, cameras and the
scenes of the benchmark configurations, built through the public API (works with any device).

Every generator takes an explicit seed and uses numpy's PCG64 (`np.random.default_rng`), so
the same bytes come out on x86 and aarch64.  All arrays handed to the device are little-endian
float32 / uint32 / uint8 (f16 for the Rgba16Float quad colours).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import api as W


# ------------------------------------------------------------------------------------ cameras
def perspective(fov_y_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """WebGPU-style right-handed perspective (view looks down -z, clip z in [0, w])."""
    f = 1.0 / math.tan(math.radians(fov_y_deg) / 2.0)
    m = np.zeros((4, 4), dtype=np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = far / (near - far)
    m[2, 3] = near * far / (near - far)
    m[3, 2] = -1.0
    return m


def look_at(eye, target, up) -> np.ndarray:
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    fwd = target - eye
    fwd /= np.linalg.norm(fwd)
    side = np.cross(fwd, up)
    side /= np.linalg.norm(side)
    up2 = np.cross(side, fwd)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = side, up2, -fwd
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def mvp_bytes(mvp: np.ndarray) -> bytes:
    """A row-major 4x4 matrix as WGSL mat4x4f bytes (column-major float32)."""
    return np.ascontiguousarray(mvp.T.astype(np.float32)).tobytes()


def camera_mvp(width: int, height: int, eye=(0.0, 0.0, 3.0), fov=60.0, near=0.1, far=100.0,
               model: Optional[np.ndarray] = None) -> np.ndarray:
    m = perspective(fov, width / height, near, far) @ look_at(eye, (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    return m @ model if model is not None else m


# ------------------------------------------------------------------------------------ meshes
def uv_sphere(segments: int = 32, rings: int = 16):
    """(rings+1) x (segments+1) vertex grid.  Per quad of band i the upper-left triangle is
    emitted unless i == 0 (north pole) and the lower-right one always, so the south-pole band
    keeps zero-area triangles: 32 x 16 gives 992 triangles and 561 vertices."""
    th = np.linspace(0.0, math.pi, rings + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, segments + 1)
    t, p = np.meshgrid(th, ph, indexing="ij")
    pos = np.stack([np.sin(t) * np.cos(p), np.cos(t), np.sin(t) * np.sin(p)], -1).reshape(-1, 3)
    idx = []
    for i in range(rings):
        for j in range(segments):
            k1 = i * (segments + 1) + j
            k2 = k1 + segments + 1
            if i != 0:
                idx.append((k1, k2, k1 + 1))
            idx.append((k1 + 1, k2, k2 + 1))
    return pos.astype(np.float32), np.asarray(idx, dtype=np.uint32)


def icosphere(level: int):
    """Unit icosphere: 20 * 4**level triangles, 10 * 4**level + 2 vertices."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        a, b, c = (inv[i * nf:(i + 1) * nf] + base for i in range(3))  # midpoints of edges 01, 12, 20
        f = np.concatenate([np.stack([f[:, 0], a, c], 1), np.stack([a, f[:, 1], b], 1),
                            np.stack([c, b, f[:, 2]], 1), np.stack([a, b, c], 1)])
    return v, f.astype(np.uint32)


def value_noise3(p: np.ndarray, seed: int, freq: float = 4.0) -> np.ndarray:
    """Trilinear value noise in [0, 1) on a seeded 16^3 lattice (periodic)."""
    rng = np.random.default_rng(seed)
    lat = rng.random((16, 16, 16))
    q = (p * freq) % 16.0
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    fr = fr * fr * (3.0 - 2.0 * fr)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = (fr[:, 0] if dx else 1 - fr[:, 0]) * (fr[:, 1] if dy else 1 - fr[:, 1]) * \
                    (fr[:, 2] if dz else 1 - fr[:, 2])
                out += w * lat[(i0[:, 0] + dx) % 16, (i0[:, 1] + dy) % 16, (i0[:, 2] + dz) % 16]
    return out


def vertex_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    p = pos.astype(np.float64)
    fn = np.cross(p[faces[:, 1]] - p[faces[:, 0]], p[faces[:, 2]] - p[faces[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n


def displaced_icosphere(level: int, seed: int, amplitude: float = 0.1):
    """Icosphere with radial value-noise displacement; returns pos, normal, uv (float32), indices."""
    v, f = icosphere(level)
    r = 1.0 + amplitude * (value_noise3(v, seed) - 0.5) * 2.0
    pos = v * r[:, None]
    nrm = vertex_normals(pos, f)
    u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2.0 * math.pi)
    vv = 0.5 - np.arcsin(np.clip(v[:, 1], -1.0, 1.0)) / math.pi
    uv = np.stack([u, vv], 1)
    return pos.astype(np.float32), nrm.astype(np.float32), uv.astype(np.float32), f


def checker_noise_texture(size: int, seed: int, cell: int = 32) -> np.ndarray:
    """size x size RGBA8: a cell-sized checkerboard mixed 50/50 with seeded value noise."""
    yy, xx = np.mgrid[0:size, 0:size]
    chk = (((xx // cell) + (yy // cell)) % 2).astype(np.float64)
    pts = np.stack([xx.ravel() / size * 4.0, yy.ravel() / size * 4.0, np.zeros(size * size)], 1)
    img = np.empty((size, size, 4), dtype=np.uint8)
    for c in range(3):
        n = value_noise3(pts + c * 5.3, seed + c, freq=2.0).reshape(size, size)
        img[:, :, c] = np.clip((0.5 * chk + 0.5 * n) * 255.0, 0, 255).astype(np.uint8)
    img[:, :, 3] = 255
    return img


def mip_chain(img: np.ndarray) -> List[np.ndarray]:
    """Box-filtered mip chain of an RGBA8 image (level 0 first)."""
    out = [img]
    cur = img.astype(np.float64)
    while cur.shape[0] > 1 or cur.shape[1] > 1:
        h, w = max(1, cur.shape[0] // 2), max(1, cur.shape[1] // 2)
        cur = cur[: h * 2, : w * 2].reshape(h, 2, w, 2, 4).mean(axis=(1, 3))
        out.append(np.clip(np.round(cur), 0, 255).astype(np.uint8))
    return out


# ------------------------------------------------------------------------------------ scenes
@dataclass
class Scene:
    """Resources of one render pass plus a recorder for it."""
    device: W.Device
    color: W.Texture
    depth: Optional[W.Texture]
    draws: list = field(default_factory=list)  # (pipeline, bind_groups, vbufs, ibuf, index_range)
    uploads: list = field(default_factory=list)  # (buffer or texture, host array) inputs of the pass
    clear_color: tuple = (0.0, 0.0, 0.0, 1.0)
    depth_clear: float = 1.0
    triangles: int = 0
    label: str = ""

    def record(self, enc: W.CommandEncoder) -> None:
        rp = enc.begin_render_pass(
            [W.RenderPassColorAttachment(self.color, self.clear_color)],
            W.RenderPassDepthStencilAttachment(self.depth, self.depth_clear) if self.depth is not None else None)
        for pipeline, groups, vbufs, ibuf, rng, base_vertex in self.draws:
            rp.set_pipeline(pipeline)
            for gi, g in enumerate(groups):
                if g is not None:
                    rp.set_bind_group(gi, g)
            for slot, vb in enumerate(vbufs):
                rp.set_vertex_buffer(slot, vb)
            if ibuf is not None:
                rp.set_index_buffer(ibuf, W.IndexFormat.UINT32)
                rp.draw_indexed(rng, base_vertex)
            else:
                rp.draw(rng)
        rp.end()

    def render(self) -> int:
        enc = self.device.create_command_encoder()
        self.record(enc)
        idx = self.device.queue.submit([enc.finish()])
        self.device.poll(True, idx)
        return idx


def _f32x3_layout(loc, offset):
    return W.VertexAttribute(W.VertexFormat.FLOAT32X3, offset, loc)


def scene_colored_sphere(dev: W.Device, width: int = 512, height: int = 512, seed: int = 1,
                         segments: int = 32, rings: int = 16, cull=W.Face.BACK) -> Scene:
    """Plain single draw: UV sphere, per-vertex colours U[0,1], perspective MVP, back-face cull,
    no depth buffer, Rgba8Unorm cleared to black (the CPU-runnable configuration)."""
    pos, idx = uv_sphere(segments, rings)
    rng = np.random.default_rng(seed)
    col = rng.random((len(pos), 3)).astype(np.float32)
    vdata = np.concatenate([pos, col], 1).astype(np.float32)
    vb = dev.create_buffer_init(vdata)
    ib = dev.create_buffer_init(idx.ravel())
    ub = dev.create_buffer_init(mvp_bytes(camera_mvp(width, height)))
    sm = dev.create_shader_module(native="mesh_color")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(24, [_f32x3_layout(0, 0), _f32x3_layout(1, 12)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, front_face=W.FrontFace.CCW, cull_mode=cull),
        None, sm, [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM)])
    bg = dev.create_bind_group([W.BindGroupEntry(0, ub)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM)
    s = Scene(dev, color, None, clear_color=(0.0, 0.0, 0.0, 1.0), triangles=len(idx), label="colored_sphere")
    s.draws.append((pl, [bg], [vb], ib, range(0, idx.size), 0))
    s._keep = [vb, ib, ub, sm, bg]
    s.uploads = [(vb, vdata), (ib, idx.ravel()), (ub, np.frombuffer(mvp_bytes(camera_mvp(width, height)), np.uint8))]
    return s


def scene_textured_icosphere(dev: W.Device, width: int = 1920, height: int = 1080, level: int = 6, seed: int = 2,
                             tex_size: int = 1024, light=(0.3, 0.5, 0.8), address=W.AddressMode.REPEAT,
                             filtering: bool = False, srgb: bool = True) -> Scene:
    """Textured mesh: displaced icosphere (level 6 = 81,920 triangles), pos/normal/uv, a
    tex_size^2 checker x noise texture, texture x Lambert shading, colour + Depth32Float Less."""
    pos, nrm, uv, f = displaced_icosphere(level, seed)
    vdata = np.concatenate([pos, nrm, uv], 1).astype(np.float32)
    vb = dev.create_buffer_init(vdata)
    ib = dev.create_buffer_init(f.ravel())
    L = np.asarray(light, dtype=np.float64)
    L = L / np.linalg.norm(L)
    ubytes = mvp_bytes(camera_mvp(width, height)) + np.array([*L, 0.0], dtype=np.float32).tobytes()
    ub = dev.create_buffer_init(ubytes)
    fmt = W.TextureFormat.RGBA8_UNORM_SRGB if srgb else W.TextureFormat.RGBA8_UNORM
    img = checker_noise_texture(tex_size, seed + 100)
    mips = mip_chain(img) if filtering else [img]
    tex = dev.create_texture(tex_size, tex_size, fmt, mip_level_count=len(mips))
    dev.queue.write_texture(tex, img)
    if filtering and dev.profile == W.Profile.EXTENSION:
        for m, im in enumerate(mips[1:], start=1):
            dev.queue.write_texture(tex, im, mip_level=m)
    flt = W.FilterMode.LINEAR if filtering else W.FilterMode.NEAREST
    samp = dev.create_sampler(address, address, address, flt, flt, flt)
    sm = dev.create_shader_module(native="mesh_tex_lambert")
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(32, [_f32x3_layout(0, 0), _f32x3_layout(1, 12),
                                       W.VertexAttribute(W.VertexFormat.FLOAT32X2, 24, 2)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, front_face=W.FrontFace.CCW, cull_mode=W.Face.NONE),
        W.DepthStencilState(True, W.CompareFunction.LESS), sm, [W.ColorTargetState(fmt)])
    g0 = dev.create_bind_group([W.BindGroupEntry(0, ub)])
    g1 = dev.create_bind_group([W.BindGroupEntry(0, tex), W.BindGroupEntry(1, samp)])
    color = dev.create_texture(width, height, fmt)
    depth = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    s = Scene(dev, color, depth, clear_color=(0.0, 0.0, 0.0, 1.0), triangles=len(f), label="textured_icosphere")
    s.draws.append((pl, [g0, g1], [vb], ib, range(0, f.size), 0))
    s._keep = [vb, ib, ub, tex, samp, sm, g0, g1]
    s.uploads = [(vb, vdata), (ib, f.ravel()), (ub, np.frombuffer(ubytes, np.uint8)), (tex, img)]
    return s


def quad_stream(n_quads: int, width: int, height: int, seed: int, size_lo: int = 16, size_hi: int = 1024):
    """Screen-aligned quads: side U[size_lo, size_hi] px, centre U over the target, z U[0,1],
    RGBA colour with alpha U[0.1, 0.9] (as f16).  Returns positions (4 per quad, clip space with
    w = 1), colours (f16x4) and indices (two triangles per quad, painter order)."""
    rng = np.random.default_rng(seed)
    side = rng.uniform(size_lo, size_hi, n_quads)
    cx = rng.uniform(0, width, n_quads)
    cy = rng.uniform(0, height, n_quads)
    z = rng.uniform(0.0, 1.0, n_quads)
    rgb = rng.uniform(0.0, 1.0, (n_quads, 3))
    a = rng.uniform(0.1, 0.9, n_quads)
    x0, x1 = (cx - side / 2) / width * 2 - 1, (cx + side / 2) / width * 2 - 1
    y0, y1 = 1 - (cy - side / 2) / height * 2, 1 - (cy + side / 2) / height * 2
    pos = np.zeros((n_quads, 4, 3))
    pos[:, 0] = np.stack([x0, y0, z], 1)
    pos[:, 1] = np.stack([x1, y0, z], 1)
    pos[:, 2] = np.stack([x1, y1, z], 1)
    pos[:, 3] = np.stack([x0, y1, z], 1)
    col = np.concatenate([rgb, a[:, None]], 1)
    col = np.repeat(col[:, None, :], 4, axis=1)
    base = (np.arange(n_quads, dtype=np.uint32) * 4)[:, None]
    idx = (base + np.array([0, 3, 2, 0, 2, 1], dtype=np.uint32)[None, :]).astype(np.uint32)
    return pos.reshape(-1, 3).astype(np.float32), col.reshape(-1, 4).astype(np.float16), idx.ravel()


def scene_blended_quads(dev: W.Device, width: int = 3840, height: int = 2160, n_quads: int = 10000, seed: int = 4,
                        size_lo: int = 16, size_hi: int = 1024, depth_always: bool = False) -> Scene:
    """Fill-rate / blend stress: quads in painter order into Rgba16Float with ALPHA_BLENDING,
    no depth (extension profile: the reference has neither blending nor f16 targets).
    depth_always adds a Depth32Float target tested with Always and never written: the same
    colours, through the generic fragment path instead of the specialised blend path."""
    pos, col, idx = quad_stream(n_quads, width, height, seed, size_lo, size_hi)
    vb_pos = dev.create_buffer_init(pos)
    vb_col = dev.create_buffer_init(col)
    ib = dev.create_buffer_init(idx)
    sm = dev.create_shader_module(native="quad_color")
    ds = W.DepthStencilState(False, W.CompareFunction.ALWAYS) if depth_always else None
    pl = dev.create_render_pipeline(
        sm, [W.VertexBufferLayout(12, [_f32x3_layout(0, 0)]),
             W.VertexBufferLayout(8, [W.VertexAttribute(W.VertexFormat.FLOAT16X4, 0, 1)])],
        W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.NONE), ds, sm,
        [W.ColorTargetState(W.TextureFormat.RGBA16_FLOAT, W.BlendState.alpha_blending())])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA16_FLOAT)
    depth = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT) if depth_always else None
    s = Scene(dev, color, depth, clear_color=(0.0, 0.0, 0.0, 0.0), triangles=n_quads * 2, label="blended_quads")
    s.draws.append((pl, [], [vb_pos, vb_col], ib, range(0, idx.size), 0))
    s._keep = [vb_pos, vb_col, ib, sm]
    s.uploads = [(vb_pos, pos), (vb_col, col), (ib, idx)]
    return s


def scene_reference_triangle(dev: W.Device, front_face: int, cull_mode: int,
                             topology: int = W.PrimitiveTopology.TRIANGLE_LIST, vertices: range = range(0, 3),
                             width: int = 512, height: int = 512) -> Scene:
    """The reference integration test scene (wgpu-cpu-tests colored_triangle.rs:11-138):
    procedural triangle, 512^2 Rgba8UnormSrgb + Depth32Float Less, cleared to black / 1.0."""
    sm = dev.create_shader_module(native="colored_triangle")
    pl = dev.create_render_pipeline(
        sm, [], W.PrimitiveState(topology, front_face=front_face, cull_mode=cull_mode),
        W.DepthStencilState(True, W.CompareFunction.LESS), sm,
        [W.ColorTargetState(W.TextureFormat.RGBA8_UNORM_SRGB)])
    color = dev.create_texture(width, height, W.TextureFormat.RGBA8_UNORM_SRGB)
    depth = dev.create_texture(width, height, W.TextureFormat.DEPTH32_FLOAT)
    s = Scene(dev, color, depth, clear_color=(0.0, 0.0, 0.0, 1.0), triangles=1, label="reference_triangle")
    s.draws.append((pl, [], [], None, vertices, 0))
    s._keep = [sm]
    return s


def random_rotation(rng) -> np.ndarray:
    """Uniform random rotation (from a random unit quaternion) as a 4x4 matrix."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    m = np.eye(4)
    m[:3, :3] = r
    return m


@dataclass
class MultiScene:
    """Several render passes (one per target) recorded into one command buffer."""
    device: W.Device
    passes: list = field(default_factory=list)  # (color, depth, [(pipeline, groups, vbufs, ibuf, range)])
    uploads: list = field(default_factory=list)
    triangles: int = 0
    label: str = ""

    @property
    def color(self):
        return self.passes[0][0]

    def record(self, enc: W.CommandEncoder) -> None:
        for color, depth, draws in self.passes:
            rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.0, 0.0, 0.0, 1.0))],
                                       W.RenderPassDepthStencilAttachment(depth, 1.0))
            for pipeline, groups, vbufs, ibuf, rng in draws:
                rp.set_pipeline(pipeline)
                for gi, g in enumerate(groups):
                    rp.set_bind_group(gi, g)
                for slot, vb in enumerate(vbufs):
                    rp.set_vertex_buffer(slot, vb)
                rp.set_index_buffer(ibuf, W.IndexFormat.UINT32)
                rp.draw_indexed(rng)
            rp.end()

    def render(self) -> int:
        enc = self.device.create_command_encoder()
        self.record(enc)
        idx = self.device.queue.submit([enc.finish()])
        self.device.poll(True, idx)
        return idx


def scene_batched(dev: W.Device, n_targets: int = 64, n_draws: int = 256, seed: int = 3, tri_lo: int = 100,
                  tri_hi: int = 200000, side_lo: int = 128, side_hi: int = 2048, tex_size: int = 1024) -> MultiScene:
    """Batching workload: n_draws draws into n_targets targets (Rgba8Unorm + Depth32Float Less),
    target sides log-uniform in [side_lo, side_hi], triangle counts log-uniform in [tri_lo, tri_hi]
    taken from the front of a displaced icosphere of the smallest sufficient level, random model
    rotations seen from a random distance (every vertex in front of the camera, so w > 0), half
    vertex-colour and half textured programs (the tex_size^2 checker x value-noise texture of the
    textured configuration, nearest, repeat), draw d into target d mod n_targets."""
    rng = np.random.default_rng(seed)
    tw = np.exp(rng.uniform(math.log(side_lo), math.log(side_hi), n_targets)).astype(int)
    th = np.exp(rng.uniform(math.log(side_lo), math.log(side_hi), n_targets)).astype(int)
    counts = np.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi), n_draws)).astype(int)
    levels = [max(0, math.ceil(math.log(max(c, 20) / 20.0, 4))) for c in counts]
    s = MultiScene(dev, label="batched")
    meshes = {}
    for lvl in sorted(set(levels)):
        pos, nrm, uv, f = displaced_icosphere(lvl, seed + lvl)
        col = rng.random((len(pos), 3)).astype(np.float32)
        vt = np.concatenate([pos, nrm, uv], 1).astype(np.float32)
        vc = np.concatenate([pos, col], 1).astype(np.float32)
        vbt, vbc, ib = dev.create_buffer_init(vt), dev.create_buffer_init(vc), dev.create_buffer_init(f.ravel())
        s.uploads += [(vbt, vt), (vbc, vc), (ib, f.ravel())]
        meshes[lvl] = (vbt, vbc, ib)
    img = checker_noise_texture(tex_size, seed + 7)
    tex = dev.create_texture(tex_size, tex_size, W.TextureFormat.RGBA8_UNORM)
    dev.queue.write_texture(tex, img)
    s.uploads.append((tex, img))
    samp = dev.create_sampler(W.AddressMode.REPEAT, W.AddressMode.REPEAT)
    sm_t = dev.create_shader_module(native="mesh_tex_lambert")
    sm_c = dev.create_shader_module(native="mesh_color")
    fmt = W.TextureFormat.RGBA8_UNORM
    prim = W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.NONE)
    depth = W.DepthStencilState(True, W.CompareFunction.LESS)
    pl_t = dev.create_render_pipeline(
        sm_t, [W.VertexBufferLayout(32, [_f32x3_layout(0, 0), _f32x3_layout(1, 12),
                                         W.VertexAttribute(W.VertexFormat.FLOAT32X2, 24, 2)])],
        prim, depth, sm_t, [W.ColorTargetState(fmt)])
    pl_c = dev.create_render_pipeline(
        sm_c, [W.VertexBufferLayout(24, [_f32x3_layout(0, 0), _f32x3_layout(1, 12)])], prim, depth, sm_c,
        [W.ColorTargetState(fmt)])
    g_tex = dev.create_bind_group([W.BindGroupEntry(0, tex), W.BindGroupEntry(1, samp)])
    targets = []
    for t in range(n_targets):
        color = dev.create_texture(int(tw[t]), int(th[t]), fmt)
        dtex = dev.create_texture(int(tw[t]), int(th[t]), W.TextureFormat.DEPTH32_FLOAT)
        targets.append((color, dtex, []))
    keep = [tex, samp, sm_t, sm_c, g_tex]
    for d in range(n_draws):
        t = d % n_targets
        color, dtex, draws = targets[t]
        dist = rng.uniform(2.6, 4.5)
        model = random_rotation(rng)
        mvp = camera_mvp(color.width, color.height, eye=(0.0, 0.0, dist), model=model)
        L = rng.normal(size=3)
        L /= np.linalg.norm(L)
        ubytes = mvp_bytes(mvp) + np.array([*L, 0.0], dtype=np.float32).tobytes()
        ub = dev.create_buffer_init(ubytes)
        s.uploads.append((ub, np.frombuffer(ubytes, np.uint8)))
        g0 = dev.create_bind_group([W.BindGroupEntry(0, ub)])
        keep += [ub, g0]
        vbt, vbc, ib = meshes[levels[d]]
        n = int(counts[d])
        if d % 2 == 0:
            draws.append((pl_t, [g0, g_tex], [vbt], ib, range(0, 3 * n)))
        else:
            draws.append((pl_c, [g0], [vbc], ib, range(0, 3 * n)))
        s.triangles += n
    s.passes = targets
    s._keep = keep + [pl_t, pl_c] + [m for v in meshes.values() for m in v]
    return s


@dataclass
class ServingSet:
    """Resident resources of the serving workload and pre-recorded submissions over them."""
    device: W.Device
    commands: list = field(default_factory=list)     # one finished command buffer per submission
    targets: list = field(default_factory=list)      # (colour, depth) of each submission
    draws: list = field(default_factory=list)        # draws per submission
    triangles: list = field(default_factory=list)    # triangles per submission
    keep: list = field(default_factory=list)


def serving_set(dev: W.Device, n_submissions: int = 256, n_meshes: int = 512, n_textures: int = 128,
                seed: int = 5, max_draws: int = 64, tri_lo: int = 100, tri_hi: int = 200000) -> ServingSet:
    """Serving workload: n_meshes displaced icospheres (seeded radial jitter of one base mesh per
    subdivision level) and n_textures 256x256 Rgba8 textures, all resident; each submission
    renders 1..max_draws draws (log-uniform) into its own Rgba8Unorm + Depth32Float (Less)
    target of width log-uniform in [256, 1920] and height in [256, 1080]; each draw takes a
    random mesh, a triangle count log-uniform in [tri_lo, tri_hi] (the first triangles of the
    mesh, capped at its size), a random rotation and distance, and either the textured Lambert
    program with a random texture or the vertex-colour program."""
    rng = np.random.default_rng(seed)
    s = ServingSet(dev)
    base = {}
    levels = []
    for m in range(n_meshes):
        lvl = int(rng.integers(2, 8))  # 320 .. 327,680 triangles
        if lvl not in base:
            v, f = icosphere(lvl)
            u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2.0 * math.pi)
            vv = 0.5 - np.arcsin(np.clip(v[:, 1], -1.0, 1.0)) / math.pi
            ib = dev.create_buffer_init(f.ravel())
            base[lvl] = (v, np.stack([u, vv], 1), f, ib)
            s.keep.append(ib)
        v, uv, f, ib = base[lvl]
        r = 1.0 + 0.1 * (rng.random(len(v)) - 0.5) * 2.0
        pos = v * r[:, None]
        nrm = v  # the unit sphere's normal: the jitter is small
        col = rng.random((len(v), 3))
        vt = dev.create_buffer_init(np.concatenate([pos, nrm, uv], 1).astype(np.float32))
        vc = dev.create_buffer_init(np.concatenate([pos, col], 1).astype(np.float32))
        s.keep += [vt, vc]
        levels.append((vt, vc, ib, len(f)))
    base_tex = [checker_noise_texture(256, seed + 100 + k) for k in range(8)]
    textures = []
    for k in range(n_textures):
        img = np.ascontiguousarray(np.roll(base_tex[k % 8], shift=(k // 8) * 16, axis=(0, 1)))
        t = dev.create_texture(256, 256, W.TextureFormat.RGBA8_UNORM)
        dev.queue.write_texture(t, img)
        textures.append(t)
    samp = dev.create_sampler(W.AddressMode.REPEAT, W.AddressMode.REPEAT)
    sm_t = dev.create_shader_module(native="mesh_tex_lambert")
    sm_c = dev.create_shader_module(native="mesh_color")
    fmt = W.TextureFormat.RGBA8_UNORM
    prim = W.PrimitiveState(W.PrimitiveTopology.TRIANGLE_LIST, cull_mode=W.Face.BACK)
    depth = W.DepthStencilState(True, W.CompareFunction.LESS)
    pl_t = dev.create_render_pipeline(
        sm_t, [W.VertexBufferLayout(32, [_f32x3_layout(0, 0), _f32x3_layout(1, 12),
                                         W.VertexAttribute(W.VertexFormat.FLOAT32X2, 24, 2)])],
        prim, depth, sm_t, [W.ColorTargetState(fmt)])
    pl_c = dev.create_render_pipeline(
        sm_c, [W.VertexBufferLayout(24, [_f32x3_layout(0, 0), _f32x3_layout(1, 12)])], prim, depth, sm_c,
        [W.ColorTargetState(fmt)])
    tex_groups = [dev.create_bind_group([W.BindGroupEntry(0, t), W.BindGroupEntry(1, samp)]) for t in textures]
    s.keep += textures + tex_groups + [samp, sm_t, sm_c, pl_t, pl_c]
    for k in range(n_submissions):
        w = int(np.exp(rng.uniform(math.log(256), math.log(1920))))
        h = int(np.exp(rng.uniform(math.log(256), math.log(1080))))
        color = dev.create_texture(w, h, fmt)
        dtex = dev.create_texture(w, h, W.TextureFormat.DEPTH32_FLOAT)
        n_draws = int(np.clip(np.round(np.exp(rng.uniform(0.0, math.log(max_draws)))), 1, max_draws))
        enc = dev.create_command_encoder()
        rp = enc.begin_render_pass([W.RenderPassColorAttachment(color, (0.0, 0.0, 0.0, 1.0))],
                                   W.RenderPassDepthStencilAttachment(dtex, 1.0))
        tris = 0
        for _ in range(n_draws):
            vt, vc, ib, nf = levels[int(rng.integers(0, n_meshes))]
            n = int(min(nf, np.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
            mvp = camera_mvp(w, h, eye=(0.0, 0.0, float(rng.uniform(2.6, 4.5))), model=random_rotation(rng))
            L = rng.normal(size=3)
            L /= np.linalg.norm(L)
            ub = dev.create_buffer_init(mvp_bytes(mvp) + np.array([*L, 0.0], dtype=np.float32).tobytes())
            g0 = dev.create_bind_group([W.BindGroupEntry(0, ub)])
            s.keep += [ub, g0]
            if rng.random() < 0.5:
                rp.set_pipeline(pl_t)
                rp.set_bind_group(1, tex_groups[int(rng.integers(0, n_textures))])
                rp.set_vertex_buffer(0, vt)
            else:
                rp.set_pipeline(pl_c)
                rp.set_vertex_buffer(0, vc)
            rp.set_bind_group(0, g0)
            rp.set_index_buffer(ib, W.IndexFormat.UINT32)
            rp.draw_indexed(range(0, 3 * n))
            tris += n
        rp.end()
        s.commands.append(enc.finish())
        s.targets.append((color, dtex))
        s.draws.append(n_draws)
        s.triangles.append(tris)
        s.keep.append(color)
        s.keep.append(dtex)
    return s


# ------------------------------------------------------------------------------------ configurations
# The benchmark configurations at their full sizes: name -> (scene builder, profile, arguments).
# The parity fixtures (tests/golden/frame_digests.json), the full-size GPU tests and bench.py all
# build their scenes from this table, so they always render the same inputs.
FULL_SIZE = {
    "colored": ("scene_colored_sphere", W.Profile.PARITY, dict(width=512, height=512)),
    "textured": ("scene_textured_icosphere", W.Profile.PARITY,
                 dict(width=1920, height=1080, level=6, tex_size=1024)),
    "textured_filtered": ("scene_textured_icosphere", W.Profile.EXTENSION,
                          dict(width=1920, height=1080, level=6, tex_size=1024, filtering=True, srgb=True)),
    "blend": ("scene_blended_quads", W.Profile.EXTENSION, dict(width=3840, height=2160, n_quads=10000)),
    "batched": ("scene_batched", W.Profile.PARITY, dict(n_targets=64, n_draws=256, seed=3, tex_size=1024)),
}


def build_config(dev: W.Device, name: str, **over):
    """The scene of configuration `name` (FULL_SIZE) on `dev`, with `over` replacing arguments."""
    builder, _, kwargs = FULL_SIZE[name]
    return globals()[builder](dev, **{**kwargs, **over})


def with_new_targets(scene):
    """A copy of `scene` that renders the same draws into new targets of the same sizes and
    formats: the second buffer of a double-buffered frame loop."""
    import copy

    dev = scene.device

    def fresh(t):
        return None if t is None else dev.create_texture(t.width, t.height, t.format)

    s = copy.copy(scene)
    if hasattr(scene, "passes"):
        s.passes = [(fresh(p[0]), fresh(p[1]), *p[2:]) for p in scene.passes]
    else:
        s.color, s.depth = fresh(scene.color), fresh(scene.depth)
    return s


def scene_targets(scene) -> list:
    """(colour, depth or None) of every render pass of a Scene or MultiScene, in pass order."""
    if hasattr(scene, "passes"):
        return [(p[0], p[1]) for p in scene.passes]
    return [(scene.color, scene.depth)]
