"""Host-side mirror of the wgpu API that wgpu-cpu implements (device, queue, pipelines, bind
groups, render passes), driving the C ABI of include/gbr.h through ctypes.

Names and argument meanings follow wgpu 28 (Device::create_*, Queue::write_buffer /
write_texture / submit, Device::poll, RenderPass::set_* / draw / draw_indexed).  Errors come
back as `GbrError` carrying the ABI status, where wgpu-cpu would panic.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _abi as A


# ------------------------------------------------------------------------------------ enums
class TextureFormat:
    R8_UNORM = 1
    RG8_UNORM = 2
    RGBA8_UNORM = 3
    RGBA8_UNORM_SRGB = 4
    BGRA8_UNORM = 5
    BGRA8_UNORM_SRGB = 6
    RGBA16_FLOAT = 7
    RGBA32_FLOAT = 8
    DEPTH32_FLOAT = 9


BYTES_PER_TEXEL = {1: 1, 2: 2, 3: 4, 4: 4, 5: 4, 6: 4, 7: 8, 8: 16, 9: 4}


class VertexFormat:
    FLOAT32 = 1
    FLOAT32X2 = 2
    FLOAT32X3 = 3
    FLOAT32X4 = 4
    UINT32 = 5
    SINT32 = 6
    FLOAT16X2 = 7
    FLOAT16X4 = 8
    UNORM8X4 = 9


class VertexStepMode:
    VERTEX = 0
    INSTANCE = 1


class IndexFormat:
    NONE = 0
    UINT16 = 1
    UINT32 = 2


class PrimitiveTopology:
    POINT_LIST = 0
    LINE_LIST = 1
    LINE_STRIP = 2
    TRIANGLE_LIST = 3
    TRIANGLE_STRIP = 4


class FrontFace:
    CCW = 0
    CW = 1


class Face:
    NONE = 0
    FRONT = 1
    BACK = 2


class CompareFunction:
    NEVER = 1
    LESS = 2
    EQUAL = 3
    LESS_EQUAL = 4
    GREATER = 5
    NOT_EQUAL = 6
    GREATER_EQUAL = 7
    ALWAYS = 8


class BlendFactor:
    ZERO = 0
    ONE = 1
    SRC = 2
    ONE_MINUS_SRC = 3
    SRC_ALPHA = 4
    ONE_MINUS_SRC_ALPHA = 5
    DST = 6
    ONE_MINUS_DST = 7
    DST_ALPHA = 8
    ONE_MINUS_DST_ALPHA = 9
    CONSTANT = 11
    ONE_MINUS_CONSTANT = 12


class BlendOperation:
    ADD = 0
    SUBTRACT = 1
    REVERSE_SUBTRACT = 2
    MIN = 3
    MAX = 4


class AddressMode:
    CLAMP_TO_EDGE = 0
    REPEAT = 1
    MIRROR_REPEAT = 2
    CLAMP_TO_BORDER = 3


class FilterMode:
    NEAREST = 0
    LINEAR = 1


class LoadOp:
    LOAD = 0
    CLEAR = 1


class Profile:
    PARITY = 0
    EXTENSION = 1


class LaunchMode:
    BATCHED = 0
    PER_DRAW = 1
    PER_PASS = 2


class RasterOrder:
    AUTO = 0
    ORDERED = 1


class RasterRule:
    SCANLINE = 0  # the reference's scanline walk at integer pixel corners (bit-exact)
    EDGE = 1      # extension profile: fixed-point edge functions, pixel centres, top-left rule


class BindingKind:
    BUFFER = 0
    SAMPLER = 1
    TEXTURE_VIEW = 2


# ------------------------------------------------------------------------------------ errors
class GbrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{A.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


def _check(lib: A.Lib, st: int) -> None:
    if st != A.OK:
        raise GbrError(st, lib.error_text())


# ------------------------------------------------------------------------------------ library
_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG_DIR, "libgbr.so")
_gpu_lib: Optional[A.Lib] = None


def gpu_lib() -> A.Lib:
    """The CUDA library (libgbr.so).  Raises if it has not been built: there is no fallback."""
    global _gpu_lib
    if _gpu_lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        _gpu_lib = A.Lib(C.CDLL(LIB_PATH), "gbr_")
    return _gpu_lib


# ------------------------------------------------------------------------------------ descriptors
@dataclass
class VertexAttribute:
    format: int
    offset: int
    shader_location: int


@dataclass
class VertexBufferLayout:
    array_stride: int
    attributes: Sequence[VertexAttribute]
    step_mode: int = VertexStepMode.VERTEX


@dataclass
class BlendComponent:
    src_factor: int = BlendFactor.ONE
    dst_factor: int = BlendFactor.ZERO
    operation: int = BlendOperation.ADD


@dataclass
class BlendState:
    color: BlendComponent
    alpha: BlendComponent

    @staticmethod
    def alpha_blending() -> "BlendState":  # wgpu::BlendState::ALPHA_BLENDING
        return BlendState(BlendComponent(BlendFactor.SRC_ALPHA, BlendFactor.ONE_MINUS_SRC_ALPHA),
                          BlendComponent(BlendFactor.ONE, BlendFactor.ONE_MINUS_SRC_ALPHA))


@dataclass
class ColorTargetState:
    format: int
    blend: Optional[BlendState] = None
    write_mask: int = 0xF


@dataclass
class PrimitiveState:
    topology: int = PrimitiveTopology.TRIANGLE_LIST
    strip_index_format: int = IndexFormat.NONE
    front_face: int = FrontFace.CCW
    cull_mode: int = Face.NONE


@dataclass
class DepthStencilState:
    depth_write_enabled: bool = True
    depth_compare: int = CompareFunction.LESS
    format: int = TextureFormat.DEPTH32_FLOAT


@dataclass
class BindGroupEntry:
    binding: int
    resource: object  # Buffer | Sampler | Texture
    offset: int = 0
    size: int = 0


@dataclass
class RenderPassColorAttachment:
    view: "Texture"
    load: object = "clear"  # "load" or a clear colour (r, g, b, a) as floats
    depth_slice: int = 0


@dataclass
class RenderPassDepthStencilAttachment:
    view: "Texture"
    depth_load: object = 1.0  # "load", None (no depth ops) or a clear value


# ------------------------------------------------------------------------------------ objects
class _Object:
    _destroy = ""

    def __init__(self, device: "Device", handle: int):
        self.device = device
        self.handle = handle

    def destroy(self) -> None:
        if self.handle and self.device.handle:
            _check(self.device.lib, getattr(self.device.lib, self._destroy)(self.device.handle, self.handle))
        self.handle = 0


class Buffer(_Object):
    _destroy = "buffer_destroy"

    def __init__(self, device, handle, size):
        super().__init__(device, handle)
        self.size = size

    def read(self, offset: int = 0, size: Optional[int] = None) -> bytes:
        size = self.size - offset if size is None else size
        out = (C.c_uint8 * size)()
        _check(self.device.lib, self.device.lib.buffer_read(self.device.handle, self.handle, offset, out, size))
        return bytes(out)


class Texture(_Object):
    _destroy = "texture_destroy"

    def __init__(self, device, handle, width, height, format, mip_level_count=1, layers=1):
        super().__init__(device, handle)
        self.width, self.height, self.format = width, height, format
        self.mip_level_count, self.layers = mip_level_count, layers

    def mip_size(self, mip: int):
        return max(1, self.width >> mip), max(1, self.height >> mip)


class Sampler(_Object):
    _destroy = "sampler_destroy"


class ShaderModule(_Object):
    _destroy = "shader_module_destroy"


class RenderPipeline(_Object):
    _destroy = "render_pipeline_destroy"

    def eval_vertices(self, first: int, count: int):
        """Runs a WGSL pipeline's vertex stage alone for `count` vertex indices (no buffers, no
        bindings): returns (positions [count, 4] f32, inter-stage values [count, 16] as raw
        32-bit words, device error code per vertex)."""
        lib = self.device.lib
        if lib.render_pipeline_eval_vertices is None:
            raise GbrError(A.ERR_UNSUPPORTED, "this library cannot evaluate vertex stages")
        out = np.zeros((count, 20), dtype=np.float32)
        errs = np.zeros(count, dtype=np.uint32)
        _check(lib, lib.render_pipeline_eval_vertices(
            self.device.handle, self.handle, first, count, out.ctypes.data_as(C.POINTER(C.c_float)),
            errs.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out[:, :4], out[:, 4:].view(np.uint32), errs


def wgsl_translate(lib: "A.Lib", source: str, vertex_entry: str, fragment_entry: Optional[str] = None) -> str:
    """The CUDA C the library emits for a WGSL vertex (+ fragment) program (no GPU needed)."""
    src = source.encode()
    need = C.c_uint64()
    buf = C.create_string_buffer(1 << 22)
    _check(lib, lib.wgsl_translate(src, len(src), vertex_entry.encode(),
                                   fragment_entry.encode() if fragment_entry else None, buf, 1 << 22, C.byref(need)))
    return buf.value.decode()


def wgsl_compile_check(lib: "A.Lib", source: str, vertex_entry: str, fragment_entry: Optional[str] = None) -> str:
    """Translates and compiles a WGSL program with NVRTC for sm_103a (no GPU needed); returns the log."""
    src = source.encode()
    buf = C.create_string_buffer(1 << 16)
    _check(lib, lib.wgsl_compile_check(src, len(src), vertex_entry.encode(),
                                       fragment_entry.encode() if fragment_entry else None, buf, 1 << 16))
    return buf.value.decode()


class BindGroup(_Object):
    _destroy = "bind_group_destroy"


# ------------------------------------------------------------------------------------ commands
class CommandBuffer:
    def __init__(self, data: bytes):
        self.data = data


class CommandEncoder:
    def __init__(self, device: "Device"):
        self.device = device
        self._chunks: list = []
        self._open_pass = False

    def _push(self, opcode: int, payload: Optional[C.Structure] = None) -> None:
        body = bytes(payload) if payload is not None else b""
        hdr = A.CmdHeader(opcode, len(body))
        pad = (-len(body)) % 8
        self._chunks.append(bytes(hdr) + body + b"\0" * pad)

    # Copies and clears outside render passes (extension profile; the reference's encoder has
    # them as todo!, command.rs:37-115).  size=None: to the end of the source / buffer.
    def copy_buffer_to_buffer(self, source: "Buffer", source_offset: int, destination: "Buffer",
                              destination_offset: int, size: Optional[int] = None) -> None:
        self._push(A.OP_COPY_BUFFER_TO_BUFFER, A.CmdCopyBufferToBuffer(
            source.handle, source_offset, destination.handle, destination_offset,
            0xFFFFFFFFFFFFFFFF if size is None else size))

    @staticmethod
    def _texture_info(texture, mip_level=0, origin=(0, 0, 0)):
        return A.TexelCopyTextureInfo(texture.handle, mip_level, *origin)

    def copy_buffer_to_texture(self, buffer: "Buffer", offset: int, bytes_per_row: int, rows_per_image: int,
                               texture: "Texture", size, mip_level: int = 0, origin=(0, 0, 0)) -> None:
        self._push(A.OP_COPY_BUFFER_TO_TEXTURE, A.CmdCopyBufferTexture(
            buffer.handle, A.TexelCopyBufferLayout(offset, bytes_per_row, rows_per_image),
            self._texture_info(texture, mip_level, origin), A.Extent3d(*size), 0))

    def copy_texture_to_buffer(self, texture: "Texture", buffer: "Buffer", offset: int, bytes_per_row: int,
                               rows_per_image: int, size, mip_level: int = 0, origin=(0, 0, 0)) -> None:
        self._push(A.OP_COPY_TEXTURE_TO_BUFFER, A.CmdCopyBufferTexture(
            buffer.handle, A.TexelCopyBufferLayout(offset, bytes_per_row, rows_per_image),
            self._texture_info(texture, mip_level, origin), A.Extent3d(*size), 0))

    def copy_texture_to_texture(self, source: "Texture", destination: "Texture", size, source_mip: int = 0,
                                source_origin=(0, 0, 0), destination_mip: int = 0,
                                destination_origin=(0, 0, 0)) -> None:
        self._push(A.OP_COPY_TEXTURE_TO_TEXTURE, A.CmdCopyTextureToTexture(
            self._texture_info(source, source_mip, source_origin),
            self._texture_info(destination, destination_mip, destination_origin), A.Extent3d(*size), 0))

    def clear_buffer(self, buffer: "Buffer", offset: int = 0, size: Optional[int] = None) -> None:
        self._push(A.OP_CLEAR_BUFFER, A.CmdClearBuffer(buffer.handle, offset,
                                                       0xFFFFFFFFFFFFFFFF if size is None else size))

    def clear_texture(self, texture: "Texture", base_mip_level: int = 0, mip_level_count: int = 0,
                      base_array_layer: int = 0, array_layer_count: int = 0) -> None:
        self._push(A.OP_CLEAR_TEXTURE, A.CmdClearTexture(texture.handle, base_mip_level, mip_level_count,
                                                         base_array_layer, array_layer_count))

    def begin_render_pass(self, color_attachments: Sequence[Optional[RenderPassColorAttachment]] = (),
                          depth_stencil_attachment: Optional[RenderPassDepthStencilAttachment] = None
                          ) -> "RenderPassEncoder":
        if self._open_pass:
            raise GbrError(A.ERR_VALIDATION, "a render pass is already open")
        b = A.CmdBeginRenderPass()
        b.color_attachment_count = len(color_attachments)
        for i, ca in enumerate(color_attachments):
            if ca is None:
                continue
            a = b.color_attachments[i]
            a.view = ca.view.handle
            a.depth_slice = ca.depth_slice
            if isinstance(ca.load, str) and ca.load == "load":
                a.load_op = LoadOp.LOAD
            else:
                a.load_op = LoadOp.CLEAR
                col = (0.0, 0.0, 0.0, 1.0) if ca.load == "clear" else ca.load
                for k in range(4):
                    a.clear_value[k] = float(col[k])
        if depth_stencil_attachment is not None:
            b.has_depth_attachment = 1
            d = b.depth_attachment
            d.view = depth_stencil_attachment.view.handle
            dl = depth_stencil_attachment.depth_load
            if dl is None:
                d.has_depth_ops = 0
            else:
                d.has_depth_ops = 1
                if isinstance(dl, str) and dl == "load":
                    d.depth_load_op = LoadOp.LOAD
                else:
                    d.depth_load_op = LoadOp.CLEAR
                    d.depth_clear_value = float(dl)
        self._push(A.OP_BEGIN_RENDER_PASS, b)
        self._open_pass = True
        return RenderPassEncoder(self)

    def finish(self) -> CommandBuffer:
        if self._open_pass:
            raise GbrError(A.ERR_VALIDATION, "render pass not ended")
        return CommandBuffer(b"".join(self._chunks))


class RenderPassEncoder:
    def __init__(self, enc: CommandEncoder):
        self.enc = enc

    def set_pipeline(self, pipeline: RenderPipeline) -> None:
        self.enc._push(A.OP_SET_PIPELINE, A.CmdSetPipeline(pipeline.handle))

    def set_bind_group(self, index: int, bind_group: Optional[BindGroup], offsets: Sequence[int] = ()) -> None:
        self.enc._push(A.OP_SET_BIND_GROUP,
                       A.CmdSetBindGroup(index, len(offsets), bind_group.handle if bind_group else 0))

    def set_index_buffer(self, buffer: Buffer, index_format: int, offset: int = 0, size: int = 0) -> None:
        self.enc._push(A.OP_SET_INDEX_BUFFER, A.CmdSetIndexBuffer(buffer.handle, index_format, 0, offset, size))

    def set_vertex_buffer(self, slot: int, buffer: Buffer, offset: int = 0, size: int = 0) -> None:
        self.enc._push(A.OP_SET_VERTEX_BUFFER, A.CmdSetVertexBuffer(slot, 0, buffer.handle, offset, size))

    def set_viewport(self, x, y, w, h, min_depth=0.0, max_depth=1.0) -> None:
        self.enc._push(A.OP_SET_VIEWPORT, A.CmdSetViewport(x, y, w, h, min_depth, max_depth))

    def set_scissor_rect(self, x, y, w, h) -> None:
        self.enc._push(A.OP_SET_SCISSOR_RECT, A.CmdSetScissorRect(x, y, w, h))

    def set_blend_constant(self, color) -> None:
        c = A.CmdSetBlendConstant()
        for k in range(4):
            c.color[k] = float(color[k])
        self.enc._push(A.OP_SET_BLEND_CONSTANT, c)

    def draw(self, vertices: range, instances: range = range(0, 1)) -> None:
        self.enc._push(A.OP_DRAW, A.CmdDraw(vertices.start, vertices.stop, instances.start, instances.stop))

    def draw_indexed(self, indices: range, base_vertex: int = 0, instances: range = range(0, 1)) -> None:
        self.enc._push(A.OP_DRAW_INDEXED, A.CmdDrawIndexed(indices.start, indices.stop, base_vertex,
                                                           instances.start, instances.stop, 0))

    def end(self) -> None:
        self.enc._push(A.OP_END_RENDER_PASS)
        self.enc._open_pass = False


# ------------------------------------------------------------------------------------ device
def _byte_array(data) -> np.ndarray:
    """The bytes of `data` as a contiguous uint8 array: a contiguous ndarray is viewed, not copied;
    other arrays and buffer objects (bytes, bytearray, memoryview, ...) are copied when needed."""
    if isinstance(data, np.ndarray):
        return np.ascontiguousarray(data).reshape(-1).view(np.uint8)
    mv = memoryview(data)
    if not mv.c_contiguous:
        return np.frombuffer(mv.tobytes(), dtype=np.uint8)
    return np.frombuffer(mv.cast("B"), dtype=np.uint8)


class PreparedWrites:
    """A fixed list of buffer writes [(buffer, offset, data)] for Queue.write_buffers.

    C-contiguous numpy arrays are referenced, not copied: their contents at each write_buffers
    call are what gets written (as with write_buffer, the bytes are captured by the call).  Every
    other input (bytes, bytearray, memoryview, non-contiguous arrays) is copied once, here, into a
    contiguous snapshot; later changes to such an object are not seen by later write_buffers
    calls — build a new PreparedWrites, or pass a contiguous ndarray, to send new contents."""

    def __init__(self, items):
        self.items = []
        for buf, off, data in items:
            if not (isinstance(data, np.ndarray) and data.flags.c_contiguous):
                data = _byte_array(data)
            self.items.append((buf, int(off), data))
        self.array = (A.BufferWrite * max(1, len(self.items)))()
        for k, (buf, off, data) in enumerate(self.items):
            self.array[k] = A.BufferWrite(buf.handle, off, data.__array_interface__["data"][0], data.nbytes)


class Queue:
    def __init__(self, device: "Device"):
        self.device = device

    def write_buffers(self, writes) -> None:
        """Many write_buffer calls in one (gbr_queue_write_buffers): `writes` is a PreparedWrites
        or a list of (buffer, offset, data).  Queued in order; nothing is queued if an entry is
        invalid.  Libraries without the batched entry point get one write_buffer per entry."""
        if not isinstance(writes, PreparedWrites):
            writes = PreparedWrites(writes)
        d = self.device
        if d.lib.queue_write_buffers is None:
            for buf, off, data in writes.items:
                self.write_buffer(buf, off, data)
            return
        _check(d.lib, d.lib.queue_write_buffers(d.handle, len(writes.items), C.cast(writes.array, C.c_void_p)))

    def write_buffer(self, buffer: Buffer, offset: int, data) -> None:
        d = self.device
        if isinstance(data, np.ndarray) and data.flags.c_contiguous:  # no copy, no view objects
            _check(d.lib, d.lib.queue_write_buffer(d.handle, buffer.handle, offset,
                                                   data.__array_interface__["data"][0], data.nbytes))
            return
        arr = _byte_array(data)
        _check(d.lib, d.lib.queue_write_buffer(d.handle, buffer.handle, offset, arr.ctypes.data, arr.nbytes))

    def write_texture(self, texture: Texture, data, bytes_per_row: int = 0, rows_per_image: int = 0,
                      mip_level: int = 0, offset: int = 0) -> None:
        arr = _byte_array(data)
        w, h = texture.mip_size(mip_level)
        layout = A.TexelCopyBufferLayout(offset, bytes_per_row or w * BYTES_PER_TEXEL[texture.format],
                                         rows_per_image or h)
        ext = A.Extent3d(w, h, texture.layers)
        d = self.device
        _check(d.lib, d.lib.queue_write_texture(d.handle, texture.handle, mip_level, arr.ctypes.data, arr.nbytes,
                                                C.byref(layout), ext))

    def submit(self, command_buffers: Sequence[CommandBuffer]) -> int:
        d = self.device
        data = b"".join(cb.data for cb in command_buffers)
        buf = C.create_string_buffer(data, len(data)) if data else None
        idx = C.c_uint64()
        _check(d.lib, d.lib.queue_submit(d.handle, buf, len(data), C.byref(idx)))
        return idx.value


class Device:
    """One device + queue + worker (wgpu_cpu::instance -> request_adapter -> request_device)."""

    def __init__(self, lib: Optional[A.Lib] = None, profile: int = Profile.PARITY, tile_size: int = 0,
                 warps_per_tile: int = 0, bin_capacity: int = 0, launch_mode: int = LaunchMode.BATCHED,
                 batch_submissions: bool = False, use_graphs: bool = False, hbm_budget_bytes: int = 0,
                 device_ordinal: int = 0, time_kernels: bool = False, raster_order: int = 0,
                 raster_rule: int = RasterRule.SCANLINE):
        self.lib = lib if lib is not None else gpu_lib()
        cfg = A.DeviceConfig()
        cfg.abi_version = A.GBR_ABI_VERSION
        cfg.profile = profile
        cfg.device_ordinal = device_ordinal
        cfg.tile_size = tile_size
        cfg.warps_per_tile = warps_per_tile
        cfg.bin_capacity = bin_capacity
        cfg.launch_mode = launch_mode
        cfg.batch_submissions = int(batch_submissions)
        cfg.use_graphs = int(use_graphs)
        cfg.time_kernels = int(time_kernels)
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.raster_order = int(raster_order)
        cfg.raster_rule = int(raster_rule)
        h = C.c_uint64()
        self.handle = 0
        _check(self.lib, self.lib.device_create(C.byref(cfg), C.byref(h)))
        self.handle = h.value
        self.profile = profile
        self.raster_rule = raster_rule
        self.queue = Queue(self)

    def close(self) -> None:
        if self.handle:
            _check(self.lib, self.lib.device_destroy(self.handle))
            self.handle = 0

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def limits(self) -> A.Limits:
        out = A.Limits()
        _check(self.lib, self.lib.device_limits(self.handle, C.byref(out)))
        return out

    # -- resources
    def create_buffer(self, size: int, usage: int = 0, data=None) -> Buffer:
        h = C.c_uint64()
        _check(self.lib, self.lib.buffer_create(self.handle, size, usage, C.byref(h)))
        b = Buffer(self, h.value, size)
        if data is not None:
            self.queue.write_buffer(b, 0, data)
        return b

    def create_buffer_init(self, data, usage: int = 0) -> Buffer:
        arr = _byte_array(data)
        return self.create_buffer(arr.nbytes, usage, arr)

    def create_texture(self, width: int, height: int, format: int, mip_level_count: int = 1, layers: int = 1,
                       usage: int = 0) -> Texture:
        desc = A.TextureDesc(A.Extent3d(width, height, layers), mip_level_count, 1, 2, format, usage, 0)
        h = C.c_uint64()
        _check(self.lib, self.lib.texture_create(self.handle, C.byref(desc), C.byref(h)))
        return Texture(self, h.value, width, height, format, mip_level_count, layers)

    def create_sampler(self, address_mode_u=AddressMode.CLAMP_TO_EDGE, address_mode_v=AddressMode.CLAMP_TO_EDGE,
                       address_mode_w=AddressMode.CLAMP_TO_EDGE, mag_filter=FilterMode.NEAREST,
                       min_filter=FilterMode.NEAREST, mipmap_filter=FilterMode.NEAREST, lod_min_clamp=0.0,
                       lod_max_clamp=32.0) -> Sampler:
        desc = A.SamplerDesc(address_mode_u, address_mode_v, address_mode_w, mag_filter, min_filter, mipmap_filter,
                             lod_min_clamp, lod_max_clamp, 0, 1)
        h = C.c_uint64()
        _check(self.lib, self.lib.sampler_create(self.handle, C.byref(desc), C.byref(h)))
        return Sampler(self, h.value)

    def create_shader_module(self, wgsl: Optional[str] = None, native: Optional[str] = None) -> ShaderModule:
        h = C.c_uint64()
        if native is not None:
            _check(self.lib, self.lib.shader_module_create_native(self.handle, native.encode(), C.byref(h)))
        else:
            if self.lib.shader_module_create is None:
                raise GbrError(A.ERR_UNSUPPORTED, "this library has no WGSL front end")
            src = wgsl.encode()
            _check(self.lib, self.lib.shader_module_create(self.handle, src, len(src), C.byref(h)))
        return ShaderModule(self, h.value)

    def create_render_pipeline(self, vertex_module: ShaderModule, vertex_buffers: Sequence[VertexBufferLayout] = (),
                               primitive: PrimitiveState = PrimitiveState(),
                               depth_stencil: Optional[DepthStencilState] = None,
                               fragment_module: Optional[ShaderModule] = None,
                               targets: Sequence[Optional[ColorTargetState]] = (),
                               vertex_entry_point: str = "vs_main", fragment_entry_point: str = "fs_main",
                               vertex_constants: Optional[dict] = None, fragment_constants: Optional[dict] = None
                               ) -> RenderPipeline:
        """wgpu's create_render_pipeline.  `vertex_constants` / `fragment_constants` are the
        stages' PipelineCompilationOptions::constants: {override @id (as a string) or name: value}."""
        d = A.RenderPipelineDesc()
        keep = []

        def constants(cs):
            if not cs:
                return None, 0
            arr = (A.PipelineConstant * len(cs))()
            for i, (k, v) in enumerate(cs.items()):
                kb = C.create_string_buffer(str(k).encode())
                keep.append(kb)
                arr[i] = A.PipelineConstant(C.cast(kb, C.c_char_p), float(v))
            keep.append(arr)
            return C.cast(arr, C.c_void_p), len(cs)

        d.vertex_constants, d.vertex_constant_count = constants(vertex_constants)
        d.fragment_constants, d.fragment_constant_count = constants(fragment_constants)
        d.vertex_module = vertex_module.handle
        d.vertex_entry_point = vertex_entry_point.encode()
        d.vertex_buffer_count = len(vertex_buffers)
        for i, vb in enumerate(vertex_buffers):
            L = d.vertex_buffers[i]
            L.array_stride = vb.array_stride
            L.step_mode = vb.step_mode
            L.attribute_count = len(vb.attributes)
            for j, at in enumerate(vb.attributes):
                L.attributes[j] = A.VertexAttribute(at.format, at.shader_location, at.offset)
        d.primitive = A.PrimitiveState(primitive.topology, primitive.strip_index_format, primitive.front_face,
                                       primitive.cull_mode, 0, 0)
        if depth_stencil is not None:
            d.has_depth_stencil = 1
            d.depth_stencil = A.DepthStencilState(depth_stencil.format, int(depth_stencil.depth_write_enabled),
                                                  depth_stencil.depth_compare, 0)
        d.multisample_count = 1
        if fragment_module is not None:
            d.has_fragment = 1
            d.fragment_module = fragment_module.handle
            d.fragment_entry_point = fragment_entry_point.encode()
            d.color_target_count = len(targets)
            for i, t in enumerate(targets):
                if t is None:
                    continue
                ct = d.color_targets[i]
                ct.format = t.format
                ct.write_mask = t.write_mask
                if t.blend is not None:
                    ct.has_blend = 1
                    ct.color = A.BlendComponent(t.blend.color.src_factor, t.blend.color.dst_factor,
                                                t.blend.color.operation)
                    ct.alpha = A.BlendComponent(t.blend.alpha.src_factor, t.blend.alpha.dst_factor,
                                                t.blend.alpha.operation)
        h = C.c_uint64()
        _check(self.lib, self.lib.render_pipeline_create(self.handle, C.byref(d), C.byref(h)))
        return RenderPipeline(self, h.value)

    def create_bind_group(self, entries: Sequence[BindGroupEntry]) -> BindGroup:
        d = A.BindGroupDesc()
        d.entry_count = len(entries)
        for i, e in enumerate(entries):
            en = d.entries[i]
            en.binding = e.binding
            en.resource = e.resource.handle
            en.offset = e.offset
            en.size = e.size
            en.kind = (BindingKind.BUFFER if isinstance(e.resource, Buffer)
                       else BindingKind.SAMPLER if isinstance(e.resource, Sampler) else BindingKind.TEXTURE_VIEW)
        h = C.c_uint64()
        _check(self.lib, self.lib.bind_group_create(self.handle, C.byref(d), C.byref(h)))
        return BindGroup(self, h.value)

    def create_command_encoder(self) -> CommandEncoder:
        return CommandEncoder(self)

    # -- synchronisation / readback
    def poll(self, wait: bool = True, submission_index: Optional[int] = None,
             timeout_s: Optional[float] = None) -> int:
        st = C.c_uint32()
        tns = 0xFFFFFFFFFFFFFFFF if timeout_s is None else int(timeout_s * 1e9)
        _check(self.lib, self.lib.device_poll(self.handle, int(wait), int(submission_index is not None),
                                              submission_index or 0, tns, C.byref(st)))
        return st.value

    def submission_stats(self, index: int) -> A.SubmissionStats:
        s = A.SubmissionStats()
        _check(self.lib, self.lib.submission_stats_get(self.handle, index, C.byref(s)))
        return s

    def elapsed_ms(self, first: int, last: int) -> float:
        """Device time from the start of submission `first` to the end of `last` (CUDA events)."""
        if self.lib.device_elapsed_ms is None:
            raise GbrError(A.ERR_UNSUPPORTED, "no device timing in this library")
        out = C.c_double()
        _check(self.lib, self.lib.device_elapsed_ms(self.handle, first, last, C.byref(out)))
        return out.value

    def memory(self) -> tuple:
        """(resident bytes of live buffers and textures, bytes of the worker's scratch arena)."""
        if self.lib.device_memory is None:
            raise GbrError(A.ERR_UNSUPPORTED, "no memory query in this library")
        r, t = C.c_uint64(), C.c_uint64()
        _check(self.lib, self.lib.device_memory(self.handle, C.byref(r), C.byref(t)))
        return r.value, t.value

    def flush_caches(self) -> None:
        if self.lib.device_flush_caches is not None:
            _check(self.lib, self.lib.device_flush_caches(self.handle))

    def read_textures_into(self, items) -> None:
        """Reads several textures in one queue operation: items = [(texture, mip_level, address,
        nbytes)], each destination at least the mip level's size (gbr_textures_read; one
        gbr_texture_read per texture where the library lacks it)."""
        items = list(items)
        if not items:
            return
        if self.lib.textures_read is None:
            for t, mip, ptr, n in items:
                _check(self.lib, self.lib.texture_read(self.handle, t.handle, mip, ptr, n))
            return
        k = len(items)
        hs = (C.c_uint64 * k)(*[t.handle for t, _, _, _ in items])
        ms = (C.c_uint32 * k)(*[m for _, m, _, _ in items])
        ps = (C.c_void_p * k)(*[p for _, _, p, _ in items])
        ns = (C.c_uint64 * k)(*[n for _, _, _, n in items])
        _check(self.lib, self.lib.textures_read(self.handle, k, hs, ms, ps, ns))

    def read_textures_into_async(self, items):
        """Enqueues the readback of several textures without waiting (gbr_queue_read_textures:
        copy_texture_to_buffer + map_async): items as for read_textures_into.  Returns the
        readback's submission index; the destinations hold the bytes once poll(True, index) has
        returned.  A library without the call reads synchronously and returns None."""
        items = list(items)
        if not items:
            return None
        if self.lib.queue_read_textures is None:
            self.read_textures_into(items)
            return None
        k = len(items)
        hs = (C.c_uint64 * k)(*[t.handle for t, _, _, _ in items])
        ms = (C.c_uint32 * k)(*[m for _, m, _, _ in items])
        ps = (C.c_void_p * k)(*[p for _, _, p, _ in items])
        ns = (C.c_uint64 * k)(*[n for _, _, _, n in items])
        idx = C.c_uint64(0)
        _check(self.lib, self.lib.queue_read_textures(self.handle, k, hs, ms, ps, ns, C.byref(idx)))
        return idx.value

    def read_textures(self, textures: Sequence[Texture], mip_level: int = 0) -> List[np.ndarray]:
        outs = []
        for t in textures:
            w, h = t.mip_size(mip_level)
            outs.append(np.empty((t.layers, h, w, BYTES_PER_TEXEL[t.format]), dtype=np.uint8))
        self.read_textures_into([(t, mip_level, o.ctypes.data, o.nbytes) for t, o in zip(textures, outs)])
        return [o[0] if t.layers == 1 else o for t, o in zip(textures, outs)]

    def read_texture(self, texture: Texture, mip_level: int = 0) -> np.ndarray:
        w, h = texture.mip_size(mip_level)
        bpp = BYTES_PER_TEXEL[texture.format]
        out = np.empty((texture.layers, h, w, bpp), dtype=np.uint8)
        _check(self.lib, self.lib.texture_read(self.handle, texture.handle, mip_level, out.ctypes.data, out.nbytes))
        return out[0] if texture.layers == 1 else out
