//! `wgpu-gb300`: the wgpu 28 `custom` backend of wgpu-cpu, with its render passes executed on a
//! GB300 by `libgbr` (the C ABI of `include/gbr.h`).
//!
//! `wgpu_gb300::instance(config)` replaces `wgpu_cpu::instance(config)` (wgpu-cpu/src/lib.rs:25-27):
//! the same `wgpu::Instance::from_custom` entry, the same trait implementations
//! (`InstanceInterface`, `AdapterInterface`, `DeviceInterface`, `QueueInterface`,
//! `CommandEncoderInterface`, `RenderPassInterface` and the resource interfaces), each method
//! forwarding to one `gbr_*` call.  Render passes are recorded as the flat command stream
//! `gbr_queue_submit` takes (the `gbr_cmd_*` records), so recording never crosses the ABI.
//!
//! Errors: where wgpu-cpu panics (`todo!`, `unwrap`, `assert!`), this crate panics with the
//! library's message (`gbr_last_error`), keeping the reference's behaviour; the library itself
//! never unwinds and stays usable.

#![allow(clippy::missing_safety_doc)]

pub mod sys;

use std::{
    ffi::CString,
    ops::Range,
    os::raw::{c_char, c_void},
    pin::Pin,
    sync::Arc,
};

use parking_lot::Mutex;
use sys::*;

// ------------------------------------------------------------------------------------ config

/// Device configuration (`gbr_device_config`); `Default` is the parity profile on CUDA device 0
/// with the batched launch mode.
#[derive(Clone, Debug, Default)]
pub struct Config {
    /// 0 = parity (exactly wgpu-cpu's results), 1 = extension (blending, f16 targets, filtering)
    pub profile: u32,
    pub device_ordinal: u32,
    /// 0 = batched, 1 = one launch sequence per draw, 2 = per pass
    pub launch_mode: u32,
    pub batch_submissions: bool,
    pub use_graphs: bool,
    pub hbm_budget_bytes: u64,
}

pub fn instance(config: Config) -> wgpu::Instance {
    wgpu::Instance::from_custom(Instance { config: Arc::new(config) })
}

/// Panics with the library's error text when `st` is not GBR_OK (the reference panics at the
/// same places: unwrap / expect / todo!).
#[track_caller]
fn check(st: gbr_status, what: &str) {
    if st != GBR_OK {
        panic!("{what}: status {st}: {}", last_error());
    }
}

/// The device handle, released when the last object of the device is dropped.
#[derive(Debug)]
struct DeviceHandle(gbr_device);

impl Drop for DeviceHandle {
    fn drop(&mut self) {
        unsafe { gbr_device_destroy(self.0) };
    }
}

/// A library object (buffer, texture, ...) with its destroy call.
#[derive(Debug)]
struct Handle {
    device: Arc<DeviceHandle>,
    handle: u64,
    destroy: unsafe extern "C" fn(gbr_device, u64) -> gbr_status,
}

impl Drop for Handle {
    fn drop(&mut self) {
        unsafe { (self.destroy)(self.device.0, self.handle) };
    }
}

// ------------------------------------------------------------------------------------ conversions

fn texture_format(f: wgpu::TextureFormat) -> u32 {
    use wgpu::TextureFormat as F;
    match f {
        F::R8Unorm => 1,
        F::Rg8Unorm => 2,
        F::Rgba8Unorm => 3,
        F::Rgba8UnormSrgb => 4,
        F::Bgra8Unorm => 5,
        F::Bgra8UnormSrgb => 6,
        F::Rgba16Float => 7,
        F::Rgba32Float => 8,
        F::Depth32Float => 9,
        other => panic!("texture format {other:?} is not supported (texture.rs:456-505)"),
    }
}

fn vertex_format(f: wgpu::VertexFormat) -> u32 {
    use wgpu::VertexFormat as V;
    match f {
        V::Float32 => 1,
        V::Float32x2 => 2,
        V::Float32x3 => 3,
        V::Float32x4 => 4,
        V::Uint32 => 5,
        V::Sint32 => 6,
        V::Float16x2 => 7,
        V::Float16x4 => 8,
        V::Unorm8x4 => 9,
        other => panic!("vertex format {other:?} is not supported"),
    }
}

fn index_format(f: Option<wgpu::IndexFormat>) -> u32 {
    match f {
        None => 0,
        Some(wgpu::IndexFormat::Uint16) => 1,
        Some(wgpu::IndexFormat::Uint32) => 2,
    }
}

fn topology(t: wgpu::PrimitiveTopology) -> u32 {
    use wgpu::PrimitiveTopology as T;
    match t {
        T::PointList => 0,
        T::LineList => 1,
        T::LineStrip => 2,
        T::TriangleList => 3,
        T::TriangleStrip => 4,
    }
}

fn compare(c: Option<wgpu::CompareFunction>) -> u32 {
    use wgpu::CompareFunction as C;
    match c {
        None => 0,
        Some(C::Never) => 1,
        Some(C::Less) => 2,
        Some(C::Equal) => 3,
        Some(C::LessEqual) => 4,
        Some(C::Greater) => 5,
        Some(C::NotEqual) => 6,
        Some(C::GreaterEqual) => 7,
        Some(C::Always) => 8,
    }
}

fn blend_factor(f: wgpu::BlendFactor) -> u32 {
    use wgpu::BlendFactor as B;
    match f {
        B::Zero => 0,
        B::One => 1,
        B::Src => 2,
        B::OneMinusSrc => 3,
        B::SrcAlpha => 4,
        B::OneMinusSrcAlpha => 5,
        B::Dst => 6,
        B::OneMinusDst => 7,
        B::DstAlpha => 8,
        B::OneMinusDstAlpha => 9,
        B::Constant => 11,
        B::OneMinusConstant => 12,
        other => panic!("blend factor {other:?} is not supported"),
    }
}

fn blend_component(c: &wgpu::BlendComponent) -> gbr_blend_component {
    use wgpu::BlendOperation as O;
    gbr_blend_component {
        src_factor: blend_factor(c.src_factor),
        dst_factor: blend_factor(c.dst_factor),
        operation: match c.operation {
            O::Add => 0,
            O::Subtract => 1,
            O::ReverseSubtract => 2,
            O::Min => 3,
            O::Max => 4,
        },
    }
}

fn address_mode(a: wgpu::AddressMode) -> u32 {
    use wgpu::AddressMode as A;
    match a {
        A::ClampToEdge => 0,
        A::Repeat => 1,
        A::MirrorRepeat => 2,
        A::ClampToBorder => 3,
    }
}

fn filter(f: wgpu::FilterMode) -> u32 {
    match f {
        wgpu::FilterMode::Nearest => 0,
        wgpu::FilterMode::Linear => 1,
    }
}

fn mipmap_filter(f: wgpu::MipmapFilterMode) -> u32 {
    match f {
        wgpu::MipmapFilterMode::Nearest => 0,
        wgpu::MipmapFilterMode::Linear => 1,
    }
}

fn entry_point_name(name: Option<&str>) -> [c_char; GBR_MAX_ENTRY_POINT_NAME] {
    let mut out = [0 as c_char; GBR_MAX_ENTRY_POINT_NAME];
    if let Some(name) = name {
        assert!(name.len() < GBR_MAX_ENTRY_POINT_NAME, "entry point name too long");
        for (o, b) in out.iter_mut().zip(name.bytes()) {
            *o = b as c_char;
        }
    }
    out
}

// ------------------------------------------------------------------------------------ command stream

/// Appends one `[opcode][payload_bytes][payload, padded to 8]` record.
fn push_record<T: Copy>(stream: &mut Vec<u8>, opcode: u32, payload: Option<&T>) {
    let size = payload.map_or(0, |_| std::mem::size_of::<T>());
    stream.extend_from_slice(&opcode.to_le_bytes());
    stream.extend_from_slice(&(size as u32).to_le_bytes());
    if let Some(p) = payload {
        let bytes = unsafe { std::slice::from_raw_parts(p as *const T as *const u8, size) };
        stream.extend_from_slice(bytes);
        stream.resize(stream.len() + (8 - size % 8) % 8, 0);
    }
}

// ------------------------------------------------------------------------------------ instance, adapter

#[derive(Debug)]
pub struct Instance {
    config: Arc<Config>,
}

impl wgpu::custom::InstanceInterface for Instance {
    fn new(_desc: wgpu::InstanceDescriptor) -> Self
    where
        Self: Sized,
    {
        unreachable!("InstanceInterface::new is not called for a custom instance");
    }

    unsafe fn create_surface(
        &self,
        _target: wgpu::SurfaceTargetUnsafe,
    ) -> Result<wgpu::custom::DispatchSurface, wgpu::CreateSurfaceError> {
        // no presentation: targets are read back with gbr_texture_read
        Err(wgpu::CreateSurfaceError::custom("wgpu-gb300 renders headless: no surfaces".to_owned()))
    }

    fn request_adapter(
        &self,
        options: &wgpu::RequestAdapterOptions,
    ) -> Pin<Box<dyn wgpu::custom::RequestAdapterFuture>> {
        let result = if options.compatible_surface.is_some() {
            Err(wgpu::RequestAdapterError::Custom("Surface not compatible".to_owned()))
        } else {
            Ok(wgpu::custom::DispatchAdapter::custom(Adapter { config: self.config.clone() }))
        };
        Box::pin(async move { result })
    }

    fn poll_all_devices(&self, _force_wait: bool) -> bool {
        true
    }

    fn enumerate_adapters(
        &self,
        _backends: wgpu::Backends,
    ) -> Pin<Box<dyn wgpu::custom::EnumerateAdapterFuture>> {
        let out = vec![wgpu::custom::DispatchAdapter::custom(Adapter { config: self.config.clone() })];
        Box::pin(async move { out })
    }

    fn wgsl_language_features(&self) -> wgpu::WgslLanguageFeatures {
        wgpu::WgslLanguageFeatures::empty()
    }
}

#[derive(Debug)]
pub struct Adapter {
    config: Arc<Config>,
}

impl wgpu::custom::AdapterInterface for Adapter {
    fn request_device(
        &self,
        desc: &wgpu::DeviceDescriptor<'_>,
    ) -> Pin<Box<dyn wgpu::custom::RequestDeviceFuture>> {
        // one gbr_device_create: device, queue and its worker (device.rs:40-74, engine.rs:12-24)
        let c = &self.config;
        let cfg = gbr_device_config {
            abi_version: GBR_ABI_VERSION,
            profile: c.profile,
            device_ordinal: c.device_ordinal,
            launch_mode: c.launch_mode,
            batch_submissions: c.batch_submissions as u32,
            use_graphs: c.use_graphs as u32,
            hbm_budget_bytes: c.hbm_budget_bytes,
            ..Default::default()
        };
        let features = desc.required_features;
        let limits = desc.required_limits.clone();
        let mut handle = 0u64;
        let st = unsafe { gbr_device_create(&cfg, &mut handle) };
        let result = if st == GBR_OK {
            let dev = Arc::new(DeviceHandle(handle));
            Ok((
                wgpu::custom::DispatchDevice::custom(Device { dev: dev.clone(), features, limits }),
                wgpu::custom::DispatchQueue::custom(Queue { dev }),
            ))
        } else {
            Err(wgpu::RequestDeviceError::custom(last_error()))
        };
        Box::pin(async move { result })
    }

    fn is_surface_supported(&self, _surface: &wgpu::custom::DispatchSurface) -> bool {
        false
    }

    fn features(&self) -> wgpu::Features {
        wgpu::Features::default()
    }

    fn limits(&self) -> wgpu::Limits {
        wgpu::Limits::downlevel_defaults()
    }

    fn downlevel_capabilities(&self) -> wgpu::DownlevelCapabilities {
        wgpu::DownlevelCapabilities::default()
    }

    fn get_info(&self) -> wgpu::AdapterInfo {
        wgpu::AdapterInfo {
            name: "wgpu-gb300".to_owned(),
            vendor: 0x10de,
            device: 0,
            device_type: wgpu::DeviceType::DiscreteGpu,
            device_pci_bus_id: String::new(),
            driver: "libgbr".to_owned(),
            driver_info: String::new(),
            backend: wgpu::Backend::Noop,
            subgroup_min_size: wgpu::MINIMUM_SUBGROUP_MIN_SIZE,
            subgroup_max_size: wgpu::MAXIMUM_SUBGROUP_MAX_SIZE,
            transient_saves_memory: false,
        }
    }

    fn get_texture_format_features(&self, _format: wgpu::TextureFormat) -> wgpu::TextureFormatFeatures {
        wgpu::TextureFormatFeatures {
            allowed_usages: wgpu::TextureUsages::COPY_SRC
                | wgpu::TextureUsages::COPY_DST
                | wgpu::TextureUsages::TEXTURE_BINDING
                | wgpu::TextureUsages::RENDER_ATTACHMENT,
            flags: wgpu::TextureFormatFeatureFlags::empty(),
        }
    }

    fn get_presentation_timestamp(&self) -> wgpu::PresentationTimestamp {
        unimplemented!("no presentation")
    }

    fn cooperative_matrix_properties(&self) -> Vec<wgpu::wgt::CooperativeMatrixProperties> {
        Vec::new()
    }
}

// ------------------------------------------------------------------------------------ resources

#[derive(Debug)]
pub struct Buffer {
    obj: Handle,
    size: u64,
    /// host copy while mapped: reads fill it at map time, writes upload it at unmap
    mapping: Mutex<Option<(wgpu::MapMode, Vec<u8>)>>,
}

impl wgpu::custom::BufferInterface for Buffer {
    fn map_async(&self, mode: wgpu::MapMode, range: Range<wgpu::BufferAddress>, callback: wgpu::custom::BufferMapCallback) {
        let mut m = self.mapping.lock();
        assert!(m.is_none(), "Buffer already mapped");
        let mut host = vec![0u8; self.size as usize];
        if mode == wgpu::MapMode::Read {
            // waits for prior submissions (buffer.rs:112-136)
            let st = unsafe {
                gbr_buffer_read(self.obj.device.0, self.obj.handle, range.start,
                                host[range.start as usize..].as_mut_ptr() as *mut c_void, range.end - range.start)
            };
            if st != GBR_OK {
                callback(Err(wgpu::BufferAsyncError));
                return;
            }
        }
        *m = Some((mode, host));
        callback(Ok(()));
    }

    fn get_mapped_range(&self, range: Range<wgpu::BufferAddress>) -> wgpu::custom::DispatchBufferMappedRange {
        let mut m = self.mapping.lock();
        let (_, host) = m.as_mut().expect("Buffer is not mapped");
        let slice = &mut host[range.start as usize..range.end as usize];
        wgpu::custom::DispatchBufferMappedRange::custom(MappedRange { ptr: slice.as_mut_ptr(), len: slice.len() })
    }

    fn unmap(&self) {
        let (mode, host) = self.mapping.lock().take().expect("Buffer is not mapped");
        if mode == wgpu::MapMode::Write {
            check(unsafe { gbr_queue_write_buffer(self.obj.device.0, self.obj.handle, 0, host.as_ptr() as *const c_void, self.size) },
                  "unmap");
        }
    }

    fn destroy(&self) {}
}

/// A view of a mapped buffer's host copy (valid until unmap, as wgpu's mapped ranges are).
#[derive(Debug)]
pub struct MappedRange {
    ptr: *mut u8,
    len: usize,
}
unsafe impl Send for MappedRange {}
unsafe impl Sync for MappedRange {}

impl wgpu::custom::BufferMappedRangeInterface for MappedRange {
    fn slice(&self) -> &[u8] {
        unsafe { std::slice::from_raw_parts(self.ptr, self.len) }
    }

    fn slice_mut(&mut self) -> &mut [u8] {
        unsafe { std::slice::from_raw_parts_mut(self.ptr, self.len) }
    }
}

#[derive(Debug)]
pub struct Texture {
    obj: Arc<Handle>,
    desc: gbr_texture_desc,
}

impl wgpu::custom::TextureInterface for Texture {
    fn create_view(&self, desc: &wgpu::TextureViewDescriptor<'_>) -> wgpu::custom::DispatchTextureView {
        // the path renders into mip 0; layers are chosen per colour attachment (depth_slice)
        assert!(desc.base_mip_level == 0, "views of mip levels other than 0 are not supported");
        wgpu::custom::DispatchTextureView::custom(TextureView { texture: self.obj.clone(), base_layer: desc.base_array_layer })
    }

    fn destroy(&self) {}
}

#[derive(Debug)]
pub struct TextureView {
    texture: Arc<Handle>,
    base_layer: u32,
}

impl wgpu::custom::TextureViewInterface for TextureView {}

#[derive(Debug)]
pub struct Sampler {
    obj: Handle,
}
impl wgpu::custom::SamplerInterface for Sampler {}

#[derive(Debug)]
pub struct ShaderModule {
    obj: Handle,
}
impl wgpu::custom::ShaderModuleInterface for ShaderModule {
    fn get_compilation_info(&self) -> Pin<Box<dyn wgpu::custom::ShaderCompilationInfoFuture>> {
        Box::pin(async move { wgpu::CompilationInfo { messages: vec![] } })
    }
}

/// Bind group layouts carry no state the library needs (bindings are resolved per draw).
#[derive(Debug)]
pub struct BindGroupLayout;
impl wgpu::custom::BindGroupLayoutInterface for BindGroupLayout {}

#[derive(Debug)]
pub struct PipelineLayout;
impl wgpu::custom::PipelineLayoutInterface for PipelineLayout {}

#[derive(Debug)]
pub struct BindGroup {
    obj: Handle,
}
impl wgpu::custom::BindGroupInterface for BindGroup {}

#[derive(Debug)]
pub struct RenderPipeline {
    obj: Handle,
}
impl wgpu::custom::RenderPipelineInterface for RenderPipeline {
    fn get_bind_group_layout(&self, _index: u32) -> wgpu::custom::DispatchBindGroupLayout {
        wgpu::custom::DispatchBindGroupLayout::custom(BindGroupLayout)
    }
}

// ------------------------------------------------------------------------------------ device

#[derive(Debug)]
pub struct Device {
    dev: Arc<DeviceHandle>,
    features: wgpu::Features,
    limits: wgpu::Limits,
}

impl Device {
    fn handle(&self, handle: u64, destroy: unsafe extern "C" fn(gbr_device, u64) -> gbr_status) -> Handle {
        Handle { device: self.dev.clone(), handle, destroy }
    }
}

impl wgpu::custom::DeviceInterface for Device {
    fn features(&self) -> wgpu::Features {
        self.features
    }

    fn limits(&self) -> wgpu::Limits {
        self.limits.clone()
    }

    fn create_shader_module(
        &self,
        desc: wgpu::ShaderModuleDescriptor<'_>,
        _checks: wgpu::ShaderRuntimeChecks,
    ) -> wgpu::custom::DispatchShaderModule {
        let src = match desc.source {
            wgpu::ShaderSource::Wgsl(src) => src,
            _ => panic!("Provided shader source variant is not supported"),
        };
        let mut h = 0u64;
        check(unsafe { gbr_shader_module_create(self.dev.0, src.as_ptr() as *const c_char, src.len() as u64, &mut h) },
              "create_shader_module");
        wgpu::custom::DispatchShaderModule::custom(ShaderModule { obj: self.handle(h, gbr_shader_module_destroy) })
    }

    unsafe fn create_shader_module_passthrough(
        &self,
        _desc: &wgpu::ShaderModuleDescriptorPassthrough<'_>,
    ) -> wgpu::custom::DispatchShaderModule {
        unimplemented!("passthrough shaders")
    }

    fn create_bind_group_layout(&self, _desc: &wgpu::BindGroupLayoutDescriptor<'_>) -> wgpu::custom::DispatchBindGroupLayout {
        wgpu::custom::DispatchBindGroupLayout::custom(BindGroupLayout)
    }

    fn create_bind_group(&self, desc: &wgpu::BindGroupDescriptor<'_>) -> wgpu::custom::DispatchBindGroup {
        let mut d = gbr_bind_group_desc::default();
        assert!(desc.entries.len() <= GBR_MAX_BIND_GROUP_ENTRIES, "too many bind group entries");
        d.entry_count = desc.entries.len() as u32;
        for (e, out) in desc.entries.iter().zip(d.entries.iter_mut()) {
            out.binding = e.binding;
            match &e.resource {
                wgpu::BindingResource::Buffer(b) => {
                    out.kind = GBR_BINDING_BUFFER;
                    out.resource = b.buffer.inner.as_custom::<Buffer>().unwrap().obj.handle;
                    out.offset = b.offset;
                    out.size = b.size.map_or(0, |s| s.get());
                }
                wgpu::BindingResource::Sampler(s) => {
                    out.kind = GBR_BINDING_SAMPLER;
                    out.resource = s.inner.as_custom::<Sampler>().unwrap().obj.handle;
                }
                wgpu::BindingResource::TextureView(v) => {
                    out.kind = GBR_BINDING_TEXTURE_VIEW;
                    out.resource = v.inner.as_custom::<TextureView>().unwrap().texture.handle;
                }
                other => panic!("binding resource {other:?} is not supported"),
            }
        }
        let mut h = 0u64;
        check(unsafe { gbr_bind_group_create(self.dev.0, &d, &mut h) }, "create_bind_group");
        wgpu::custom::DispatchBindGroup::custom(BindGroup { obj: self.handle(h, gbr_bind_group_destroy) })
    }

    fn create_pipeline_layout(&self, _desc: &wgpu::PipelineLayoutDescriptor<'_>) -> wgpu::custom::DispatchPipelineLayout {
        wgpu::custom::DispatchPipelineLayout::custom(PipelineLayout)
    }

    fn create_render_pipeline(&self, desc: &wgpu::RenderPipelineDescriptor<'_>) -> wgpu::custom::DispatchRenderPipeline {
        let mut d = gbr_render_pipeline_desc::default();
        d.vertex_module = desc.vertex.module.inner.as_custom::<ShaderModule>().unwrap().obj.handle;
        d.vertex_entry_point = entry_point_name(desc.vertex.entry_point);
        assert!(desc.vertex.buffers.len() <= GBR_MAX_VERTEX_BUFFERS, "too many vertex buffers");
        d.vertex_buffer_count = desc.vertex.buffers.len() as u32;
        for (b, out) in desc.vertex.buffers.iter().zip(d.vertex_buffers.iter_mut()) {
            out.array_stride = b.array_stride;
            out.step_mode = match b.step_mode {
                wgpu::VertexStepMode::Vertex => 0,
                wgpu::VertexStepMode::Instance => 1,
            };
            out.attribute_count = b.attributes.len() as u32;
            for (a, o) in b.attributes.iter().zip(out.attributes.iter_mut()) {
                *o = gbr_vertex_attribute { format: vertex_format(a.format), shader_location: a.shader_location, offset: a.offset };
            }
        }
        let p = &desc.primitive;
        d.primitive = gbr_primitive_state {
            topology: topology(p.topology),
            strip_index_format: index_format(p.strip_index_format),
            front_face: match p.front_face {
                wgpu::FrontFace::Ccw => 0,
                wgpu::FrontFace::Cw => 1,
            },
            cull_mode: match p.cull_mode {
                None => 0,
                Some(wgpu::Face::Front) => 1,
                Some(wgpu::Face::Back) => 2,
            },
            polygon_mode: match p.polygon_mode {
                wgpu::PolygonMode::Fill => 0,
                wgpu::PolygonMode::Line => 1,
                wgpu::PolygonMode::Point => 2,
            },
            unclipped_depth: p.unclipped_depth as u32,
        };
        if let Some(ds) = &desc.depth_stencil {
            d.has_depth_stencil = 1;
            d.depth_stencil = gbr_depth_stencil_state {
                format: texture_format(ds.format),
                depth_write_enabled: ds.depth_write_enabled.unwrap_or(false) as u32,
                depth_compare: compare(ds.depth_compare),
                _pad: 0,
            };
        }
        d.multisample_count = desc.multisample.count;
        // PipelineCompilationOptions::constants of both stages (shader.rs:52-74)
        let keep_keys: Vec<CString>;
        let mut vconsts = Vec::new();
        let mut fconsts = Vec::new();
        {
            let mut keys = Vec::new();
            for (k, _) in desc.vertex.compilation_options.constants.iter() {
                keys.push(CString::new(*k).unwrap());
            }
            if let Some(f) = &desc.fragment {
                for (k, _) in f.compilation_options.constants.iter() {
                    keys.push(CString::new(*k).unwrap());
                }
            }
            keep_keys = keys;
            let mut it = keep_keys.iter();
            for (_, v) in desc.vertex.compilation_options.constants.iter() {
                vconsts.push(gbr_pipeline_constant { key: it.next().unwrap().as_ptr(), value: *v });
            }
            if let Some(f) = &desc.fragment {
                for (_, v) in f.compilation_options.constants.iter() {
                    fconsts.push(gbr_pipeline_constant { key: it.next().unwrap().as_ptr(), value: *v });
                }
            }
        }
        d.vertex_constants = vconsts.as_ptr();
        d.vertex_constant_count = vconsts.len() as u32;
        if let Some(f) = &desc.fragment {
            d.has_fragment = 1;
            d.fragment_module = f.module.inner.as_custom::<ShaderModule>().unwrap().obj.handle;
            d.fragment_entry_point = entry_point_name(f.entry_point);
            d.fragment_constants = fconsts.as_ptr();
            d.fragment_constant_count = fconsts.len() as u32;
            assert!(f.targets.len() <= GBR_MAX_COLOR_TARGETS, "too many colour targets");
            d.color_target_count = f.targets.len() as u32;
            for (t, out) in f.targets.iter().zip(d.color_targets.iter_mut()) {
                if let Some(t) = t {
                    out.format = texture_format(t.format);
                    out.write_mask = t.write_mask.bits();
                    if let Some(b) = &t.blend {
                        out.has_blend = 1;
                        out.color = blend_component(&b.color);
                        out.alpha = blend_component(&b.alpha);
                    }
                }
            }
        }
        let mut h = 0u64;
        check(unsafe { gbr_render_pipeline_create(self.dev.0, &d, &mut h) }, "create_render_pipeline");
        drop(keep_keys);
        wgpu::custom::DispatchRenderPipeline::custom(RenderPipeline { obj: self.handle(h, gbr_render_pipeline_destroy) })
    }

    fn create_mesh_pipeline(&self, _desc: &wgpu::MeshPipelineDescriptor<'_>) -> wgpu::custom::DispatchRenderPipeline {
        unimplemented!("mesh pipelines")
    }

    fn create_compute_pipeline(&self, _desc: &wgpu::ComputePipelineDescriptor<'_>) -> wgpu::custom::DispatchComputePipeline {
        unimplemented!("compute pipelines")
    }

    unsafe fn create_pipeline_cache(&self, _desc: &wgpu::PipelineCacheDescriptor<'_>) -> wgpu::custom::DispatchPipelineCache {
        unimplemented!("pipeline caches")
    }

    fn create_buffer(&self, desc: &wgpu::BufferDescriptor<'_>) -> wgpu::custom::DispatchBuffer {
        let mut h = 0u64;
        check(unsafe { gbr_buffer_create(self.dev.0, desc.size, desc.usage.bits(), &mut h) }, "create_buffer");
        let mapping = if desc.mapped_at_creation { Some((wgpu::MapMode::Write, vec![0u8; desc.size as usize])) } else { None };
        wgpu::custom::DispatchBuffer::custom(Buffer { obj: self.handle(h, gbr_buffer_destroy), size: desc.size, mapping: Mutex::new(mapping) })
    }

    fn create_texture(&self, desc: &wgpu::TextureDescriptor<'_>) -> wgpu::custom::DispatchTexture {
        let d = gbr_texture_desc {
            size: gbr_extent3d { width: desc.size.width, height: desc.size.height, depth_or_array_layers: desc.size.depth_or_array_layers },
            mip_level_count: desc.mip_level_count,
            sample_count: desc.sample_count,
            dimension: 2,
            format: texture_format(desc.format),
            usage: desc.usage.bits(),
            _pad: 0,
        };
        let mut h = 0u64;
        check(unsafe { gbr_texture_create(self.dev.0, &d, &mut h) }, "create_texture");
        wgpu::custom::DispatchTexture::custom(Texture { obj: Arc::new(self.handle(h, gbr_texture_destroy)), desc: d })
    }

    fn create_external_texture(&self, _desc: &wgpu::ExternalTextureDescriptor<'_>, _planes: &[&wgpu::TextureView])
        -> wgpu::custom::DispatchExternalTexture {
        unimplemented!("external textures")
    }

    fn create_blas(&self, _desc: &wgpu::CreateBlasDescriptor<'_>, _sizes: wgpu::BlasGeometrySizeDescriptors)
        -> (Option<u64>, wgpu::custom::DispatchBlas) {
        unimplemented!("acceleration structures")
    }

    fn create_tlas(&self, _desc: &wgpu::CreateTlasDescriptor<'_>) -> wgpu::custom::DispatchTlas {
        unimplemented!("acceleration structures")
    }

    fn create_sampler(&self, desc: &wgpu::SamplerDescriptor<'_>) -> wgpu::custom::DispatchSampler {
        let d = gbr_sampler_desc {
            address_mode_u: address_mode(desc.address_mode_u),
            address_mode_v: address_mode(desc.address_mode_v),
            address_mode_w: address_mode(desc.address_mode_w),
            mag_filter: filter(desc.mag_filter),
            min_filter: filter(desc.min_filter),
            mipmap_filter: mipmap_filter(desc.mipmap_filter),
            lod_min_clamp: desc.lod_min_clamp,
            lod_max_clamp: desc.lod_max_clamp,
            compare: compare(desc.compare),
            anisotropy_clamp: desc.anisotropy_clamp as u32,
        };
        let mut h = 0u64;
        check(unsafe { gbr_sampler_create(self.dev.0, &d, &mut h) }, "create_sampler");
        wgpu::custom::DispatchSampler::custom(Sampler { obj: self.handle(h, gbr_sampler_destroy) })
    }

    fn create_query_set(&self, _desc: &wgpu::QuerySetDescriptor<'_>) -> wgpu::custom::DispatchQuerySet {
        unimplemented!("query sets")
    }

    fn create_command_encoder(&self, _desc: &wgpu::CommandEncoderDescriptor<'_>) -> wgpu::custom::DispatchCommandEncoder {
        wgpu::custom::DispatchCommandEncoder::custom(CommandEncoder { stream: Arc::new(Mutex::new(Vec::new())) })
    }

    fn create_render_bundle_encoder(&self, _desc: &wgpu::RenderBundleEncoderDescriptor<'_>)
        -> wgpu::custom::DispatchRenderBundleEncoder {
        unimplemented!("render bundles")
    }

    fn set_device_lost_callback(&self, _callback: wgpu::custom::BoxDeviceLostCallback) {}

    fn on_uncaptured_error(&self, _handler: Arc<dyn wgpu::UncapturedErrorHandler>) {}

    fn push_error_scope(&self, _filter: wgpu::ErrorFilter) -> u32 {
        0
    }

    fn pop_error_scope(&self, _index: u32) -> Pin<Box<dyn wgpu::custom::PopErrorScopeFuture>> {
        Box::pin(async move { None })
    }

    unsafe fn start_graphics_debugger_capture(&self) {}

    unsafe fn stop_graphics_debugger_capture(&self) {}

    fn poll(&self, poll_type: wgpu::wgt::PollType<u64>) -> Result<wgpu::PollStatus, wgpu::PollError> {
        // DeviceInterface::poll (device.rs:237-295) over gbr_device_poll
        let (wait, has_index, index, timeout) = match poll_type {
            wgpu::wgt::PollType::Wait { submission_index, timeout } => (
                1u32,
                submission_index.is_some() as u32,
                submission_index.unwrap_or(0),
                timeout.map_or(u64::MAX, |t| t.as_nanos().min(u64::MAX as u128 - 1) as u64),
            ),
            wgpu::wgt::PollType::Poll => (0, 0, 0, 0),
        };
        let mut out = 0u32;
        match unsafe { gbr_device_poll(self.dev.0, wait, has_index, index, timeout, &mut out) } {
            GBR_OK => Ok(match out {
                GBR_POLL_WAIT_SUCCEEDED => wgpu::PollStatus::WaitSucceeded,
                GBR_POLL_QUEUE_EMPTY => wgpu::PollStatus::QueueEmpty,
                _ => wgpu::PollStatus::Poll,
            }),
            GBR_ERR_TIMEOUT => Err(wgpu::PollError::Timeout),
            st => panic!("poll: status {st}: {}", last_error()),
        }
    }

    fn get_internal_counters(&self) -> wgpu::InternalCounters {
        wgpu::InternalCounters::default()
    }

    fn generate_allocator_report(&self) -> Option<wgpu::AllocatorReport> {
        None
    }

    fn destroy(&self) {}
}

// ------------------------------------------------------------------------------------ queue

#[derive(Debug)]
pub struct Queue {
    dev: Arc<DeviceHandle>,
}

impl wgpu::custom::QueueInterface for Queue {
    fn write_buffer(&self, buffer: &wgpu::custom::DispatchBuffer, offset: wgpu::BufferAddress, data: &[u8]) {
        let b = buffer.as_custom::<Buffer>().unwrap();
        check(unsafe { gbr_queue_write_buffer(self.dev.0, b.obj.handle, offset, data.as_ptr() as *const c_void, data.len() as u64) },
              "write_buffer");
    }

    fn create_staging_buffer(&self, _size: wgpu::BufferSize) -> Option<wgpu::custom::DispatchQueueWriteBuffer> {
        unimplemented!("staging buffers")
    }

    fn validate_write_buffer(&self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress,
                             _size: wgpu::BufferSize) -> Option<()> {
        Some(())
    }

    fn write_staging_buffer(&self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress,
                            _staging: &wgpu::custom::DispatchQueueWriteBuffer) {
        unimplemented!("staging buffers")
    }

    fn write_texture(&self, texture: wgpu::TexelCopyTextureInfo<'_>, data: &[u8], layout: wgpu::TexelCopyBufferLayout,
                     size: wgpu::Extent3d) {
        let t = texture.texture.inner.as_custom::<Texture>().unwrap();
        let l = gbr_texel_copy_buffer_layout {
            offset: layout.offset,
            bytes_per_row: layout.bytes_per_row.unwrap_or(0),
            rows_per_image: layout.rows_per_image.unwrap_or(0),
        };
        let e = gbr_extent3d { width: size.width, height: size.height, depth_or_array_layers: size.depth_or_array_layers };
        check(unsafe {
            gbr_queue_write_texture(self.dev.0, t.obj.handle, texture.mip_level, data.as_ptr() as *const c_void,
                                    data.len() as u64, &l, e)
        }, "write_texture");
    }

    fn submit(&self, command_buffers: &mut dyn Iterator<Item = wgpu::custom::DispatchCommandBuffer>) -> u64 {
        // one stream for all command buffers of the submission (device.rs:436-462)
        let mut stream = Vec::new();
        for cb in command_buffers {
            stream.extend_from_slice(&cb.as_custom::<CommandBuffer>().unwrap().take());
        }
        let mut index = 0u64;
        check(unsafe { gbr_queue_submit(self.dev.0, stream.as_ptr() as *const c_void, stream.len() as u64, &mut index) },
              "submit");
        index
    }

    fn get_timestamp_period(&self) -> f32 {
        1.0
    }

    fn on_submitted_work_done(&self, callback: wgpu::custom::BoxSubmittedWorkDoneCallback) {
        let mut out = 0u32;
        unsafe { gbr_device_poll(self.dev.0, 1, 0, 0, u64::MAX, &mut out) };
        callback();
    }

    fn compact_blas(&self, _blas: &wgpu::custom::DispatchBlas) -> (Option<u64>, wgpu::custom::DispatchBlas) {
        unimplemented!("acceleration structures")
    }
}

// ------------------------------------------------------------------------------------ encoders

#[derive(Debug, Clone)]
pub struct CommandEncoder {
    stream: Arc<Mutex<Vec<u8>>>,
}

#[derive(Debug, Default)]
pub struct CommandBuffer {
    stream: Mutex<Vec<u8>>,
}

impl CommandBuffer {
    /// consumed at submit (command.rs:179-183)
    fn take(&self) -> Vec<u8> {
        std::mem::take(&mut *self.stream.lock())
    }
}
impl wgpu::custom::CommandBufferInterface for CommandBuffer {}

fn texel_info(t: &wgpu::TexelCopyTextureInfo<'_>) -> gbr_texel_copy_texture_info {
    gbr_texel_copy_texture_info {
        texture: t.texture.inner.as_custom::<Texture>().unwrap().obj.handle,
        mip_level: t.mip_level,
        origin_x: t.origin.x,
        origin_y: t.origin.y,
        origin_z: t.origin.z,
    }
}

fn extent(e: wgpu::Extent3d) -> gbr_extent3d {
    gbr_extent3d { width: e.width, height: e.height, depth_or_array_layers: e.depth_or_array_layers }
}

impl wgpu::custom::CommandEncoderInterface for CommandEncoder {
    // The copies and clears are todo!() in the reference (command.rs:37-115); the library runs
    // them under the extension profile and rejects them under the parity profile at submit.
    fn copy_buffer_to_buffer(&self, source: &wgpu::custom::DispatchBuffer, source_offset: wgpu::BufferAddress,
                             destination: &wgpu::custom::DispatchBuffer, destination_offset: wgpu::BufferAddress,
                             copy_size: Option<wgpu::BufferAddress>) {
        let c = gbr_cmd_copy_buffer_to_buffer {
            source: source.as_custom::<Buffer>().unwrap().obj.handle,
            source_offset,
            destination: destination.as_custom::<Buffer>().unwrap().obj.handle,
            destination_offset,
            size: copy_size.unwrap_or(u64::MAX),
        };
        push_record(&mut self.stream.lock(), GBR_OP_COPY_BUFFER_TO_BUFFER, Some(&c));
    }

    fn copy_buffer_to_texture(&self, source: wgpu::TexelCopyBufferInfo<'_>, destination: wgpu::TexelCopyTextureInfo<'_>,
                              copy_size: wgpu::Extent3d) {
        let c = gbr_cmd_copy_buffer_texture {
            buffer: source.buffer.inner.as_custom::<Buffer>().unwrap().obj.handle,
            layout: gbr_texel_copy_buffer_layout {
                offset: source.layout.offset,
                bytes_per_row: source.layout.bytes_per_row.unwrap_or(0),
                rows_per_image: source.layout.rows_per_image.unwrap_or(0),
            },
            texture: texel_info(&destination),
            size: extent(copy_size),
            _pad: 0,
        };
        push_record(&mut self.stream.lock(), GBR_OP_COPY_BUFFER_TO_TEXTURE, Some(&c));
    }

    fn copy_texture_to_buffer(&self, source: wgpu::TexelCopyTextureInfo<'_>, destination: wgpu::TexelCopyBufferInfo<'_>,
                              copy_size: wgpu::Extent3d) {
        let c = gbr_cmd_copy_buffer_texture {
            buffer: destination.buffer.inner.as_custom::<Buffer>().unwrap().obj.handle,
            layout: gbr_texel_copy_buffer_layout {
                offset: destination.layout.offset,
                bytes_per_row: destination.layout.bytes_per_row.unwrap_or(0),
                rows_per_image: destination.layout.rows_per_image.unwrap_or(0),
            },
            texture: texel_info(&source),
            size: extent(copy_size),
            _pad: 0,
        };
        push_record(&mut self.stream.lock(), GBR_OP_COPY_TEXTURE_TO_BUFFER, Some(&c));
    }

    fn copy_texture_to_texture(&self, source: wgpu::TexelCopyTextureInfo<'_>, destination: wgpu::TexelCopyTextureInfo<'_>,
                               copy_size: wgpu::Extent3d) {
        let c = gbr_cmd_copy_texture_to_texture { source: texel_info(&source), destination: texel_info(&destination),
                                                  size: extent(copy_size), _pad: 0 };
        push_record(&mut self.stream.lock(), GBR_OP_COPY_TEXTURE_TO_TEXTURE, Some(&c));
    }

    fn begin_compute_pass(&self, _desc: &wgpu::ComputePassDescriptor<'_>) -> wgpu::custom::DispatchComputePass {
        unimplemented!("compute passes")
    }

    fn begin_render_pass(&self, desc: &wgpu::RenderPassDescriptor<'_>) -> wgpu::custom::DispatchRenderPass {
        let mut b = gbr_cmd_begin_render_pass::default();
        assert!(desc.color_attachments.len() <= GBR_MAX_COLOR_TARGETS, "too many colour attachments");
        b.color_attachment_count = desc.color_attachments.len() as u32;
        for (ca, out) in desc.color_attachments.iter().zip(b.color_attachments.iter_mut()) {
            let Some(ca) = ca else { continue };
            let view = ca.view.inner.as_custom::<TextureView>().unwrap();
            out.view = view.texture.handle;
            out.depth_slice = ca.depth_slice.unwrap_or(view.base_layer);
            out.store_op = match ca.ops.store {
                wgpu::StoreOp::Store => GBR_STORE_OP_STORE,
                wgpu::StoreOp::Discard => GBR_STORE_OP_DISCARD,
            };
            match ca.ops.load {
                wgpu::LoadOp::Clear(c) => {
                    out.load_op = GBR_LOAD_OP_CLEAR;
                    out.clear_value = [c.r, c.g, c.b, c.a];
                }
                _ => out.load_op = GBR_LOAD_OP_LOAD,
            }
        }
        if let Some(ds) = &desc.depth_stencil_attachment {
            b.has_depth_attachment = 1;
            b.depth_attachment.view = ds.view.inner.as_custom::<TextureView>().unwrap().texture.handle;
            if let Some(ops) = &ds.depth_ops {
                b.depth_attachment.has_depth_ops = 1;
                b.depth_attachment.depth_store_op = match ops.store {
                    wgpu::StoreOp::Store => GBR_STORE_OP_STORE,
                    wgpu::StoreOp::Discard => GBR_STORE_OP_DISCARD,
                };
                match ops.load {
                    wgpu::LoadOp::Clear(v) => {
                        b.depth_attachment.depth_load_op = GBR_LOAD_OP_CLEAR;
                        b.depth_attachment.depth_clear_value = v;
                    }
                    _ => b.depth_attachment.depth_load_op = GBR_LOAD_OP_LOAD,
                }
            }
        }
        let mut commands = Vec::new();
        push_record(&mut commands, GBR_OP_BEGIN_RENDER_PASS, Some(&b));
        wgpu::custom::DispatchRenderPass::custom(RenderPass { encoder: self.clone(), commands: Some(commands) })
    }

    fn finish(&mut self) -> wgpu::custom::DispatchCommandBuffer {
        let stream = std::mem::take(&mut *self.stream.lock());
        wgpu::custom::DispatchCommandBuffer::custom(CommandBuffer { stream: Mutex::new(stream) })
    }

    fn clear_texture(&self, texture: &wgpu::custom::DispatchTexture, range: &wgpu::ImageSubresourceRange) {
        let c = gbr_cmd_clear_texture {
            texture: texture.as_custom::<Texture>().unwrap().obj.handle,
            base_mip_level: range.base_mip_level,
            mip_level_count: range.mip_level_count.unwrap_or(0),
            base_array_layer: range.base_array_layer,
            array_layer_count: range.array_layer_count.unwrap_or(0),
        };
        push_record(&mut self.stream.lock(), GBR_OP_CLEAR_TEXTURE, Some(&c));
    }

    fn clear_buffer(&self, buffer: &wgpu::custom::DispatchBuffer, offset: wgpu::BufferAddress, size: Option<wgpu::BufferAddress>) {
        let c = gbr_cmd_clear_buffer { buffer: buffer.as_custom::<Buffer>().unwrap().obj.handle, offset, size: size.unwrap_or(u64::MAX) };
        push_record(&mut self.stream.lock(), GBR_OP_CLEAR_BUFFER, Some(&c));
    }

    fn insert_debug_marker(&self, _label: &str) {}
    fn push_debug_group(&self, _label: &str) {}
    fn pop_debug_group(&self) {}

    fn write_timestamp(&self, _query_set: &wgpu::custom::DispatchQuerySet, _query_index: u32) {
        unimplemented!("timestamp queries")
    }

    fn resolve_query_set(&self, _query_set: &wgpu::custom::DispatchQuerySet, _first_query: u32, _query_count: u32,
                         _destination: &wgpu::custom::DispatchBuffer, _destination_offset: wgpu::BufferAddress) {
        unimplemented!("queries")
    }

    fn mark_acceleration_structures_built<'a>(&self, _blas: &mut dyn Iterator<Item = &'a wgpu::Blas>,
                                              _tlas: &mut dyn Iterator<Item = &'a wgpu::Tlas>) {
        unimplemented!("acceleration structures")
    }

    fn build_acceleration_structures<'a>(&self, _blas: &mut dyn Iterator<Item = &'a wgpu::BlasBuildEntry<'a>>,
                                         _tlas: &mut dyn Iterator<Item = &'a wgpu::Tlas>) {
        unimplemented!("acceleration structures")
    }

    fn transition_resources<'a>(
        &mut self,
        _buffer_transitions: &mut dyn Iterator<Item = wgpu::wgt::BufferTransition<&'a wgpu::custom::DispatchBuffer>>,
        _texture_transitions: &mut dyn Iterator<Item = wgpu::wgt::TextureTransition<&'a wgpu::custom::DispatchTexture>>,
    ) {
        // the library orders every command on one stream: nothing to transition
    }
}

/// A render pass being recorded: its records go to the encoder's stream at `end`
/// (render_pass/mod.rs:300-322).
#[derive(Debug)]
pub struct RenderPass {
    encoder: CommandEncoder,
    commands: Option<Vec<u8>>,
}

impl RenderPass {
    fn push<T: Copy>(&mut self, opcode: u32, payload: &T) {
        push_record(self.commands.as_mut().expect("render pass already ended"), opcode, Some(payload));
    }
}

impl wgpu::custom::RenderPassInterface for RenderPass {
    fn set_pipeline(&mut self, pipeline: &wgpu::custom::DispatchRenderPipeline) {
        let p = gbr_cmd_set_pipeline { pipeline: pipeline.as_custom::<RenderPipeline>().unwrap().obj.handle };
        self.push(GBR_OP_SET_PIPELINE, &p);
    }

    fn set_bind_group(&mut self, index: u32, bind_group: Option<&wgpu::custom::DispatchBindGroup>, offsets: &[wgpu::DynamicOffset]) {
        let p = gbr_cmd_set_bind_group {
            index,
            dynamic_offset_count: offsets.len() as u32,
            bind_group: bind_group.map_or(0, |g| g.as_custom::<BindGroup>().unwrap().obj.handle),
        };
        self.push(GBR_OP_SET_BIND_GROUP, &p);
    }

    fn set_index_buffer(&mut self, buffer: &wgpu::custom::DispatchBuffer, index_format: wgpu::IndexFormat,
                        offset: wgpu::BufferAddress, size: Option<wgpu::BufferSize>) {
        let p = gbr_cmd_set_index_buffer {
            buffer: buffer.as_custom::<Buffer>().unwrap().obj.handle,
            index_format: crate::index_format(Some(index_format)),
            _pad: 0,
            offset,
            size: size.map_or(0, |s| s.get()),
        };
        self.push(GBR_OP_SET_INDEX_BUFFER, &p);
    }

    fn set_vertex_buffer(&mut self, slot: u32, buffer: &wgpu::custom::DispatchBuffer, offset: wgpu::BufferAddress,
                         size: Option<wgpu::BufferSize>) {
        let p = gbr_cmd_set_vertex_buffer {
            slot,
            _pad: 0,
            buffer: buffer.as_custom::<Buffer>().unwrap().obj.handle,
            offset,
            size: size.map_or(0, |s| s.get()),
        };
        self.push(GBR_OP_SET_VERTEX_BUFFER, &p);
    }

    fn set_immediates(&mut self, _offset: u32, _data: &[u8]) {
        unimplemented!("immediates")
    }

    fn set_blend_constant(&mut self, color: wgpu::Color) {
        self.push(GBR_OP_SET_BLEND_CONSTANT, &gbr_cmd_set_blend_constant { color: [color.r, color.g, color.b, color.a] });
    }

    fn set_scissor_rect(&mut self, x: u32, y: u32, width: u32, height: u32) {
        self.push(GBR_OP_SET_SCISSOR_RECT, &gbr_cmd_set_scissor_rect { x, y, width, height });
    }

    fn set_viewport(&mut self, x: f32, y: f32, width: f32, height: f32, min_depth: f32, max_depth: f32) {
        self.push(GBR_OP_SET_VIEWPORT, &gbr_cmd_set_viewport { x, y, width, height, min_depth, max_depth });
    }

    fn set_stencil_reference(&mut self, reference: u32) {
        self.push(GBR_OP_SET_STENCIL_REFERENCE, &[reference, 0u32]);
    }

    fn draw(&mut self, vertices: Range<u32>, instances: Range<u32>) {
        self.push(GBR_OP_DRAW, &gbr_cmd_draw { vertex_start: vertices.start, vertex_end: vertices.end,
                                              instance_start: instances.start, instance_end: instances.end });
    }

    fn draw_indexed(&mut self, indices: Range<u32>, base_vertex: i32, instances: Range<u32>) {
        self.push(GBR_OP_DRAW_INDEXED, &gbr_cmd_draw_indexed { index_start: indices.start, index_end: indices.end,
                                                               base_vertex, instance_start: instances.start,
                                                               instance_end: instances.end, _pad: 0 });
    }

    fn draw_mesh_tasks(&mut self, _x: u32, _y: u32, _z: u32) {
        unimplemented!("mesh shading")
    }

    fn draw_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress) {
        unimplemented!("indirect draws")
    }

    fn draw_indexed_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress) {
        unimplemented!("indirect draws")
    }

    fn draw_mesh_tasks_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress) {
        unimplemented!("mesh shading")
    }

    fn multi_draw_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress, _count: u32) {
        unimplemented!("indirect draws")
    }

    fn multi_draw_indexed_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress, _count: u32) {
        unimplemented!("indirect draws")
    }

    fn multi_draw_indirect_count(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress,
                                 _count_buffer: &wgpu::custom::DispatchBuffer, _count_offset: wgpu::BufferAddress,
                                 _max_count: u32) {
        unimplemented!("indirect draws")
    }

    fn multi_draw_mesh_tasks_indirect(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress,
                                      _count: u32) {
        unimplemented!("mesh shading")
    }

    fn multi_draw_indexed_indirect_count(&mut self, _buffer: &wgpu::custom::DispatchBuffer, _offset: wgpu::BufferAddress,
                                         _count_buffer: &wgpu::custom::DispatchBuffer,
                                         _count_offset: wgpu::BufferAddress, _max_count: u32) {
        unimplemented!("indirect draws")
    }

    fn multi_draw_mesh_tasks_indirect_count(&mut self, _buffer: &wgpu::custom::DispatchBuffer,
                                            _offset: wgpu::BufferAddress, _count_buffer: &wgpu::custom::DispatchBuffer,
                                            _count_offset: wgpu::BufferAddress, _max_count: u32) {
        unimplemented!("mesh shading")
    }

    fn insert_debug_marker(&mut self, _label: &str) {}
    fn push_debug_group(&mut self, _label: &str) {}
    fn pop_debug_group(&mut self) {}

    fn write_timestamp(&mut self, _query_set: &wgpu::custom::DispatchQuerySet, _query_index: u32) {
        unimplemented!("timestamp queries")
    }

    fn begin_occlusion_query(&mut self, _query_index: u32) {
        unimplemented!("occlusion queries")
    }

    fn end_occlusion_query(&mut self) {
        unimplemented!("occlusion queries")
    }

    fn begin_pipeline_statistics_query(&mut self, _query_set: &wgpu::custom::DispatchQuerySet, _query_index: u32) {
        unimplemented!("pipeline statistics")
    }

    fn end_pipeline_statistics_query(&mut self) {
        unimplemented!("pipeline statistics")
    }

    fn execute_bundles(&mut self, _bundles: &mut dyn Iterator<Item = &wgpu::custom::DispatchRenderBundle>) {
        unimplemented!("render bundles")
    }

    fn end(&mut self) {
        if let Some(mut commands) = self.commands.take() {
            push_record::<u8>(&mut commands, GBR_OP_END_RENDER_PASS, None);
            self.encoder.stream.lock().extend_from_slice(&commands);
        }
    }
}

impl Drop for RenderPass {
    fn drop(&mut self) {
        wgpu::custom::RenderPassInterface::end(self)
    }
}

// ------------------------------------------------------------------------------------ readback

/// The headless stand-in for wgpu-cpu's `image::rgba_texture_image` (lib.rs:158-173): waits for
/// prior submissions and copies mip 0 of `texture` (tightly packed rows).
pub fn read_texture(device: &wgpu::Device, texture: &wgpu::Texture) -> Vec<u8> {
    let dev = device.as_custom::<Device>().expect("not a wgpu-gb300 device");
    let t = texture.as_custom::<Texture>().expect("not a wgpu-gb300 texture");
    let bpp: u64 = match t.desc.format {
        1 => 1,
        2 => 2,
        7 => 8,
        8 => 16,
        _ => 4,
    };
    let n = t.desc.size.width as u64 * t.desc.size.height as u64 * t.desc.size.depth_or_array_layers as u64 * bpp;
    let mut out = vec![0u8; n as usize];
    check(unsafe { gbr_texture_read(dev.dev.0, t.obj.handle, 0, out.as_mut_ptr() as *mut c_void, n) }, "read_texture");
    out
}
