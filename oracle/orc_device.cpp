// TEST INFRASTRUCTURE — the oracle (see orc_core.hpp).  Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline leg load liborc.so, as the checker.
//
// orc_device.cpp — a CPU device behind the same C ABI as the GPU library (include/gbr.h), with
// every symbol prefixed `orc_` instead of `gbr_`.  It restates wgpu-cpu's engine: resources are
// host byte vectors (buffer.rs:22-52, texture.rs:34-43), a submission executes its render
// passes immediately and in order (engine.rs:26-46), and each pass replays its sub-commands
// through the reference's draw loop (render_pass/mod.rs:345-395, render_pass/state.rs:239-593)
// and fragment processing (render_pass/fragment.rs:127-214, 427-489).
//
// Threading: with orc_set_threads(n > 1) a pass is executed by n threads, each owning a band of
// framebuffer rows.  Every thread runs the whole draw loop but emits only fragments of its
// rows, so the per-pixel fragment order — and therefore every output bit — is the same as
// with one thread.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gbr.h"
#include "orc_core.hpp"
#include "orc_programs.hpp"
#include "srgb_tables.h"  // extension-profile sRGB tables, shared with the kernels

#define ORC_API extern "C" __attribute__((visibility("default")))

namespace orc {

static thread_local std::string g_last_error;
static int g_threads = 1;

struct Error {
    gbr_status status;
    std::string msg;
};
[[noreturn]] static void fail(gbr_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error{st, buf};
}

// [offset, offset + size) inside [0, total) with no wrapping sum: the reference's try_into and
// slice bounds (buffer.rs, device.rs:332-344) reject such ranges with a panic.
static inline bool range_fits(uint64_t offset, uint64_t size, uint64_t total) {
    return size <= total && offset <= total - size;
}
// a + b * c + d, or UINT64_MAX when it does not fit in 64 bits
static inline uint64_t span_end(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    uint64_t p, s, r;
    if (__builtin_mul_overflow(b, c, &p) || __builtin_add_overflow(a, p, &s) || __builtin_add_overflow(s, d, &r))
        return UINT64_MAX;
    return r;
}

// ---------------------------------------------------------------- texture formats
// bytes_per_texel (texture.rs:456-505) for the formats this ABI exposes.
static uint32_t bytes_per_texel(uint32_t f) {
    switch (f) {
        case GBR_TEXTURE_FORMAT_R8_UNORM: return 1;
        case GBR_TEXTURE_FORMAT_RG8_UNORM: return 2;
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM:
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB:
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM:
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB:
        case GBR_TEXTURE_FORMAT_DEPTH32_FLOAT: return 4;
        case GBR_TEXTURE_FORMAT_RGBA16_FLOAT: return 8;
        case GBR_TEXTURE_FORMAT_RGBA32_FLOAT: return 16;
        default: return 0;
    }
}

// ---------------------------------------------------------------- objects
struct Object {
    virtual ~Object() {}
};
struct Buffer : Object {
    std::vector<uint8_t> data;
};
struct Texture : Object {
    gbr_texture_desc desc;
    uint32_t bpp;
    uint32_t mips_stored;
    std::vector<std::vector<uint8_t>> mips;  // mip level -> bytes (layer-major, row-major)
    uint32_t mip_w(uint32_t m) const { return std::max(1u, desc.size.width >> m); }
    uint32_t mip_h(uint32_t m) const { return std::max(1u, desc.size.height >> m); }
};
struct TextureView {
    const Texture* tex;
};
struct SamplerState {
    gbr_sampler_desc desc;
};
struct Sampler : Object {
    SamplerState s;
};
struct ShaderModule : Object {
    const Program* prog;
};
struct Pipeline : Object {
    gbr_render_pipeline_desc desc;
    const Program* vs;
    const Program* fs;
    // shader input location -> (buffer index, offset, format)
    struct Loc {
        bool present;
        uint32_t buffer;
        uint64_t offset;
        uint32_t format;
    } loc[16];
};
struct BindGroup : Object {
    gbr_bind_group_desc desc;
};

struct Device {
    uint32_t profile = GBR_PROFILE_PARITY;
    uint32_t raster_rule = GBR_RASTER_RULE_SCANLINE;
    std::mutex mu;
    uint64_t next_handle = 1;
    std::unordered_map<uint64_t, std::unique_ptr<Object>> objects;
    uint64_t next_submission = 0;
    std::unordered_map<uint64_t, gbr_submission_stats> stats;

    template <class T>
    T* get(uint64_t h, const char* what) {
        auto it = objects.find(h);
        if (it == objects.end()) fail(GBR_ERR_INVALID_ARGUMENT, "invalid %s handle %llu", what, (unsigned long long)h);
        T* p = dynamic_cast<T*>(it->second.get());
        if (!p) fail(GBR_ERR_INVALID_ARGUMENT, "handle %llu is not a %s", (unsigned long long)h, what);
        return p;
    }
    uint64_t add(Object* o) {
        uint64_t h = next_handle++;
        objects[h].reset(o);
        return h;
    }
};

static std::mutex g_devices_mu;
static std::unordered_map<uint64_t, std::unique_ptr<Device>> g_devices;
static uint64_t g_next_device = 1;

static Device* get_device(gbr_device d) {
    std::lock_guard<std::mutex> lk(g_devices_mu);
    auto it = g_devices.find(d);
    if (it == g_devices.end()) fail(GBR_ERR_INVALID_ARGUMENT, "invalid device handle");
    return it->second.get();
}

// ---------------------------------------------------------------- sampling
// texel_coordinate (render_pass/binding.rs:150-164)
static uint32_t texel_coordinate(float x, uint32_t mode, uint32_t size) {
    switch (mode) {
        case GBR_ADDRESS_CLAMP_TO_EDGE:
            if (x < 0.0f) x = 0.0f;
            if (x > 1.0f) x = 1.0f;
            break;
        case GBR_ADDRESS_REPEAT: {
            float r = std::fmod(x, 1.0f);
            x = (r < 0.0f) ? r + 1.0f : r;  // f32::rem_euclid(1.0)
            break;
        }
        case GBR_ADDRESS_MIRROR_REPEAT: {
            float r = std::fmod(x, 2.0f);
            r = (r < 0.0f) ? r + 2.0f : r;  // f32::rem_euclid(2.0)
            x = (r <= 1.0f) ? r : 2.0f - r;
            break;
        }
        default: fail(GBR_ERR_UNSUPPORTED, "ClampToBorder is not implemented (binding.rs:160)");
    }
    float scaled = x * (float)(size - 1u);
    return rust_f32_to_u32(std::round(scaled));
}

// TextureReadGuard::get_pixel (texture.rs:170-188): Rgba8Unorm / Rgba8UnormSrgb only.
static V4 get_pixel_rgba8(const Texture* t, uint32_t mip, uint32_t x, uint32_t y) {
    uint32_t w = t->mip_w(mip);
    const uint8_t* p = t->mips[mip].data() + ((size_t)y * w + x) * 4;
    return {(float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f, (float)p[3] / 255.0f};
}


// image_sample (render_pass/binding.rs:93-140).  Nearest, mip 0, layer 0; filters ignored.
static V4 sample_parity(const TextureView* tv, const SamplerState* s, float u, float v) {
    const Texture* t = tv->tex;
    if (t->desc.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM && t->desc.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB)
        fail(GBR_ERR_UNSUPPORTED, "sampling format %u is not implemented (texture.rs:186)", t->desc.format);
    uint32_t x = texel_coordinate(u, s->desc.address_mode_u, t->desc.size.width);
    uint32_t y = texel_coordinate(v, s->desc.address_mode_v, t->desc.size.height);
    return get_pixel_rgba8(t, 0, x, y);
}

// ---------------------------------------------------------------- extension-profile sampling
// The reference has no filtering, mips or sRGB decode; the extension profile follows the WebGPU
// sampling model with these exact steps (restated in the kernels' sampling.cuh):
//   LOD = 0.5 * log2(max(|d(uv)/dx|^2, |d(uv)/dy|^2)) in level-0 texels, clamped to the sampler's
//   [lod_min, lod_max]; LOD <= 0 magnifies (mag filter, level 0); the mip filter picks level
//   ceil(LOD + 0.5) - 1 (nearest) or blends floor(LOD) and the next level (linear); nearest texel
//   floor(u * w), linear taps at u * w - 0.5; integer coordinates wrap per address mode; sRGB
//   texels decode through kSrgbToLinear; lerp(a, b, t) = a + (b - a) * t.

// log2 from IEEE basic operations: r = m * 2^e, m in [sqrt(1/2), sqrt(2)), ln(m) = 2 atanh(s),
// s = (m - 1) / (m + 1), series s + s^3/3 + s^5/5 + s^7/7 (Horner in z = s^2).
static float log2_spec(float r) {
    if (!(r > 0.0f)) return -std::numeric_limits<float>::infinity();
    if (std::isinf(r)) return r;
    uint32_t bits;
    std::memcpy(&bits, &r, 4);
    int e = (int)((bits >> 23) & 0xFFu);
    if (e == 0) {  // subnormal
        float q = r * 0x1p24f;
        std::memcpy(&bits, &q, 4);
        e = (int)((bits >> 23) & 0xFFu) - 24;
    }
    e -= 127;
    uint32_t mb = (bits & 0x7FFFFFu) | 0x3F800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 0x1.6a09e6p+0f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float z = s * s;
    float p = 0x1.249250p-3f;
    p = p * z + 0x1.99999ap-3f;
    p = p * z + 0x1.555556p-2f;
    p = p * z + 1.0f;
    float ln = (2.0f * s) * p;
    return (float)e + ln * 0x1.715476p+0f;
}

static float lod_from_grad(const float g[4], uint32_t w, uint32_t h, float lod_min, float lod_max) {
    float sx = g[0] * (float)w, tx = g[1] * (float)h, sy = g[2] * (float)w, ty = g[3] * (float)h;
    float px2 = sx * sx + tx * tx, py2 = sy * sy + ty * ty;
    float r2 = px2 >= py2 ? px2 : py2;
    float lod = 0.5f * log2_spec(r2);
    if (!(lod >= lod_min)) lod = lod_min;
    if (lod > lod_max) lod = lod_max;
    return lod;
}

static int wrap_texel(int i, int n, uint32_t mode) {
    if (mode == GBR_ADDRESS_REPEAT) {
        int r = i % n;
        return r < 0 ? r + n : r;
    }
    if (mode == GBR_ADDRESS_MIRROR_REPEAT) {
        int p = 2 * n;
        int t = i % p;
        if (t < 0) t += p;
        return t < n ? t : p - 1 - t;
    }
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

static float texel_space(float u, uint32_t size, float bias) {
    float x = u * (float)size - bias;
    if (!(x >= -16777216.0f)) x = std::isnan(x) ? 0.0f : -16777216.0f;
    if (x > 16777216.0f) x = 16777216.0f;
    return x;
}

static V4 decode_texel(const uint8_t* p, bool srgb) {
    if (srgb) return {kSrgbToLinear[p[0]], kSrgbToLinear[p[1]], kSrgbToLinear[p[2]], (float)p[3] / 255.0f};
    return {(float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f, (float)p[3] / 255.0f};
}
static V4 lerp4(V4 a, V4 b, float t) {
    return {a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t};
}

static V4 sample_level(const Texture* t, const gbr_sampler_desc& s, uint32_t level, bool linear, float u, float v) {
    const bool srgb = t->desc.format == GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB;
    const int w = (int)t->mip_w(level), h = (int)t->mip_h(level);
    const uint8_t* base = t->mips[level].data();
    auto at = [&](int x, int y) { return decode_texel(base + ((size_t)y * w + x) * 4, srgb); };
    if (!linear) {
        int x = wrap_texel((int)std::floor(texel_space(u, (uint32_t)w, 0.0f)), w, s.address_mode_u);
        int y = wrap_texel((int)std::floor(texel_space(v, (uint32_t)h, 0.0f)), h, s.address_mode_v);
        return at(x, y);
    }
    float xs = texel_space(u, (uint32_t)w, 0.5f), ys = texel_space(v, (uint32_t)h, 0.5f);
    float xf = std::floor(xs), yf = std::floor(ys);
    float fx = xs - xf, fy = ys - yf;
    int x0 = wrap_texel((int)xf, w, s.address_mode_u), x1 = wrap_texel((int)xf + 1, w, s.address_mode_u);
    int y0 = wrap_texel((int)yf, h, s.address_mode_v), y1 = wrap_texel((int)yf + 1, h, s.address_mode_v);
    return lerp4(lerp4(at(x0, y0), at(x1, y0), fx), lerp4(at(x0, y1), at(x1, y1), fx), fy);
}

static V4 sample_ext(const TextureView* tv, const SamplerState* ss, float u, float v, const float grad[4]) {
    const Texture* t = tv->tex;
    const gbr_sampler_desc& s = ss->desc;
    if (t->desc.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM && t->desc.format != GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB)
        fail(GBR_ERR_UNSUPPORTED, "sampling format %u is not implemented", t->desc.format);
    if (s.address_mode_u == GBR_ADDRESS_CLAMP_TO_BORDER || s.address_mode_v == GBR_ADDRESS_CLAMP_TO_BORDER)
        fail(GBR_ERR_UNSUPPORTED, "ClampToBorder is todo!() (binding.rs:160)");
    const float lod = lod_from_grad(grad, t->desc.size.width, t->desc.size.height, s.lod_min_clamp, s.lod_max_clamp);
    const uint32_t last = t->mips_stored - 1;
    if (lod <= 0.0f) return sample_level(t, s, 0, s.mag_filter == GBR_FILTER_LINEAR, u, v);
    const bool lin = s.min_filter == GBR_FILTER_LINEAR;
    if (s.mipmap_filter != GBR_FILTER_LINEAR) {
        float lv = std::ceil(lod + 0.5f) - 1.0f;
        uint32_t level = lv >= (float)last ? last : (uint32_t)lv;
        return sample_level(t, s, level, lin, u, v);
    }
    float lc = lod < (float)last ? lod : (float)last;
    float lf = std::floor(lc);
    uint32_t l0 = (uint32_t)lf;
    float f = lc - lf;
    V4 c0 = sample_level(t, s, l0, lin, u, v);
    if (f == 0.0f || l0 >= last) return c0;
    return lerp4(c0, sample_level(t, s, l0 + 1, lin, u, v), f);
}

// `grad` = (du/dx, dv/dx, du/dy, dv/dy) of the sampled coordinate (extension profile only).
static V4 sample_cb(const TextureView* tv, const SamplerState* s, float u, float v, const float grad[4],
                    const void* ctx) {
    if (!tv || !s) fail(GBR_ERR_VALIDATION, "No such binding resource");
    if (*static_cast<const uint32_t*>(ctx) == GBR_PROFILE_EXTENSION) return sample_ext(tv, s, u, v, grad);
    return sample_parity(tv, s, u, v);
}

// ---------------------------------------------------------------- texel writers
// f32_to_u8 (texture.rs:378-381): (v * 255).clamp(0, 255) as u8, i.e. truncation.
static inline uint8_t unorm8_trunc(float v) {
    float s = v * 255.0f;
    if (s < 0.0f) s = 0.0f;
    if (s > 255.0f) s = 255.0f;
    return rust_f32_to_u8(s);
}

// Extension profile, sRGB targets: linear -> unorm8 sRGB = number of encode thresholds <= v
// (round to nearest of the encoded value; NaN and negatives 0, v >= the last threshold 255).
static inline uint8_t linear_to_srgb8(float v) {
    uint32_t k = 0;
    for (uint32_t step = 128; step > 0; step >>= 1)
        if (k + step <= 255u && v >= kSrgbEncodeThreshold[k + step]) k += step;
    return (uint8_t)k;
}
// Extension profile: WebGPU float -> unorm8, clamp then round to nearest even (the alpha of sRGB
// targets).
static inline uint8_t unorm8_round(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.0f) return 255;
    return (uint8_t)std::nearbyint(v * 255.0f);
}

// TexelWriter::from_color (texture.rs:373-411) + put_pixel (texture.rs:213-218).
static void write_color(Texture* t, uint32_t x, uint32_t y, uint32_t slice, V4 c, uint32_t profile) {
    uint32_t w = t->desc.size.width, h = t->desc.size.height;
    uint8_t* p = t->mips[0].data() + (((size_t)slice * h + y) * w + x) * t->bpp;
    switch (t->desc.format) {
        case GBR_TEXTURE_FORMAT_R8_UNORM: p[0] = unorm8_trunc(c.x); break;
        case GBR_TEXTURE_FORMAT_RG8_UNORM:
            p[0] = unorm8_trunc(c.x);
            p[1] = unorm8_trunc(c.y);
            break;
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB:
            if (profile == GBR_PROFILE_EXTENSION) {  // WebGPU: linear -> sRGB on write
                p[0] = linear_to_srgb8(c.x);
                p[1] = linear_to_srgb8(c.y);
                p[2] = linear_to_srgb8(c.z);
                p[3] = unorm8_round(c.w);
                break;
            }
            [[fallthrough]];
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM:
            p[0] = unorm8_trunc(c.x);
            p[1] = unorm8_trunc(c.y);
            p[2] = unorm8_trunc(c.z);
            p[3] = unorm8_trunc(c.w);
            break;
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB:
            if (profile == GBR_PROFILE_EXTENSION) {
                p[0] = linear_to_srgb8(c.z);
                p[1] = linear_to_srgb8(c.y);
                p[2] = linear_to_srgb8(c.x);
                p[3] = unorm8_round(c.w);
                break;
            }
            [[fallthrough]];
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM:
            p[0] = unorm8_trunc(c.z);
            p[1] = unorm8_trunc(c.y);
            p[2] = unorm8_trunc(c.x);
            p[3] = unorm8_trunc(c.w);
            break;
        case GBR_TEXTURE_FORMAT_RGBA16_FLOAT:
            if (profile != GBR_PROFILE_EXTENSION)
                fail(GBR_ERR_UNSUPPORTED, "Unsupported texture format: Rgba16Float (texture.rs:407)");
            {
                uint16_t hv[4] = {f32_to_f16_rne(c.x), f32_to_f16_rne(c.y), f32_to_f16_rne(c.z), f32_to_f16_rne(c.w)};
                std::memcpy(p, hv, 8);
            }
            break;
        case GBR_TEXTURE_FORMAT_RGBA32_FLOAT:
            if (profile != GBR_PROFILE_EXTENSION)
                fail(GBR_ERR_UNSUPPORTED, "Unsupported texture format: Rgba32Float (texture.rs:407)");
            {
                float fv[4] = {c.x, c.y, c.z, c.w};
                std::memcpy(p, fv, 16);
            }
            break;
        default: fail(GBR_ERR_UNSUPPORTED, "Unsupported colour target format %u", t->desc.format);
    }
}

// Decoded read of a colour target texel (extension-profile blending only; sRGB targets decode).
static V4 read_color(const Texture* t, uint32_t x, uint32_t y, uint32_t slice) {
    uint32_t w = t->desc.size.width, h = t->desc.size.height;
    const uint8_t* p = t->mips[0].data() + (((size_t)slice * h + y) * w + x) * t->bpp;
    switch (t->desc.format) {
        case GBR_TEXTURE_FORMAT_RGBA16_FLOAT: {
            uint16_t hv[4];
            std::memcpy(hv, p, 8);
            return {f16_to_f32(hv[0]), f16_to_f32(hv[1]), f16_to_f32(hv[2]), f16_to_f32(hv[3])};
        }
        case GBR_TEXTURE_FORMAT_RGBA32_FLOAT: {
            float fv[4];
            std::memcpy(fv, p, 16);
            return {fv[0], fv[1], fv[2], fv[3]};
        }
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM:
            return {p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f};
        case GBR_TEXTURE_FORMAT_RGBA8_UNORM_SRGB:
            return {kSrgbToLinear[p[0]], kSrgbToLinear[p[1]], kSrgbToLinear[p[2]], p[3] / 255.0f};
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM:
            return {p[2] / 255.0f, p[1] / 255.0f, p[0] / 255.0f, p[3] / 255.0f};
        case GBR_TEXTURE_FORMAT_BGRA8_UNORM_SRGB:
            return {kSrgbToLinear[p[2]], kSrgbToLinear[p[1]], kSrgbToLinear[p[0]], p[3] / 255.0f};
        default: fail(GBR_ERR_UNSUPPORTED, "blend: unsupported target format %u", t->desc.format);
    }
}

// WebGPU blend factor (extension profile; the reference never reads the blend state).
static float blend_factor(uint32_t f, float src, float src_a, float dst, float dst_a, float konst) {
    switch (f) {
        case GBR_BLEND_ZERO: return 0.0f;
        case GBR_BLEND_ONE: return 1.0f;
        case GBR_BLEND_SRC: return src;
        case GBR_BLEND_ONE_MINUS_SRC: return 1.0f - src;
        case GBR_BLEND_SRC_ALPHA: return src_a;
        case GBR_BLEND_ONE_MINUS_SRC_ALPHA: return 1.0f - src_a;
        case GBR_BLEND_DST: return dst;
        case GBR_BLEND_ONE_MINUS_DST: return 1.0f - dst;
        case GBR_BLEND_DST_ALPHA: return dst_a;
        case GBR_BLEND_ONE_MINUS_DST_ALPHA: return 1.0f - dst_a;
        case GBR_BLEND_CONSTANT: return konst;
        case GBR_BLEND_ONE_MINUS_CONSTANT: return 1.0f - konst;
        default: fail(GBR_ERR_UNSUPPORTED, "blend factor %u", f);
    }
}
static float blend_op(uint32_t op, float s, float d) {
    switch (op) {
        case GBR_BLEND_OP_ADD: return s + d;
        case GBR_BLEND_OP_SUBTRACT: return s - d;
        case GBR_BLEND_OP_REVERSE_SUBTRACT: return d - s;
        case GBR_BLEND_OP_MIN: return std::fmin(s, d);
        case GBR_BLEND_OP_MAX: return std::fmax(s, d);
        default: fail(GBR_ERR_UNSUPPORTED, "blend op %u", op);
    }
}
// One channel: (src * srcFactor) op (dst * dstFactor); MIN/MAX ignore the factors.
static float blend_channel(const gbr_blend_component& bc, float s, float sa, float d, float da, float k) {
    if (bc.operation == GBR_BLEND_OP_MIN || bc.operation == GBR_BLEND_OP_MAX) return blend_op(bc.operation, s, d);
    float fs = blend_factor(bc.src_factor, s, sa, d, da, k);
    float fd = blend_factor(bc.dst_factor, s, sa, d, da, k);
    return blend_op(bc.operation, s * fs, d * fd);
}
static V4 blend_colors(const gbr_color_target_state& ct, V4 s, V4 d, const double konst[4]) {
    V4 r;
    r.x = blend_channel(ct.color, s.x, s.w, d.x, d.w, (float)konst[0]);
    r.y = blend_channel(ct.color, s.y, s.w, d.y, d.w, (float)konst[1]);
    r.z = blend_channel(ct.color, s.z, s.w, d.z, d.w, (float)konst[2]);
    r.w = blend_channel(ct.alpha, s.w, s.w, d.w, d.w, (float)konst[3]);
    return r;
}

// ---------------------------------------------------------------- pass state
struct BoundSlice {
    const Buffer* buf = nullptr;
    uint64_t offset = 0, size = 0;
};

struct PassState {  // render_pass/state.rs:57-74
    const Pipeline* pipeline = nullptr;
    BoundSlice index;
    uint32_t index_format = 0;
    BoundSlice vb[GBR_MAX_VERTEX_BUFFERS];
    const BindGroup* groups[GBR_MAX_BIND_GROUPS] = {};
    float viewport[6];
    uint32_t scissor[4];
    double blend_constant[4] = {0, 0, 0, 0};
};

struct PassTargets {
    Texture* color[GBR_MAX_COLOR_TARGETS] = {};
    uint32_t color_slice[GBR_MAX_COLOR_TARGETS] = {};
    Texture* depth = nullptr;
    uint32_t width = 0, height = 0;
};

struct Counters {
    uint64_t fragments = 0;
    uint64_t primitives = 0;
    uint64_t fs_runs = 0;   // fragment-stage invocations
    uint64_t tex_runs = 0;  // those of programs with a texture binding
};

static bool program_samples_texture(const Program* p) {
    for (int b = 0; b < p->num_bindings; ++b)
        if (p->bindings[b].kind == 1) return true;
    return false;
}

struct Exec {
    Device* dev;
    uint32_t profile;
    PassTargets* tg;
    uint32_t band_y0, band_y1;  // rows [y0, y1) this thread owns
    Counters cnt;
};

// Per-draw resolved bindings for the program callbacks.
static void resolve_bindings(Device* dev, const PassState& st, ProgramBindings& pb) {
    std::memset(&pb, 0, sizeof pb);
    for (int g = 0; g < GBR_MAX_BIND_GROUPS; ++g) {
        const BindGroup* bg = st.groups[g];
        if (!bg) continue;
        for (uint32_t e = 0; e < bg->desc.entry_count; ++e) {
            const gbr_bind_group_entry& en = bg->desc.entries[e];
            if (en.binding >= 8) continue;
            if (en.kind == GBR_BINDING_BUFFER) {
                Buffer* b = dev->get<Buffer>(en.resource, "buffer");
                if (en.offset > b->data.size()) fail(GBR_ERR_VALIDATION, "bind group buffer range out of bounds");
                uint64_t size = en.size ? en.size : b->data.size() - en.offset;
                if (!range_fits(en.offset, size, b->data.size())) fail(GBR_ERR_VALIDATION, "bind group buffer range out of bounds");
                pb.uniform[g][en.binding] = b->data.data() + en.offset;
                pb.uniform_size[g][en.binding] = size;
            } else if (en.kind == GBR_BINDING_TEXTURE_VIEW) {
                Texture* t = dev->get<Texture>(en.resource, "texture");
                pb.texture[g][en.binding] = new TextureView{t};  // freed in free_bindings
            } else if (en.kind == GBR_BINDING_SAMPLER) {
                Sampler* s = dev->get<Sampler>(en.resource, "sampler");
                pb.sampler[g][en.binding] = &s->s;
            }
        }
    }
    pb.sample = sample_cb;
    pb.sample_ctx = &dev->profile;
}
static void free_bindings(ProgramBindings& pb) {
    for (int g = 0; g < 4; ++g)
        for (int b = 0; b < 8; ++b) delete pb.texture[g][b];
}

// Vertex attribute fetch (render_pass/vertex.rs:128-156, 191-195).
static void fetch_vertex(const PassState& st, const Pipeline* pl, uint32_t profile, uint32_t vertex, uint32_t instance,
                         VsIn& in) {
    std::memset(in.attr, 0, sizeof in.attr);
    in.vertex_index = vertex;
    in.instance_index = instance;
    const Program* prog = pl->vs;
    for (int i = 0; i < prog->num_inputs; ++i) {
        int loc = prog->inputs[i].location;
        const Pipeline::Loc& L = pl->loc[loc];
        if (!L.present) fail(GBR_ERR_VALIDATION, "No vertex attribute at location %d", loc);
        const gbr_vertex_buffer_layout& lay = pl->desc.vertex_buffers[L.buffer];
        const BoundSlice& bs = st.vb[L.buffer];
        if (!bs.buf) fail(GBR_ERR_VALIDATION, "Buffer %u not bound", L.buffer);
        uint64_t stride_v = lay.step_mode == GBR_STEP_VERTEX ? lay.array_stride : 0;
        uint64_t stride_i = lay.step_mode == GBR_STEP_INSTANCE ? lay.array_stride : 0;
        uint64_t start = (uint64_t)instance * stride_i + (uint64_t)vertex * stride_v + L.offset;
        uint32_t fsize = 0;
        switch (L.format) {
            case GBR_VERTEX_FORMAT_FLOAT32:
            case GBR_VERTEX_FORMAT_UINT32:
            case GBR_VERTEX_FORMAT_SINT32:
            case GBR_VERTEX_FORMAT_UNORM8X4:
            case GBR_VERTEX_FORMAT_FLOAT16X2: fsize = 4; break;
            case GBR_VERTEX_FORMAT_FLOAT32X2:
            case GBR_VERTEX_FORMAT_FLOAT16X4: fsize = 8; break;
            case GBR_VERTEX_FORMAT_FLOAT32X3: fsize = 12; break;
            case GBR_VERTEX_FORMAT_FLOAT32X4: fsize = 16; break;
            default: fail(GBR_ERR_UNSUPPORTED, "vertex format %u", L.format);
        }
        if (start + fsize > bs.size) fail(GBR_ERR_VALIDATION, "vertex attribute read out of bounds (vertex %u)", vertex);
        const uint8_t* src = bs.buf->data.data() + bs.offset + start;
        int comps = prog->inputs[i].components;
        if (profile == GBR_PROFILE_EXTENSION && L.format == GBR_VERTEX_FORMAT_FLOAT16X4 && comps == 4) {
            uint16_t h[4];
            std::memcpy(h, src, 8);
            for (int k = 0; k < 4; ++k) in.attr[loc][k] = f16_to_f32(h[k]);
        } else if (profile == GBR_PROFILE_EXTENSION && L.format == GBR_VERTEX_FORMAT_UNORM8X4 && comps == 4) {
            for (int k = 0; k < 4; ++k) in.attr[loc][k] = (float)src[k] / 255.0f;
        } else {
            // The reference copies exactly `format.size()` bytes into the shader input, so the
            // shader type must have the same size (vertex.rs:150-154).
            if ((uint32_t)comps * 4u != fsize)
                fail(GBR_ERR_VALIDATION, "vertex format %u does not match a %d-component shader input", L.format, comps);
            std::memcpy(in.attr[loc], src, fsize);
        }
    }
}

// evaluate_compare_function (render_pass/mod.rs:434-452)
static bool compare(uint32_t f, float v, float r) {
    switch (f) {
        case GBR_COMPARE_NEVER: return false;
        case GBR_COMPARE_LESS: return v < r;
        case GBR_COMPARE_EQUAL: return v == r;
        case GBR_COMPARE_LESS_EQUAL: return v <= r;
        case GBR_COMPARE_GREATER: return v > r;
        case GBR_COMPARE_NOT_EQUAL: return v != r;
        case GBR_COMPARE_GREATER_EQUAL: return v >= r;
        case GBR_COMPARE_ALWAYS: return true;
        default: fail(GBR_ERR_VALIDATION, "invalid compare function %u", f);
    }
}

// The per-fragment work of FragmentProcessingState::process (fragment.rs:127-214),
// FragmentOutput::depth_test (fragment.rs:427-453) and ::read_from (fragment.rs:456-489).
// `coeff` are the interpolation coefficients for the FS inputs (N = 1, 2 or 3 vertices),
// `vars` the inter-stage variables of the primitive's unclipped vertices.
static const float kZero3[3] = {0.0f, 0.0f, 0.0f};

struct FragCtx {
    Exec* ex;
    const PassState* st;
    const Pipeline* pl;
    const ProgramBindings* pb;
};

// `dcx` / `dcy`: screen-space derivatives of the coefficients (extension-profile sampling; zero
// for lines and points).
static void process_fragment(FragCtx& fc, uint32_t fx, uint32_t fy, V4 fragment, bool front_facing,
                             uint32_t primitive_index, int nverts, const float coeff[3], const VsOut* const verts[3],
                             const float inv_w[3], const float dcx[3], const float dcy[3]) {
    Exec* ex = fc.ex;
    const Pipeline* pl = fc.pl;
    const Program* fs = pl->fs;
    ex->cnt.fragments++;
    FsIn in;
    in.position = fragment;
    in.front_facing = front_facing;
    in.primitive_index = primitive_index;
    in.sample_index = 0;
    in.sample_mask = ~0u;
    std::memset(in.dvar_dx, 0, sizeof in.dvar_dx);
    std::memset(in.dvar_dy, 0, sizeof in.dvar_dy);
    for (int v = 0; v < fs->num_varyings; ++v) {
        const ProgramVarying& pv = fs->varyings[v];
        for (int c = 0; c < pv.components; ++c) {
            float x;
            if (pv.interp == INTERP_FLAT) {
                x = verts[0]->var[pv.location][c];  // FlatSampling: inputs[0] (fragment.rs:395-405)
            } else if (pv.interp == INTERP_LINEAR) {
                // Interpolate::interpolate on the inter-stage values (fragment.rs:346-366)
                float accu = verts[0]->var[pv.location][c] * coeff[0];
                for (int k = 1; k < nverts; ++k) accu = accu + verts[k]->var[pv.location][c] * coeff[k];
                x = accu;
                // d/dx and d/dy of the interpolated value, summed in the same order
                float gx = verts[0]->var[pv.location][c] * dcx[0], gy = verts[0]->var[pv.location][c] * dcy[0];
                for (int k = 1; k < nverts; ++k) {
                    gx = gx + verts[k]->var[pv.location][c] * dcx[k];
                    gy = gy + verts[k]->var[pv.location][c] * dcy[k];
                }
                in.dvar_dx[pv.location][c] = gx;
                in.dvar_dy[pv.location][c] = gy;
            } else {
                if (ex->profile != GBR_PROFILE_EXTENSION)
                    fail(GBR_ERR_UNSUPPORTED, "perspective interpolation is todo!() (fragment.rs:343-345)");
                // Extension: perspective-correct, (sum v_k c_k / w_k) / (sum c_k / w_k).
                float num = (verts[0]->var[pv.location][c] * coeff[0]) * inv_w[0];
                float den = coeff[0] * inv_w[0];
                for (int k = 1; k < nverts; ++k) {
                    num = num + (verts[k]->var[pv.location][c] * coeff[k]) * inv_w[k];
                    den = den + coeff[k] * inv_w[k];
                }
                x = num / den;
            }
            in.var[pv.location][c] = x;
        }
    }
    PassTargets* tg = ex->tg;
    // FragmentOutput::depth_test (fragment.rs:427-453): compare with the stored depth, write on a
    // pass when depth writes are on; true when there is no depth attachment or no depth state
    auto depth_test = [&]() {
        if (!(tg->depth && pl->desc.has_depth_stencil)) return true;
        Texture* d = tg->depth;
        float* dp = reinterpret_cast<float*>(d->mips[0].data()) + (size_t)fy * d->desc.size.width + fx;
        if (!compare(pl->desc.depth_stencil.depth_compare, fragment.z, *dp)) return false;
        if (pl->desc.depth_stencil.depth_write_enabled) *dp = fragment.z;
        return true;
    };
    // @early_depth_test (fragment.rs:166-194): none = late test only; Force = early test only
    // (its result stands at the colour output); Allow = early test, then the late test again
    bool have_result = false, result = true;
    if (fs->early_depth != 0) {
        if (!depth_test()) return;  // early depth test reject: the fragment stage does not run
        if (fs->early_depth == 1) have_result = true;
    }
    FsOut out;
    out.killed = false;
    ex->cnt.fs_runs++;
    if (program_samples_texture(fs)) ex->cnt.tex_runs++;
    fs->fs(in, *fc.pb, out);
    if (out.killed) return;  // EntryPointError::Killed (fragment.rs:204-208)
    if (fs->num_outputs == 0) return;
    // Late depth test at the first @location output (fragment.rs:470-479).
    const bool pass = have_result ? result : depth_test();
    if (!pass) return;
    for (int o = 0; o < fs->num_outputs; ++o) {
        Texture* t = tg->color[o];
        if (!t) fail(GBR_ERR_VALIDATION, "no colour attachment at location %d (fragment.rs:482-483)", o);
        V4 c = out.color[o];
        if (ex->profile == GBR_PROFILE_EXTENSION && o < (int)pl->desc.color_target_count) {
            const gbr_color_target_state& ct = pl->desc.color_targets[o];
            if (ct.has_blend) c = blend_colors(ct, c, read_color(t, fx, fy, tg->color_slice[o]), fc.st->blend_constant);
            uint32_t wm = ct.write_mask;
            if (wm != 0xF) {
                V4 d = read_color(t, fx, fy, tg->color_slice[o]);
                if (!(wm & 1)) c.x = d.x;
                if (!(wm & 2)) c.y = d.y;
                if (!(wm & 4)) c.z = d.z;
                if (!(wm & 8)) c.w = d.w;
            }
        }
        write_color(t, fx, fy, tg->color_slice[o], c, ex->profile);
    }
}

// ------------------------------------------------------------------ the draw loop
// DrawCall::execute + draw (render_pass/state.rs:239-593)
static void execute_draw(Exec* ex, const PassState& st, bool indexed, uint32_t start, uint32_t end, int32_t base_vertex,
                         uint32_t inst_start, uint32_t inst_end) {
    Device* dev = ex->dev;
    const Pipeline* pl = st.pipeline;
    if (!pl) fail(GBR_ERR_VALIDATION, "No pipeline bound");
    const gbr_primitive_state& ps = pl->desc.primitive;
    if (ps.polygon_mode != GBR_POLYGON_FILL) fail(GBR_ERR_UNSUPPORTED, "Unsupported polygon mode %u", ps.polygon_mode);
    bool is_strip = ps.topology == GBR_TOPOLOGY_LINE_STRIP || ps.topology == GBR_TOPOLOGY_TRIANGLE_STRIP;
    bool separated = false;
    if (indexed) {
        if (!st.index.buf) fail(GBR_ERR_VALIDATION, "No index buffer bound");
        if (ps.strip_index_format != GBR_INDEX_NONE) {
            if (!is_strip) fail(GBR_ERR_VALIDATION, "List can't be separated");
            if (ps.strip_index_format != st.index_format) fail(GBR_ERR_VALIDATION, "strip_index_format mismatch");
            separated = true;
        }
    }
    ProgramBindings pb;
    resolve_bindings(dev, st, pb);
    struct Guard {
        ProgramBindings* p;
        ~Guard() { free_bindings(*p); }
    } guard{&pb};

    ToRaster tr = make_to_raster(st.viewport, st.scissor);
    FragCtx fc{ex, &st, pl, &pb};
    bool has_fs = pl->desc.has_fragment && pl->fs;
    uint32_t n = end > start ? end - start : 0;

    for (uint32_t instance = inst_start; instance < inst_end; ++instance) {
        // index resolution + vertex processing, once per index (state.rs:521-535)
        std::vector<VsOut> vout(n);
        std::vector<uint8_t> is_sep(n, 0);
        for (uint32_t k = 0; k < n; ++k) {
            uint32_t vertex;
            if (indexed) {
                uint32_t pos = start + k;
                uint64_t isz = st.index_format == GBR_INDEX_UINT16 ? 2 : 4;
                if ((uint64_t)(pos + 1) * isz > st.index.size) fail(GBR_ERR_VALIDATION, "index %u out of range", pos);
                const uint8_t* ip = st.index.buf->data.data() + st.index.offset + (uint64_t)pos * isz;
                uint32_t raw;
                if (isz == 2) {
                    uint16_t h;
                    std::memcpy(&h, ip, 2);
                    raw = h;
                    if (separated && h == 0xFFFFu) {
                        is_sep[k] = 1;
                        continue;
                    }
                } else {
                    std::memcpy(&raw, ip, 4);
                    if (separated && raw == 0xFFFFFFFFu) {
                        is_sep[k] = 1;
                        continue;
                    }
                }
                int64_t v = (int64_t)raw + (int64_t)base_vertex;  // u32::strict_add_signed (index.rs:55-57)
                if (v < 0 || v > 0xFFFFFFFFll) fail(GBR_ERR_VALIDATION, "index + base_vertex overflows u32");
                vertex = (uint32_t)v;
            } else {
                vertex = start + k;
            }
            VsIn in;
            fetch_vertex(st, pl, ex->profile, vertex, instance, in);
            std::memset(vout[k].var, 0, sizeof vout[k].var);
            if (!pl->vs->vs(in, pb, vout[k])) fail(GBR_ERR_VALIDATION, "vertex processing failed");
        }
        if (!has_fs) continue;  // vertex shaders still ran (state.rs:584-589)

        // primitive assembly (primitive.rs:206-487) -> list of vertex positions per primitive
        int nv = (ps.topology == GBR_TOPOLOGY_POINT_LIST) ? 1
                 : (ps.topology == GBR_TOPOLOGY_LINE_LIST || ps.topology == GBR_TOPOLOGY_LINE_STRIP) ? 2
                                                                                                    : 3;
        std::vector<std::array<uint32_t, 3>> prims;
        if (ps.topology == GBR_TOPOLOGY_POINT_LIST || ps.topology == GBR_TOPOLOGY_LINE_LIST ||
            ps.topology == GBR_TOPOLOGY_TRIANGLE_LIST) {
            for (uint32_t k = 0; k + nv <= n; k += nv) {  // array_chunks_ drops a partial chunk
                std::array<uint32_t, 3> p = {k, nv > 1 ? k + 1 : 0, nv > 2 ? k + 2 : 0};
                prims.push_back(p);
            }
        } else if (ps.topology == GBR_TOPOLOGY_LINE_STRIP) {
            if (!separated) {
                for (uint32_t k = 0; k + 1 < n; ++k) prims.push_back({k, k + 1, 0});  // tuple_windows
            } else {  // Strip<2> with separators (primitive.rs:287-322)
                int cnt = 0;
                uint32_t last = 0;
                for (uint32_t k = 0; k < n; ++k) {
                    if (is_sep[k]) {
                        cnt = 0;
                        continue;
                    }
                    if (cnt == 1) prims.push_back({last, k, 0});
                    last = k;
                    cnt = 1;
                }
            }
        } else {  // triangle strip
            if (!separated) {  // TriStripIter (primitive.rs:394-426)
                for (uint32_t p = 0; p + 2 < n; ++p) {
                    uint32_t t[3];
                    strip_tri(p, t);
                    prims.push_back({t[0], t[1], t[2]});
                }
            } else {  // ResetTriStripIter (primitive.rs:428-487)
                uint32_t seg[3];
                int fill = 0;
                bool odd = false;
                uint32_t buf[2];
                for (uint32_t k = 0; k < n; ++k) {
                    if (is_sep[k]) {
                        fill = 0;
                        continue;
                    }
                    if (fill < 2) {
                        seg[fill] = k;
                        ++fill;
                        if (fill == 2) {
                            buf[0] = seg[0];
                            buf[1] = seg[1];
                            odd = false;
                        }
                        continue;
                    }
                    prims.push_back({buf[0], buf[1], k});  // TriStripGenerator::push
                    buf[odd ? 1 : 0] = k;
                    odd = !odd;
                }
            }
        }

        for (size_t prim_index = 0; prim_index < prims.size(); ++prim_index) {
            const auto& pr = prims[prim_index];
            ex->cnt.primitives++;
            if (nv == 3) {
                const VsOut* verts[3] = {&vout[pr[0]], &vout[pr[1]], &vout[pr[2]]};
                V4 pos[3] = {verts[0]->position, verts[1]->position, verts[2]->position};
                bool ccw;
                if (!tri_face_ccw(pos, &ccw)) fail(GBR_ERR_VALIDATION, "clip position w=0 (primitive.rs:177)");
                bool front_facing = (ccw ? GBR_FRONT_FACE_CCW : GBR_FRONT_FACE_CW) == ps.front_face;
                bool cull = ps.cull_mode == GBR_CULL_FRONT ? front_facing
                            : ps.cull_mode == GBR_CULL_BACK ? !front_facing
                                                            : false;
                if (cull) continue;
                float inv_w[3] = {1.0f / pos[0].w, 1.0f / pos[1].w, 1.0f / pos[2].w};
                std::vector<ClipTri> subs;
                clip_tri(pos, subs);
                for (const ClipTri& sub : subs) {
                    // TriRasterizer::rasterize (raster.rs:280-363)
                    RasterPoint rp[3];
                    for (int i = 0; i < 3; ++i)
                        if (!to_raster(tr, sub.v[i].position, &rp[i])) fail(GBR_ERR_VALIDATION, "w=0 (raster.rs:146)");
                    P2 va = {rp[0].frag.x, rp[0].frag.y}, vb = {rp[1].frag.x, rp[1].frag.y},
                       vc = {rp[2].frag.x, rp[2].frag.y};
                    float total = shoelace(va, vb, vc);
                    if (total == 0.0f) continue;
                    Bary3 clipb[3] = {sub.v[0].bary, sub.v[1].bary, sub.v[2].bary};
                    V4 frags[3] = {rp[0].frag, rp[1].frag, rp[2].frag};
                    // d(lambda)/dx, d(lambda)/dy of the shoelace barycentrics (lambda_0 = S(p, b, c) / A:
                    // (b.y - c.y) / A and (c.x - b.x) / A, cyclically), composed with the clip
                    // barycentrics like the barycentrics themselves
                    Bary3 lgx = {{(vb.y - vc.y) / total, (vc.y - va.y) / total, (va.y - vb.y) / total}};
                    Bary3 lgy = {{(vc.x - vb.x) / total, (va.x - vc.x) / total, (vb.x - va.x) / total}};
                    Bary3 dcx = compose_bary(clipb, lgx), dcy = compose_bary(clipb, lgy);
                    auto emit = [&](uint32_t px, uint32_t py, P2 p) {
                        if (!in_scissor(tr, px, py)) return;
                        Bary3 lam = {{shoelace(p, vb, vc) / total, shoelace(va, p, vc) / total,
                                      shoelace(va, vb, p) / total}};
                        Bary3 comp = compose_bary(clipb, lam);
                        V4 fragment = interp3_v4(frags, comp);
                        process_fragment(fc, px, py, fragment, front_facing, (uint32_t)prim_index, 3, comp.c, verts,
                                         inv_w, dcx.c, dcy.c);
                    };
                    if (ex->dev->raster_rule == GBR_RASTER_RULE_EDGE) {
                        // extension: pixel centres inside the snapped edges (top-left rule),
                        // attributes sampled at the centre
                        const float vxs[3] = {va.x, vb.x, vc.x}, vys[3] = {va.y, vb.y, vc.y};
                        for (int i = 0; i < 3; ++i)
                            if (!(std::fabs(vxs[i]) < 4194304.0f && std::fabs(vys[i]) < 4194304.0f))
                                fail(GBR_ERR_VALIDATION, "raster coordinates out of range for the edge rule");
                        int64_t X[3], Y[3];
                        if (snap_triangle(vxs, vys, X, Y) == 0) continue;
                        const int64_t ylo = std::min(Y[0], std::min(Y[1], Y[2]));
                        const int64_t yhi = std::max(Y[0], std::max(Y[1], Y[2]));
                        int64_t r0 = std::max(ceil_div64(ylo - 128, 256), (int64_t)ex->band_y0);
                        int64_t r1 = std::min(floor_div64(yhi - 128, 256), (int64_t)ex->band_y1 - 1);
                        for (int64_t y = r0; y <= r1; ++y) {
                            int64_t x1, x2;
                            span_edge(X, Y, y, &x1, &x2);
                            for (int64_t x = std::max<int64_t>(x1, 0); x <= x2; ++x)
                                emit((uint32_t)x, (uint32_t)y, P2{(float)x + 0.5f, (float)y + 0.5f});
                        }
                        continue;
                    }
                    uint32_t fxs[3] = {rp[0].fbx, rp[1].fbx, rp[2].fbx}, fys[3] = {rp[0].fby, rp[1].fby, rp[2].fby};
                    bool ok = scanlines(fxs, fys, [&](const Scanline& sl) {
                        if (sl.y < (int64_t)ex->band_y0 || sl.y >= (int64_t)ex->band_y1) return;
                        for (int64_t x = sl.x1; x <= sl.x2; ++x) {
                            uint32_t px = (uint32_t)x, py = (uint32_t)sl.y;
                            emit(px, py, P2{(float)px, (float)py});
                        }
                    });
                    if (!ok) fail(GBR_ERR_VALIDATION, "scanlines generated points that don't fit u32");
                }
            } else if (nv == 2) {
                const VsOut* verts[3] = {&vout[pr[0]], &vout[pr[1]], nullptr};
                V4 pts[2] = {verts[0]->position, verts[1]->position};
                float alphas[2];
                if (!clip_line(pts, alphas)) continue;
                RasterPoint s, e;
                if (!to_raster(tr, pts[0], &s) || !to_raster(tr, pts[1], &e)) fail(GBR_ERR_VALIDATION, "w=0");
                float inv_w[3] = {1.0f / verts[0]->position.w, 1.0f / verts[1]->position.w, 0.0f};
                bresenham(s.fbx, s.fby, e.fbx, e.fby, [&](uint32_t px, uint32_t py, float t) {
                    if (py < ex->band_y0 || py >= ex->band_y1) return;
                    if (!in_scissor(tr, px, py)) return;
                    // Lerp(t).interpolate([Lerp(a0), Lerp(a1)]) (raster.rs:248-254)
                    float T = alphas[0] * (1.0f - t) + alphas[1] * t;
                    V4 fragment = v4_add(v4_mul(s.frag, 1.0f - T), v4_mul(e.frag, T));
                    float coeff[3] = {1.0f - T, T, 0.0f};
                    // Lerp::interpolate for the inter-stage values: v0*(1-T) + v1*T
                    process_fragment(fc, px, py, fragment, true, (uint32_t)prim_index, 2, coeff, verts, inv_w, kZero3,
                                     kZero3);
                });
            } else {
                const VsOut* verts[3] = {&vout[pr[0]], nullptr, nullptr};
                RasterPoint r;
                if (!to_raster(tr, verts[0]->position, &r)) fail(GBR_ERR_VALIDATION, "w=0");
                if (r.fby < ex->band_y0 || r.fby >= ex->band_y1) continue;
                if (!in_scissor(tr, r.fbx, r.fby)) continue;
                float coeff[3] = {1.0f, 0.0f, 0.0f};
                float inv_w[3] = {1.0f / verts[0]->position.w, 0.0f, 0.0f};
                process_fragment(fc, r.fbx, r.fby, r.frag, true, (uint32_t)prim_index, 1, coeff, verts, inv_w, kZero3,
                                 kZero3);
            }
        }
    }
}

// ------------------------------------------------------------------ command stream
struct Cursor {
    const uint8_t* p;
    const uint8_t* end;
};

template <class T>
static const T* payload(const gbr_cmd_header* h, const uint8_t* body) {
    if (h->payload_bytes < sizeof(T)) fail(GBR_ERR_INVALID_ARGUMENT, "command %u payload too short", h->opcode);
    return reinterpret_cast<const T*>(body);
}

struct DecodedPass {
    gbr_cmd_begin_render_pass begin;
    std::vector<std::pair<gbr_cmd_header, std::vector<uint8_t>>> cmds;
    bool is_copy = false;  // an encoder copy / clear between passes: cmds holds that one record
};

static std::vector<DecodedPass> decode_stream(const uint8_t* data, uint64_t len) {
    std::vector<DecodedPass> passes;
    uint64_t off = 0;
    DecodedPass* cur = nullptr;
    while (off < len) {
        if (len - off < sizeof(gbr_cmd_header)) fail(GBR_ERR_INVALID_ARGUMENT, "truncated command header");
        gbr_cmd_header h;
        std::memcpy(&h, data + off, sizeof h);
        off += sizeof h;
        uint64_t padded = (h.payload_bytes + 7ull) & ~7ull;
        if (len - off < padded) fail(GBR_ERR_INVALID_ARGUMENT, "truncated command payload");
        const uint8_t* body = data + off;
        off += padded;
        if (h.opcode == GBR_OP_BEGIN_RENDER_PASS) {
            if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "nested render pass");
            passes.emplace_back();
            cur = &passes.back();
            std::memcpy(&cur->begin, payload<gbr_cmd_begin_render_pass>(&h, body), sizeof cur->begin);
        } else if (h.opcode == GBR_OP_END_RENDER_PASS) {
            if (!cur) fail(GBR_ERR_INVALID_ARGUMENT, "end without begin");
            cur = nullptr;
        } else if (h.opcode >= GBR_OP_COPY_BUFFER_TO_BUFFER && h.opcode <= GBR_OP_CLEAR_TEXTURE) {
            if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "command %u inside a render pass", h.opcode);
            passes.emplace_back();
            std::memset(&passes.back().begin, 0, sizeof passes.back().begin);
            passes.back().is_copy = true;
            passes.back().cmds.emplace_back(h, std::vector<uint8_t>(body, body + h.payload_bytes));
        } else {
            if (!cur) fail(GBR_ERR_INVALID_ARGUMENT, "command %u outside a render pass", h.opcode);
            cur->cmds.emplace_back(h, std::vector<uint8_t>(body, body + h.payload_bytes));
        }
    }
    if (cur) fail(GBR_ERR_INVALID_ARGUMENT, "render pass not ended");
    return passes;
}

// texture.rs:199-211 (clear_color / clear_depth) for rows [y0, y1).
static void clear_targets(Exec* ex, const DecodedPass& dp) {
    PassTargets* tg = ex->tg;
    for (uint32_t a = 0; a < dp.begin.color_attachment_count && a < GBR_MAX_COLOR_TARGETS; ++a) {
        const gbr_color_attachment& ca = dp.begin.color_attachments[a];
        Texture* t = tg->color[a];
        if (!t || ca.load_op != GBR_LOAD_OP_CLEAR) continue;
        V4 c = {(float)ca.clear_value[0], (float)ca.clear_value[1], (float)ca.clear_value[2], (float)ca.clear_value[3]};
        for (uint32_t y = ex->band_y0; y < ex->band_y1; ++y)
            for (uint32_t x = 0; x < t->desc.size.width; ++x) write_color(t, x, y, tg->color_slice[a], c, ex->profile);
    }
    if (tg->depth && dp.begin.depth_attachment.has_depth_ops &&
        dp.begin.depth_attachment.depth_load_op == GBR_LOAD_OP_CLEAR) {
        float* d = reinterpret_cast<float*>(tg->depth->mips[0].data());
        uint32_t w = tg->depth->desc.size.width;
        for (uint32_t y = ex->band_y0; y < ex->band_y1; ++y)
            std::fill(d + (size_t)y * w, d + (size_t)(y + 1) * w, dp.begin.depth_attachment.depth_clear_value);
    }
}

static void run_pass_band(Exec* ex, const DecodedPass& dp) {
    Device* dev = ex->dev;
    clear_targets(ex, dp);
    PassState st;
    st.viewport[0] = 0.0f;
    st.viewport[1] = 0.0f;
    st.viewport[2] = (float)ex->tg->width;
    st.viewport[3] = (float)ex->tg->height;
    st.viewport[4] = 0.0f;
    st.viewport[5] = 1.0f;
    st.scissor[0] = 0;
    st.scissor[1] = 0;
    st.scissor[2] = ex->tg->width;
    st.scissor[3] = ex->tg->height;
    for (const auto& c : dp.cmds) {
        const gbr_cmd_header& h = c.first;
        const uint8_t* b = c.second.data();
        switch (h.opcode) {
            case GBR_OP_SET_PIPELINE:
                st.pipeline = dev->get<Pipeline>(payload<gbr_cmd_set_pipeline>(&h, b)->pipeline, "pipeline");
                break;
            case GBR_OP_SET_BIND_GROUP: {
                auto* p = payload<gbr_cmd_set_bind_group>(&h, b);
                if (p->index >= GBR_MAX_BIND_GROUPS) fail(GBR_ERR_VALIDATION, "bind group index");
                st.groups[p->index] = p->bind_group ? dev->get<BindGroup>(p->bind_group, "bind group") : nullptr;
                break;
            }
            case GBR_OP_SET_INDEX_BUFFER: {
                auto* p = payload<gbr_cmd_set_index_buffer>(&h, b);
                Buffer* buf = dev->get<Buffer>(p->buffer, "buffer");
                uint64_t size = p->size ? p->size : buf->data.size() - p->offset;
                if (!range_fits(p->offset, size, buf->data.size())) fail(GBR_ERR_VALIDATION, "index buffer slice out of range");
                st.index = {buf, p->offset, size};
                st.index_format = p->index_format;
                break;
            }
            case GBR_OP_SET_VERTEX_BUFFER: {
                auto* p = payload<gbr_cmd_set_vertex_buffer>(&h, b);
                if (p->slot >= GBR_MAX_VERTEX_BUFFERS) fail(GBR_ERR_VALIDATION, "vertex buffer slot");
                Buffer* buf = dev->get<Buffer>(p->buffer, "buffer");
                uint64_t size = p->size ? p->size : buf->data.size() - p->offset;
                if (!range_fits(p->offset, size, buf->data.size())) fail(GBR_ERR_VALIDATION, "vertex buffer slice out of range");
                st.vb[p->slot] = {buf, p->offset, size};
                break;
            }
            case GBR_OP_SET_VIEWPORT: {
                auto* p = payload<gbr_cmd_set_viewport>(&h, b);
                st.viewport[0] = p->x;
                st.viewport[1] = p->y;
                st.viewport[2] = p->width;
                st.viewport[3] = p->height;
                st.viewport[4] = p->min_depth;
                st.viewport[5] = p->max_depth;
                break;
            }
            case GBR_OP_SET_SCISSOR_RECT: {
                auto* p = payload<gbr_cmd_set_scissor_rect>(&h, b);
                st.scissor[0] = p->x;
                st.scissor[1] = p->y;
                st.scissor[2] = p->width;
                st.scissor[3] = p->height;
                break;
            }
            case GBR_OP_SET_BLEND_CONSTANT: {
                auto* p = payload<gbr_cmd_set_blend_constant>(&h, b);
                for (int k = 0; k < 4; ++k) st.blend_constant[k] = p->color[k];
                break;
            }
            case GBR_OP_SET_STENCIL_REFERENCE: break;
            case GBR_OP_DRAW: {
                auto* p = payload<gbr_cmd_draw>(&h, b);
                execute_draw(ex, st, false, p->vertex_start, p->vertex_end, 0, p->instance_start, p->instance_end);
                break;
            }
            case GBR_OP_DRAW_INDEXED: {
                auto* p = payload<gbr_cmd_draw_indexed>(&h, b);
                execute_draw(ex, st, true, p->index_start, p->index_end, p->base_vertex, p->instance_start,
                             p->instance_end);
                break;
            }
            default: fail(GBR_ERR_INVALID_ARGUMENT, "unknown opcode %u", h.opcode);
        }
    }
}

static void execute_pass(Device* dev, const DecodedPass& dp, Counters& total, int threads) {
    // State::new (render_pass/state.rs:77-133): all attachments must have the same size.
    PassTargets tg;
    bool have = false;
    auto size_of = [&](Texture* t) {
        if (!have) {
            tg.width = t->desc.size.width;
            tg.height = t->desc.size.height;
            have = true;
        } else if (tg.width != t->desc.size.width || tg.height != t->desc.size.height) {
            fail(GBR_ERR_VALIDATION, "All render attachments must be the same size");
        }
    };
    for (uint32_t a = 0; a < dp.begin.color_attachment_count && a < GBR_MAX_COLOR_TARGETS; ++a) {
        const gbr_color_attachment& ca = dp.begin.color_attachments[a];
        if (!ca.view) continue;
        Texture* t = dev->get<Texture>(ca.view, "texture");
        tg.color[a] = t;
        tg.color_slice[a] = ca.depth_slice;
        size_of(t);
    }
    if (dp.begin.has_depth_attachment && dp.begin.depth_attachment.view) {
        Texture* t = dev->get<Texture>(dp.begin.depth_attachment.view, "texture");
        if (t->desc.format != GBR_TEXTURE_FORMAT_DEPTH32_FLOAT) fail(GBR_ERR_UNSUPPORTED, "depth format");
        tg.depth = t;
        size_of(t);
    }
    int nt = std::max(1, threads);
    if ((uint32_t)nt > tg.height) nt = std::max(1u, tg.height);
    std::vector<Exec> ex(nt);
    std::vector<std::string> errs(nt);
    std::vector<gbr_status> sts(nt, GBR_OK);
    auto work = [&](int i) {
        ex[i].dev = dev;
        ex[i].profile = dev->profile;
        ex[i].tg = &tg;
        ex[i].band_y0 = (uint32_t)((uint64_t)tg.height * i / nt);
        ex[i].band_y1 = (uint32_t)((uint64_t)tg.height * (i + 1) / nt);
        try {
            run_pass_band(&ex[i], dp);
        } catch (const Error& e) {
            sts[i] = e.status;
            errs[i] = e.msg;
        }
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (int i = 0; i < nt; ++i) th.emplace_back(work, i);
        for (auto& t : th) t.join();
    }
    for (int i = 0; i < nt; ++i)
        if (sts[i] != GBR_OK) throw Error{sts[i], errs[i]};
    for (int i = 0; i < nt; ++i) {
        total.fragments += ex[i].cnt.fragments;
        total.fs_runs += ex[i].cnt.fs_runs;
        total.tex_runs += ex[i].cnt.tex_runs;
    }
    total.primitives += ex[0].cnt.primitives;  // every thread assembles all primitives
}

// The textures a render pass renders to (its attachments) and samples (texture views of the bind
// groups it sets).
static void pass_textures(Device* dev, const DecodedPass& dp, std::set<Texture*>& writes, std::set<Texture*>& reads) {
    for (uint32_t a = 0; a < dp.begin.color_attachment_count && a < GBR_MAX_COLOR_TARGETS; ++a)
        if (dp.begin.color_attachments[a].view) writes.insert(dev->get<Texture>(dp.begin.color_attachments[a].view, "texture"));
    if (dp.begin.has_depth_attachment && dp.begin.depth_attachment.view)
        writes.insert(dev->get<Texture>(dp.begin.depth_attachment.view, "texture"));
    for (const auto& c : dp.cmds) {
        if (c.first.opcode != GBR_OP_SET_BIND_GROUP || c.second.size() < sizeof(gbr_cmd_set_bind_group)) continue;
        gbr_cmd_set_bind_group sb;
        std::memcpy(&sb, c.second.data(), sizeof sb);
        if (!sb.bind_group) continue;
        const BindGroup* g = dev->get<BindGroup>(sb.bind_group, "bind group");
        for (uint32_t e = 0; e < g->desc.entry_count; ++e)
            if (g->desc.entries[e].kind == GBR_BINDING_TEXTURE_VIEW)
                reads.insert(dev->get<Texture>(g->desc.entries[e].resource, "texture"));
    }
}

// End of the run of render passes from `first` that do not depend on one another: none renders
// to a texture another one renders to or samples.  Their results do not depend on their order.
static size_t independent_run(Device* dev, const std::vector<DecodedPass>& passes, size_t first) {
    std::set<Texture*> writes, reads;
    size_t j = first;
    for (; j < passes.size() && !passes[j].is_copy; ++j) {
        std::set<Texture*> w, r;
        try {
            pass_textures(dev, passes[j], w, r);
        } catch (const Error&) {
            return j == first ? first + 1 : j;  // the pass reports its own error when it runs
        }
        bool clash = false;
        for (Texture* t : w) clash = clash || writes.count(t) || reads.count(t);
        for (Texture* t : r) clash = clash || writes.count(t);
        if (clash) break;
        writes.insert(w.begin(), w.end());
        reads.insert(r.begin(), r.end());
    }
    return std::max(j, first + 1);
}

// Independent passes [first, last) on g_threads host threads, one pass per thread at a time
// (largest target first).  The first error in pass order is reported.
static void execute_passes_parallel(Device* dev, const std::vector<DecodedPass>& passes, size_t first, size_t last,
                                    Counters& total) {
    const size_t n = last - first;
    std::vector<size_t> order(n);
    std::vector<uint64_t> area(n, 0);
    for (size_t k = 0; k < n; ++k) {
        order[k] = first + k;
        const gbr_cmd_begin_render_pass& b = passes[first + k].begin;
        const uint64_t h = b.color_attachment_count && b.color_attachments[0].view ? b.color_attachments[0].view
                           : b.has_depth_attachment                                ? b.depth_attachment.view
                                                                                   : 0;
        if (h) {
            const Texture* t = dev->get<Texture>(h, "texture");
            area[k] = (uint64_t)t->desc.size.width * t->desc.size.height;
        }
    }
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return area[a - first] > area[b - first]; });
    std::vector<Counters> cnt(n);
    std::vector<gbr_status> sts(n, GBR_OK);
    std::vector<std::string> errs(n);
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t k; (k = next.fetch_add(1)) < n;) {
            const size_t p = order[k];
            try {
                execute_pass(dev, passes[p], cnt[p - first], 1);
            } catch (const Error& e) {
                sts[p - first] = e.status;
                errs[p - first] = e.msg;
            }
        }
    };
    std::vector<std::thread> th;
    const int nt = (int)std::min<size_t>((size_t)g_threads, n);
    for (int i = 0; i < nt; ++i) th.emplace_back(work);
    for (auto& t : th) t.join();
    for (size_t k = 0; k < n; ++k)
        if (sts[k] != GBR_OK) throw Error{sts[k], errs[k]};
    for (const Counters& c : cnt) {
        total.fragments += c.fragments;
        total.primitives += c.primitives;
        total.fs_runs += c.fs_runs;
        total.tex_runs += c.tex_runs;
    }
}

}  // namespace orc

using namespace orc;

#define ORC_TRY(...)                               \
    try {                                          \
        __VA_ARGS__;                                   \
        return GBR_OK;                             \
    } catch (const Error& e) {                     \
        g_last_error = e.msg;                      \
        return e.status;                           \
    } catch (const std::exception& e) {            \
        g_last_error = e.what();                   \
        return GBR_ERR_OUT_OF_MEMORY;              \
    }

ORC_API size_t orc_last_error(char* buf, size_t len) {
    if (buf && len) {
        size_t n = std::min(len - 1, g_last_error.size());
        std::memcpy(buf, g_last_error.data(), n);
        buf[n] = 0;
    }
    return g_last_error.size();
}
ORC_API uint32_t orc_abi_version(void) { return GBR_ABI_VERSION; }
ORC_API void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

ORC_API gbr_status orc_device_create(const gbr_device_config* cfg, gbr_device* out) {
    ORC_TRY({
        if (!cfg || !out) fail(GBR_ERR_INVALID_ARGUMENT, "null argument");
        if (cfg->abi_version != GBR_ABI_VERSION) fail(GBR_ERR_INVALID_ARGUMENT, "ABI version mismatch");
        auto d = std::make_unique<Device>();
        d->profile = cfg->profile;
        if (cfg->raster_rule > GBR_RASTER_RULE_EDGE) fail(GBR_ERR_INVALID_ARGUMENT, "raster_rule");
        if (cfg->raster_rule == GBR_RASTER_RULE_EDGE && cfg->profile != GBR_PROFILE_EXTENSION)
            fail(GBR_ERR_INVALID_ARGUMENT, "the edge-function raster rule belongs to the extension profile");
        d->raster_rule = cfg->raster_rule;
        std::lock_guard<std::mutex> lk(g_devices_mu);
        uint64_t h = g_next_device++;
        g_devices[h] = std::move(d);
        *out = h;
    })
}
ORC_API gbr_status orc_device_destroy(gbr_device d) {
    ORC_TRY({
        std::lock_guard<std::mutex> lk(g_devices_mu);
        if (!g_devices.erase(d)) fail(GBR_ERR_INVALID_ARGUMENT, "invalid device handle");
    })
}
ORC_API gbr_status orc_device_limits(gbr_device d, gbr_limits* out) {
    ORC_TRY({
        get_device(d);
        out->max_texture_dimension_2d = 16384;
        out->max_bind_groups = GBR_MAX_BIND_GROUPS;
        out->max_vertex_buffers = GBR_MAX_VERTEX_BUFFERS;
        out->max_vertex_attributes = GBR_MAX_VERTEX_ATTRIBUTES;
        out->max_color_attachments = GBR_MAX_COLOR_TARGETS;
        out->max_inter_stage_components = 32;
        out->max_buffer_size = 1ull << 36;
    })
}
ORC_API gbr_status orc_buffer_create(gbr_device d, uint64_t size, uint32_t usage, gbr_buffer* out) {
    ORC_TRY({
        (void)usage;
        Device* dev = get_device(d);
        auto* b = new Buffer;
        b->data.assign(size, 0);
        std::lock_guard<std::mutex> lk(dev->mu);
        *out = dev->add(b);
    })
}
ORC_API gbr_status orc_buffer_destroy(gbr_device d, gbr_buffer b) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<Buffer>(b, "buffer");
        dev->objects.erase(b);
    })
}
ORC_API gbr_status orc_queue_write_buffer(gbr_device d, gbr_buffer b, uint64_t offset, const void* data, uint64_t size) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        Buffer* buf = dev->get<Buffer>(b, "buffer");
        if (!range_fits(offset, size, buf->data.size())) fail(GBR_ERR_VALIDATION, "write_buffer out of range");
        std::memcpy(buf->data.data() + offset, data, size);
    })
}
ORC_API gbr_status orc_buffer_read(gbr_device d, gbr_buffer b, uint64_t offset, void* dst, uint64_t size) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        Buffer* buf = dev->get<Buffer>(b, "buffer");
        if (!range_fits(offset, size, buf->data.size())) fail(GBR_ERR_VALIDATION, "buffer read out of range");
        std::memcpy(dst, buf->data.data() + offset, size);
    })
}
ORC_API gbr_status orc_texture_create(gbr_device d, const gbr_texture_desc* desc, gbr_texture* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        uint32_t bpp = bytes_per_texel(desc->format);
        if (!bpp) fail(GBR_ERR_UNSUPPORTED, "Unsupported texture format: %u", desc->format);
        auto* t = new Texture;
        t->desc = *desc;
        if (t->desc.size.depth_or_array_layers == 0) t->desc.size.depth_or_array_layers = 1;
        t->bpp = bpp;
        // The reference stores mip 0 only (texture.rs:34-43); the extension profile keeps the chain.
        uint32_t mips = desc->mip_level_count ? desc->mip_level_count : 1;
        t->mips_stored = dev->profile == GBR_PROFILE_EXTENSION ? std::min(mips, 16u) : 1;
        t->mips.resize(t->mips_stored);
        for (uint32_t m = 0; m < t->mips_stored; ++m)
            t->mips[m].assign((size_t)t->mip_w(m) * t->mip_h(m) * t->desc.size.depth_or_array_layers * bpp, 0);
        std::lock_guard<std::mutex> lk(dev->mu);
        *out = dev->add(t);
    })
}
ORC_API gbr_status orc_texture_destroy(gbr_device d, gbr_texture t) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<Texture>(t, "texture");
        dev->objects.erase(t);
    })
}
// QueueInterface::write_texture (device.rs:371-434): whole texture, whole rows.
ORC_API gbr_status orc_queue_write_texture(gbr_device d, gbr_texture tex, uint32_t mip, const void* data,
                                           uint64_t data_size, const gbr_texel_copy_buffer_layout* layout,
                                           gbr_extent3d size) {
    ORC_TRY({
        (void)size;  // shadowed by the texture size in the reference (device.rs:388)
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        Texture* t = dev->get<Texture>(tex, "texture");
        if (mip >= t->mips_stored) fail(GBR_ERR_UNSUPPORTED, "write to mip_level %u (device.rs:378-380)", mip);
        uint32_t w = t->mip_w(mip), h = t->mip_h(mip), layers = t->desc.size.depth_or_array_layers;
        uint64_t row = layout->bytes_per_row ? layout->bytes_per_row : data_size;
        uint64_t rows_per_image = layout->rows_per_image ? layout->rows_per_image : h;
        uint64_t dst_row = (uint64_t)w * t->bpp;
        if (row < dst_row) fail(GBR_ERR_VALIDATION, "bytes_per_row too small");
        const uint8_t* src = static_cast<const uint8_t*>(data);
        uint8_t* dst = t->mips[mip].data();
        for (uint32_t z = 0; z < layers; ++z)
            for (uint32_t y = 0; y < h; ++y) {
                uint64_t so = span_end(layout->offset, (uint64_t)z * rows_per_image + y, row, 0);
                if (!range_fits(so, dst_row, data_size)) fail(GBR_ERR_VALIDATION, "write_texture source out of range");
                std::memcpy(dst + ((uint64_t)z * h + y) * dst_row, src + so, dst_row);
            }
    })
}
ORC_API gbr_status orc_texture_read(gbr_device d, gbr_texture tex, uint32_t mip, void* dst, uint64_t size) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        Texture* t = dev->get<Texture>(tex, "texture");
        if (mip >= t->mips_stored) fail(GBR_ERR_VALIDATION, "mip level not stored");
        if (size < t->mips[mip].size()) fail(GBR_ERR_VALIDATION, "destination too small");
        std::memcpy(dst, t->mips[mip].data(), t->mips[mip].size());
    })
}
ORC_API gbr_status orc_sampler_create(gbr_device d, const gbr_sampler_desc* desc, gbr_sampler* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        auto* s = new Sampler;
        s->s.desc = *desc;
        std::lock_guard<std::mutex> lk(dev->mu);
        *out = dev->add(s);
    })
}
ORC_API gbr_status orc_sampler_destroy(gbr_device d, gbr_sampler s) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<Sampler>(s, "sampler");
        dev->objects.erase(s);
    })
}
ORC_API gbr_status orc_shader_module_create_native(gbr_device d, const char* name, gbr_shader_module* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        const Program* p = find_program(name);
        if (!p) fail(GBR_ERR_SHADER, "unknown native program '%s'", name);
        auto* m = new ShaderModule;
        m->prog = p;
        std::lock_guard<std::mutex> lk(dev->mu);
        *out = dev->add(m);
    })
}
ORC_API gbr_status orc_shader_module_destroy(gbr_device d, gbr_shader_module m) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<ShaderModule>(m, "shader module");
        dev->objects.erase(m);
    })
}
ORC_API gbr_status orc_render_pipeline_create(gbr_device d, const gbr_render_pipeline_desc* desc,
                                              gbr_render_pipeline* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        auto pl = std::make_unique<Pipeline>();
        pl->desc = *desc;
        pl->vs = dev->get<ShaderModule>(desc->vertex_module, "shader module")->prog;
        pl->fs = desc->has_fragment ? dev->get<ShaderModule>(desc->fragment_module, "shader module")->prog : nullptr;
        std::memset(pl->loc, 0, sizeof pl->loc);
        if (desc->vertex_buffer_count > GBR_MAX_VERTEX_BUFFERS) fail(GBR_ERR_VALIDATION, "too many vertex buffers");
        // VertexState::new (vertex.rs:50-94): location -> (buffer, offset, size); duplicates panic.
        for (uint32_t b = 0; b < desc->vertex_buffer_count; ++b) {
            const gbr_vertex_buffer_layout& L = desc->vertex_buffers[b];
            for (uint32_t a = 0; a < L.attribute_count && a < GBR_MAX_VERTEX_ATTRIBUTES; ++a) {
                const gbr_vertex_attribute& at = L.attributes[a];
                if (at.shader_location >= 16) fail(GBR_ERR_VALIDATION, "shader location out of range");
                if (pl->loc[at.shader_location].present)
                    fail(GBR_ERR_VALIDATION, "Duplicate vertex attribute at location %u", at.shader_location);
                pl->loc[at.shader_location] = {true, b, at.offset, at.format};
            }
        }
        *out = dev->add(pl.release());
    })
}
ORC_API gbr_status orc_render_pipeline_destroy(gbr_device d, gbr_render_pipeline p) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<Pipeline>(p, "pipeline");
        dev->objects.erase(p);
    })
}
ORC_API gbr_status orc_bind_group_create(gbr_device d, const gbr_bind_group_desc* desc, gbr_bind_group* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        if (!desc || desc->entry_count > GBR_MAX_BIND_GROUP_ENTRIES) fail(GBR_ERR_INVALID_ARGUMENT, "bad descriptor");
        std::lock_guard<std::mutex> lk(dev->mu);
        // buffer entries must lie inside their buffer (a BufferSlice of the reference, bind_group.rs:58-72)
        for (uint32_t e = 0; e < desc->entry_count; ++e) {
            const gbr_bind_group_entry& en = desc->entries[e];
            if (en.kind != GBR_BINDING_BUFFER) continue;
            Buffer* b = dev->get<Buffer>(en.resource, "buffer");
            if (en.offset > b->data.size() || (en.size && !range_fits(en.offset, en.size, b->data.size())))
                fail(GBR_ERR_VALIDATION, "bind group buffer range out of bounds");
        }
        auto* g = new BindGroup;
        g->desc = *desc;
        *out = dev->add(g);
    })
}
ORC_API gbr_status orc_bind_group_destroy(gbr_device d, gbr_bind_group g) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        dev->get<BindGroup>(g, "bind group");
        dev->objects.erase(g);
    })
}
// Submission executes immediately on the calling thread (the engine loop of engine.rs:26-46
// without the thread hop).
// Encoder copies and clears (extension profile; the reference has them as todo!,
// command.rs:37-115), with WebGPU's validation rules, on the host copies of the resources.
static void execute_copy(Device* dev, const gbr_cmd_header& h, const uint8_t* b) {
    static const char* const kNames[] = {"copy_buffer_to_buffer", "copy_buffer_to_texture", "copy_texture_to_buffer",
                                         "copy_texture_to_texture", "clear_buffer", "clear_texture"};
    static const char* const kLines[] = {"37-46", "48-55", "57-64", "66-73", "108-115", "100-106"};
    const uint32_t k = h.opcode - GBR_OP_COPY_BUFFER_TO_BUFFER;
    if (dev->profile != GBR_PROFILE_EXTENSION)
        fail(GBR_ERR_UNSUPPORTED, "%s is todo!() (command.rs:%s)", kNames[k], kLines[k]);
    auto region_ok = [](const Texture* t, uint32_t mip, uint32_t x, uint32_t y, uint32_t z, const gbr_extent3d& e) {
        const uint32_t layers = t->desc.size.depth_or_array_layers ? t->desc.size.depth_or_array_layers : 1;
        if (mip >= t->mips_stored) fail(GBR_ERR_VALIDATION, "copy: mip level %u not stored", mip);
        if ((uint64_t)x + e.width > t->mip_w(mip) || (uint64_t)y + e.height > t->mip_h(mip) ||
            (uint64_t)z + e.depth_or_array_layers > layers)
            fail(GBR_ERR_VALIDATION, "copy: texture region out of range");
    };
    auto texel = [](Texture* t, uint32_t mip, uint32_t x, uint32_t y, uint32_t z) {
        return t->mips[mip].data() + (((size_t)z * t->mip_h(mip) + y) * t->mip_w(mip) + x) * t->bpp;
    };
    switch (h.opcode) {
        case GBR_OP_COPY_BUFFER_TO_BUFFER: {
            auto* p = payload<gbr_cmd_copy_buffer_to_buffer>(&h, b);
            Buffer* src = dev->get<Buffer>(p->source, "buffer");
            Buffer* dst = dev->get<Buffer>(p->destination, "buffer");
            const uint64_t size = p->size == UINT64_MAX ? src->data.size() - std::min<uint64_t>(p->source_offset,
                                                                                              src->data.size())
                                                        : p->size;
            if (src == dst) fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: source and destination are the same buffer");
            if (p->source_offset % 4 || p->destination_offset % 4 || size % 4)
                fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: alignment");
            if (!range_fits(p->source_offset, size, src->data.size()) || !range_fits(p->destination_offset, size, dst->data.size()))
                fail(GBR_ERR_VALIDATION, "copy_buffer_to_buffer: range out of bounds");
            std::memcpy(dst->data.data() + p->destination_offset, src->data.data() + p->source_offset, size);
            break;
        }
        case GBR_OP_COPY_BUFFER_TO_TEXTURE:
        case GBR_OP_COPY_TEXTURE_TO_BUFFER: {
            auto* p = payload<gbr_cmd_copy_buffer_texture>(&h, b);
            Buffer* buf = dev->get<Buffer>(p->buffer, "buffer");
            Texture* t = dev->get<Texture>(p->texture.texture, "texture");
            const gbr_extent3d e = p->size;
            region_ok(t, p->texture.mip_level, p->texture.origin_x, p->texture.origin_y, p->texture.origin_z, e);
            const uint64_t width = (uint64_t)e.width * t->bpp;
            const uint64_t bpr = p->layout.bytes_per_row ? p->layout.bytes_per_row : width;
            const uint64_t rpi = p->layout.rows_per_image ? p->layout.rows_per_image : e.height;
            if ((e.height > 1 || e.depth_or_array_layers > 1) && (p->layout.bytes_per_row % 256 || !p->layout.bytes_per_row))
                fail(GBR_ERR_VALIDATION, "%s: bytes_per_row must be a multiple of 256", kNames[k]);
            if (bpr < width || rpi < e.height) fail(GBR_ERR_VALIDATION, "%s: layout smaller than the copy", kNames[k]);
            if (p->layout.offset % t->bpp) fail(GBR_ERR_VALIDATION, "%s: offset not a multiple of the texel size", kNames[k]);
            if (!e.width || !e.height || !e.depth_or_array_layers) break;
            const uint64_t need = span_end(p->layout.offset, (uint64_t)(e.depth_or_array_layers - 1) * rpi + (e.height - 1), bpr, width);
            if (need > buf->data.size()) fail(GBR_ERR_VALIDATION, "%s: buffer range out of bounds", kNames[k]);
            for (uint32_t z = 0; z < e.depth_or_array_layers; ++z)
                for (uint32_t y = 0; y < e.height; ++y) {
                    uint8_t* tp = texel(t, p->texture.mip_level, p->texture.origin_x, p->texture.origin_y + y,
                                        p->texture.origin_z + z);
                    uint8_t* bp = buf->data.data() + p->layout.offset + (z * rpi + y) * bpr;
                    if (h.opcode == GBR_OP_COPY_BUFFER_TO_TEXTURE) std::memcpy(tp, bp, width);
                    else std::memcpy(bp, tp, width);
                }
            break;
        }
        case GBR_OP_COPY_TEXTURE_TO_TEXTURE: {
            auto* p = payload<gbr_cmd_copy_texture_to_texture>(&h, b);
            Texture* a = dev->get<Texture>(p->source.texture, "texture");
            Texture* c = dev->get<Texture>(p->destination.texture, "texture");
            const gbr_extent3d e = p->size;
            if (a->desc.format != c->desc.format) fail(GBR_ERR_VALIDATION, "copy_texture_to_texture: formats differ");
            region_ok(a, p->source.mip_level, p->source.origin_x, p->source.origin_y, p->source.origin_z, e);
            region_ok(c, p->destination.mip_level, p->destination.origin_x, p->destination.origin_y,
                      p->destination.origin_z, e);
            if (a == c && p->source.mip_level == p->destination.mip_level &&
                p->source.origin_z < p->destination.origin_z + e.depth_or_array_layers &&
                p->destination.origin_z < p->source.origin_z + e.depth_or_array_layers)
                fail(GBR_ERR_VALIDATION, "copy_texture_to_texture: source and destination overlap");
            for (uint32_t z = 0; z < e.depth_or_array_layers; ++z)
                for (uint32_t y = 0; y < e.height; ++y)
                    std::memcpy(texel(c, p->destination.mip_level, p->destination.origin_x, p->destination.origin_y + y,
                                      p->destination.origin_z + z),
                                texel(a, p->source.mip_level, p->source.origin_x, p->source.origin_y + y,
                                      p->source.origin_z + z),
                                (size_t)e.width * a->bpp);
            break;
        }
        case GBR_OP_CLEAR_BUFFER: {
            auto* p = payload<gbr_cmd_clear_buffer>(&h, b);
            Buffer* buf = dev->get<Buffer>(p->buffer, "buffer");
            const uint64_t size = p->size == UINT64_MAX ? buf->data.size() - std::min<uint64_t>(p->offset, buf->data.size())
                                                        : p->size;
            if (p->offset % 4 || size % 4) fail(GBR_ERR_VALIDATION, "clear_buffer: alignment");
            if (!range_fits(p->offset, size, buf->data.size())) fail(GBR_ERR_VALIDATION, "clear_buffer: range out of bounds");
            std::memset(buf->data.data() + p->offset, 0, size);
            break;
        }
        case GBR_OP_CLEAR_TEXTURE: {
            auto* p = payload<gbr_cmd_clear_texture>(&h, b);
            Texture* t = dev->get<Texture>(p->texture, "texture");
            const uint32_t layers = t->desc.size.depth_or_array_layers ? t->desc.size.depth_or_array_layers : 1;
            if (p->base_mip_level >= t->mips_stored || p->base_array_layer >= layers)
                fail(GBR_ERR_VALIDATION, "clear_texture: subresource range out of range");
            const uint32_t mc = p->mip_level_count ? p->mip_level_count : t->mips_stored - p->base_mip_level;
            const uint32_t lc = p->array_layer_count ? p->array_layer_count : layers - p->base_array_layer;
            if ((uint64_t)p->base_mip_level + mc > t->mips_stored || (uint64_t)p->base_array_layer + lc > layers)
                fail(GBR_ERR_VALIDATION, "clear_texture: subresource range out of range");
            for (uint32_t m = p->base_mip_level; m < p->base_mip_level + mc; ++m) {
                const size_t layer = (size_t)t->mip_w(m) * t->mip_h(m) * t->bpp;
                std::memset(t->mips[m].data() + p->base_array_layer * layer, 0, lc * layer);
            }
            break;
        }
        default: break;
    }
}

ORC_API gbr_status orc_queue_submit(gbr_device d, const void* cmds, uint64_t len, uint64_t* out_index) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        auto passes = decode_stream(static_cast<const uint8_t*>(cmds), len);
        uint64_t idx = dev->next_submission++;
        Counters total;
        uint64_t draws = 0;
        for (const auto& p : passes)
            for (const auto& c : p.cmds)
                if (c.first.opcode == GBR_OP_DRAW || c.first.opcode == GBR_OP_DRAW_INDEXED) ++draws;
        for (size_t i = 0; i < passes.size();) {
            if (passes[i].is_copy) {
                execute_copy(dev, passes[i].cmds[0].first, passes[i].cmds[0].second.data());
                ++i;
                continue;
            }
            const size_t j = independent_run(dev, passes, i);
            if (g_threads > 1 && j - i > 1) {
                execute_passes_parallel(dev, passes, i, j, total);
            } else {
                for (size_t k = i; k < j; ++k) execute_pass(dev, passes[k], total, g_threads);
            }
            i = j;
        }
        gbr_submission_stats s;
        std::memset(&s, 0, sizeof s);
        s.submission_index = idx;
        s.draws = draws;
        s.primitives_in = total.primitives;
        s.fragments_shaded = total.fragments;
        s.fs_invocations = total.fs_runs;
        s.texture_fs_invocations = total.tex_runs;
        s.batched_with = 1;
        dev->stats[idx] = s;
        if (out_index) *out_index = idx;
    })
}
ORC_API gbr_status orc_device_poll(gbr_device d, uint32_t wait, uint32_t has_index, uint64_t index, uint64_t timeout_ns,
                                   uint32_t* out_status) {
    ORC_TRY({
        (void)has_index;
        (void)index;
        (void)timeout_ns;
        get_device(d);
        if (out_status) *out_status = wait ? GBR_POLL_QUEUE_EMPTY : GBR_POLL_POLL;
    })
}
ORC_API gbr_status orc_submission_stats_get(gbr_device d, uint64_t index, gbr_submission_stats* out) {
    ORC_TRY({
        Device* dev = get_device(d);
        std::lock_guard<std::mutex> lk(dev->mu);
        auto it = dev->stats.find(index);
        if (it == dev->stats.end()) fail(GBR_ERR_INVALID_ARGUMENT, "unknown submission");
        *out = it->second;
    })
}

// ------------------------------------------------------------------ stage-level entry points
// used by the known-answer tests that replay the reference's unit tests.

// TriClipper::clip_tri; out: per triangle 3 x (x, y, z, w, b0, b1, b2).  Returns the count.
ORC_API int orc_kat_clip_tri(const float* pos12, float* out, int max_tris) {
    V4 pos[3];
    for (int i = 0; i < 3; ++i) pos[i] = {pos12[4 * i], pos12[4 * i + 1], pos12[4 * i + 2], pos12[4 * i + 3]};
    std::vector<ClipTri> r;
    clip_tri(pos, r);
    int n = (int)r.size();
    for (int t = 0; t < n && t < max_tris; ++t)
        for (int i = 0; i < 3; ++i) {
            float* o = out + (t * 3 + i) * 7;
            const ClipVertex& v = r[t].v[i];
            o[0] = v.position.x;
            o[1] = v.position.y;
            o[2] = v.position.z;
            o[3] = v.position.w;
            o[4] = v.bary.c[0];
            o[5] = v.bary.c[1];
            o[6] = v.bary.c[2];
        }
    return n;
}
// cohen_sutherland::clip; returns 1 with out8/alphas2 filled, 0 for None.
ORC_API int orc_kat_clip_line(const float* pos8, float* out8, float* alphas2) {
    V4 p[2] = {{pos8[0], pos8[1], pos8[2], pos8[3]}, {pos8[4], pos8[5], pos8[6], pos8[7]}};
    if (!clip_line(p, alphas2)) return 0;
    float v[8] = {p[0].x, p[0].y, p[0].z, p[0].w, p[1].x, p[1].y, p[1].z, p[1].w};
    std::memcpy(out8, v, sizeof v);
    return 1;
}
// scanlines; out rows of (y, x1, x2).  Returns the row count or -1 when the reference panics.
ORC_API int orc_kat_scanlines(const uint32_t* xy6, int64_t* out, int max_rows) {
    uint32_t fx[3] = {xy6[0], xy6[2], xy6[4]}, fy[3] = {xy6[1], xy6[3], xy6[5]};
    int n = 0;
    bool ok = scanlines(fx, fy, [&](const Scanline& s) {
        if (n < max_rows) {
            out[3 * n] = s.y;
            out[3 * n + 1] = s.x1;
            out[3 * n + 2] = s.x2;
        }
        ++n;
    });
    return ok ? n : -1;
}
ORC_API void orc_kat_bubblesort3(int64_t* v) {
    bubblesort3(v, [](int64_t x) { return x; });
}
ORC_API int orc_kat_bresenham(uint32_t sx, uint32_t sy, uint32_t ex, uint32_t ey, uint32_t* out_xy, float* out_t,
                              int max_pts) {
    int n = 0;
    bresenham(sx, sy, ex, ey, [&](uint32_t x, uint32_t y, float t) {
        if (n < max_pts) {
            out_xy[2 * n] = x;
            out_xy[2 * n + 1] = y;
            out_t[n] = t;
        }
        ++n;
    });
    return n;
}
// TriFace::front_face: 1 = Ccw, 0 = Cw, -1 = w == 0.
ORC_API int orc_kat_tri_face(const float* pos12) {
    V4 pos[3];
    for (int i = 0; i < 3; ++i) pos[i] = {pos12[4 * i], pos12[4 * i + 1], pos12[4 * i + 2], pos12[4 * i + 3]};
    bool ccw;
    if (!tri_face_ccw(pos, &ccw)) return -1;
    return ccw ? 1 : 0;
}
ORC_API void orc_kat_strip_tri(uint32_t p, uint32_t* out3) { strip_tri(p, out3); }
ORC_API uint16_t orc_kat_f32_to_f16(float f) { return f32_to_f16_rne(f); }
ORC_API float orc_kat_f16_to_f32(uint16_t h) { return f16_to_f32(h); }
// TextureDataLayout::byte_size (texture.rs:251-302)
ORC_API uint64_t orc_kat_texture_byte_size(uint32_t w, uint32_t h, uint32_t layers, uint32_t format) {
    return (uint64_t)w * h * layers * bytes_per_texel(format);
}
