// wgsl.h — WGSL front end and CUDA emitter for the render-pass programs.
//
// A WGSL module is parsed into an AST (the subset naga-cranelift executes: scalar / vector /
// matrix f32, i32, u32, bool; structs; let / var / const, private and uniform globals;
// if / for / loop / while / switch / break / continue / return / discard; user functions;
// casts; select; textureSample; plus swizzles and splats, which are exact copies).  A vertex and
// a fragment entry point are then emitted as CUDA device functions (`jit_vs`, `jit_fs`) with
// naga-cranelift's arithmetic: one rounded IEEE operation per WGSL operator in source order, no
// contraction, mat4x4 * vec4 as the column sum ((v0*c0 + v1*c1) + v2*c2) + v3*c3
// (naga-cranelift/src/expression/binary.rs:273-325), Rust `as` casts (expression/as.rs:60-160),
// integer division and remainder by zero as traps (tests.rs, trap_divide_by_zero).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbr {
namespace wgsl {

// A parse / validation failure: `unsupported` marks features outside the subset.
struct Error : std::runtime_error {
    bool unsupported;
    Error(const std::string& m, bool u) : std::runtime_error(m), unsupported(u) {}
};

struct Module;  // parsed module (opaque)

std::shared_ptr<Module> parse(const std::string& source);

// Entry points of a module: name and stage (0 = vertex, 1 = fragment).
std::vector<std::pair<std::string, int>> entry_points(const Module& m);

// What the raster path needs to know about an emitted vertex + fragment program.
struct ProgramCode {
    std::string cuda;               // defines jit_vs and (if any) jit_fs
    uint32_t num_varyings = 0;      // f32 inter-stage values per vertex
    bool perspective = false;       // interpolation of the non-flat inter-stage values (one mode per program)
    uint32_t flat_mask = 0;         // bit k: inter-stage float k is @interpolate(flat)
    uint32_t early_depth = 0;       // fragment entry point's @early_depth_test: 0 none, 1 force, 2 allow
    bool may_discard = false;
    bool uses_position = false;     // the fragment stage reads @builtin(position)
    int input_loc[16];              // vertex inputs: location and f32 component count
    int input_comps[16];
    int input_kind[16];             // 0 = f32, 1 = i32, 2 = u32
    int num_inputs = 0;
    uint32_t uniform_size[4][8] = {};  // bytes each uniform binding must hold (0 = unused)
    int tex_group = -1, tex_binding = -1, samp_group = -1, samp_binding = -1;
};

// Pipeline-overridable constants of one stage (PipelineCompilationOptions::constants): key (an
// override's @id as a decimal string, or its name) -> value.
using Constants = std::map<std::string, double>;

// Emits the program of `vs_entry` (in vs) and, when fs is given, `fs_entry` (in fs), with the
// stages' override values.
ProgramCode emit_program(const Module& vs, const std::string& vs_entry, const Module* fs, const std::string& fs_entry,
                         const Constants& vertex_constants = {}, const Constants& fragment_constants = {});

}  // namespace wgsl
}  // namespace gbr
