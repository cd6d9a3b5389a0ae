// Per-flame device code generation.
//
// Plays the role of flame_compiler::make_source + assets/templates/flame.tpl
// (src/librefrakt/src/flame_compiler.cpp:448-580): for each xform it emits a
// function that applies the vlink chain (affine, then the sum of weighted
// variations with the vlink's commons computed first, flame.tpl:46-79), blends
// the colour (INTERP, flame.tpl:154) and returns the opacity; a dispatch
// switch over the standard xforms (flame.tpl:146-160); and the variation
// precalc code (flame.tpl:59-66). Parameters are read from the per-sample
// parameter block at compile-time offsets that follow the pack_sample layout.
#pragma once

#include <string>
#include <vector>

#include "flamedb.h"
#include "genome.h"

namespace rfk {

struct xform_info {
    size_t base = 0;          // offset of weight in the packed sample
    int rand_calls = 0;       // upper bound of uniform draws per application
    int sfu_ops = 0;          // transcendental calls per application
    int affines = 0;          // vlink affines per application
};

struct generated_flame {
    std::string source;       // device code (defines + functions)
    size_t size_reals = 0;
    size_t num_xforms = 0;
    bool has_final = false;
    bool chaos = false;
    std::vector<size_t> affine_indices;
    std::vector<xform_info> xforms;  // standard xforms, then the final xform
};

generated_flame generate_flame_code(const flamedb& db, const flame& f);

}  // namespace rfk
