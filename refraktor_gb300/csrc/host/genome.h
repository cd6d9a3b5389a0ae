// Flame genome and its packed sample layout.
//
// Value types mirror rfkt::affine / vardata / vlink / xform / flame
// (src/librefrakt/include/librefrakt/flame_types.h:109-807). Animated values
// (anima with a call) are host-side parameter curves that this library does
// not evaluate: every value is its t0, as anima::sample returns when no call
// is attached (flame_types.h:67-71).
//
// pack_sample() produces exactly the reference layout (flame_types.h:634-672),
// which the device code addresses with compile-time offsets:
//   [0..5]   screen-space affine a,d,b,e,c,f      (flame_types.h:616-622)
//   [6..11]  plane-space affine a,d,b,e,c,f       (flame_types.h:624-631)
//   [12]     weight-sum slot (filled on device)
//   chaos:   per xform row: sum slot + one weight per xform
//   xforms:  weight, color, color_speed, opacity, then per vlink the affine
//            (after mod_scale / mod_rotate / mod_x,y) and per variation in
//            name order: weight, ordinary params in name order, one zero per
//            precalc param (flame_types.h:250-260, 375-400, 484-494)
//   final xform (if any), then 256 x (hue, saturation, value).
#pragma once

#include <array>
#include <map>
#include <optional>
#include <string>
#include <vector>

#include "flamedb.h"
#include "value.h"

namespace rfk {

struct affine {
    // [a b c]
    // [d e f]
    double a = 0, d = 0, b = 0, e = 0, c = 0, f = 0;

    static affine identity() { return {1, 0, 0, 1, 0, 0}; }
    affine translated(double x, double y) const;  // flame_types.h:142-148
    affine scaled(double s) const;                // flame_types.h:138-140
    affine rotated(double deg) const;             // flame_types.h:121-136
};

struct vardata {
    double weight = 0;
    std::map<std::string, double> params;  // ordinary params, sorted
    size_t precalc_count = 0;
    size_t size_reals() const { return 1 + params.size() + precalc_count; }
};

struct vlink {
    affine transform;
    double mod_x = 0, mod_y = 0, mod_scale = 1, mod_rotate = 0;
    std::map<std::string, vardata> variations;  // sorted by name
    size_t size_reals() const;
};

struct xform {
    double weight = 0, color = 0, color_speed = 0, opacity = 1;
    std::vector<vlink> vchain;
    size_t size_reals() const;
};

struct flame {
    std::string name;
    std::vector<xform> xforms;
    std::optional<xform> final_xform;
    std::optional<std::vector<std::vector<double>>> chaos;  // [from][to]

    double center_x = 0, center_y = 0, scale = 1, rotate = 0;
    double gamma = 4, brightness = 1, vibrancy = 1, highlight_power = -1, gamma_threshold = 0.01;
    double mod_hue = 0, mod_sat = 0, mod_val = 0;
    std::vector<std::array<double, 3>> palette;  // HSV: hue in degrees, s and v in [0, 1]

    size_t size_reals() const;                      // flame_types.h:602-613
    std::vector<size_t> affine_indices() const;     // flame_types.h:674-705
    affine screen_space(int w, int h) const;        // flame_types.h:616-622
    affine plane_space(int w, int h) const;         // flame_types.h:624-631
    void pack_sample(std::vector<double>& out, int w, int h) const;

    // Structure key: what forces a new kernel (xform count, vlink chains and
    // their variation names, final xform, chaos) - flame_types.h:578-592.
    std::string structure_key() const;
    uint64_t structure_hash() const { return fnv1a(structure_key()); }
};

constexpr size_t palette_reals = 256 * 3;

// Genome JSON in the reference format (flame_types.cpp:241-485). The palette
// may be the reference's zlib+base64 string of 256 x 3 doubles, or a plain
// array of [h, s, v] triples.
flame flame_from_json(const flamedb& db, const value& js);
value flame_to_json(const flame& f);

// flam3 XML import (flame_types.cpp:33-239).
flame flame_from_flam3(const flamedb& db, const std::string& xml);

// New vardata with defaults for `name` (flame_info.cpp:224-237).
vardata make_vardata(const flamedb& db, const std::string& name);

// A vlink that maps (nearly) as the identity but carries the variations of
// `vl`, to pad a vlink chain (flamedb::make_padder, flame_info.cpp:239-320).
vlink make_padder(const flamedb& db, const vlink& vl);

// Gives genomes one structure (xform count, vlink chains, variation sets,
// final xform, chaos rows) without changing what each one renders: the
// reference interpolator's alignment (src/refraktor/src/refraktor.cpp:117-191)
// for any number of genomes. by_weight: every genome carries all genomes'
// xforms, the foreign ones with weight 0; otherwise xforms align by position.
std::vector<flame> align_structures(const flamedb& db, const std::vector<flame>& flames, bool by_weight);

// FP64 rotation fix-up of packed samples before spline interpolation
// (src/librefrakt/src/flame_compiler.cpp:957-1035): every affine's linear
// columns become (angle, log magnitude) with angles unwrapped across samples,
// and palette hues are unwrapped across +-180 degrees.
void fix_rotation(std::vector<double>& samples, size_t sample_size, size_t flame_size,
                  const std::vector<size_t>& affine_indices);

// RGB <-> HSV (src/librefrakt/src/util/color.cpp).
std::array<double, 3> rgb_to_hsv(double r, double g, double b);

}  // namespace rfk
