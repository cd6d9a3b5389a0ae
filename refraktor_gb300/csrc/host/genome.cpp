#include "genome.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <sstream>

#include "inflate.h"

namespace rfk {

static constexpr double kPi = 3.14159265358979323846;

affine affine::translated(double x, double y) const {
    return {a, d, b, e, a * x + b * y + c, d * x + e * y + f};
}

affine affine::scaled(double s) const { return {a * s, d * s, b * s, e * s, c, f}; }

affine affine::rotated(double deg) const {
    // The reference builds the 2x2 part into a matrix and post-multiplies a
    // rotation by -deg about z (glm::rotate). Written out:
    //   a' = a cos + d sin,  d' = d cos - a sin,
    //   b' = b cos + e sin,  e' = e cos - b sin.
    double rad = -deg * kPi / 180.0;
    double cs = std::cos(rad), sn = std::sin(rad);
    return {a * cs + d * sn, -a * sn + d * cs, b * cs + e * sn, -b * sn + e * cs, c, f};
}

size_t vlink::size_reals() const {
    size_t s = 6;
    for (auto& [_, v] : variations) s += v.size_reals();
    return s;
}

size_t xform::size_reals() const {
    size_t s = 4;
    for (auto& vl : vchain) s += vl.size_reals();
    return s;
}

size_t flame::size_reals() const {
    size_t s = final_xform ? final_xform->size_reals() : 0;
    if (chaos) s += xforms.size() * (xforms.size() + 1);
    for (auto& xf : xforms) s += xf.size_reals();
    return s + 13;
}

std::vector<size_t> flame::affine_indices() const {
    std::vector<size_t> ret = {0, 6};
    size_t index = 13 + (chaos ? xforms.size() * (xforms.size() + 1) : 0);
    auto walk = [&](const xform& xf) {
        index += 4;
        for (auto& vl : xf.vchain) {
            ret.push_back(index);
            index += vl.size_reals();
        }
    };
    for (auto& xf : xforms) walk(xf);
    if (final_xform) walk(*final_xform);
    return ret;
}

affine flame::screen_space(int w, int h) const {
    return affine::identity()
        .translated(w / 2.0, h / 2.0)
        .scaled(scale * h)
        .rotated(rotate)
        .translated(-center_x, -center_y);
}

affine flame::plane_space(int w, int h) const {
    return affine::identity()
        .translated(center_x, center_y)
        .rotated(-rotate)
        .scaled(1 / (scale * h))
        .translated(w / -2.0, h / -2.0);
}

static void pack_affine(std::vector<double>& o, const affine& a) {
    o.push_back(a.a);
    o.push_back(a.d);
    o.push_back(a.b);
    o.push_back(a.e);
    o.push_back(a.c);
    o.push_back(a.f);
}

static void pack_xform(std::vector<double>& o, const xform& xf) {
    o.push_back(xf.weight);
    o.push_back(xf.color);
    o.push_back(xf.color_speed);
    o.push_back(xf.opacity);
    for (auto& vl : xf.vchain) {
        pack_affine(o, vl.transform.scaled(vl.mod_scale).rotated(vl.mod_rotate).translated(vl.mod_x, vl.mod_y));
        for (auto& [_, v] : vl.variations) {
            o.push_back(v.weight);
            for (auto& [__, pv] : v.params) o.push_back(pv);
            for (size_t i = 0; i < v.precalc_count; i++) o.push_back(0.0);
        }
    }
}

void flame::pack_sample(std::vector<double>& o, int w, int h) const {
    if (palette.size() != 256) throw format_error("palette must have 256 entries, has " + std::to_string(palette.size()));
    pack_affine(o, screen_space(w, h));
    pack_affine(o, plane_space(w, h));
    o.push_back(0.0);
    if (chaos) {
        for (auto& row : *chaos) {
            o.push_back(0.0);
            for (double v : row) o.push_back(v);
        }
    }
    for (auto& xf : xforms) pack_xform(o, xf);
    if (final_xform) pack_xform(o, *final_xform);
    for (auto& hsv : palette) {
        o.push_back(std::fmod(hsv[0] + mod_hue, 360.0));
        o.push_back(std::clamp(hsv[1] + mod_sat, 0.0, 1.0));
        o.push_back(std::clamp(hsv[2] + mod_val, 0.0, 1.0));
    }
}

std::string flame::structure_key() const {
    std::ostringstream k;
    auto xk = [&](const xform& xf) {
        k << "{";
        for (auto& vl : xf.vchain) {
            k << "[";
            for (auto& [n, _] : vl.variations) k << n << ",";
            k << "]";
        }
        k << "}";
    };
    k << "X" << xforms.size();
    for (auto& xf : xforms) xk(xf);
    if (final_xform) {
        k << "F";
        xk(*final_xform);
    }
    if (chaos) k << "C";
    return k.str();
}

vardata make_vardata(const flamedb& db, const std::string& name) {
    const auto& def = db.get_variation(name);
    vardata v;
    for (auto& [pn, p] : def.params) {
        if (p.is_precalc()) v.precalc_count++;
        else v.params[pn] = p.default_value.value_or(0.0);
    }
    return v;
}

// ---------------------------------------------------------------- JSON ----
namespace {

double anima_value(const value& v, const char* what) {
    if (v.is_number()) return v.num;
    if (v.is_object()) {
        if (auto* t0 = v.find("t0"); t0 && t0->is_number()) return t0->num;
    }
    throw format_error(std::string("bad value for ") + what);
}

double field(const value& js, const char* name) {
    auto* v = js.find(name);
    if (!v) throw format_error(std::string("missing field '") + name + "'");
    return anima_value(*v, name);
}

vardata vardata_from_json(const flamedb& db, const std::string& name, const value& js) {
    if (!db.is_variation(name)) throw format_error("unknown variation '" + name + "'");
    vardata v = make_vardata(db, name);
    if (js.is_number() || (js.is_object() && js.contains("t0"))) {
        if (!v.params.empty()) throw format_error("variation '" + name + "' needs a parameter object");
        v.weight = anima_value(js, "weight");
        return v;
    }
    if (!js.is_object()) throw format_error("bad variation entry '" + name + "'");
    v.weight = field(js, "weight");
    if (auto* ps = js.find("parameters")) {
        if (!ps->is_object()) throw format_error("parameters of '" + name + "' must be an object");
        for (auto& [pn, pv] : ps->obj) {
            if (!v.params.count(pn)) throw format_error("variation '" + name + "' has no parameter '" + pn + "'");
            v.params[pn] = anima_value(pv, pn.c_str());
        }
    }
    return v;
}

affine affine_from_json(const value& js) {
    if (!js.is_array() || js.arr.size() != 6) throw format_error("affine must be an array of 6");
    return {anima_value(js.arr[0], "a"), anima_value(js.arr[1], "d"), anima_value(js.arr[2], "b"),
            anima_value(js.arr[3], "e"), anima_value(js.arr[4], "c"), anima_value(js.arr[5], "f")};
}

xform xform_from_json(const flamedb& db, const value& js) {
    if (!js.is_object()) throw format_error("xform must be an object");
    xform xf;
    xf.weight = field(js, "weight");
    xf.color = field(js, "color");
    xf.color_speed = field(js, "color_speed");
    xf.opacity = field(js, "opacity");
    auto* vc = js.find("vchain");
    if (!vc || !vc->is_array()) throw format_error("xform needs a vchain array");
    for (auto& l : vc->arr) {
        if (!l.is_object()) throw format_error("vlink must be an object");
        vlink vl;
        vl.transform = affine_from_json(l.at("transform"));
        vl.mod_x = field(l, "mod_x");
        vl.mod_y = field(l, "mod_y");
        vl.mod_scale = field(l, "mod_scale");
        vl.mod_rotate = field(l, "mod_rotate");
        auto* vars = l.find("variations");
        if (!vars || !vars->is_object()) throw format_error("vlink needs a variations object");
        for (auto& [vn, vv] : vars->obj) vl.variations[vn] = vardata_from_json(db, vn, vv);
        xf.vchain.push_back(std::move(vl));
    }
    return xf;
}

value num(double d) { return value::make_number(d); }

value xform_to_json(const xform& xf) {
    value o = value::make_object();
    o.set("weight", num(xf.weight));
    o.set("color", num(xf.color));
    o.set("color_speed", num(xf.color_speed));
    o.set("opacity", num(xf.opacity));
    value chain = value::make_array();
    for (auto& vl : xf.vchain) {
        value l = value::make_object();
        value t = value::make_array();
        for (double c : {vl.transform.a, vl.transform.d, vl.transform.b, vl.transform.e, vl.transform.c, vl.transform.f})
            t.arr.push_back(num(c));
        l.set("transform", t);
        l.set("mod_x", num(vl.mod_x));
        l.set("mod_y", num(vl.mod_y));
        l.set("mod_scale", num(vl.mod_scale));
        l.set("mod_rotate", num(vl.mod_rotate));
        value vars = value::make_object();
        for (auto& [vn, vd] : vl.variations) {
            if (vd.params.empty()) {
                vars.set(vn, num(vd.weight));
            } else {
                value e = value::make_object();
                e.set("weight", num(vd.weight));
                value ps = value::make_object();
                for (auto& [pn, pv] : vd.params) ps.set(pn, num(pv));
                e.set("parameters", ps);
                vars.set(vn, e);
            }
        }
        l.set("variations", vars);
        chain.arr.push_back(l);
    }
    o.set("vchain", chain);
    return o;
}

}  // namespace

flame flame_from_json(const flamedb& db, const value& js) {
    if (!js.is_object()) throw format_error("flame must be a JSON object");
    flame f;
    if (auto* n = js.find("name"); n && n->is_string()) f.name = n->str;
    f.center_x = field(js, "center_x");
    f.center_y = field(js, "center_y");
    f.scale = field(js, "scale");
    f.rotate = field(js, "rotate");
    f.gamma = field(js, "gamma");
    f.brightness = field(js, "brightness");
    f.vibrancy = field(js, "vibrancy");
    f.highlight_power = field(js, "highlight_power");
    f.gamma_threshold = field(js, "gamma_threshold");
    f.mod_hue = field(js, "mod_hue");
    f.mod_sat = field(js, "mod_sat");
    f.mod_val = field(js, "mod_val");
    auto* xfs = js.find("xforms");
    if (!xfs || !xfs->is_array()) throw format_error("flame needs an xforms array");
    for (auto& x : xfs->arr) f.xforms.push_back(xform_from_json(db, x));
    if (auto* fx = js.find("final_xform")) f.final_xform = xform_from_json(db, *fx);
    if (auto* ch = js.find("chaos")) {
        if (!ch->is_array() || ch->arr.size() != f.xforms.size()) throw format_error("chaos must be an X by X array");
        std::vector<std::vector<double>> rows;
        for (auto& r : ch->arr) {
            if (!r.is_array() || r.arr.size() != f.xforms.size()) throw format_error("chaos must be an X by X array");
            std::vector<double> row;
            for (auto& c : r.arr) row.push_back(anima_value(c, "chaos"));
            rows.push_back(row);
        }
        f.chaos = rows;
    }
    auto* pal = js.find("palette");
    if (!pal) throw format_error("flame needs a palette");
    if (pal->is_string()) {
        // zlib stream of 256 x 3 doubles, base64 encoded (flame_types.cpp:429-432)
        std::vector<uint8_t> raw = zlib_uncompress(base64_decode(pal->str));
        if (raw.size() % (3 * sizeof(double)) != 0) throw format_error("palette blob has a bad size");
        size_t n = raw.size() / (3 * sizeof(double));
        f.palette.resize(n);
        for (size_t i = 0; i < n; i++) std::memcpy(f.palette[i].data(), raw.data() + i * 24, 24);
    } else if (pal->is_array()) {
        for (auto& e : pal->arr) {
            if (!e.is_array() || e.arr.size() != 3) throw format_error("palette entries must be [h, s, v]");
            f.palette.push_back({e.arr[0].as_number(), e.arr[1].as_number(), e.arr[2].as_number()});
        }
    } else {
        throw format_error("palette must be a string or an array");
    }
    return f;
}

value flame_to_json(const flame& f) {
    value o = value::make_object();
    if (!f.name.empty()) o.set("name", value::make_string(f.name));
    o.set("center_x", num(f.center_x));
    o.set("center_y", num(f.center_y));
    o.set("scale", num(f.scale));
    o.set("rotate", num(f.rotate));
    o.set("gamma", num(f.gamma));
    o.set("brightness", num(f.brightness));
    o.set("vibrancy", num(f.vibrancy));
    o.set("highlight_power", num(f.highlight_power));
    o.set("gamma_threshold", num(f.gamma_threshold));
    o.set("mod_hue", num(f.mod_hue));
    o.set("mod_sat", num(f.mod_sat));
    o.set("mod_val", num(f.mod_val));
    value xfs = value::make_array();
    for (auto& xf : f.xforms) xfs.arr.push_back(xform_to_json(xf));
    o.set("xforms", xfs);
    if (f.final_xform) o.set("final_xform", xform_to_json(*f.final_xform));
    if (f.chaos) {
        value ch = value::make_array();
        for (auto& r : *f.chaos) {
            value row = value::make_array();
            for (double c : r) row.arr.push_back(num(c));
            ch.arr.push_back(row);
        }
        o.set("chaos", ch);
    }
    value pal = value::make_array();
    for (auto& e : f.palette) {
        value t = value::make_array();
        for (double c : e) t.arr.push_back(num(c));
        pal.arr.push_back(t);
    }
    o.set("palette", pal);
    return o;
}

std::array<double, 3> rgb_to_hsv(double r, double g, double b) {
    double cmax = std::max({r, g, b}), cmin = std::min({r, g, b});
    double delta = cmax - cmin;
    std::array<double, 3> out = {0.0, 0.0, cmax};
    if (delta > 0.0) {
        out[1] = delta / cmax;
        if (r == cmax) out[0] = 60.0 * std::fmod((g - b) / delta, 6.0);
        else if (g == cmax) out[0] = 60.0 * (((b - r) / delta) + 2.0);
        else out[0] = 60.0 * (((r - g) / delta) + 4.0);
    }
    return out;
}

void fix_rotation(std::vector<double>& s, size_t sample_size, size_t flame_size, const std::vector<size_t>& idxs) {
    const double eps = 1e-10;
    const size_t n = s.size() / sample_size;
    for (size_t idx : idxs) {
        for (size_t i = 0; i < n; i++) {
            size_t o = idx + i * sample_size;
            double ax = std::atan2(s[o + 1], s[o]);
            double mx = std::sqrt(s[o] * s[o] + s[o + 1] * s[o + 1]);
            double ay = std::atan2(s[o + 3], s[o + 2]);
            double my = std::sqrt(s[o + 2] * s[o + 2] + s[o + 3] * s[o + 3]);
            bool zx = (mx == 0.0), zy = (my == 0.0);
            if (zx && !zy) ax = ay;
            if (zy && !zx) ay = ax;
            s[o] = ax;
            s[o + 1] = ay;
            s[o + 2] = std::log(mx);
            s[o + 3] = std::log(my);
        }
        for (size_t i = 1; i < n; i++) {
            for (size_t j = 0; j < 2; j++) {
                size_t me = idx + i * sample_size + j, prev = idx + (i - 1) * sample_size + j;
                double diff = s[me] - s[prev];
                if (diff > kPi + eps) s[me] -= 2 * kPi;
                else if (diff < -(kPi - eps)) s[me] += 2 * kPi;
            }
        }
    }
    for (size_t i = flame_size; i < sample_size; i += 3) {
        for (size_t j = 1; j < n; j++) {
            size_t me = i + j * sample_size, prev = i + (j - 1) * sample_size;
            double diff = s[me] - s[prev];
            if (diff > 180.0 + eps) s[me] -= 360.0;
            else if (diff < -(180.0 - eps)) s[me] += 360.0;
        }
    }
}

}  // namespace rfk
