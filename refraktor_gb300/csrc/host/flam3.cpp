// flam3 XML genome import, following rfkt::import_flam3 and from_flam3_xml
// (src/librefrakt/src/flame_types.cpp:33-239): `coefs` is the main vlink's
// affine; `pre_*` variations form a vlink before it (identity affine,
// pre_blur meaning gaussian_blur) and `post` / `post_*` a vlink after it
// (linear 1 when only a post affine is given); `<finalxform>` becomes the
// final xform; xaos / chaos rows fill the chaos table; colours become HSV.
#include <cctype>
#include <cstdlib>

#include "genome.h"

namespace rfk {

namespace {

struct xml_node {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<xml_node> kids;
    std::string text;
    const std::string* attr(const std::string& n) const {
        for (auto& [k, v] : attrs)
            if (k == n) return &v;
        return nullptr;
    }
};

struct xml_reader {
    const std::string& s;
    size_t i = 0;
    [[noreturn]] void fail(const char* m) { throw format_error(std::string("flam3 xml: ") + m + " at offset " + std::to_string(i)); }
    void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) i++; }
    void skip_misc() {
        for (;;) {
            ws();
            if (s.compare(i, 4, "<!--") == 0) {
                size_t e = s.find("-->", i);
                if (e == std::string::npos) fail("unterminated comment");
                i = e + 3;
            } else if (s.compare(i, 2, "<?") == 0) {
                size_t e = s.find("?>", i);
                if (e == std::string::npos) fail("unterminated declaration");
                i = e + 2;
            } else if (s.compare(i, 2, "<!") == 0) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) fail("unterminated doctype");
                i = e + 1;
            } else {
                return;
            }
        }
    }
    std::string name() {
        size_t st = i;
        while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == ':' || s[i] == '.')) i++;
        if (st == i) fail("expected a name");
        return s.substr(st, i - st);
    }
    static std::string unescape(const std::string& v) {
        std::string o;
        for (size_t k = 0; k < v.size(); k++) {
            if (v[k] == '&') {
                size_t e = v.find(';', k);
                if (e != std::string::npos) {
                    std::string ent = v.substr(k + 1, e - k - 1);
                    if (ent == "lt") o += '<';
                    else if (ent == "gt") o += '>';
                    else if (ent == "amp") o += '&';
                    else if (ent == "quot") o += '"';
                    else if (ent == "apos") o += '\'';
                    else o += v.substr(k, e - k + 1);
                    k = e;
                    continue;
                }
            }
            o += v[k];
        }
        return o;
    }
    xml_node element() {
        skip_misc();
        if (i >= s.size() || s[i] != '<') fail("expected '<'");
        i++;
        xml_node n;
        n.name = name();
        for (;;) {
            ws();
            if (i >= s.size()) fail("unterminated tag");
            if (s[i] == '/') {
                if (i + 1 >= s.size() || s[i + 1] != '>') fail("expected '/>'");
                i += 2;
                return n;
            }
            if (s[i] == '>') {
                i++;
                break;
            }
            std::string an = name();
            ws();
            if (s[i] != '=') fail("expected '='");
            i++;
            ws();
            char q = s[i];
            if (q != '"' && q != '\'') fail("expected quoted attribute");
            size_t e = s.find(q, i + 1);
            if (e == std::string::npos) fail("unterminated attribute");
            n.attrs.emplace_back(an, unescape(s.substr(i + 1, e - i - 1)));
            i = e + 1;
        }
        for (;;) {
            size_t st = i;
            while (i < s.size() && s[i] != '<') i++;
            n.text += s.substr(st, i - st);
            if (i >= s.size()) fail("unterminated element");
            if (s.compare(i, 4, "<!--") == 0) {
                skip_misc();
                continue;
            }
            if (s.compare(i, 2, "</") == 0) {
                i += 2;
                std::string en = name();
                if (en != n.name) fail("mismatched closing tag");
                ws();
                if (s[i] != '>') fail("expected '>'");
                i++;
                return n;
            }
            n.kids.push_back(element());
        }
    }
};

std::vector<double> doubles(const std::string& s) {
    std::vector<double> out;
    const char* p = s.c_str();
    char* end = nullptr;
    for (;;) {
        while (*p && std::isspace((unsigned char)*p)) p++;
        if (!*p) break;
        double v = std::strtod(p, &end);
        if (end == p) break;
        out.push_back(v);
        p = end;
    }
    return out;
}

double as_double(const std::string& s) { return std::strtod(s.c_str(), nullptr); }

xform xform_from_xml(const flamedb& db, const xml_node& node) {
    xform xf;
    vlink vls[3];
    bool has_post_affine = false;

    auto longest_prefix_variation = [&](const std::string& attr) -> std::pair<std::string, std::string> {
        std::string match;
        for (auto& [vn, _] : db.variations())
            if (attr.rfind(vn, 0) == 0 && attr.size() > vn.size() + 1 && attr[vn.size()] == '_' && vn.size() > match.size())
                match = vn;
        if (match.empty()) return {};
        return {match, attr.substr(match.size() + 1)};
    };

    for (auto& [raw_name, val] : node.attrs) {
        std::string an = raw_name;
        int which = 1;
        if (an.rfind("pre_", 0) == 0) {
            which = 0;
            an = an.substr(4);
            if (an == "blur") an = "gaussian_blur";
        } else if (an.rfind("post_", 0) == 0) {
            which = 2;
            an = an.substr(5);
        }
        vlink& cur = vls[which];
        if (an == "weight") xf.weight = as_double(val);
        else if (an == "color") xf.color = as_double(val);
        else if (an == "color_speed") xf.color_speed = as_double(val);
        else if (an == "symmetry") xf.color_speed = (1.0 - as_double(val)) / 2.0;
        else if (an == "opacity") xf.opacity = as_double(val);
        else if (raw_name == "coefs" || raw_name == "post") {
            if (raw_name == "post") has_post_affine = true;
            auto v = doubles(val);
            while (v.size() < 6) v.push_back(0.0);
            vls[raw_name == "coefs" ? 1 : 2].transform = {v[0], v[1], v[2], v[3], v[4], v[5]};
        } else if (db.is_variation(an)) {
            if (!cur.variations.count(an)) cur.variations[an] = make_vardata(db, an);
            cur.variations[an].weight = as_double(val);
        } else if (auto [vn, pn] = longest_prefix_variation(an); !vn.empty()) {
            if (!cur.variations.count(vn)) cur.variations[vn] = make_vardata(db, vn);
            auto& vd = cur.variations[vn];
            if (vd.params.count(pn)) vd.params[pn] = as_double(val);
        }
        // other attributes (animate, chaos, name, ...) carry no render state here
    }
    if (!vls[0].variations.empty()) {
        vls[0].transform = affine::identity();
        xf.vchain.push_back(vls[0]);
    }
    xf.vchain.push_back(vls[1]);
    if (!vls[2].variations.empty() || has_post_affine) {
        if (vls[2].variations.empty()) {
            vls[2].variations["linear"] = make_vardata(db, "linear");
            vls[2].variations["linear"].weight = 1.0;
        }
        xf.vchain.push_back(vls[2]);
    }
    return xf;
}

int hexval(char c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'f') return c - 'a' + 10;
    if (c >= 'A' && c <= 'F') return c - 'A' + 10;
    return -1;
}

}  // namespace

flame flame_from_flam3(const flamedb& db, const std::string& xml) {
    xml_reader r{xml};
    xml_node root = r.element();
    const xml_node* fn = nullptr;
    if (root.name == "flame") fn = &root;
    else
        for (auto& k : root.kids)
            if (k.name == "flame") { fn = &k; break; }
    if (!fn) throw format_error("flam3 xml: no <flame> element");

    flame f;
    auto A = [&](const char* n) -> const std::string* { return fn->attr(n); };
    if (auto* v = A("name")) f.name = *v;
    auto size = A("size") ? doubles(*A("size")) : std::vector<double>{};
    if (size.size() < 2) throw format_error("flam3 xml: flame needs a size");
    f.scale = (A("scale") ? as_double(*A("scale")) : 1.0) / size[1];
    f.rotate = A("rotate") ? as_double(*A("rotate")) : 0.0;
    auto center = A("center") ? doubles(*A("center")) : std::vector<double>{};
    center.resize(2, 0.0);
    f.center_x = center[0];
    f.center_y = center[1];
    f.gamma = A("gamma") ? as_double(*A("gamma")) : 0.0;
    f.brightness = A("brightness") ? as_double(*A("brightness")) : 0.0;
    f.vibrancy = A("vibrancy") ? as_double(*A("vibrancy")) : 0.0;
    f.highlight_power = A("highlight_power") ? as_double(*A("highlight_power")) : 0.0;
    f.gamma_threshold = A("gamma_threshold") ? as_double(*A("gamma_threshold")) : 0.0;

    std::vector<std::pair<size_t, std::string>> chaos_rows;
    for (auto& k : fn->kids) {
        if (k.name == "xform") {
            if (auto* c = k.attr("chaos")) chaos_rows.emplace_back(f.xforms.size(), *c);
            f.xforms.push_back(xform_from_xml(db, k));
        } else if (k.name == "finalxform") {
            f.final_xform = xform_from_xml(db, k);
        }
    }

    const xml_node* pal = nullptr;
    for (auto& k : fn->kids)
        if (k.name == "palette") pal = &k;
    if (pal) {
        size_t count = pal->attr("count") ? (size_t)as_double(*pal->attr("count")) : 256;
        f.palette.assign(count, {0, 0, 0});
        std::string hex;
        size_t idx = 0;
        for (char c : pal->text) {
            if (hexval(c) < 0) continue;
            hex += c;
            if (hex.size() == 6) {
                double rgb[3];
                for (int j = 0; j < 3; j++) rgb[j] = hexval(hex[2 * j]) * 16 + hexval(hex[2 * j + 1]);
                if (idx < count) f.palette[idx] = rgb_to_hsv(rgb[0] / 255.0, rgb[1] / 255.0, rgb[2] / 255.0);
                idx++;
                hex.clear();
            }
        }
    } else {
        size_t n = 0;
        for (auto& k : fn->kids)
            if (k.name == "color") n++;
        f.palette.assign(n, {0, 0, 0});
        for (auto& k : fn->kids) {
            if (k.name != "color") continue;
            size_t index = k.attr("index") ? (size_t)as_double(*k.attr("index")) : 0;
            auto rgb = k.attr("rgb") ? doubles(*k.attr("rgb")) : std::vector<double>{};
            rgb.resize(3, 0.0);
            if (index < n) f.palette[index] = rgb_to_hsv(rgb[0] / 255.0, rgb[1] / 255.0, rgb[2] / 255.0);
        }
    }

    if (!chaos_rows.empty()) {
        std::vector<std::vector<double>> table(f.xforms.size(), std::vector<double>(f.xforms.size(), 1.0));
        for (auto& [row, txt] : chaos_rows) {
            auto v = doubles(txt);
            for (size_t j = 0; j < f.xforms.size() && j < v.size(); j++) table[row][j] = v[j];
        }
        f.chaos = table;
    }
    return f;
}

}  // namespace rfk
