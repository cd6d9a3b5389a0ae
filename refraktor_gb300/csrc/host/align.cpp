// Structure alignment of several genomes: after it they pack to one layout and
// run on one kernel, so that keyframes of different structure interpolate
// and unrelated flames render in one batch.
//
// The two-keyframe case is the reference interpolator's rebuild_sides /
// interp_xforms (src/refraktor/src/refraktor.cpp:117-191) with the padding
// vlinks of flamedb::make_padder (src/librefrakt/src/flame_info.cpp:239-320).
// For n genomes the side that lacks a vlink is padded from the first genome
// (in argument order) that has it, and every vlink carries the union of the
// variations used there, the added ones with weight 0 and the parameters of
// the first genome that has them.
#include <algorithm>

#include "genome.h"

namespace rfk {

vlink make_padder(const flamedb& db, const vlink& vl) {
    vlink ret = vl;
    ret.transform = affine::identity();
    ret.mod_rotate = 0.0;
    ret.mod_scale = 1.0;
    ret.mod_x = 0.0;
    ret.mod_y = 0.0;
    for (auto& [name, vd] : ret.variations) vd.weight = 0.0;
    auto ensure_linear = [&] {
        if (!ret.variations.count("linear")) ret.variations["linear"] = make_vardata(db, "linear");
    };

    // a variation that maps through a half turn: linear -1 after a -1 affine
    for (const auto& name : db.pad_set(pad_type::rotated)) {
        if (!vl.variations.count(name)) continue;
        ensure_linear();
        ret.variations["linear"].weight = -1.0;
        ret.transform.a = -1.0;
        ret.transform.e = -1.0;
        return ret;
    }

    // variations with parameter values that make them the identity
    int found = 0;
    for (const auto& name : db.pad_set(pad_type::identity)) {
        if (!vl.variations.count(name)) continue;
        vardata& vd = ret.variations[name];
        vd.weight = 1.0;
        found++;
        for (const auto& [pn, pdef] : db.get_variation(name).params)
            if (pdef.identity_value && vd.params.count(pn)) vd.params[pn] = *pdef.identity_value;
    }
    if (found > 0) {
        for (auto& [name, vd] : ret.variations) vd.weight /= found;
        return ret;
    }

    // variations that are the identity after swapping x and y in the affine
    for (const auto& name : db.pad_set(pad_type::affine)) {
        if (!vl.variations.count(name)) continue;
        ret.variations[name].weight = 1.0;
        found++;
    }
    if (found > 0) {
        ret.transform = affine{0.0, 1.0, 1.0, 0.0, 0.0, 0.0};
        for (auto& [name, vd] : ret.variations) vd.weight /= found;
        return ret;
    }

    ensure_linear();
    ret.variations["linear"].weight = 1.0;
    return ret;
}

namespace {

// Gives the xforms at one position the same vlink chain and variation sets.
void align_xforms(const flamedb& db, std::vector<xform*>& xs) {
    size_t max_vl = 0;
    for (auto* x : xs) max_vl = std::max(max_vl, x->vchain.size());
    for (size_t j = 0; j < max_vl; j++) {
        const vlink* src = nullptr;
        for (auto* x : xs)
            if (x->vchain.size() > j) {
                src = &x->vchain[j];
                break;
            }
        for (auto* x : xs)
            if (x->vchain.size() == j) x->vchain.push_back(make_padder(db, *src));
    }
    for (size_t j = 0; j < max_vl; j++) {
        std::map<std::string, vardata> first;
        for (auto* x : xs)
            for (auto& [name, vd] : x->vchain[j].variations)
                if (!first.count(name)) first[name] = vd;
        for (auto* x : xs)
            for (auto& [name, vd] : first)
                if (!x->vchain[j].variations.count(name)) {
                    vardata z = vd;
                    z.weight = 0.0;
                    x->vchain[j].variations[name] = z;
                }
    }
}

}  // namespace

std::vector<flame> align_structures(const flamedb& db, const std::vector<flame>& in, bool by_weight) {
    std::vector<flame> out = in;
    if (out.size() < 2) return out;

    std::vector<size_t> nx;
    for (auto& f : in) nx.push_back(f.xforms.size());
    const bool any_chaos = std::any_of(in.begin(), in.end(), [](const flame& f) { return f.chaos.has_value(); });

    if (by_weight) {
        // every genome gets all genomes' xforms; the foreign ones weigh 0
        std::vector<xform> all;
        for (auto& f : in) all.insert(all.end(), f.xforms.begin(), f.xforms.end());
        size_t first = 0;
        for (size_t i = 0; i < out.size(); i++) {
            out[i].xforms = all;
            for (size_t k = 0; k < all.size(); k++)
                if (k < first || k >= first + nx[i]) out[i].xforms[k].weight = 0.0;
            first += nx[i];
        }
    } else {
        const size_t max_x = *std::max_element(nx.begin(), nx.end());
        for (auto& f : out)
            while (f.xforms.size() < max_x) f.xforms.push_back(xform{});
        for (size_t k = 0; k < max_x; k++) {
            std::vector<xform*> xs;
            for (auto& f : out) xs.push_back(&f.xforms[k]);
            align_xforms(db, xs);
        }
    }

    if (std::any_of(out.begin(), out.end(), [](const flame& f) { return f.final_xform.has_value(); })) {
        std::vector<xform*> xs;
        for (auto& f : out) {
            if (!f.final_xform) f.final_xform = xform{};
            xs.push_back(&*f.final_xform);
        }
        align_xforms(db, xs);
    }

    // chaos rows: a genome without them behaves as all ones; new xforms get 1
    if (any_chaos) {
        size_t first = 0;
        for (size_t i = 0; i < out.size(); i++) {
            const size_t n = out[i].xforms.size();
            std::vector<std::vector<double>> m(n, std::vector<double>(n, 1.0));
            if (in[i].chaos) {
                const size_t off = by_weight ? first : 0;
                const auto& c = *in[i].chaos;
                for (size_t r = 0; r < c.size() && r + off < n; r++)
                    for (size_t col = 0; col < c[r].size() && col + off < n; col++) m[r + off][col + off] = c[r][col];
            }
            out[i].chaos = m;
            first += nx[i];
        }
    }
    return out;
}

}  // namespace rfk
