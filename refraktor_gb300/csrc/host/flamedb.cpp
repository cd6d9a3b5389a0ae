#include "flamedb.h"

#include <fstream>
#include <functional>
#include <sstream>

#include "value.h"

namespace rfk {

uint64_t fnv1a(const std::string& s, uint64_t h) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::vector<std::string> variation_def::plain_params() const {
    std::vector<std::string> out;
    for (auto& [n, p] : params)
        if (!p.is_precalc()) out.push_back(n);
    return out;
}

std::vector<std::string> variation_def::precalc_params() const {
    std::vector<std::string> out;
    for (auto& [n, p] : params)
        if (p.is_precalc()) out.push_back(n);
    return out;
}

const std::set<std::string>& flamedb::pad_set(pad_type t) const { return pads_.at(t); }

namespace {

// Checks names a body may use: p, result, weight, declared locals (not
// scoped precisely: a name must be declared somewhere before its first use in
// source order), param.*, aff.*, common.*, math.*; calls to library functions
// are checked by the emitter.
void check_body(const dsl::node& root, const variation_def& def, const flamedb& db) {
    std::set<std::string> declared = {"p", "result", "weight"};
    std::function<void(const dsl::node&)> visit = [&](const dsl::node& n) {
        using K = dsl::node_kind;
        if (n.kind == K::decl) {
            for (auto& k : n.kids) visit(*k);
            declared.insert(n.text);
            return;
        }
        if (n.kind == K::variable && !declared.count(n.text))
            throw dsl::parse_error("variation '" + def.name + "' uses undeclared name '" + n.text + "'");
        if (n.kind == K::member) {
            if (n.text == "param" && !def.params.count(n.text2))
                throw dsl::parse_error("variation '" + def.name + "' uses unknown param." + n.text2);
            if (n.text == "common" && !db.is_common(n.text2))
                throw dsl::parse_error("variation '" + def.name + "' uses unknown common." + n.text2);
            if (n.text != "param" && n.text != "common" && n.text != "aff" && n.text != "math" &&
                !declared.count(n.text))
                throw dsl::parse_error("variation '" + def.name + "' uses undeclared name '" + n.text + "'");
        }
        for (auto& k : n.kids) visit(*k);
    };
    visit(root);
    // Emitting also validates function names and member names.
    dsl::emit_env env;
    env.variation = def.name;
    for (auto& [pn, _] : def.params) env.param_expr[pn] = "P_" + pn;
    dsl::emit_body(root, env);
}

}  // namespace

bool flamedb::add_or_update_variation(const variation_def& in, std::string& err) {
    variation_def def = in;
    try {
        def.apply_ast = dsl::parse_body(def.source);
        check_body(*def.apply_ast, def, *this);
        def.apply_usage = dsl::analyze(*def.apply_ast);
        if (def.precalc_source) {
            def.precalc_ast = dsl::parse_body(*def.precalc_source);
            check_body(*def.precalc_ast, def, *this);
        }
    } catch (const std::exception& e) {
        err = "cannot load variation '" + def.name + "': " + e.what();
        return false;
    }
    if (auto it = variations_.find(def.name); it != variations_.end() && it->second.pad)
        pads_[*it->second.pad].erase(def.name);
    if (def.pad) pads_[*def.pad].insert(def.name);
    variations_[def.name] = std::move(def);
    recalc_hash();
    return true;
}

bool flamedb::add_or_update_common(const std::string& name, const std::string& source, std::string& err) {
    try {
        auto ast = dsl::parse_expression(source);
        common_ast_[name] = std::shared_ptr<dsl::node>(std::move(ast));
    } catch (const std::exception& e) {
        err = "cannot load common '" + name + "': " + e.what();
        return false;
    }
    commons_[name] = source;
    recalc_hash();
    return true;
}

bool flamedb::remove_variation(const std::string& name) {
    auto it = variations_.find(name);
    if (it == variations_.end()) return false;
    if (it->second.pad) pads_[*it->second.pad].erase(name);
    variations_.erase(it);
    recalc_hash();
    return true;
}

bool flamedb::remove_common(const std::string& name) {
    if (!commons_.erase(name)) return false;
    common_ast_.erase(name);
    recalc_hash();
    return true;
}

std::vector<std::string> flamedb::common_closure(const std::set<std::string>& direct) const {
    std::vector<std::string> order;
    std::set<std::string> seen;
    std::function<void(const std::string&)> add = [&](const std::string& n) {
        if (seen.count(n)) return;
        seen.insert(n);
        auto u = dsl::analyze(*common_ast_.at(n));
        for (auto& d : u.commons) add(d);
        order.push_back(n);
    };
    for (auto& d : direct) add(d);
    return order;
}

void flamedb::recalc_hash() {
    uint64_t h = 1469598103934665603ull;
    for (auto& [n, v] : variations_) {
        h = fnv1a(n, h);
        h = fnv1a(v.source, h);
        if (v.precalc_source) h = fnv1a(*v.precalc_source, h);
        for (auto& [pn, p] : v.params) {
            h = fnv1a(pn, h);
            for (auto& t : p.tags) h = fnv1a(t, h);
        }
    }
    for (auto& [n, s] : commons_) {
        h = fnv1a(n, h);
        h = fnv1a(s, h);
    }
    hash_ = h;
}

static std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw format_error("cannot open " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

void load_flamedb(flamedb& db, const std::string& dir) {
    const std::string vtext = read_file(dir + "/variations_new.yml");
    value cdefs = parse_yaml(read_file(dir + "/common.yml"));
    std::string err;
    for (auto& [name, src] : cdefs.obj) {
        if (!db.add_or_update_common(name, src.as_string(), err)) throw format_error(err);
    }
    add_variations_yaml(db, vtext);
}

void add_variations_yaml(flamedb& db, const std::string& yaml_text) {
    value vdefs = parse_yaml(yaml_text);
    if (!vdefs.is_object()) throw format_error("a variation document is a mapping of names to definitions");
    std::string err;
    std::vector<std::string> names;
    for (auto& [name, _] : vdefs.obj) names.push_back(name);
    std::sort(names.begin(), names.end());
    for (auto& name : names) {
        const value& y = vdefs.at(name);
        variation_def def;
        def.name = name;
        if (y.is_string()) {
            def.source = y.str;
        } else if (y.is_object()) {
            def.source = y.at("src").as_string();
            if (auto* pc = y.find("precalc"); pc && pc->is_string()) def.precalc_source = pc->str;
            if (auto* tags = y.find("tags"); tags && tags->is_array()) {
                for (auto& t : tags->arr) {
                    std::string ts = t.as_string();
                    def.tags.insert(ts);
                    if (ts == "pad_affine") def.pad = pad_type::affine;
                    else if (ts == "pad_rotated") def.pad = pad_type::rotated;
                    else if (ts == "pad_identity") def.pad = pad_type::identity;
                }
            }
            if (auto* prm = y.find("param"); prm && prm->is_object()) {
                for (auto& [pn, pv] : prm->obj) {
                    param_def pd;
                    pd.name = pn;
                    if (pv.is_object()) {
                        if (auto* d = pv.find("default"); d && !d->is_null()) pd.default_value = d->as_number();
                        if (auto* d = pv.find("identity"); d && !d->is_null()) pd.identity_value = d->as_number();
                        if (auto* t = pv.find("tags"); t && t->is_array())
                            for (auto& tv : t->arr) pd.tags.insert(tv.as_string());
                    }
                    def.params[pn] = pd;
                }
            }
        } else {
            throw format_error("variation '" + name + "' is neither a body nor a mapping");
        }
        if (!db.add_or_update_variation(def, err)) throw format_error(err);
    }
}

}  // namespace rfk
