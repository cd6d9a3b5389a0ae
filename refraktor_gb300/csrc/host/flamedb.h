// Variation database: the plugin surface that defines what a genome may use.
//
// Mirrors rfkt::flamedb (src/librefrakt/include/librefrakt/flame_info.h:18-157)
// and rfkt::initialize (src/librefrakt/src/flame_info.cpp:60-148): a config
// directory holds variations_new.yml (one entry per variation: a DSL body, or
// a mapping with src / precalc / param / tags) and common.yml (shared named
// sub-expressions). Parameters are kept sorted by name, as std::map does in
// the reference, because that order fixes the packed genome layout.
#pragma once

#include <map>
#include <optional>
#include <set>
#include <string>

#include "dsl.h"

namespace rfk {

enum class pad_type { rotated, identity, affine };

struct param_def {
    std::string name;
    std::optional<double> default_value;
    std::optional<double> identity_value;
    std::set<std::string> tags;
    bool is_precalc() const { return tags.count("precalc") > 0; }
};

struct variation_def {
    std::string name;
    std::string source;
    std::optional<std::string> precalc_source;
    std::set<std::string> tags;
    std::map<std::string, param_def> params;  // sorted by name
    std::optional<pad_type> pad;

    std::shared_ptr<dsl::node> apply_ast;
    std::shared_ptr<dsl::node> precalc_ast;
    dsl::usage apply_usage;

    // Names of ordinary (non-precalc) parameters, sorted.
    std::vector<std::string> plain_params() const;
    std::vector<std::string> precalc_params() const;
};

class flamedb {
public:
    // Adds or replaces; returns false and sets `err` when the source does not
    // parse or refers to unknown parameters / commons / functions
    // (flame_info.cpp:152-194 semantics).
    bool add_or_update_variation(const variation_def& def, std::string& err);
    bool add_or_update_common(const std::string& name, const std::string& source, std::string& err);

    // flamedb::remove_variation / remove_common (flame_info.h:113-129): false
    // when the name is not present
    bool remove_variation(const std::string& name);
    bool remove_common(const std::string& name);

    bool is_variation(const std::string& n) const { return variations_.count(n) > 0; }
    bool is_common(const std::string& n) const { return commons_.count(n) > 0; }
    bool is_parameter(const std::string& v, const std::string& p) const {
        auto it = variations_.find(v);
        return it != variations_.end() && it->second.params.count(p) > 0;
    }
    const variation_def& get_variation(const std::string& n) const { return variations_.at(n); }
    const dsl::node& common_ast(const std::string& n) const { return *common_ast_.at(n); }
    const std::map<std::string, variation_def>& variations() const { return variations_; }
    const std::map<std::string, std::string>& commons() const { return commons_; }
    const std::set<std::string>& pad_set(pad_type t) const;

    // Commons needed by a set of direct references, in dependency order.
    std::vector<std::string> common_closure(const std::set<std::string>& direct) const;

    uint64_t hash() const { return hash_; }

private:
    void recalc_hash();
    std::map<std::string, variation_def> variations_;
    std::map<std::string, std::string> commons_;
    std::map<std::string, std::shared_ptr<dsl::node>> common_ast_;
    std::map<pad_type, std::set<std::string>> pads_ = {{pad_type::rotated, {}}, {pad_type::identity, {}}, {pad_type::affine, {}}};
    uint64_t hash_ = 0;
};

// Loads `<dir>/variations_new.yml` and `<dir>/common.yml` into `db`
// (flame_info.cpp:60-148). Throws rfk::format_error on failure.
void load_flamedb(flamedb& db, const std::string& dir);
// Adds or replaces the variations of a document in variations_new.yml format
// (name: body, or name: {src, precalc, param, tags}), in name order; the
// first failure throws rfk::format_error and leaves the earlier ones added.
void add_variations_yaml(flamedb& db, const std::string& yaml_text);

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull);

}  // namespace rfk
