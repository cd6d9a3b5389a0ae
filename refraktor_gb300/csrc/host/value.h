// Tree value shared by the JSON reader/writer and the YAML-subset reader.
//
// The reference reads its variation database with yaml-cpp
// (src/librefrakt/src/flame_info.cpp:78-146) and genomes with nlohmann::json
// (src/librefrakt/src/flame_types.cpp:241-485). Neither library is available
// here, so the library carries its own readers for the subset those files use.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace rfk {

struct format_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct value {
    enum class kind { null, boolean, number, string, array, object };
    kind k = kind::null;
    bool b = false;
    double num = 0.0;
    bool num_is_int = false;
    std::string str;
    std::vector<value> arr;
    std::vector<std::pair<std::string, value>> obj;  // insertion ordered

    bool is_null() const { return k == kind::null; }
    bool is_number() const { return k == kind::number; }
    bool is_string() const { return k == kind::string; }
    bool is_array() const { return k == kind::array; }
    bool is_object() const { return k == kind::object; }
    bool is_bool() const { return k == kind::boolean; }

    const value* find(const std::string& key) const {
        for (auto& [n, v] : obj)
            if (n == key) return &v;
        return nullptr;
    }
    bool contains(const std::string& key) const { return find(key) != nullptr; }
    const value& at(const std::string& key) const {
        auto* v = find(key);
        if (!v) throw format_error("missing key '" + key + "'");
        return *v;
    }
    value& set(const std::string& key, value v) {
        for (auto& [n, old] : obj)
            if (n == key) { old = std::move(v); return old; }
        obj.emplace_back(key, std::move(v));
        return obj.back().second;
    }
    double as_number() const;  // numbers, and strings holding numbers (YAML scalars)
    std::string as_string() const;

    static value make_number(double d) { value v; v.k = kind::number; v.num = d; return v; }
    static value make_string(std::string s) { value v; v.k = kind::string; v.str = std::move(s); return v; }
    static value make_object() { value v; v.k = kind::object; return v; }
    static value make_array() { value v; v.k = kind::array; return v; }
};

value parse_json(const std::string& text);
std::string write_json(const value& v, int indent = -1);

// YAML subset: block mappings by indentation, plain / quoted scalars,
// literal block scalars (| and |-), flow mappings {a: b} and flow
// sequences [a, "b"], comments. Scalars are kept as strings.
value parse_yaml(const std::string& text);

}  // namespace rfk
