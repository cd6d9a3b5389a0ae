#include "value.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>

namespace rfk {

double value::as_number() const {
    if (k == kind::number) return num;
    if (k == kind::string) {
        char* end = nullptr;
        double d = std::strtod(str.c_str(), &end);
        if (end == str.c_str()) throw format_error("not a number: '" + str + "'");
        return d;
    }
    if (k == kind::boolean) return b ? 1.0 : 0.0;
    throw format_error("value is not a number");
}

std::string value::as_string() const {
    if (k == kind::string) return str;
    if (k == kind::number) {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g", num);
        return buf;
    }
    throw format_error("value is not a string");
}

// ---------------------------------------------------------------- JSON ----
namespace {

struct json_reader {
    const std::string& s;
    size_t i = 0;

    [[noreturn]] void fail(const char* m) { throw format_error(std::string("json: ") + m + " at offset " + std::to_string(i)); }
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    bool lit(const char* w) {
        size_t n = std::char_traits<char>::length(w);
        if (s.compare(i, n, w) == 0) { i += n; return true; }
        return false;
    }
    std::string string_lit() {
        if (s[i] != '"') fail("expected string");
        i++;
        std::string out;
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) fail("bad escape");
                char e = s[i++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (i + 4 > s.size()) fail("bad \\u escape");
                    unsigned cp = std::stoul(s.substr(i, 4), nullptr, 16);
                    i += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size()) fail("unterminated string");
        i++;
        return out;
    }
    value parse() {
        ws();
        if (i >= s.size()) fail("unexpected end");
        char c = s[i];
        value v;
        if (c == '{') {
            i++;
            v.k = value::kind::object;
            ws();
            if (s[i] == '}') { i++; return v; }
            for (;;) {
                ws();
                std::string key = string_lit();
                ws();
                if (s[i] != ':') fail("expected ':'");
                i++;
                v.obj.emplace_back(std::move(key), parse());
                ws();
                if (s[i] == ',') { i++; continue; }
                if (s[i] == '}') { i++; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            i++;
            v.k = value::kind::array;
            ws();
            if (s[i] == ']') { i++; return v; }
            for (;;) {
                v.arr.push_back(parse());
                ws();
                if (s[i] == ',') { i++; continue; }
                if (s[i] == ']') { i++; return v; }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') return value::make_string(string_lit());
        if (lit("true")) { v.k = value::kind::boolean; v.b = true; return v; }
        if (lit("false")) { v.k = value::kind::boolean; v.b = false; return v; }
        if (lit("null")) return v;
        if (c == '-' || std::isdigit((unsigned char)c)) {
            size_t st = i;
            if (s[i] == '-') i++;
            bool is_int = true;
            while (i < s.size() && (std::isdigit((unsigned char)s[i]) || s[i] == '.' || s[i] == 'e' || s[i] == 'E' ||
                                    s[i] == '+' || s[i] == '-')) {
                if (s[i] == '.' || s[i] == 'e' || s[i] == 'E') is_int = false;
                i++;
            }
            v = value::make_number(std::strtod(s.substr(st, i - st).c_str(), nullptr));
            v.num_is_int = is_int;
            return v;
        }
        fail("unexpected character");
    }
};

void write_json_rec(std::ostringstream& o, const value& v, int indent, int depth) {
    auto nl = [&](int d) {
        if (indent >= 0) {
            o << '\n' << std::string(d * indent, ' ');
        }
    };
    switch (v.k) {
    case value::kind::null: o << "null"; break;
    case value::kind::boolean: o << (v.b ? "true" : "false"); break;
    case value::kind::number: {
        if (!std::isfinite(v.num)) { o << "null"; break; }
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g", v.num);
        o << buf;
        break;
    }
    case value::kind::string: {
        o << '"';
        for (char c : v.str) {
            if (c == '"' || c == '\\') o << '\\' << c;
            else if (c == '\n') o << "\\n";
            else if ((unsigned char)c < 0x20) { char b[8]; std::snprintf(b, sizeof b, "\\u%04x", c); o << b; }
            else o << c;
        }
        o << '"';
        break;
    }
    case value::kind::array:
        o << '[';
        for (size_t i = 0; i < v.arr.size(); i++) {
            if (i) o << ',';
            nl(depth + 1);
            write_json_rec(o, v.arr[i], indent, depth + 1);
        }
        if (!v.arr.empty()) nl(depth);
        o << ']';
        break;
    case value::kind::object:
        o << '{';
        for (size_t i = 0; i < v.obj.size(); i++) {
            if (i) o << ',';
            nl(depth + 1);
            write_json_rec(o, value::make_string(v.obj[i].first), indent, depth + 1);
            o << (indent >= 0 ? ": " : ":");
            write_json_rec(o, v.obj[i].second, indent, depth + 1);
        }
        if (!v.obj.empty()) nl(depth);
        o << '}';
        break;
    }
}

}  // namespace

value parse_json(const std::string& text) {
    json_reader r{text};
    value v = r.parse();
    r.ws();
    if (r.i != text.size()) r.fail("trailing characters");
    return v;
}

std::string write_json(const value& v, int indent) {
    std::ostringstream o;
    write_json_rec(o, v, indent, 0);
    return o.str();
}

// ---------------------------------------------------------------- YAML ----
namespace {

struct yline {
    int indent;
    std::string text;  // without indentation, comments kept (handled later)
    size_t number;
};

std::string rstrip(std::string s) {
    while (!s.empty() && std::isspace((unsigned char)s.back())) s.pop_back();
    return s;
}

std::string strip(const std::string& s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

// Removes a trailing " # comment" that is outside quotes.
std::string drop_comment(const std::string& s) {
    bool sq = false, dq = false;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (c == '\'' && !dq) sq = !sq;
        else if (c == '"' && !sq) dq = !dq;
        else if (c == '#' && !sq && !dq && (i == 0 || std::isspace((unsigned char)s[i - 1]))) return rstrip(s.substr(0, i));
    }
    return s;
}

struct flow_reader {
    const std::string& s;
    size_t i = 0;
    void ws() { while (i < s.size() && std::isspace((unsigned char)s[i])) i++; }
    [[noreturn]] void fail(const char* m) { throw format_error(std::string("yaml flow: ") + m + " in '" + s + "'"); }
    std::string scalar(const char* stops) {
        ws();
        if (i < s.size() && (s[i] == '"' || s[i] == '\'')) {
            char q = s[i++];
            std::string out;
            while (i < s.size() && s[i] != q) {
                if (s[i] == '\\' && q == '"' && i + 1 < s.size()) { out += s[i + 1]; i += 2; continue; }
                out += s[i++];
            }
            if (i >= s.size()) fail("unterminated quote");
            i++;
            return out;
        }
        size_t st = i;
        while (i < s.size() && !std::strchr(stops, s[i])) i++;
        return strip(s.substr(st, i - st));
    }
    value node() {
        ws();
        if (i < s.size() && s[i] == '{') {
            i++;
            value v = value::make_object();
            ws();
            if (i < s.size() && s[i] == '}') { i++; return v; }
            for (;;) {
                std::string key = scalar(":,}");
                ws();
                if (i >= s.size() || s[i] != ':') fail("expected ':'");
                i++;
                v.set(key, node());
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == '}') { i++; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (i < s.size() && s[i] == '[') {
            i++;
            value v = value::make_array();
            ws();
            if (i < s.size() && s[i] == ']') { i++; return v; }
            for (;;) {
                v.arr.push_back(node());
                ws();
                if (i < s.size() && s[i] == ',') { i++; continue; }
                if (i < s.size() && s[i] == ']') { i++; return v; }
                fail("expected ',' or ']'");
            }
        }
        return value::make_string(scalar(",}]"));
    }
};

value scalar_or_flow(const std::string& raw) {
    std::string t = strip(raw);
    if (!t.empty() && (t[0] == '{' || t[0] == '[')) {
        flow_reader r{t};
        value v = r.node();
        return v;
    }
    if (t.size() >= 2 && ((t[0] == '"' && t.back() == '"') || (t[0] == '\'' && t.back() == '\'')))
        return value::make_string(t.substr(1, t.size() - 2));
    return value::make_string(t);
}

// Position of the mapping colon in "key: value" / "key:" (outside quotes and flow brackets).
size_t key_colon(const std::string& t) {
    int depth = 0;
    bool sq = false, dq = false;
    for (size_t i = 0; i < t.size(); i++) {
        char c = t[i];
        if (c == '\'' && !dq) sq = !sq;
        else if (c == '"' && !sq) dq = !dq;
        else if (sq || dq) continue;
        else if (c == '{' || c == '[') depth++;
        else if (c == '}' || c == ']') depth--;
        else if (c == ':' && depth == 0 && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) return i;
    }
    return std::string::npos;
}

struct yaml_reader {
    std::vector<yline> lines;
    size_t pos = 0;

    [[noreturn]] void fail(const std::string& m) {
        size_t ln = pos < lines.size() ? lines[pos].number : 0;
        throw format_error("yaml line " + std::to_string(ln + 1) + ": " + m);
    }

    // Parses a block mapping whose keys sit at exactly `indent`.
    value mapping(int indent, const std::vector<std::string>& raw) {
        value m = value::make_object();
        while (pos < lines.size()) {
            const yline& L = lines[pos];
            if (L.indent < indent) break;
            if (L.indent > indent) fail("unexpected indentation");
            std::string t = drop_comment(L.text);
            size_t c = key_colon(t);
            if (c == std::string::npos) fail("expected 'key:'");
            std::string key = strip(t.substr(0, c));
            if (key.size() >= 2 && (key[0] == '"' || key[0] == '\'')) key = key.substr(1, key.size() - 2);
            std::string rest = strip(t.substr(c + 1));
            pos++;
            if (rest == "|" || rest == "|-" || rest == "|+" || rest == ">" || rest == ">-") {
                m.set(key, block_scalar(indent, rest, raw));
            } else if (rest.empty()) {
                if (pos < lines.size() && lines[pos].indent > indent) {
                    m.set(key, mapping(lines[pos].indent, raw));
                } else {
                    m.set(key, value());
                }
            } else {
                // a plain scalar may continue on more-indented lines
                std::string acc = rest;
                while (pos < lines.size() && lines[pos].indent > indent && rest[0] != '{' && rest[0] != '[') {
                    acc += " " + strip(drop_comment(lines[pos].text));
                    pos++;
                }
                m.set(key, scalar_or_flow(acc));
            }
        }
        return m;
    }

    value block_scalar(int parent_indent, const std::string& style, const std::vector<std::string>& raw) {
        // collect every following raw line more indented than the parent (blank lines included)
        size_t first_raw = pos < lines.size() ? lines[pos].number : raw.size();
        size_t end_raw = first_raw;
        int block_indent = -1;
        while (pos < lines.size() && lines[pos].indent > parent_indent) {
            if (block_indent < 0) block_indent = lines[pos].indent;
            end_raw = lines[pos].number + 1;
            pos++;
        }
        std::string out;
        for (size_t r = first_raw; r < end_raw; r++) {
            std::string l = raw[r];
            if (strip(l).empty()) { out += "\n"; continue; }
            out += (block_indent >= 0 && (int)l.size() >= block_indent) ? l.substr(block_indent) : strip(l);
            out += "\n";
        }
        if (style == "|-" || style == ">-") {
            while (!out.empty() && out.back() == '\n') out.pop_back();
        } else if (style == "|") {
            while (out.size() >= 2 && out[out.size() - 1] == '\n' && out[out.size() - 2] == '\n') out.pop_back();
        }
        return value::make_string(rstrip(out) == out ? out : out);
    }
};

}  // namespace

value parse_yaml(const std::string& text) {
    std::vector<std::string> raw;
    {
        std::string cur;
        for (char c : text) {
            if (c == '\n') { raw.push_back(cur); cur.clear(); }
            else if (c != '\r') cur += c;
        }
        raw.push_back(cur);
    }
    yaml_reader r;
    for (size_t i = 0; i < raw.size(); i++) {
        std::string l = raw[i];
        size_t ind = 0;
        while (ind < l.size() && (l[ind] == ' ' || l[ind] == '\t')) ind++;
        std::string body = l.substr(ind);
        if (strip(body).empty()) continue;
        if (body[0] == '#') continue;
        if (body == "---") continue;
        r.lines.push_back({(int)ind, rstrip(body), i});
    }
    if (r.lines.empty()) return value::make_object();
    value v = r.mapping(r.lines[0].indent, raw);
    if (r.pos != r.lines.size()) r.fail("unparsed content");
    return v;
}

}  // namespace rfk
