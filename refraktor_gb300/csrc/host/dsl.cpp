#include "dsl.h"

#include <cctype>
#include <functional>
#include <sstream>

namespace rfk::dsl {

namespace {

enum class tok { ident, number, op, end };

struct token {
    tok kind;
    std::string text;
    bool is_int = false;
    size_t pos = 0;
};

std::vector<token> lex(const std::string& s) {
    std::vector<token> out;
    size_t i = 0, n = s.size();
    static const std::vector<std::string> ops2 = {"**", "==", "!=", "<=", ">=", "&&", "||",
                                                  "+=", "-=", "*=", "/=", ":="};
    while (i < n) {
        char c = s[i];
        if (std::isspace((unsigned char)c)) { i++; continue; }
        if (c == '#') {  // comment to end of line
            while (i < n && s[i] != '\n') i++;
            continue;
        }
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t j = i;
            while (j < n && (std::isalnum((unsigned char)s[j]) || s[j] == '_')) j++;
            out.push_back({tok::ident, s.substr(i, j - i), false, i});
            i = j;
            continue;
        }
        if (std::isdigit((unsigned char)c)) {
            size_t j = i;
            while (j < n && std::isdigit((unsigned char)s[j])) j++;
            bool is_int = true;
            if (j + 1 < n && s[j] == '.' && std::isdigit((unsigned char)s[j + 1])) {
                is_int = false;
                j++;
                while (j < n && std::isdigit((unsigned char)s[j])) j++;
            }
            out.push_back({tok::number, s.substr(i, j - i), is_int, i});
            i = j;
            continue;
        }
        bool matched = false;
        if (i + 1 < n) {
            std::string two = s.substr(i, 2);
            for (auto& o : ops2) {
                if (two == o) {
                    out.push_back({tok::op, two, false, i});
                    i += 2;
                    matched = true;
                    break;
                }
            }
        }
        if (matched) continue;
        if (std::string("+-*/<>=!(){};,.?:").find(c) != std::string::npos) {
            out.push_back({tok::op, std::string(1, c), false, i});
            i++;
            continue;
        }
        throw parse_error("unexpected character '" + std::string(1, c) + "' at offset " + std::to_string(i));
    }
    out.push_back({tok::end, "", false, n});
    return out;
}

node_ptr mk(node_kind k, std::string t = {}, std::string t2 = {}) {
    auto p = std::make_unique<node>();
    p->kind = k;
    p->text = std::move(t);
    p->text2 = std::move(t2);
    return p;
}

class parser {
public:
    explicit parser(const std::string& src) : t_(lex(src)) {}

    node_ptr body() {
        auto root = mk(node_kind::block, "root");
        while (!at_end()) root->kids.push_back(statement());
        if (root->kids.empty()) throw parse_error("empty body");
        return root;
    }

    node_ptr single_expression() {
        auto e = expression();
        if (!at_end()) fail("trailing tokens after expression");
        return e;
    }

private:
    std::vector<token> t_;
    size_t i_ = 0;

    const token& peek(size_t o = 0) const { return t_[std::min(i_ + o, t_.size() - 1)]; }
    bool at_end() const { return peek().kind == tok::end; }
    bool is_op(const char* o, size_t off = 0) const { return peek(off).kind == tok::op && peek(off).text == o; }
    bool is_ident(const char* s, size_t off = 0) const { return peek(off).kind == tok::ident && peek(off).text == s; }
    [[noreturn]] void fail(const std::string& m) const {
        throw parse_error(m + " near offset " + std::to_string(peek().pos) + " ('" + peek().text + "')");
    }
    void expect(const char* o) {
        if (!is_op(o)) fail(std::string("expected '") + o + "'");
        i_++;
    }

    node_ptr statement() {
        if (is_ident("if")) {
            i_++;
            auto s = mk(node_kind::if_stmt);
            s->kids.push_back(expression());
            s->kids.push_back(statement());
            if (is_ident("else")) {
                i_++;
                s->kids.push_back(statement());
            }
            return s;
        }
        if (is_op("{")) {
            i_++;
            auto b = mk(node_kind::block, "scope");
            while (!is_op("}")) {
                if (at_end()) fail("unterminated block");
                b->kids.push_back(statement());
            }
            i_++;
            if (b->kids.empty()) fail("empty block");
            return b;
        }
        if (is_ident("break")) {
            i_++;
            expect(";");
            return mk(node_kind::brk);
        }
        // declaration or assignment, both start with an lvalue
        auto lv = lvalue();
        if (is_op(":=")) {
            i_++;
            if (lv->kind != node_kind::variable) fail("declaration target must be a plain name");
            auto d = mk(node_kind::decl, lv->text);
            d->kids.push_back(expression());
            expect(";");
            return d;
        }
        static const char* aops[] = {"=", "+=", "-=", "*=", "/="};
        for (auto o : aops) {
            if (is_op(o)) {
                i_++;
                auto a = mk(node_kind::assign, o);
                a->kids.push_back(std::move(lv));
                a->kids.push_back(expression());
                expect(";");
                return a;
            }
        }
        fail("expected statement");
    }

    node_ptr lvalue() {
        if (peek().kind != tok::ident) fail("expected a name");
        std::string a = peek().text;
        i_++;
        if (is_op(".")) {
            i_++;
            if (peek().kind != tok::ident) fail("expected a member name");
            std::string b = peek().text;
            i_++;
            return mk(node_kind::member, a, b);
        }
        return mk(node_kind::variable, a);
    }

    node_ptr expression() {
        // '(' boolean ')' '?' boolean ':' boolean
        if (is_op("(")) {
            size_t save = i_;
            try {
                i_++;
                auto c = boolean();
                if (is_op(")") && is_op("?", 1)) {
                    i_ += 2;
                    auto a = boolean();
                    expect(":");
                    auto b = boolean();
                    auto t = mk(node_kind::ternary);
                    t->kids.push_back(std::move(c));
                    t->kids.push_back(std::move(a));
                    t->kids.push_back(std::move(b));
                    return t;
                }
            } catch (const parse_error&) {
            }
            i_ = save;
        }
        return boolean();
    }

    node_ptr left_assoc(const std::function<node_ptr()>& sub, const std::vector<std::string>& ops) {
        auto lhs = sub();
        for (;;) {
            std::string found;
            if (peek().kind == tok::op) {
                for (auto& o : ops)
                    if (peek().text == o) found = o;
            } else if (peek().kind == tok::ident) {
                for (auto& o : ops)
                    if (peek().text == o) found = o;
            }
            if (found.empty()) return lhs;
            i_++;
            if (found == "and") found = "&&";
            if (found == "or") found = "||";
            auto b = mk(node_kind::binary, found);
            b->kids.push_back(std::move(lhs));
            b->kids.push_back(sub());
            lhs = std::move(b);
        }
    }

    node_ptr boolean() {
        return left_assoc([this] { return equality(); }, {"&&", "||", "and", "or"});
    }
    node_ptr equality() {
        return left_assoc([this] { return comparison(); }, {"==", "!="});
    }
    node_ptr comparison() {
        return left_assoc([this] { return sum(); }, {"<", "<=", ">", ">="});
    }
    node_ptr sum() {
        return left_assoc([this] { return product(); }, {"+", "-"});
    }
    node_ptr product() {
        return left_assoc([this] { return power(); }, {"*", "/"});
    }
    node_ptr power() {
        return left_assoc([this] { return unary(); }, {"**"});
    }
    node_ptr unary() {
        if (is_op("-") || is_op("!")) {
            std::string o = peek().text;
            i_++;
            auto u = mk(node_kind::unary, o);
            u->kids.push_back(value());
            return u;
        }
        return value();
    }
    node_ptr value() {
        const token& t = peek();
        if (t.kind == tok::number) {
            i_++;
            auto n = mk(node_kind::number, t.text);
            n->is_int = t.is_int;
            return n;
        }
        if (t.kind == tok::ident && (t.text == "true" || t.text == "false")) {
            i_++;
            return mk(node_kind::boolean, t.text);
        }
        if (is_op("(")) {
            i_++;
            auto e = expression();
            expect(")");
            auto p = mk(node_kind::unary, "()");
            p->kids.push_back(std::move(e));
            return p;
        }
        auto lv = lvalue();
        if (is_op("(")) {
            i_++;
            auto c = mk(node_kind::call, lv->kind == node_kind::member ? lv->text + "." + lv->text2 : lv->text);
            if (!is_op(")")) {
                c->kids.push_back(expression());
                while (is_op(",")) {
                    i_++;
                    c->kids.push_back(expression());
                }
            }
            expect(")");
            return c;
        }
        return lv;
    }
};

const std::set<std::string>& sfu_functions() {
    static const std::set<std::string> s = {"sin", "cos", "tan", "sinh", "cosh", "exp", "log", "log2", "log10",
                                            "sqrt", "rsqrt", "acos", "pow", "atan2", "hypot", "sinpi", "cospi",
                                            "sincos", "cossin", "sincospi", "cossinpi"};
    return s;
}

const std::set<std::string>& known_functions() {
    static const std::set<std::string> s = {
        "sin", "sinpi", "cos", "cospi", "cosh", "sinh", "exp", "sqrt", "eps", "tan", "abs", "log",
        "log10", "log2", "rsqrt", "acos", "sincos", "cossin", "sincospi", "cossinpi", "copysign", "modf",
        "pow", "atan2", "hypot", "rand01", "randbit", "randgauss", "elmul", "floor", "trunc", "rint",
        "is_even", "vec2"};
    return s;
}

void walk(const node& n, const std::function<void(const node&)>& f) {
    f(n);
    for (auto& k : n.kids) walk(*k, f);
}

std::string emit_stmt(const node& n, const emit_env& env, int indent);

std::string pad(int indent) { return std::string(indent * 4, ' '); }

}  // namespace

node_ptr parse_body(const std::string& src) { return parser(src).body(); }
node_ptr parse_expression(const std::string& src) { return parser(src).single_expression(); }

usage analyze(const node& root) {
    usage u;
    walk(root, [&](const node& n) {
        if (n.kind == node_kind::member) {
            if (n.text == "common") u.commons.insert(n.text2);
            if (n.text == "param") u.params.insert(n.text2);
        }
        if (n.kind == node_kind::call) {
            if (n.text == "rand01" || n.text == "randbit") u.rand_calls += 1;
            if (n.text == "randgauss") u.rand_calls += 5;
            if (sfu_functions().count(n.text)) u.sfu_ops += (n.text == "sincos" || n.text == "cossin" ||
                                                             n.text == "sincospi" || n.text == "cossinpi" ||
                                                             n.text == "pow" || n.text == "hypot")
                                                                ? 2
                                                                : 1;
        }
        if (n.kind == node_kind::brk) u.has_break = true;
    });
    return u;
}

std::string emit_expression(const node& e, const emit_env& env) {
    switch (e.kind) {
    case node_kind::number:
        if (e.is_int) return e.text;
        return "R(" + e.text + ")";
    case node_kind::boolean:
        return e.text;
    case node_kind::variable:
        if (e.text == "p") return "p";
        if (e.text == "result") return "r_";
        if (e.text == "weight") return "w_";
        return "u_" + e.text;
    case node_kind::member: {
        if (e.text == "aff") {
            static const std::set<std::string> ok = {"a", "b", "c", "d", "e", "f"};
            if (!ok.count(e.text2)) throw parse_error("unknown affine member aff." + e.text2);
            return env.aff_prefix + e.text2;
        }
        if (e.text == "param") {
            auto it = env.param_expr.find(e.text2);
            if (it == env.param_expr.end())
                throw parse_error("variation '" + env.variation + "' uses undeclared param." + e.text2);
            return it->second;
        }
        if (e.text == "math") {
            if (e.text2 == "pi") return "RFK_PI";
            if (e.text2 == "inv_pi") return "RFK_INV_PI";
            throw parse_error("unknown constant math." + e.text2);
        }
        if (e.text == "common") return env.common_prefix + e.text2;
        std::string base = (e.text == "p") ? "p" : (e.text == "result") ? "r_" : "u_" + e.text;
        if (e.text2 != "x" && e.text2 != "y") throw parse_error("unknown vector member ." + e.text2);
        return base + "." + e.text2;
    }
    case node_kind::call: {
        const std::string& f = e.text;
        if (!known_functions().count(f)) throw parse_error("unknown function " + f + "()");
        if (f == "rand01") return "RNG_U01()";
        if (f == "randbit") return "RNG_BIT()";
        if (f == "randgauss") return "RNG_GAUSS()";
        std::string args;
        for (size_t i = 0; i < e.kids.size(); i++) {
            if (i) args += ", ";
            args += emit_expression(*e.kids[i], env);
        }
        return "fl_" + f + "(" + args + ")";
    }
    case node_kind::unary:
        if (e.text == "()") return "(" + emit_expression(*e.kids[0], env) + ")";
        return e.text + emit_expression(*e.kids[0], env);
    case node_kind::binary:
        if (e.text == "**")
            return "fl_pow(" + emit_expression(*e.kids[0], env) + ", " + emit_expression(*e.kids[1], env) + ")";
    {
        // The DSL gives && and || one precedence level; C++ does not, so every
        // nested binary operand is parenthesised.
        auto side = [&](const node& k) {
            std::string s = emit_expression(k, env);
            return k.kind == node_kind::binary ? "(" + s + ")" : s;
        };
        return side(*e.kids[0]) + " " + e.text + " " + side(*e.kids[1]);
    }
    case node_kind::ternary:
        return "((" + emit_expression(*e.kids[0], env) + ") ? (" + emit_expression(*e.kids[1], env) + ") : (" +
               emit_expression(*e.kids[2], env) + "))";
    default:
        throw parse_error("statement used as expression");
    }
}

namespace {

std::string emit_stmt(const node& n, const emit_env& env, int indent) {
    std::ostringstream o;
    switch (n.kind) {
    case node_kind::block: {
        o << pad(indent) << "{\n";
        for (auto& k : n.kids) o << emit_stmt(*k, env, indent + 1);
        o << pad(indent) << "}\n";
        break;
    }
    case node_kind::if_stmt: {
        o << pad(indent) << "if (" << emit_expression(*n.kids[0], env) << ")\n";
        const node& th = *n.kids[1];
        o << (th.kind == node_kind::block ? emit_stmt(th, env, indent) : emit_stmt(th, env, indent + 1));
        if (n.kids.size() == 3) {
            o << pad(indent) << "else\n";
            const node& el = *n.kids[2];
            o << (el.kind == node_kind::block ? emit_stmt(el, env, indent) : emit_stmt(el, env, indent + 1));
        }
        break;
    }
    case node_kind::assign:
        o << pad(indent) << emit_expression(*n.kids[0], env) << " " << n.text << " "
          << emit_expression(*n.kids[1], env) << ";\n";
        break;
    case node_kind::decl:
        o << pad(indent) << "auto u_" << n.text << " = " << emit_expression(*n.kids[0], env) << ";\n";
        break;
    case node_kind::brk:
        o << pad(indent) << "break;\n";
        break;
    default:
        o << pad(indent) << emit_expression(n, env) << ";\n";
    }
    return o.str();
}

}  // namespace

std::string emit_body(const node& root, const emit_env& env) {
    usage u = analyze(root);
    std::ostringstream o;
    o << "do {\n";
    for (auto& k : root.kids) o << emit_stmt(*k, env, 1);
    o << "} while (0);\n";
    (void)u;
    return o.str();
}

}  // namespace rfk::dsl
