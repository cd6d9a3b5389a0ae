// Variation DSL ("flang") front end: lexer, recursive-descent parser, AST and
// a CUDA/C++ emitter.
//
// The grammar follows the reference PEG grammar
// (src/librefrakt/depend/flang/src/grammar_defs.h:15-112):
//   statement   := if-statement | assignment ';' | declaration ';' | '{' statement+ '}' | 'break' ';'
//   declaration := lvalue ':=' expression
//   assignment  := lvalue ('=' | '+=' | '-=' | '*=' | '/=') expression
//   expression  := '(' boolean ')' '?' boolean ':' boolean | boolean
//   boolean     := equality (('&&' | '||' | 'and' | 'or') equality)*
//   equality    := comparison (('==' | '!=') comparison)*
//   comparison  := sum (('<' | '<=' | '>' | '>=') sum)*
//   sum         := product (('+' | '-') product)*
//   product     := power (('*' | '/') power)*
//   power       := unary ('**' unary)*
//   unary       := ('-' | '!')? value
//   value       := literal | call | lvalue | '(' expression ')'
//   lvalue      := ident ('.' ident)?
// and the translation rules of the reference code generator
// (src/librefrakt/src/flame_compiler.cpp:108-391): `p` is the vlink input,
// `result` the accumulated output, `weight` the variation weight, `param.*`,
// `aff.*`, `common.*` and `math.*` are the four groups, rand01/randbit/
// randgauss draw from the chain's random stream, a root body containing
// `break` is wrapped in do { } while(0).
#pragma once

#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace rfk::dsl {

struct parse_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

enum class node_kind {
    number,   // text = literal, is_int
    boolean,  // text = true/false
    variable, // text = name
    member,   // text = group, text2 = member
    call,     // text = function name (may be "a.b"), kids = args
    unary,    // text = op, kids[0]
    binary,   // text = op, kids[0], kids[1]
    ternary,  // kids = cond, a, b
    block,    // kids = statements
    if_stmt,  // kids = cond, then, [else]
    assign,   // text = op, kids = lvalue, expr
    decl,     // text = name, kids[0] = expr
    brk,
};

struct node {
    node_kind kind;
    std::string text, text2;
    bool is_int = false;
    std::vector<std::unique_ptr<node>> kids;
};

using node_ptr = std::unique_ptr<node>;

// Parses a statement list (a variation body or precalc body).
node_ptr parse_body(const std::string& src);
// Parses a single expression (a `common` definition).
node_ptr parse_expression(const std::string& src);

// What a body needs from its surroundings.
struct usage {
    std::set<std::string> commons;  // common.<name>
    std::set<std::string> params;   // param.<name>
    int rand_calls = 0;             // upper bound of uniform draws per evaluation
    int sfu_ops = 0;                // transcendental calls (for the roofline)
    bool has_break = false;
};
usage analyze(const node& root);

// How each group maps to code. The emitter writes expressions in terms of
// the names below; the surrounding generated code defines them.
struct emit_env {
    std::string variation;                          // for diagnostics
    std::map<std::string, std::string> param_expr;  // param name -> C expression (lvalue in precalc)
    std::string aff_prefix = "aff_";                // aff.a -> aff_a
    std::string common_prefix = "c_";               // common.x -> c_x
    bool precalc = false;
};

// Emits the body as C++ statements valid in both CUDA (R = float) and host
// C++ (R = double), using the names of rfk_device.cuh.
std::string emit_body(const node& root, const emit_env& env);
std::string emit_expression(const node& e, const emit_env& env);

}  // namespace rfk::dsl
