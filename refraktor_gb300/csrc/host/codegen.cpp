#include "codegen.h"

#include <sstream>

namespace rfk {

namespace {

std::string indent(const std::string& s, int n) {
    std::string pad(n * 4, ' '), out;
    size_t st = 0;
    while (st < s.size()) {
        size_t e = s.find('\n', st);
        if (e == std::string::npos) e = s.size();
        std::string line = s.substr(st, e - st);
        if (!line.empty()) out += pad + line;
        out += "\n";
        st = e + 1;
    }
    return out;
}

struct emitter {
    const flamedb& db;
    std::ostringstream fn;       // xform functions
    std::ostringstream precalc;  // body of rfk_precalc

    // Emits one xform function; `base` is the offset of its weight.
    xform_info xform_fn(const xform& xf, size_t base, int id) {
        xform_info info;
        info.base = base;
        fn << "RFK_FN R rfk_xf_" << id << "(V2& pt, R& col, const PT* RFK_RESTRICT P, Rng& rng) {\n";
        fn << "    V2 in = pt;\n";
        size_t off = base + 4;
        for (size_t li = 0; li < xf.vchain.size(); li++) {
            const vlink& vl = xf.vchain[li];
            const size_t aff = off;
            fn << "    { // vlink " << li << "\n";
            info.affines++;
            fn << "        const R aff_a = P[" << aff << "], aff_d = P[" << aff + 1 << "], aff_b = P[" << aff + 2
               << "], aff_e = P[" << aff + 3 << "], aff_c = P[" << aff + 4 << "], aff_f = P[" << aff + 5 << "];\n";
            fn << "        (void)aff_a; (void)aff_b; (void)aff_c; (void)aff_d; (void)aff_e; (void)aff_f;\n";
            // affine as flame.tpl:10-14 (fma order)
            fn << "        V2 p = fl_vec2(fl_fma(aff_a, in.x, fl_fma(aff_b, in.y, aff_c)), "
                  "fl_fma(aff_d, in.x, fl_fma(aff_e, in.y, aff_f)));\n";
            fn << "        V2 r_ = fl_vec2(R(0), R(0));\n";
            off += 6;
            std::set<std::string> direct;
            for (auto& [vn, _] : vl.variations) {
                const auto& def = db.get_variation(vn);
                for (auto& c : def.apply_usage.commons) direct.insert(c);
            }
            for (auto& cn : db.common_closure(direct)) {
                dsl::emit_env cenv;
                cenv.variation = "common." + cn;
                fn << "        const R c_" << cn << " = " << dsl::emit_expression(db.common_ast(cn), cenv) << ";\n";
            }
            std::ostringstream pc;  // precalc statements for this vlink
            for (auto& [vn, vd] : vl.variations) {
                const auto& def = db.get_variation(vn);
                const size_t v0 = off;
                auto plain = def.plain_params();
                auto pre = def.precalc_params();
                if (plain.size() != vd.params.size() || pre.size() != vd.precalc_count)
                    throw format_error("genome parameters of '" + vn + "' do not match the variation database");
                dsl::emit_env env;
                env.variation = vn;
                env.aff_prefix = "aff_";
                for (size_t i = 0; i < plain.size(); i++) env.param_expr[plain[i]] = "P_" + plain[i];
                for (size_t i = 0; i < pre.size(); i++) env.param_expr[pre[i]] = "P_" + pre[i];
                fn << "        { // " << vn << "\n";
                fn << "            const R w_ = P[" << v0 << "];\n";
                for (size_t i = 0; i < plain.size(); i++)
                    fn << "            const R P_" << plain[i] << " = P[" << v0 + 1 + i << "]; (void)P_" << plain[i] << ";\n";
                for (size_t i = 0; i < pre.size(); i++)
                    fn << "            const R P_" << pre[i] << " = P[" << v0 + 1 + plain.size() + i << "]; (void)P_" << pre[i] << ";\n";
                // a zero-weight variation (padding, or a union kernel's slot
                // that this flame does not use) adds nothing and draws no
                // random numbers; skipping it also keeps 0 * inf out of the sum
                fn << "            if (w_ != R(0)) {\n";
                fn << indent(dsl::emit_body(*def.apply_ast, env), 4);
                fn << "            }\n";
                fn << "        }\n";
                info.rand_calls += def.apply_usage.rand_calls;
                info.sfu_ops += def.apply_usage.sfu_ops;

                if (def.precalc_ast) {
                    dsl::emit_env penv;
                    penv.variation = vn;
                    penv.precalc = true;
                    for (size_t i = 0; i < plain.size(); i++) penv.param_expr[plain[i]] = "P[" + std::to_string(v0 + 1 + i) + "]";
                    for (size_t i = 0; i < pre.size(); i++)
                        penv.param_expr[pre[i]] = "P[" + std::to_string(v0 + 1 + plain.size() + i) + "]";
                    pc << "    { // " << vn << " precalc\n";
                    pc << "        const R w_ = P[" << v0 << "]; (void)w_;\n";
                    pc << indent(dsl::emit_body(*def.precalc_ast, penv), 2);
                    pc << "    }\n";
                }
                off += 1 + plain.size() + pre.size();
            }
            fn << "        in = r_;\n";
            fn << "    }\n";
            if (!pc.str().empty()) {
                precalc << "  { // xform " << id << " vlink " << li << "\n";
                precalc << "    const R aff_a = P[" << aff << "], aff_d = P[" << aff + 1 << "], aff_b = P[" << aff + 2
                        << "], aff_e = P[" << aff + 3 << "], aff_c = P[" << aff + 4 << "], aff_f = P[" << aff + 5 << "];\n";
                precalc << "    (void)aff_a; (void)aff_b; (void)aff_c; (void)aff_d; (void)aff_e; (void)aff_f;\n";
                precalc << pc.str();
                precalc << "  }\n";
            }
        }
        fn << "    pt = in;\n";
        // INTERP(in.z, color, color_speed) = in.z * (1 - cs) + color * cs
        fn << "    col = col * (R(1) - P[" << base + 2 << "]) + P[" << base + 1 << "] * P[" << base + 2 << "];\n";
        fn << "    return P[" << base + 3 << "];\n";
        fn << "}\n\n";
        end = off;
        return info;
    }
    size_t end = 0;
};

}  // namespace

generated_flame generate_flame_code(const flamedb& db, const flame& f) {
    generated_flame g;
    if (f.xforms.empty()) throw format_error("flame has no xforms");
    if (f.xforms.size() > 254) throw format_error("too many xforms");
    for (auto& xf : f.xforms)
        if (xf.vchain.empty()) throw format_error("xform has an empty vchain");
    g.size_reals = f.size_reals();
    g.num_xforms = f.xforms.size();
    g.has_final = f.final_xform.has_value();
    g.chaos = f.chaos.has_value();
    g.affine_indices = f.affine_indices();

    emitter em{db};
    size_t off = 13 + (g.chaos ? g.num_xforms * (g.num_xforms + 1) : 0);
    for (size_t i = 0; i < f.xforms.size(); i++) {
        g.xforms.push_back(em.xform_fn(f.xforms[i], off, (int)i));
        off = em.end;
    }
    if (f.final_xform) {
        g.xforms.push_back(em.xform_fn(*f.final_xform, off, (int)g.num_xforms));
        off = em.end;
    }
    if (off != g.size_reals) throw format_error("internal: packed layout mismatch");

    std::ostringstream s;
    s << "// generated for structure " << f.structure_key() << "\n";
    s << "#ifndef RFK_PARAM_T\n#define RFK_PARAM_T float\n#endif\n";
    s << "typedef RFK_PARAM_T PT;\n";
    s << "#define RFK_NX " << g.num_xforms << "\n";
    s << "#define RFK_HAS_FINAL " << (g.has_final ? 1 : 0) << "\n";
    s << "#define RFK_CHAOS " << (g.chaos ? 1 : 0) << "\n";
    s << "#define RFK_SIZE_REALS " << g.size_reals << "\n";
    s << "#define RFK_NUM_AFFINES " << g.affine_indices.size() << "\n";
    s << "#ifdef RFK_HOST_TWIN\nstatic const unsigned\n#else\n__constant__ unsigned\n#endif\n";
    s << "rfk_affine_idx[RFK_NUM_AFFINES] = {";
    for (size_t i = 0; i < g.affine_indices.size(); i++) s << (i ? ", " : "") << g.affine_indices[i];
    s << "};\n";
    s << "#ifdef RFK_HOST_TWIN\nstatic const unsigned\n#else\n__constant__ unsigned\n#endif\n";
    s << "rfk_xf_base[" << g.xforms.size() << "] = {";
    for (size_t i = 0; i < g.xforms.size(); i++) s << (i ? ", " : "") << g.xforms[i].base;
    s << "};\n\n";
    s << em.fn.str();
    s << "RFK_FN R rfk_dispatch(int k, V2& pt, R& col, const PT* RFK_RESTRICT P, Rng& rng) {\n";
    s << "    switch (k) {\n";
    for (size_t i = 1; i < g.num_xforms; i++) s << "    case " << i << ": return rfk_xf_" << i << "(pt, col, P, rng);\n";
    s << "    default: return rfk_xf_0(pt, col, P, rng);\n";
    s << "    }\n}\n\n";
    if (g.has_final) {
        s << "RFK_FN R rfk_final(V2& pt, R& col, const PT* RFK_RESTRICT P, Rng& rng) {\n";
        s << "    return rfk_xf_" << g.num_xforms << "(pt, col, P, rng);\n}\n\n";
    }
    s << "RFK_FN void rfk_precalc(PT* P, Rng& rng) {\n    (void)P; (void)rng;\n" << em.precalc.str() << "}\n";
    g.source = s.str();
    return g;
}

}  // namespace rfk
