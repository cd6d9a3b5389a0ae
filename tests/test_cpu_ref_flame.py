"""The generator of the reference's per-flame kernel header (oracle/
ref_flame.py), which lets the reference's own chaos-game kernels run in the
GPU parity tests: the flang-to-CUDA rules of flame_compiler.cpp:108-391 on
known variation bodies, and the template subset of flame.tpl."""
from oracle import ref_flame as rf


def tr(name: str, src: str) -> str:
    return rf.translate(name, rf.parse_program(src))


def test_fma_folding_and_names():
    assert tr("linear", "result += weight * p;") == "outp = fl::fma<FloatT>(v_linear, inp, outp);"
    assert tr("spherical", "result += weight / eps(common.sumsq) * p;") == \
        "outp = fl::fma<FloatT>(v_spherical / fl::eps<FloatT>(common_sumsq), inp, outp);"
    # minus-assign negates the multiplier's right operand; a product on the
    # right of a minus negates the addend
    assert tr("heart", "result.y -= r * sca.y;") == "outp.y = fl::fma<FloatT>(u_r__, -(u_sca__.y), outp.y);"
    assert tr("x", "result.x += weight * (a.x * p.x - a.y * p.y);") == \
        "outp.x = fl::fma<FloatT>(v_x, (fl::fma<FloatT>(u_a__.x, inp.x, -(u_a__.y * inp.y))), outp.x);"
    # a quotient is not folded
    assert tr("hyperbolic", "result.x += weight * common.sina / coeff;") == \
        "outp.x += v_hyperbolic * common_sina / u_coeff__;"


def test_literals_members_calls_and_declarations():
    assert tr("polar", "result += weight * vec2(common.atan / math.pi, common.sqrt - 1.0);") == \
        ("outp = fl::fma<FloatT>(v_polar, vec2<FloatT>{common_atan / fl::math::pi<FloatT>, "
         "common_sqrt - static_cast<FloatT>(1.0)}, outp);")
    assert tr("julia", "result += weight * cossin(math.pi * randbit());") == \
        "outp = fl::fma<FloatT>(v_julia, fl::cossin<FloatT>(fl::math::pi<FloatT> * rs->randbit()), outp);"
    src = tr("swirl", "s := sincos(common.sumsq); result.x += weight * s.x;")
    assert src.startswith("{\n") and "const auto u_s__ = fl::sincos<FloatT>(common_sumsq);" in src
    # a local that is assigned later is not const; parameters are p_<var>_<name>
    src = tr("v", "t := param.a; t += 1; result += weight * t;")
    assert "auto u_t__ = p_v_a;" in src and "const auto u_t__" not in src
    assert "fl::is_even(u_n__)" in tr("v", "k := is_even(n);")
    assert tr("v", "if a < 1 { break; } result += weight * p;").startswith("do {")


def test_template_subset():
    tpl = ("A @n@ @n < length(xs)@\n"
           "<# for x in xs #>\n"
           "  <# if not loop.is_last #>\n"
           "  v@loop.index@=@x.name@,\n"
           "  <# else #>\n"
           "  last=@x.name@\n"
           "  <# endif #>\n"
           "<# endfor #>\n"
           "<# for k, v in d #>@k@:@v@ <# endfor #>\n"
           "<# set y=at(xs, 1) #>\n"
           "    @-f(y.name, \"> \")@\n")
    out = rf.render_template(tpl, {"n": 2, "xs": [{"name": "a"}, {"name": "b"}, {"name": "c"}], "d": {"p": 1, "q": 2}},
                             {"f": lambda s, ind: ind + s.upper()})
    # trim_blocks drops the newline after each statement, so the last two
    # lines join
    assert out == "A 2 true\n  v0=a,\n  v1=b,\n  last=c\np:1 q:2 > B\n"
