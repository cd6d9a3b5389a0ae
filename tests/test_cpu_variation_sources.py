"""The bundled variation database against the reference's own definitions,
in FP64 on the host (needs the reference checkout; skipped without it).

(a) Every variation of the bundled refraktor_gb300/config/variations_new.yml
    against the same variation of the reference's config/variations_new.yml:
    both translated by the library's translator into host twins
    (tests/twin.py) of one flame, evaluated on the same points with the same
    random draws. The bundled file restates the reference's formulas, so the
    two must agree to rounding.
(b) The 14 variations of the 1080p workload's set against the reference's
    legacy raw-CUDA definitions (config/variations.yml), compiled here as C++
    with their xcommon macros and random-number calls supplied: an
    independent statement of the same formulas. The legacy file adds M_EPS
    (1e-20) to denominators where the new one replaces an exact 0 by 1e-20,
    which changes nothing at these points.
"""
import re
import shutil
import subprocess

import numpy as np
import pytest

from oracle.build_ref import REFERENCE_ROOT as REFERENCE
from refraktor_gb300 import build
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn
from tests.twin import ITERATE_MARK, Twin, variation_params

pytestmark = pytest.mark.skipif(not (REFERENCE / "config" / "variations_new.yml").exists(),
                                reason="reference checkout not present")

HD_SET = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc", "spiral",
          "hyperbolic", "julia", "exponential", "power"]
N = 512


def _flame(names, params, seed=23):
    rng = np.random.default_rng(seed)
    g = syn.plain_flame(2)
    xfs = []
    for name in names:
        w = float(rng.uniform(0.3, 1.0))
        ps = params.get(name, [])
        entry = w
        if ps:
            entry = {"weight": w, "parameters": {
                p: float((d if d is not None else rng.uniform(0.3, 1.0)) * rng.uniform(0.6, 1.4)) for p, d in ps}}
        xfs.append({"weight": 1.0, "color": float(rng.uniform()), "color_speed": 0.5, "opacity": 1.0,
                    "vchain": [{"transform": [1.0, 0.0, 0.0, 1.0, 0.0, 0.0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {name: entry}}]})
    g["xforms"] = xfs
    return g


def _points(seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(-1.5, 1.5, N), rng.uniform(-1.5, 1.5, N), rng.uniform(0, 1, N)], 1)


def test_bundled_variations_match_the_reference_file(tmp_path):
    bundled = lr.flamedb()
    ref = lr.flamedb(REFERENCE / "config")
    names = bundled.variations()
    assert all(ref.is_variation(n) for n in names)
    params = variation_params((build.PKG / "config" / "variations_new.yml").read_text())
    g = _flame(names, params)
    fb, fr = lr.flame.from_json(bundled, g), lr.flame.from_json(ref, g)
    assert fb.size_reals() == fr.size_reals()
    tb, tr = Twin(bundled, fb, tmp_path / "b"), Twin(ref, fr, tmp_path / "r")
    # the packed reals of a static genome stand in for the prepared block (the
    # precalc slots are computed by the twins' own code paths below)
    P = np.asarray(fb.pack_sample(256, 256), dtype=np.float64)[:fb.size_reals()]
    assert np.array_equal(P, np.asarray(fr.pack_sample(256, 256), dtype=np.float64)[:fr.size_reals()])
    worst = {}
    for k, name in enumerate(names):
        pts = _points(100 + k)
        a = tb.apply(P, k, pts, np.arange(N), seed=3)
        b = tr.apply(P, k, pts, np.arange(N), seed=3)
        fin = np.all(np.isfinite(a[:, :2]) & np.isfinite(b[:, :2]), axis=1)
        assert np.array_equal(fin, np.all(np.isfinite(b[:, :2]), axis=1)), name
        scale = np.maximum(np.abs(b[fin, :2]).max(axis=1), 1e-300)
        rel = np.abs(a[fin, :2] - b[fin, :2]).max(axis=1) / scale
        worst[name] = float(rel.max())
        np.testing.assert_allclose(a[:, 2:], b[:, 2:], rtol=1e-14, atol=1e-15, err_msg=name)
    bad = {n: v for n, v in worst.items() if not v <= 1e-9}
    assert not bad, bad


LEGACY_MAIN = r"""
using FloatT = double;
constexpr FloatT operator""_r(long double v) { return (FloatT)v; }
#define M_EPS (1e-20)
struct legacy_rng {
    Rng* r;
    unsigned rand() { return r->next(); }
    FloatT rand_uniform() { return (FloatT)r->u01(); }
};
%(functions)s
#include <cstdio>
typedef void (*legacy_fn)(FloatT, FloatT, FloatT, FloatT&, FloatT&, legacy_rng*);
static const legacy_fn legacy[] = {%(table)s};
int main() {
    unsigned n = 0, np = 0, seed = 0;
    int k = 0;
    if (std::scanf("%%u %%u %%d %%u", &n, &np, &k, &seed) != 4) return 2;
    std::vector<double> P(np);
    for (unsigned i = 0; i < np; i++)
        if (std::scanf("%%lf", &P[i]) != 1) return 3;
    for (unsigned j = 0; j < n; j++) {
        unsigned idx = 0;
        double x = 0, y = 0, c = 0;
        if (std::scanf("%%u %%lf %%lf %%lf", &idx, &x, &y, &c) != 4) return 4;
        Rng r1, r2;
        r1.start(idx, 0xFFFCu, 0ull, seed, 0u);
        r2.start(idx, 0xFFFCu, 0ull, seed, 0u);
        V2 p = fl_vec2(x, y);
        R col = c;
        rfk_dispatch(k, p, col, P.data(), r1);
        legacy_rng rs{&r2};
        FloatT nx = 0, ny = 0;
        legacy[k](x, y, P[rfk_xf_base[k] + 4 + 6], nx, ny, &rs);
        std::printf("%%.17g %%.17g %%.17g %%.17g\n", (double)p.x, (double)p.y, nx, ny);
    }
    return 0;
}
"""


def _legacy_snippets(text: str) -> tuple[dict, dict]:
    xc = {}
    head = text[text.index("xcommon:"):text.index("variations:")]
    for m in re.finditer(r"^    (\w+):\s*(.+)$", head, re.M):
        xc[m.group(1)] = m.group(2).strip()
    body = text[text.index("variations:"):]
    out = {}
    for name in HD_SET:
        m = re.search(r"^    %s: \|-\n((?:        .*\n|[ \t]*\n)*)" % name, body, re.M)
        assert m, name
        out[name] = m.group(1)
    return xc, out


def _xc(expr: str) -> str:
    return re.sub(r"xcommon\((\w+)\)", r"xc_\1", expr)


def test_hd_set_matches_the_legacy_definitions(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    xc, snippets = _legacy_snippets((REFERENCE / "config" / "variations.yml").read_text())
    db = lr.flamedb()
    g = _flame(HD_SET, {})
    f = lr.flame.from_json(db, g)
    order = ["sumsq", "sqrt", "atan", "phi", "sina", "cosa", "sinr", "cosr"]
    assert set(order) <= set(xc)
    funcs = []
    for name in HD_SET:
        commons = "".join(f"    const FloatT xc_{c} = {_xc(xc[c])};\n" for c in order)
        funcs.append(f"static void legacy_{name}(FloatT px, FloatT py, FloatT weight, FloatT& nx, FloatT& ny, "
                     f"legacy_rng* rs) {{\n    using std::sin; using std::cos; using std::exp; using std::pow;\n"
                     f"    (void)rs;\n{commons}" + "".join(f"    (void)xc_{c};\n" for c in order) +
                     _xc(snippets[name]) + "}\n")
    src = lr.generate_source(db, f)
    prog = ("#define RFK_HOST_TWIN 1\n#define RFK_REAL double\n#define RFK_PARAM_T double\n#include <vector>\n"
            "#include <cmath>\n#define sincos(a, s, c) (*(s) = std::sin(a), *(c) = std::cos(a))\n"
            + src[:src.index(ITERATE_MARK)]
            + LEGACY_MAIN % {"functions": "\n".join(funcs), "table": ", ".join(f"legacy_{n}" for n in HD_SET)})
    (tmp_path / "legacy.cpp").write_text(prog)
    exe = tmp_path / "legacy"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-ffp-contract=off", "-w", str(tmp_path / "legacy.cpp"), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    P = np.asarray(f.pack_sample(256, 256), dtype=np.float64)[:f.size_reals()]
    for k, name in enumerate(HD_SET):
        pts = _points(300 + k)
        head = f"{N} {P.size} {k} 9\n" + " ".join(repr(float(v)) for v in P) + "\n"
        body = "".join(f"{i} {x!r} {y!r} {c!r}\n" for i, (x, y, c) in enumerate(pts.tolist()))
        out = subprocess.run([str(exe)], input=head + body, capture_output=True, text=True, check=True).stdout
        v = np.array([[float(t) for t in line.split()] for line in out.strip().split("\n")])
        new, old = v[:, :2], v[:, 2:]
        scale = np.maximum(np.abs(old).max(axis=1), 1e-300)
        rel = np.abs(new - old).max(axis=1) / scale
        assert rel.max() <= 1e-12, (name, float(rel.max()))
