"""Generates tests/golden/oracle_vectors.json: known answers computed with
mpmath at 40 significant digits from a second, independent restatement of the
reference formulas (config/variations_new.yml of the reference for the
variations, assets/kernels/tonemap.cu:67-104 with tonemapper.cpp:52 for the
tonemap, assets/kernels/catmull.cu:11-28 for the spline). The FP64 oracle must
reproduce them (tests/test_cpu_oracle.py::test_golden_vectors).

Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import ctypes

import mpmath as mp
import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

mp.mp.dps = 40
PI = mp.pi


def eps(a):
    return mp.mpf("1e-20") if a == 0 else a


def variation(name, w, x, y, bit=0):
    sumsq = x * x + y * y
    sq = mp.sqrt(sumsq)
    rs = 1 / mp.sqrt(sumsq)
    at = mp.atan2(x, y)
    sina, cosa = x * rs, y * rs
    if name == "linear":
        return w * x, w * y
    if name == "sinusoidal":
        return w * mp.sin(x), w * mp.sin(y)
    if name == "spherical":
        k = w / eps(sumsq)
        return k * x, k * y
    if name == "swirl":
        s, c = mp.sin(sumsq), mp.cos(sumsq)
        return w * (s * x - c * y), w * (c * x + s * y)
    if name == "horseshoe":
        k = w / eps(sq)
        return k * (x + y) * (x - y), k * 2 * x * y
    if name == "polar":
        return w * at / PI, w * (sq - 1)
    if name == "handkerchief":
        return w * sq * mp.sin(at + sq), w * sq * mp.cos(at - sq)
    if name == "heart":
        a, r = sq * at, w * sq
        return r * mp.sin(a), -r * mp.cos(a)
    if name == "disc":
        k = w * at / PI
        return k * mp.sin(PI * sq), k * mp.cos(PI * sq)
    if name == "spiral":
        r = eps(sq)
        return w / r * (cosa + mp.sin(r)), w / r * (sina - mp.cos(r))
    if name == "hyperbolic":
        r = eps(sq)
        return w * sina / r, w * cosa * r
    if name == "julia":
        a, r = at / 2 + PI * bit, w * mp.sqrt(sq)
        return r * mp.cos(a), r * mp.sin(a)
    if name == "exponential":
        r = w * mp.exp(x - 1)
        return r * mp.cos(PI * y), r * mp.sin(PI * y)
    if name == "power":
        r = w * mp.power(sq, sina)
        return r * cosa, r * sina
    if name == "fisheye":
        r = 2 * w / (sq + 1)
        return r * y, r * x
    if name == "bubble":
        r = w / (sumsq / 4 + 1)
        return r * x, r * y
    raise KeyError(name)


SET = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc", "spiral",
       "hyperbolic", "julia", "exponential", "power", "fisheye", "bubble"]


def apply_cases(rng):
    from refraktor_gb300 import synthetic as syn

    cases = []
    for i, name in enumerate(SET):
        g = syn.plain_flame(0)
        aff = [float(v) for v in rng.uniform(-1, 1, 6)]
        wv = float(rng.uniform(0.2, 1.5))
        cs, col, op = float(rng.uniform(0, 1)), float(rng.uniform(0, 1)), float(rng.uniform(0.1, 1))
        g["xforms"] = [{"weight": 1.0, "color": col, "color_speed": cs, "opacity": op,
                        "vchain": [{"transform": aff, "mod_x": 0.0, "mod_y": 0.0, "mod_scale": 1.0, "mod_rotate": 0.0,
                                    "variations": {name: wv}}]}]
        pts, outs = [], []
        for _ in range(6):
            x, y, c = (float(v) for v in (rng.uniform(-2, 2), rng.uniform(-2, 2), rng.uniform(0, 1)))
            a, d, b, e, cc, f = (mp.mpf(v) for v in aff)
            px, py = a * x + b * y + cc, d * x + e * y + f
            # julia's random bit: the oracle draws it from u[1] < 0.5 -> bit 0 with the zero uniforms used here
            ox, oy = variation(name, mp.mpf(wv), px, py, bit=0)
            oc = mp.mpf(c) * (1 - mp.mpf(cs)) + mp.mpf(col) * mp.mpf(cs)
            pts.append([x, y, c])
            outs.append([float(ox), float(oy), float(oc), op])
        cases.append({"variation": name, "genome": g, "xform": 0, "points": pts, "out": outs})
    return cases


def _scale_constant(q: float) -> float:
    """10^(-log10(q) - 0.5) in single precision with libm, as tonemapper.cpp:52."""
    m = ctypes.CDLL("libm.so.6")
    m.powf.restype = m.log10f.restype = ctypes.c_float
    m.powf.argtypes = [ctypes.c_float, ctypes.c_float]
    m.log10f.argtypes = [ctypes.c_float]
    return float(m.powf(10.0, -m.log10f(q) - np.float32(0.5)))


def tonemap_cases(rng):
    cases = []
    for q, gamma, B, V in [(16.0, 2.2, 4.0, 1.0), (1024.0, 4.0, 64.0783, 0.5), (2.0, 1.5, 1.0, 0.0)]:
        dens = np.concatenate([[0.0, 1e-6, 0.5, 1.0, 3.0], np.exp(rng.uniform(-3, 10, 11))]).astype(np.float32)
        col = rng.uniform(0, 1, (dens.size, 3)).astype(np.float32)
        bins = np.concatenate([col * dens[:, None], dens[:, None]], 1).astype(np.float32)
        k2 = mp.mpf(_scale_constant(q))
        g = mp.mpf(float(np.float32(gamma)))
        Bf, Vf = mp.mpf(float(np.float32(B))), mp.mpf(float(np.float32(V)))
        out = []
        for px in bins:
            w_in = mp.mpf(float(px[3]))
            if w_in == 0:
                out.append([0.0] * 4)
                continue
            f = Bf / 2 * mp.log10(1 + w_in * k2) / w_in
            c = [mp.mpf(float(v)) * f for v in px[:3]]
            wf = w_in * f
            gf = mp.power(wf, 1 / g) / wf
            o = []
            for ch in c:
                a = mp.power(ch, 1 / g) if ch > 0 else mp.mpf(0)
                o.append(float(min(max(a + Vf * (ch * gf - a), 0), 1)))
            o.append(float(min(max(mp.log(w_in) * (4 / mp.log(2)) / 96, 0), 1)))
            out.append(o)
        cases.append({"args": [q, gamma, B, V], "bins": bins.reshape(1, -1, 4).tolist(), "out": [out]})
    return cases


def catmull_cases(rng):
    cases = []
    for n in (3, 7):
        s = rng.uniform(-4, 4, 4 * n)
        coeff = []
        for r in range(n):
            p0, p1, p2, p3 = (mp.mpf(float(s[k * n + r])) for k in range(4))
            t01, t12, t23 = (mp.sqrt(mp.sqrt(d * d + 1)) for d in (p1 - p0, p2 - p1, p3 - p2))
            m1 = p2 - p1 + t12 * ((p1 - p0) / t01 - (p2 - p0) / (t01 + t12))
            m2 = p2 - p1 + t12 * ((p3 - p2) / t23 - (p3 - p1) / (t12 + t23))
            coeff.append([float(2 * (p1 - p2) + m1 + m2), float(-3 * (p1 - p2) - 2 * m1 - m2), float(m1), float(p1)])
        cases.append({"n": n, "samples": s.tolist(), "coeff": [coeff]})
    return cases


def main():
    rng = np.random.default_rng(20240)
    gold = {"generator": "tests/golden/make_golden.py (mpmath, 40 digits)", "apply": apply_cases(rng),
            "tonemap": tonemap_cases(rng), "catmull": catmull_cases(rng)}
    (HERE / "oracle_vectors.json").write_text(json.dumps(gold))
    print("wrote", HERE / "oracle_vectors.json")


if __name__ == "__main__":
    main()
