"""The best any FP32 evaluation of a variation formula, as it is written, can
do: every operation of the formula rounded once to FP32 (numpy's float32
arithmetic is IEEE round-to-nearest; sin, cos, atan2, hypot and 1/sqrt are
evaluated in float64 and rounded once, i.e. correctly rounded functions, more
accurate than any FP32 library). The operations and their order follow the
bundled refraktor_gb300/config/variations_new.yml and common.yml (the same
formulas as the reference's config/variations_new.yml:16-60), with the FP64
formulas of oracle/oracle.c beside them for the error measure.

Used to show, on the CPU, which variations cannot meet "every point within 4
ulp of the FP64 result" in FP32 however accurate the arithmetic: if even this
evaluation misses the bar at some input, the rounding of the formula's own
intermediate values (an angle sum such as atan + sqrt rounded to FP32 before
its sine, a cancellation such as sqrt - 1) is what misses it.
"""
from __future__ import annotations

import zlib

import numpy as np

# Variations held to distribution bounds in tests/test_gpu_render.py instead of
# the per-point 4-ulp bound, with the measured bounds there: forward-error
# median / 90th percentile in ulp, and the fraction of points whose backward
# error is within 4 ulp. tests/test_cpu_fp32_bounds.py shows for each of them
# that the correctly rounded evaluation above misses the per-point bound too.
ANGLE_COMPOSED = {"polar": (2.0, 4.0, 0.99), "handkerchief": (2.0, 4.0, 0.99), "disc": (2.0, 4.0, 0.99),
                  "diamond": (2.0, 4.0, 0.99), "spiral": (2.0, 4.0, 0.95), "ex": (2.0, 8.0, 0.97)}

# Variations held to the per-point backward bound whose forward error at the
# exact input is above 4 ulp at more than 1% of the points even when correctly
# rounded (the formula's conditioning, not its rounding: heart's sin(atan *
# sqrt) moves by more than 4 ulp of the output between neighbouring FP32
# inputs), with the forward fraction the GPU test requires instead of 0.99.
FORWARD_WITHIN_4 = {"heart": 0.97}

IDEAL = ("polar", "handkerchief", "heart", "disc", "spiral", "diamond", "ex")


def _f(v) -> np.ndarray:
    return np.asarray(v, dtype=np.float64).astype(np.float32)


_INV_PI = _f(1.0 / np.pi)


def _sin(v):
    return _f(np.sin(v.astype(np.float64)))


def _cos(v):
    return _f(np.cos(v.astype(np.float64)))


def _common(x: np.ndarray, y: np.ndarray):
    """common.yml: sumsq, sqrt (hypot), rsqrt, atan = atan2(x, y), sina, cosa."""
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    sumsq = _f(x64 * x64 + y64 * y64)
    sq = _f(np.hypot(x64, y64))
    rs = _f(1.0 / np.sqrt(sumsq.astype(np.float64)))
    at = _f(np.arctan2(x64, y64))
    return sumsq, sq, rs, at, _f(x64 * rs), _f(y64 * rs)


def ideal(name: str, w: float, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """(n, 2) FP32 result of one variation at FP32 points (x, y), weight w,
    with every operation of its formula correctly rounded."""
    w = np.float32(w)
    one = np.float32(1.0)
    _, sq, _, at, sina, cosa = _common(x, y)
    if name == "polar":  # weight * vec2(atan * inv_pi, sqrt - 1)
        r = (_f(w * _f(at * _INV_PI)), _f(w * _f(sq - one)))
    elif name == "handkerchief":  # (weight * sqrt) * vec2(sin(atan + sqrt), cos(atan - sqrt))
        ws = _f(w * sq)
        r = (_f(ws * _sin(_f(at + sq))), _f(ws * _cos(_f(at - sq))))
    elif name == "heart":  # sincos(atan * sqrt), amp = weight * sqrt; x += amp sin, y -= amp cos
        a = _f(at * sq)
        amp = _f(w * sq)
        r = (_f(amp * _sin(a)), -_f(amp * _cos(a)))
    elif name == "disc":  # (weight * atan * inv_pi) * sincospi(sqrt)
        k = _f(_f(w * at) * _INV_PI)
        s = sq.astype(np.float64)
        r = (_f(k * _f(np.sin(np.pi * s))), _f(k * _f(np.cos(np.pi * s))))
    elif name == "spiral":  # rad = eps(sqrt); (weight / rad) * vec2(cosa + sin rad, sina - cos rad)
        rad = np.where(sq == 0, np.float32(1e-20), sq).astype(np.float32)
        k = _f(w / rad)
        r = (_f(k * _f(cosa + _sin(rad))), _f(k * _f(sina - _cos(rad))))
    elif name == "diamond":  # weight * sina * cos(sqrt), weight * cosa * sin(sqrt)
        r = (_f(_f(w * sina) * _cos(sq)), _f(_f(w * cosa) * _sin(sq)))
    elif name == "ex":  # a = sin(atan + sqrt), b = cos(atan - sqrt); a^3 sqrt +- b^3 sqrt
        a = _sin(_f(at + sq))
        b = _cos(_f(at - sq))
        a3 = _f(_f(_f(a * a) * a) * sq)
        b3 = _f(_f(_f(b * b) * b) * sq)
        r = (_f(w * _f(a3 + b3)), _f(w * _f(a3 - b3)))
    else:
        raise KeyError(name)
    return np.stack(r, 1)


def exact(name: str, w: float, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """(n, 2) FP64 result (oracle/oracle.c: variation, cases 5-9, 16, 17)."""
    x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
    sq = np.hypot(x, y)
    rs = 1.0 / np.sqrt(x * x + y * y)
    at = np.arctan2(x, y)
    sina, cosa = x * rs, y * rs
    if name == "polar":
        r = (w * at / np.pi, w * (sq - 1.0))
    elif name == "handkerchief":
        r = (w * sq * np.sin(at + sq), w * sq * np.cos(at - sq))
    elif name == "heart":
        a = sq * at
        r = (w * sq * np.sin(a), -w * sq * np.cos(a))
    elif name == "disc":
        k = w * at / np.pi
        r = (k * np.sin(np.pi * sq), k * np.cos(np.pi * sq))
    elif name == "spiral":
        rad = np.where(sq == 0, 1e-20, sq)
        r = (w / rad * (cosa + np.sin(rad)), w / rad * (sina - np.cos(rad)))
    elif name == "diamond":
        r = (w * sina * np.cos(sq), w * cosa * np.sin(sq))
    elif name == "ex":
        a, b = np.sin(at + sq), np.cos(at - sq)
        r = (w * (a ** 3 * sq + b ** 3 * sq), w * (a ** 3 * sq - b ** 3 * sq))
    else:
        raise KeyError(name)
    return np.stack(r, 1)


def single_map_points(name: str):
    """The weight and the 2048 points of test_single_map_within_4_ulp for this
    variation: the weight is the value the variation's seeded generator gives
    after the affine's six (_one_variation_flame), rounded to FP32 as the
    prepared flame holds it; the points are uniform in [-1.5, 1.5]^2 from
    seed 12."""
    rng = np.random.default_rng(zlib.crc32(name.encode()) % 1000)
    rng.uniform(-1, 1, size=(2, 2))
    rng.uniform(-0.5, 0.5, 2)
    w = float(np.float32(rng.uniform(0.2, 1.0)))
    rng = np.random.default_rng(12)
    n = 2048
    pts = np.stack([rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n)], 1).astype(np.float32)
    return w, pts


def ulp_errors(name: str, w: float, pts: np.ndarray, out: np.ndarray):
    """Forward error at the given input and backward error (the smallest over
    inputs within 2 ulp per coordinate) of an FP32 result `out`, in ulp of the
    larger FP64 output component, as test_single_map_within_4_ulp measures
    them; also the mask of points with a finite, moderate FP64 result."""
    x, y = pts[:, 0], pts[:, 1]
    ref = exact(name, w, x, y)
    ok = np.all(np.isfinite(ref), axis=1) & (np.abs(ref).max(axis=1) < 1e6)
    scale = np.abs(ref).max(axis=1)
    ulp = np.spacing(np.maximum(scale, 1e-30).astype(np.float32)).astype(np.float64)
    out = out.astype(np.float64)
    fwd = np.abs(out - ref).max(axis=1) / ulp
    best = fwd.copy()
    sx, sy = np.spacing(x).astype(np.float64), np.spacing(y).astype(np.float64)
    for i in range(-2, 3):
        for j in range(-2, 3):
            r2 = exact(name, w, x.astype(np.float64) + i * sx, y.astype(np.float64) + j * sy)
            best = np.minimum(best, np.abs(out - r2).max(axis=1) / ulp)
    return fwd, best, ok
