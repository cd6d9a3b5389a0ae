"""Python side of the FP64 CPU oracle. TEST INFRASTRUCTURE ONLY: imported by
tests/, __graft_entry__.smoke() and bench.py's CPU legs as the oracle; the
library never uses it.

Restates from the reference (paths relative to its root):
  pack_sample        src/librefrakt/include/librefrakt/flame_types.h:634-672
                     (affine helpers :121-148, screen/plane :616-631)
  size_reals         flame_types.h:602-613, affine_indices :674-705
and wraps liboracle.so (oracle.c) for the numeric steps.
"""
from __future__ import annotations

import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None

# parameter slots (ordinary + precalc) of the variations the oracle knows
PARAM_SLOTS = {n: 0 for n in ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart",
                              "disc", "spiral", "hyperbolic", "julia", "exponential", "power", "fisheye", "bubble",
                              "diamond", "ex", "bent", "cylinder", "exp", "eyefish", "blur", "gaussian_blur", "cosine"]}


def build() -> Path:
    so = HERE / "liboracle.so"
    src = [HERE / "oracle.c", HERE / "oracle.h", HERE / "Makefile"]
    if not so.exists() or any(p.stat().st_mtime > so.stat().st_mtime for p in src):
        subprocess.run(["make", "-C", str(HERE), "-s"], check=True)
    return so


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        L = C.CDLL(str(build()))
        L.oracle_variation_id.argtypes = [C.c_char_p]
        L.oracle_variation_id.restype = C.c_int
        L.oracle_catmull.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]
        L.oracle_fix_rotation.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t]
        L.oracle_interpolate.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_double, C.c_void_p, C.c_size_t,
                                         C.c_void_p, C.c_void_p]
        L.oracle_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_void_p, C.POINTER(C.c_int)]
        L.oracle_apply.restype = C.c_double
        L.oracle_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                    C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_apply_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_size_t, C.c_void_p, C.c_void_p]
        L.oracle_render.restype = C.c_uint64
        L.oracle_tonemap.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.c_void_p]
        L.oracle_density_histogram.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
        L.oracle_density_blur.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_void_p]
        _LIB = L
    return _LIB


# ------------------------------------------------------------ genome layout --
def _rotated(a, d, b, e, c, f, deg):
    rad = -deg * math.pi / 180.0
    cs, sn = math.cos(rad), math.sin(rad)
    return (a * cs + d * sn, -a * sn + d * cs, b * cs + e * sn, -b * sn + e * cs, c, f)


def _translated(a, d, b, e, c, f, x, y):
    return (a, d, b, e, a * x + b * y + c, d * x + e * y + f)


def _scaled(a, d, b, e, c, f, s):
    return (a * s, d * s, b * s, e * s, c, f)


def screen_space(g: dict, w: int, h: int):
    m = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    m = _translated(*m, w / 2.0, h / 2.0)
    m = _scaled(*m, g["scale"] * h)
    m = _rotated(*m, g["rotate"])
    return _translated(*m, -g["center_x"], -g["center_y"])


def plane_space(g: dict, w: int, h: int):
    m = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    m = _translated(*m, g["center_x"], g["center_y"])
    m = _rotated(*m, -g["rotate"])
    m = _scaled(*m, 1.0 / (g["scale"] * h))
    return _translated(*m, w / -2.0, h / -2.0)


def _val(v):
    return v["t0"] if isinstance(v, dict) else v


def _xforms(g: dict):
    out = list(g["xforms"])
    if "final_xform" in g:
        out.append(g["final_xform"])
    return out


def pack_sample(g: dict, w: int, h: int, precalc_slots: dict | None = None) -> np.ndarray:
    """flame_types.h:634-672 for a JSON genome whose values are plain numbers."""
    precalc_slots = precalc_slots or {}
    out: list[float] = []
    out += list(screen_space(g, w, h))
    out += list(plane_space(g, w, h))
    out.append(0.0)
    if "chaos" in g:
        for row in g["chaos"]:
            out.append(0.0)
            out += [float(_val(c)) for c in row]
    for xf in _xforms(g):
        out += [float(_val(xf["weight"])), float(_val(xf["color"])), float(_val(xf["color_speed"])),
                float(_val(xf["opacity"]))]
        for vl in xf["vchain"]:
            t = [float(_val(v)) for v in vl["transform"]]
            m = _scaled(*t, float(_val(vl["mod_scale"])))
            m = _rotated(*m, float(_val(vl["mod_rotate"])))
            m = _translated(*m, float(_val(vl["mod_x"])), float(_val(vl["mod_y"])))
            out += list(m)
            for name in sorted(vl["variations"]):
                v = vl["variations"][name]
                if isinstance(v, dict) and "weight" in v:
                    out.append(float(_val(v["weight"])))
                    for pn in sorted(v.get("parameters", {})):
                        out.append(float(_val(v["parameters"][pn])))
                else:
                    out.append(float(_val(v)))
                out += [0.0] * precalc_slots.get(name, 0)
    for hh, s, v in g["palette"]:
        out += [math.fmod(hh + g.get("mod_hue", 0.0), 360.0), min(max(s + g.get("mod_sat", 0.0), 0.0), 1.0),
                min(max(v + g.get("mod_val", 0.0), 0.0), 1.0)]
    return np.array(out, dtype=np.float64)


def size_reals(g: dict) -> int:
    n = 13
    if "chaos" in g:
        n += len(g["xforms"]) * (len(g["xforms"]) + 1)
    for xf in _xforms(g):
        n += 4
        for vl in xf["vchain"]:
            n += 6
            for name, v in vl["variations"].items():
                n += 1 + (len(v.get("parameters", {})) if isinstance(v, dict) else 0) + PARAM_SLOTS.get(name, 0)
    return n


def affine_indices(g: dict) -> list[int]:
    ret = [0, 6]
    idx = 13 + (len(g["xforms"]) * (len(g["xforms"]) + 1) if "chaos" in g else 0)
    for xf in _xforms(g):
        idx += 4
        for vl in xf["vchain"]:
            ret.append(idx)
            idx += 6
            for name, v in vl["variations"].items():
                idx += 1 + (len(v.get("parameters", {})) if isinstance(v, dict) else 0) + PARAM_SLOTS.get(name, 0)
    return ret


def structure(g: dict) -> np.ndarray:
    s = [len(g["xforms"]), 1 if "final_xform" in g else 0, 1 if "chaos" in g else 0]
    for xf in _xforms(g):
        s.append(len(xf["vchain"]))
        for vl in xf["vchain"]:
            names = sorted(vl["variations"])
            s.append(len(names))
            for n in names:
                vid = lib().oracle_variation_id(n.encode())
                if vid < 0:
                    raise ValueError(f"oracle has no restatement of variation '{n}'")
                v = vl["variations"][n]
                s += [vid, (len(v.get("parameters", {})) if isinstance(v, dict) else 0) + PARAM_SLOTS[n]]
    return np.array(s, dtype=np.int32)


# -------------------------------------------------------------- numerics ----
def catmull(samples: np.ndarray, sample_size: int) -> np.ndarray:
    s = np.ascontiguousarray(samples, dtype=np.float64)
    nseg = s.size // sample_size - 3
    out = np.zeros((nseg, sample_size, 4))
    lib().oracle_catmull(s.ctypes.data, sample_size, nseg, out.ctypes.data)
    return out


def fix_rotation(samples: np.ndarray, sample_size: int, flame_size: int, aff) -> np.ndarray:
    s = np.ascontiguousarray(samples, dtype=np.float64).copy()
    a = np.ascontiguousarray(aff, dtype=np.uint64)
    lib().oracle_fix_rotation(s.ctypes.data, s.size // sample_size, sample_size, flame_size, a.ctypes.data, a.size)
    return s


def prepared(g: dict, w: int, h: int, t: float = 0.0, seg: int = 0, samples: np.ndarray | None = None):
    """Flame params (FP64) and 8-bit palette at time t, as the device prepares them."""
    R = size_reals(g)
    ss = R + 768
    if samples is None:
        samples = np.tile(pack_sample(g, w, h), 4)
    aff = np.array(affine_indices(g), dtype=np.uint64)
    fixed = fix_rotation(samples, ss, R, aff)
    coeff = catmull(fixed, ss)
    params = np.zeros(R)
    pal = np.zeros((256, 3))
    lib().oracle_interpolate(coeff.ctypes.data, ss, R, seg, t, aff.ctypes.data, aff.size, params.ctypes.data, pal.ctypes.data)
    return params, pal


def apply(g: dict, params: np.ndarray, xf: int, x: float, y: float, c: float, u=None):
    s = structure(g)
    uu = np.ascontiguousarray(u if u is not None else np.zeros(40), dtype=np.float64)
    xx, yy, cc = C.c_double(x), C.c_double(y), C.c_double(c)
    used = C.c_int(0)
    op = lib().oracle_apply(s.ctypes.data, np.ascontiguousarray(params, dtype=np.float64).ctypes.data, xf, C.byref(xx),
                            C.byref(yy), C.byref(cc), uu.ctypes.data, C.byref(used))
    return xx.value, yy.value, cc.value, op


def render(g: dict, w: int, h: int, chains: int, passes: int, warmup: int = 20, seed: int = 1, threads: int = 1,
           n_jitter: int = 1024, params=None, palette=None, jitter=None, hammersley: bool = False
           ) -> tuple[np.ndarray, int]:
    """FP64 chaos game. `jitter` (n x 2) gives the screen offsets to cycle
    over the chains; by default n_jitter Gaussian(1/3 px) offsets are drawn."""
    if params is None:
        params, palette = prepared(g, w, h)
    s = structure(g)
    hist = np.zeros((h, w, 4))
    P = np.ascontiguousarray(params, dtype=np.float64)
    pal = np.ascontiguousarray(palette, dtype=np.float64)
    jp = None
    if jitter is not None:
        j = np.ascontiguousarray(jitter, dtype=np.float64).reshape(-1, 2)
        n_jitter = j.shape[0]
        jp = j.ctypes.data
    draws = lib().oracle_render(s.ctypes.data, P.ctypes.data, pal.ctypes.data, w, h, chains, warmup, passes, seed, threads,
                                n_jitter, jp, 1 if hammersley else 0, hist.ctypes.data)
    return hist, int(draws)


def apply_many(g: dict, params: np.ndarray, xf: int, pts: np.ndarray) -> np.ndarray:
    """oracle_apply over an (n, 3) array of (x, y, colour); random draws are 0."""
    s = structure(g)
    P = np.ascontiguousarray(params, dtype=np.float64)
    p = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros((p.shape[0], 4))
    lib().oracle_apply_many(s.ctypes.data, P.ctypes.data, xf, p.shape[0], p.ctypes.data, out.ctypes.data)
    return out


def hermite_eval(seg4: np.ndarray, t: float) -> np.ndarray:
    """Evaluates (p1, p2, m1, m2) Hermite segments at t in FP64."""
    s = np.asarray(seg4, dtype=np.float64)
    h01 = t * t * (3 - 2 * t)
    h00 = 1 - h01
    h10 = t * (1 - t) ** 2
    h11 = t * t * (t - 1)
    return h00 * s[..., 0] + h01 * s[..., 1] + h10 * s[..., 2] + h11 * s[..., 3]


def cubic_eval(coeff: np.ndarray, t: float) -> np.ndarray:
    """Evaluates (a, b, c, d) segments (catmull.cu layout) at t in FP64."""
    c = np.asarray(coeff, dtype=np.float64)
    return ((c[..., 0] * t + c[..., 1]) * t + c[..., 2]) * t + c[..., 3]


def tonemap(bins: np.ndarray, quality: float, gamma: float, brightness: float, vibrancy: float,
            highlight_power: float = -1.0) -> np.ndarray:
    b = np.ascontiguousarray(bins, dtype=np.float32).reshape(-1, 4)
    out = np.zeros((b.shape[0], 4))
    lib().oracle_tonemap(b.ctypes.data, b.shape[0], quality, gamma, brightness, vibrancy, highlight_power, out.ctypes.data)
    return out.reshape(bins.shape[:-1] + (4,))


def density_histogram(bins: np.ndarray) -> tuple[np.ndarray, int]:
    b = np.ascontiguousarray(bins, dtype=np.float32).reshape(-1, 4)
    hist = np.zeros(97, dtype=np.uint64)
    mx = C.c_uint64(0)
    lib().oracle_density_histogram(b.ctypes.data, b.shape[0], hist.ctypes.data, C.byref(mx))
    return hist, mx.value


def density_blur(bins: np.ndarray, max_radius: float = 9.0, min_radius: float = 0.0, curve: float = 0.5) -> np.ndarray:
    b = np.ascontiguousarray(bins, dtype=np.float32)
    h, w = b.shape[:2]
    out = np.zeros((h, w, 4))
    lib().oracle_density_blur(b.ctypes.data, w, h, max_radius, min_radius, curve, out.ctypes.data)
    return out
