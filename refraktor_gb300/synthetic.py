"""Seeded synthetic genomes for the benchmark workloads.

The reference publishes no benchmark genomes, so the workloads are generated:
  plain_flame(seed)          512x512, 3 xforms (weights 0.5/0.3/0.2), variations
                             from {linear, sinusoidal, spherical}
  hd_flame(seed)             1920x1080, 8 xforms with Dirichlet(1) weights plus a
                             final xform, 1-3 variations each from the 14-set
Affine 2x2 parts are uniform in [-1, 1] rescaled to spectral norm <= 0.9,
translations uniform in [-1, 1]; variation weights U[0, 1]; colour per xform
U[0, 1]; colour speed 0.5; opacity 1; the palette is an HSV cubic spline
through 8 seeded knots. The default camera is centre (0, 0), scale 0.25
(the image height spans 4 units); frame_on_gpu() refits centre and scale to
the 1% / 99% quantiles of the chain positions after a GPU warm-up.
Genomes are emitted in the reference JSON layout (flame_types.cpp:399-485)
with the palette as [h, s, v] triples.
"""
from __future__ import annotations

import json
import math

import numpy as np

PLAIN_SET = ["linear", "sinusoidal", "spherical"]
HD_SET = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc", "spiral",
          "hyperbolic", "julia", "exponential", "power"]


def _affine(rng: np.random.Generator) -> list[float]:
    m = rng.uniform(-1.0, 1.0, size=(2, 2))
    n = np.linalg.norm(m, 2)
    if n > 0.9:
        m *= 0.9 / n
    c, f = rng.uniform(-1.0, 1.0, size=2)
    # reference order a, d, b, e, c, f for [[a b c], [d e f]]
    return [float(m[0, 0]), float(m[1, 0]), float(m[0, 1]), float(m[1, 1]), float(c), float(f)]


def palette(rng: np.random.Generator) -> list[list[float]]:
    """256 HSV entries from a periodic cubic spline through 8 seeded knots."""
    knots = rng.uniform(0.0, 1.0, size=(8, 3))
    knots[:, 0] *= 360.0
    knots[:, 1] = 0.4 + 0.6 * knots[:, 1]
    knots[:, 2] = 0.5 + 0.5 * knots[:, 2]
    out = []
    for i in range(256):
        u = i / 256.0 * 8.0
        k = int(math.floor(u))
        t = u - k
        p = [knots[(k + j - 1) % 8] for j in range(4)]
        # Catmull-Rom through the knots (uniform)
        v = 0.5 * ((2 * p[1]) + (-p[0] + p[2]) * t + (2 * p[0] - 5 * p[1] + 4 * p[2] - p[3]) * t * t +
                   (-p[0] + 3 * p[1] - 3 * p[2] + p[3]) * t ** 3)
        h = float(v[0] % 360.0)
        out.append([h, float(np.clip(v[1], 0.0, 1.0)), float(np.clip(v[2], 0.0, 1.0))])
    return out


def _xform(rng: np.random.Generator, weight: float, names: list[str]) -> dict:
    return {
        "weight": float(weight),
        "color": float(rng.uniform(0.0, 1.0)),
        "color_speed": 0.5,
        "opacity": 1.0,
        "vchain": [{
            "transform": _affine(rng),
            "mod_x": 0.0, "mod_y": 0.0, "mod_scale": 1.0, "mod_rotate": 0.0,
            "variations": {n: float(rng.uniform(0.0, 1.0)) for n in sorted(set(names))},
        }],
    }


def _quantile_box(dens: np.ndarray, g: dict, rw: int, rh: int, q: float = 0.01):
    """Plane-space box holding the q..1-q mass of a low-resolution render."""
    col = dens.sum(axis=0)
    row = dens.sum(axis=1)
    if col.sum() <= 0:
        return None

    def qi(m):
        c = np.cumsum(m) / m.sum()
        return int(np.searchsorted(c, q)), int(np.searchsorted(c, 1 - q))

    x0, x1 = qi(col)
    y0, y1 = qi(row)
    s = g["scale"] * rh
    to_x = lambda px: (px - rw / 2.0) / s + g["center_x"]  # noqa: E731
    to_y = lambda py: (py - rh / 2.0) / s + g["center_y"]  # noqa: E731
    return to_x(x0), to_x(x1 + 1), to_y(y0), to_y(y1 + 1)


def frame_on_gpu(db, genome: dict, w: int, h: int, seed: int = 0, with_coverage: bool = False):
    """Refits centre and scale so that the 1%..99% box of the drawn points
    (after the final xform) fills the image: a wide low-resolution render on
    the GPU locates the attractor, a second one at the located box refines it.
    With `with_coverage`, also returns the lit fraction of a third render at
    the final framing."""
    from . import librefrakt as lr

    rw = 256
    rh = max(16, int(round(rw * h / w)))
    g = dict(genome, center_x=0.0, center_y=0.0, scale=1.0 / 40.0)  # view spans 40 units vertically
    comp = lr.flame_compiler()
    coverage = 0.0
    for it in range(3 if with_coverage else 2):
        f = lr.flame.from_json(db, g)
        k = comp.get_flame_kernel(db, f)
        st = k.warmup(f.pack_samples(4, rw, rh), (rw, rh), seed, 64)
        k.bin(st, lr.bailout_args(iters=0, millis=2000, quality=16.0))
        dens = st.bins()[..., 3].double().cpu().numpy()
        if it == 2:
            coverage = float((dens > 0).mean())
            break
        box = _quantile_box(dens, g, rw, rh)
        if box is None:
            return (dict(genome), 0.0) if with_coverage else dict(genome)
        x0, x1, y0, y1 = box
        span_x, span_y = max(x1 - x0, 1e-4), max(y1 - y0, 1e-4)
        # screen = (p - centre) * scale * h + (w/2, h/2): fit both extents, 5% margin
        g = dict(g, center_x=float((x0 + x1) / 2), center_y=float((y0 + y1) / 2),
                 scale=float(min(rw / (span_x * rh), 1.0 / span_y) * 0.95))
    out = dict(genome, center_x=g["center_x"], center_y=g["center_y"],
               scale=float(g["scale"]) * (rh / rw) / (h / w))
    return (out, coverage) if with_coverage else out


def visible_flame(db, make, seed: int, w: int, h: int, min_coverage: float = 0.25, tries: int = 64) -> dict:
    """First genome make(seed * 1000 + j), j = 0, 1, ..., whose framed render
    lights at least `min_coverage` of a 256-pixel-wide preview: the visibility
    rejection that random flame generators apply (flam3-genome rejects
    candidates whose test render is mostly empty), so that benchmark genomes
    are images rather than a few collapsed points."""
    best = None
    for j in range(tries):
        g, cov = frame_on_gpu(db, make(seed * 1000 + j), w, h, seed=j, with_coverage=True)
        if cov >= min_coverage:
            return dict(g, name=f"seed{seed}.{j}")
        if best is None or cov > best[1]:
            best = (g, cov, j)
    return dict(best[0], name=f"seed{seed}.{best[2]}")


def _base(rng: np.random.Generator, gamma: float, brightness: float) -> dict:
    return {
        "center_x": 0.0, "center_y": 0.0, "scale": 0.25, "rotate": 0.0,
        "gamma": gamma, "brightness": brightness, "vibrancy": 1.0, "highlight_power": -1.0, "gamma_threshold": 0.01,
        "mod_hue": 0.0, "mod_sat": 0.0, "mod_val": 0.0,
        "xforms": [],
    }


def plain_flame(seed: int = 0) -> dict:
    rng = np.random.default_rng(seed)
    g = _base(rng, 2.2, 4.0)
    for wt in (0.5, 0.3, 0.2):
        k = int(rng.integers(1, 4))
        names = list(rng.choice(PLAIN_SET, size=k, replace=False))
        g["xforms"].append(_xform(rng, wt, names))
    g["palette"] = palette(rng)
    return g


def hd_flame(seed: int = 0, n_xforms: int = 8, final: bool = True, var_set: list[str] | None = None) -> dict:
    rng = np.random.default_rng(seed + 1_000_003)
    g = _base(rng, 2.2, 4.0)
    weights = rng.dirichlet(np.ones(n_xforms))
    for wt in weights:
        k = int(rng.integers(1, 4))
        names = list(rng.choice(var_set or HD_SET, size=k, replace=False))
        g["xforms"].append(_xform(rng, wt, names))
    if final:
        k = int(rng.integers(1, 4))
        names = list(rng.choice(var_set or HD_SET, size=k, replace=False))
        fx = _xform(rng, 0.0, names)
        g["final_xform"] = fx
    g["palette"] = palette(rng)
    return g


def keyframe_of(g: dict, seed: int) -> dict:
    """A keyframe with the structure (xforms, variation sets) of `g` and its own
    affines, xform weights (Dirichlet(1)) and variation weights (U[0, 1])."""
    rng = np.random.default_rng(seed + 2_000_003)
    out = json.loads(json.dumps(g))
    weights = rng.dirichlet(np.ones(len(out["xforms"])))
    for xf, wt in zip(out["xforms"], weights):
        xf["weight"] = float(wt)
        for vl in xf["vchain"]:
            vl["transform"] = _affine(rng)
            vl["variations"] = {n: float(rng.uniform(0.0, 1.0)) for n in vl["variations"]}
    return out


def animation_keyframes(db, seed: int, w: int, h: int, n_xforms: int = 6, count: int = 4) -> list[dict]:
    """`count` keyframes of one structure (n_xforms xforms, 1-3 variations each
    from the 14-variation set, no final xform), each framed for w x h and
    passing the visibility rejection."""
    base = visible_flame(db, lambda s: hd_flame(s, n_xforms=n_xforms, final=False), seed, w, h)
    keys = [base]
    j = 1
    while len(keys) < count:
        g, cov = frame_on_gpu(db, keyframe_of(base, seed * 1000 + j), w, h, seed=j, with_coverage=True)
        if cov >= 0.25:
            keys.append(dict(g, name=f"{base['name']}.key{j}"))
        j += 1
        if j > 256:
            raise RuntimeError("no visible keyframes")
    return keys


HETERO_SIZES = [(256, 256), (512, 512), (1024, 768), (1280, 720), (1920, 1080), (2048, 1152)]
HETERO_SPP = [64, 256, 1024]


def hetero_batch(db, seed: int, count: int = 64) -> list[dict]:
    """`count` independent flames: resolution uniform over HETERO_SIZES, xform
    count uniform in 2..12, spp uniform over HETERO_SPP, 1-3 variations per
    xform from the 14-variation set, no final xform; each framed for its size
    and passing the visibility rejection. Returns [{"genome", "width",
    "height", "spp"}]."""
    rng = np.random.default_rng(seed + 3_000_003)
    out = []
    for i in range(count):
        w, h = HETERO_SIZES[int(rng.integers(0, len(HETERO_SIZES)))]
        nx = int(rng.integers(2, 13))
        spp = HETERO_SPP[int(rng.integers(0, len(HETERO_SPP)))]
        g = visible_flame(db, lambda s, nx=nx: hd_flame(s, n_xforms=nx, final=False), seed * 100 + i, w, h)
        out.append({"genome": g, "width": w, "height": h, "spp": spp})
    return out
