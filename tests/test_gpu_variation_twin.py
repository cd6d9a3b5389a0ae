"""Every variation of the bundled database, deterministic and stochastic, in
one map application on the GPU (precise-math build, FP32) against the
translator's FP64 host twin of the same generated code (tests/twin.py),
which replays the device's random draws.

One flame holds one xform per variation (identity affine, seeded weight and
parameter values), so one NVRTC module and one host build cover all of them.
Per variation, 1024 seeded points in [-1.5, 1.5]^2: the forward error in FP32
ulps of the larger output component, and, for points beyond 4 ulps, the
backward error (the nearest FP64 result over inputs within 2 ulps, the
rounding an FP32 input carries). The bounds are the ones the tests of the
22 classic variations use (tests/test_gpu_render.py): every point within 4
ulps backward, median forward error at most 1 ulp; variations whose formulas
compose FP32-rounded angles with radii, cancel, or compose three or more
libm results are held to measured distribution bounds instead (BOUNDED)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from refraktor_gb300 import build
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn
from tests.twin import Twin, variation_params

pytestmark = pytest.mark.gpu

N = 1024
SEED = 5

# variation -> (median forward ulp bound, fraction of points within 4 ulps
# backward), measured on GB300 (1024 points). Beside the angle-composing
# variations of the classic set: popcorn's tan(3y) amplifies the input's
# rounding near its poles; cross cancels in x^2 - y^2 near the
# diagonals; gaussian_blur sums four FP32 uniforms and subtracts 2 (the
# reference's Irwin-Hall gaussian), which cancels near 0; curl, log,
# juliascope and rectangles compose a rounded intermediate (a quotient, a
# logarithm's argument, a power, a floor) with the output.
BOUNDED = {"polar": (2.0, 0.985), "handkerchief": (2.0, 0.99), "disc": (2.0, 0.99), "heart": (2.0, 0.99),
           "diamond": (2.0, 0.99), "spiral": (2.0, 0.95), "ex": (2.0, 0.97), "cosine": (1.0, 0.999),
           "cross": (1.0, 0.90), "gaussian_blur": (2.0, 0.75), "curl": (1.0, 0.995), "log": (1.0, 0.995),
           "juliascope": (1.0, 0.98), "rectangles": (1.0, 0.995), "popcorn": (1.0, 0.85)}

# Variations that read the vlink's affine offsets (aff.c, aff.f): they get
# offsets (0.25, -0.375) instead of the identity's zeros (waves divides by
# their squares), with inputs on a 2^-12 grid so that the affine's additions
# are exact in FP32 and the variation sees the same point in both precisions.
AFF_OFFSET = {"fan": (0.25, -0.375), "popcorn": (0.25, -0.375), "rings": (0.25, -0.375), "waves": (0.25, -0.375)}


def _flame(names, params):
    rng = np.random.default_rng(17)
    g = syn.plain_flame(2)
    xfs = []
    for name in names:
        w = float(rng.uniform(0.3, 1.0))
        ps = params.get(name, [])
        entry = w
        if ps:
            # around the default, or in [0.3, 1] without one (0 would make
            # some of them degenerate)
            entry = {"weight": w, "parameters": {
                p: float((d if d is not None else rng.uniform(0.3, 1.0)) * rng.uniform(0.6, 1.4)) for p, d in ps}}
        c, f = AFF_OFFSET.get(name, (0.0, 0.0))
        xfs.append({"weight": 1.0, "color": float(rng.uniform()), "color_speed": 0.5, "opacity": 1.0,
                    "vchain": [{"transform": [1.0, 0.0, 0.0, 1.0, c, f], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {name: entry}}]})
    g["xforms"] = xfs
    return g


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    db = lr.flamedb()
    names = db.variations()
    params = variation_params((build.PKG / "config" / "variations_new.yml").read_text())
    g = _flame(names, params)
    f = lr.flame.from_json(db, g)
    k = lr.flame_compiler().get_flame_kernel(db, f, precise_math=1)
    prep = k.prepare_samples(f.pack_samples(4, 256, 256), [0], [0.0])[0]
    twin = Twin(db, f, tmp_path_factory.mktemp("twin"))
    return names, f, k, prep, twin


def _ulps(out, ref):
    scale = np.maximum(np.abs(ref[:, 0]), np.abs(ref[:, 1]))
    ulp = np.spacing(np.maximum(scale, 1e-30).astype(np.float32)).astype(np.float64)
    return np.max(np.abs(out[:, :2] - ref[:, :2]), axis=1) / ulp


@pytest.mark.parametrize("xi", range(47))
def test_variation_matches_fp64_twin(setup, xi):
    names, f, k, prep, twin = setup
    assert len(names) == 47
    name = names[xi]
    rng = np.random.default_rng(1000 + xi)
    pts = np.stack([rng.uniform(-1.5, 1.5, N), rng.uniform(-1.5, 1.5, N), rng.uniform(0, 1, N)], 1).astype(np.float32)
    c, fo = AFF_OFFSET.get(name, (0.0, 0.0))
    if name in AFF_OFFSET:
        pts[:, :2] = np.round(pts[:, :2] * 4096.0) / 4096.0
    out = k.apply_xform(prep, xi, pts, seed=SEED).astype(np.float64)
    P = prep[:f.size_reals()].astype(np.float64)
    idx = np.arange(N)
    ref = twin.apply(P, xi, pts.astype(np.float64), idx, seed=SEED)
    ok = np.all(np.isfinite(ref[:, :2]), axis=1) & (np.abs(ref[:, :2]).max(axis=1) < 1e6)
    assert ok.mean() > 0.9, (name, ok.mean())
    fwd = _ulps(out, ref)
    best = fwd.copy()
    bad = np.nonzero(ok & (fwd > 4))[0]
    if bad.size:
        # backward: the nearest FP64 result over inputs within 2 ulps per coordinate
        q0 = pts[bad].astype(np.float64)
        # ulps of the point the variation sees (after the affine's exact offsets)
        sx = np.spacing((pts[bad, 0] + np.float32(c)).astype(np.float32)).astype(np.float64)
        sy = np.spacing((pts[bad, 1] + np.float32(fo)).astype(np.float32)).astype(np.float64)
        qs, ids = [], []
        for i in range(-2, 3):
            for j in range(-2, 3):
                q = q0.copy()
                q[:, 0] += i * sx
                q[:, 1] += j * sy
                qs.append(q)
                ids.append(bad)
        r2 = twin.apply(P, xi, np.concatenate(qs), np.concatenate(ids), seed=SEED).reshape(25, bad.size, 4)
        for r in r2:
            best[bad] = np.minimum(best[bad], _ulps(out[bad], r))
    p50 = float(np.median(fwd[ok]))
    within = float(np.mean(best[ok] <= 4))
    print(f"{name:14s} forward p50 {p50:.2f} p99 {np.percentile(fwd[ok], 99):.2f} max {fwd[ok].max():.1f} "
          f"backward within 4 ulp {within:.4f} max {best[ok].max():.1f}")
    med, frac = BOUNDED.get(name, (1.0, 1.0))
    assert p50 <= med, (name, p50)
    assert within >= frac, (name, within, float(best[ok].max()))
    np.testing.assert_allclose(out[ok, 2], ref[ok, 2], rtol=1e-6, atol=1e-7)  # colour blend
    assert np.all(out[:, 3] == ref[:, 3])
