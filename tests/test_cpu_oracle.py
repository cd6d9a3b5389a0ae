"""Known-answer checks of the FP64 oracle itself (no GPU): the reference
ships no golden vectors for this path, so the oracle is pinned by cases with
closed-form answers, by the committed golden vectors in tests/golden/, and on
the GPU by the reference's own kernels (tests/test_gpu_image.py)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc
from refraktor_gb300 import synthetic as syn

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_catmull_linear_and_constant_knots():
    # equally spaced linear knots: the centripetal spline is the straight line
    n = 5
    d = np.array([0.5, -2.0, 0.0, 3.0, 1e-3])
    samples = np.concatenate([d * i + 7.0 for i in range(4)])
    c = orc.catmull(samples, n)[0]
    for t in (0.0, 0.3, 0.5, 1.0):
        np.testing.assert_allclose(orc.cubic_eval(c, t), 7.0 + d * (1 + t), rtol=1e-14, atol=1e-14)
    # constant knots: a = b = c = 0, d = p
    c = orc.catmull(np.full(4 * n, 2.5), n)[0]
    np.testing.assert_array_equal(c, np.tile([0.0, 0.0, 0.0, 2.5], (n, 1)))


def test_hsv_palette_known_colours():
    g = syn.plain_flame(0)
    g["palette"] = [[0.0, 1.0, 1.0]] * 64 + [[120.0, 1.0, 1.0]] * 64 + [[240.0, 0.5, 1.0]] * 64 + [[0.0, 0.0, 0.2]] * 64
    _, pal = orc.prepared(g, 64, 64)
    np.testing.assert_allclose(pal[0], [1, 0, 0])
    np.testing.assert_allclose(pal[64], [0, 1, 0])
    np.testing.assert_allclose(pal[128], [127 / 255, 127 / 255, 1])  # 0.5 * 255 = 127.5 truncates to 127
    np.testing.assert_allclose(pal[255], [51 / 255] * 3)


def test_fix_rotation_round_trip():
    g = syn.hd_flame(0)
    R = orc.size_reals(g)
    s = np.tile(orc.pack_sample(g, 320, 200), 4)
    aff = orc.affine_indices(g)
    params, _ = orc.prepared(g, 320, 200)
    # prepared = interpolate(fix_rotation(samples)) of identical knots = the sample itself
    np.testing.assert_allclose(params, s[:R], rtol=1e-12, atol=1e-9)


def test_tonemap_known_values():
    bins = np.zeros((1, 3, 4), np.float32)
    bins[0, 1] = [2.0, 1.0, 0.0, 2.0]
    bins[0, 2] = [0.0, 0.0, 0.0, 16.0]
    q, gamma, B, V = 1.0, 2.0, 4.0, 1.0
    out = orc.tonemap(bins, q, gamma, B, V)
    assert np.all(out[0, 0] == 0)
    k2 = float(np.float32(10.0) ** (-np.log10(np.float32(1.0)) - np.float32(0.5)))
    f = 0.5 * B * math.log10(1 + 2.0 * k2) / 2.0
    w = 2.0 * f
    gf = w ** 0.5 / w
    np.testing.assert_allclose(out[0, 1, :3], [min(2 * f * gf, 1), 1 * f * gf, 0], rtol=1e-12)
    np.testing.assert_allclose(out[0, 1, 3], math.log(2.0) * (4 / math.log(2)) / 96, rtol=1e-12)
    np.testing.assert_allclose(out[0, 2, 3], math.log(16.0) * (4 / math.log(2)) / 96, rtol=1e-12)


def test_density_histogram_known_bins():
    v = np.array([0.0, 0.5, 1.0, 1.9, 2.0, 4.0, 1000.0], np.float32)
    bins = np.zeros((1, v.size, 4), np.float32)
    bins[0, :, 3] = v
    h, mx = orc.density_histogram(bins)
    assert mx == 1000
    assert h[0] == 2 and h[1] == 1  # log2(1) * 4 = 0 -> bin 1
    assert h[4] == 1 and h[5] == 1   # 1.9 -> floor(3.7) + 1 = 4; 2.0 -> 5
    assert h[9] == 1 and h[40] == 1  # 4.0 -> 9; 1000 -> floor(39.86) + 1 = 40
    assert h.sum() == v.size


def test_density_blur_identity_and_conservation():
    rng = np.random.default_rng(0)
    bins = np.zeros((40, 50, 4), np.float32)
    bins[20, 25] = [1, 2, 3, 1.0]   # density 1 -> radius 9: spreads
    bins[5, 5] = [4, 4, 4, 400.0]   # density 400 -> radius 0.45 -> 2 quarter steps: tight
    out = orc.density_blur(bins, 9.0, 0.0, 0.5)
    np.testing.assert_allclose(out.sum(axis=(0, 1)), bins.sum(axis=(0, 1)), rtol=1e-12)
    assert np.count_nonzero(out[..., 3] > 0) > 200
    ident = orc.density_blur(bins, 0.0, 0.0, 0.5)
    np.testing.assert_allclose(ident, bins, rtol=1e-7)


def test_render_single_fixed_point():
    """linear 0.5 toward the origin: every draw lands on the centre pixel."""
    g = syn.plain_flame(0)
    g["xforms"] = [{"weight": 1.0, "color": 0.0, "color_speed": 1.0, "opacity": 1.0,
                    "vchain": [{"transform": [0.5, 0, 0, 0.5, 0, 0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {"linear": 1.0}}]}]
    g["palette"] = [[0.0, 1.0, 1.0]] * 256
    hist, draws = orc.render(g, 64, 64, chains=100, passes=50, warmup=60, threads=2,
                             jitter=np.zeros((1, 2)))
    assert draws == 100 * 50
    assert hist[32, 32, 3] == 5000 and hist[..., 3].sum() == 5000
    np.testing.assert_allclose(hist[32, 32, :3], [5000, 0, 0])


def two_point_chaos_flame() -> dict:
    """Two near-constant maps (to x = -0.25 and x = +0.25; a zero matrix has
    no polar form) with weights 0.9 / 0.1
    and chaos rows that forbid repeating an xform: a chain alternates
    between the two points, so they get equal counts (0.9 / 0.1 without the
    chaos rows)."""
    g = syn.plain_flame(0)
    g["xforms"] = [{"weight": wt, "color": col, "color_speed": 1.0, "opacity": 1.0,
                    "vchain": [{"transform": [1e-6, 0, 0, 1e-6, tx, 0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {"linear": 1.0}}]}
                   for wt, col, tx in ((0.9, 0.0, -0.25), (0.1, 1.0, 0.25))]
    g["chaos"] = [[0.0, 1.0], [1.0, 0.0]]
    g["palette"] = [[0.0, 1.0, 1.0]] * 256
    return g


def test_render_chaos_rows_alternate():
    """Chaos (xaos) rows weight the next pick by the previous xform
    (flame.tpl:170-177): with rows [[0, 1], [1, 0]] every chain alternates."""
    g = two_point_chaos_flame()
    hist, draws = orc.render(g, 64, 64, chains=100, passes=50, warmup=60, threads=2, jitter=np.zeros((1, 2)))
    assert draws == 100 * 50
    left, right = hist[:, :32, 3].sum(), hist[:, 32:, 3].sum()
    assert left == right == 2500
    assert np.count_nonzero(hist[..., 3]) == 2
    del g["chaos"]
    hist, _ = orc.render(g, 64, 64, chains=100, passes=50, warmup=60, threads=2, jitter=np.zeros((1, 2)))
    assert abs(hist[:, :32, 3].sum() - 4500) < 200


def test_apply_known_points():
    g = syn.plain_flame(0)
    g["xforms"] = [{"weight": 1.0, "color": 0.25, "color_speed": 0.5, "opacity": 0.7,
                    "vchain": [{"transform": [1, 0, 0, 1, 0, 0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {"spherical": 2.0}}]}]
    params, _ = orc.prepared(g, 64, 64)
    x, y, c, op = orc.apply(g, params, 0, 0.5, 0.0, 1.0)
    assert (x, y) == pytest.approx((4.0, 0.0))  # 2 * p / |p|^2
    assert c == pytest.approx(0.625) and op == pytest.approx(0.7)


def test_golden_vectors():
    """Committed FP64 vectors (tests/golden/make_golden.py): the oracle keeps
    producing them."""
    path = GOLDEN / "oracle_vectors.json"
    gold = json.loads(path.read_text())
    for case in gold["apply"]:
        g = case["genome"]
        params, _ = orc.prepared(g, 64, 64)
        for (x, y, c), want in zip(case["points"], case["out"]):
            got = orc.apply(g, params, case["xform"], x, y, c)
            np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)
    for case in gold["tonemap"]:
        bins = np.array(case["bins"], np.float32)
        got = orc.tonemap(bins, *case["args"])
        np.testing.assert_allclose(got, np.array(case["out"]), rtol=1e-13, atol=1e-15)
    for case in gold["catmull"]:
        got = orc.catmull(np.array(case["samples"]), case["n"])
        np.testing.assert_allclose(got, np.array(case["coeff"]), rtol=1e-14, atol=1e-15)
