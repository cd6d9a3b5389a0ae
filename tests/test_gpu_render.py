"""GPU parity of the chaos game: interpolation, single map application,
converged renders against the FP64 oracle, and the bailout / resume / abort
behaviour of warmup + bin."""
import threading
import time
import zlib

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as orc
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn
from tests import fp32_ideal as fi
from tests.pick_tables import alias_distribution

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def comp():
    return lr.flame_compiler()


def _one_variation_flame(name, seed):
    rng = np.random.default_rng(seed)
    g = syn.plain_flame(seed)
    m = rng.uniform(-1, 1, size=(2, 2))
    g["xforms"] = [{"weight": 1.0, "color": 0.3, "color_speed": 0.5, "opacity": 1.0,
                    "vchain": [{"transform": [m[0, 0], m[1, 0], m[0, 1], m[1, 1], *rng.uniform(-0.5, 0.5, 2)],
                                "mod_x": 0, "mod_y": 0, "mod_scale": 1, "mod_rotate": 0,
                                "variations": {name: float(rng.uniform(0.2, 1.0))}}]}]
    return g


def test_warmup_and_bin_reach_quality(db, comp):
    g = syn.plain_flame(0)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    assert not k.info["has_final"]
    assert k.info["fma_per_iter"] == pytest.approx(8.0)  # one vlink affine per xform + the projection
    w, h = 256, 192
    st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=1, count=20)
    r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=64.0))
    assert r.status & 1
    # the overshoot is at most one round of passes of every chain
    chains = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    assert 64.0 <= r.quality <= 64.0 * 1.13 + chains / (w * h)
    assert r.total_bins == w * h
    bins = st.bins().cpu().numpy()
    # opacity 1 everywhere: density sum = draws = quality * pixels
    assert abs(bins[..., 3].sum() - r.draw_count) <= 1e-4 * r.draw_count
    assert r.total_draws == int(r.quality * w * h)
    assert r.max_density == pytest.approx(float(np.floor(bins[..., 3].max())), abs=1.0)
    # resume: a second call keeps accumulating
    r2 = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=16.0))
    assert st.quality == pytest.approx(r.quality + r2.quality)
    bins2 = st.bins().cpu().numpy()
    assert bins2[..., 3].sum() == pytest.approx(r.draw_count + r2.draw_count, rel=1e-5)


def test_pass_cap_and_time_bailouts(db, comp):
    f = lr.flame.from_json(db, syn.plain_flame(1))
    k = comp.get_flame_kernel(db, f)
    st = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=2, count=10)
    r = k.bin(st, lr.bailout_args(iters=64, millis=0, quality=0))
    assert r.status == 8
    chains = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    assert r.total_passes == 64 * chains
    t0 = time.time()
    r = k.bin(st, lr.bailout_args(iters=0, millis=50, quality=0))
    assert r.status & 2
    assert 40 <= r.elapsed_ms < 2000
    assert time.time() - t0 < 5


def test_abort_from_another_thread(db, comp):
    f = lr.flame.from_json(db, syn.plain_flame(2))
    k = comp.get_flame_kernel(db, f)
    st = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=3, count=10)
    k.bin_async(st, lr.bailout_args(iters=0, millis=20000, quality=0))
    threading.Timer(0.2, st.abort_binning).start()
    t0 = time.time()
    r = st.wait()
    assert r.status & 4
    assert time.time() - t0 < 10


def test_abort_right_after_bin_async_on_a_busy_stream(db, comp):
    """An abort issued as soon as bin_async returns, while earlier work (a
    500 ms time-budget bin of another state) still occupies the stream, stops
    the new call at its first check: the stop flag is cleared on the host
    before the call queues anything, so nothing queued later can wipe out the
    abort."""
    import torch

    f = lr.flame.from_json(db, syn.plain_flame(2))
    k = comp.get_flame_kernel(db, f)
    s = torch.cuda.Stream()
    busy = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=5, count=10, stream=s)
    st = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=6, count=10, stream=s)
    k.bin_async(busy, lr.bailout_args(iters=0, millis=500, quality=0), stream=s)
    k.bin_async(st, lr.bailout_args(iters=0, millis=20000, quality=0), stream=s)
    st.abort_binning()
    t0 = time.time()
    rb = busy.wait()
    r = st.wait()
    assert rb.status & 2
    assert r.status & 4, r
    assert r.elapsed_ms < 1000, r
    assert time.time() - t0 < 5


def test_second_bin_async_while_pending_is_rejected(db, comp):
    """One bin call per state at a time: a second bin_async before the first
    is waited for fails and leaves the pending call and its result intact."""
    f = lr.flame.from_json(db, syn.plain_flame(2))
    k = comp.get_flame_kernel(db, f)
    st = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=3, count=10)
    k.bin_async(st, lr.bailout_args(iters=0, millis=0, quality=2.0))
    with pytest.raises(lr.RfkError):
        k.bin_async(st, lr.bailout_args(iters=0, millis=0, quality=2.0))
    r = st.wait()
    assert r.status & 1 and r.quality >= 2.0
    assert abs(st.quality - r.quality) < 1e-9
    r2 = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=1.0))
    assert r2.status & 1


def _guard_flame(bad_xform: dict, final: dict | None = None) -> dict:
    """Two xforms of weight 0.5: `bad_xform`, whose every step leaves a bad
    value, and the identity; the camera maps [-1, 1]^2 exactly onto a square
    image."""
    g = syn.plain_flame(3)
    g.update(center_x=0.0, center_y=0.0, scale=0.5, rotate=0.0)
    ident = {"weight": 0.5, "color": 0.8, "color_speed": 0.5, "opacity": 1.0,
             "vchain": [{"transform": [1.0, 0.0, 0.0, 1.0, 0.0, 0.0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                         "mod_rotate": 0, "variations": {"linear": 1.0}}]}
    g["xforms"] = [bad_xform, ident]
    if final is not None:
        g["final_xform"] = final
    return g


def _bad_xform(transform, variation):
    return {"weight": 0.5, "color": 0.2, "color_speed": 0.5, "opacity": 1.0,
            "vchain": [{"transform": transform, "mod_x": 0, "mod_y": 0, "mod_scale": 1, "mod_rotate": 0,
                        "variations": {variation: 1.0}}]}


@pytest.mark.parametrize("kind", ["overflow", "nan"])
def test_bad_value_guard_resets_uniformly_with_zero_opacity(kind):
    """The bad-value guard (refactor.cu:195-199, flamelib.h:25): a point that
    leaves an xform as NaN or beyond 1e10 restarts uniformly in [-1, 1]^2 and
    the step draws nothing (opacity 0). Xform 0 always leaves a bad value (an
    offset of 1e12, or a variation whose log of a negative number is NaN),
    xform 1 is the identity. (a) Every identity step draws the restarted
    point, so half the steps draw and the density is flat over the image.
    (b) With a final xform that maps every point to the image centre, a draw
    of xform 0's step would land there too: draws stay at half the steps, so
    the reset step's opacity is 0."""
    db = lr.flamedb()
    if kind == "nan":
        db.add_or_update_variations("nan_probe: result += (weight * log(-1.0 - p.x * p.x)) * p;\n")
        bad = _bad_xform([1.0, 0.0, 0.0, 1.0, 0.0, 0.0], "nan_probe")
    else:
        bad = _bad_xform([1.0, 0.0, 0.0, 1.0, 1e12, 0.0], "linear")
    comp = lr.flame_compiler()
    w = h = 64
    squash = {"weight": 0.0, "color": 0.5, "color_speed": 0.0, "opacity": 1.0,
              "vchain": [{"transform": [1e-6, 0.0, 0.0, 1e-6, 0.0, 0.0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                          "mod_rotate": 0, "variations": {"linear": 1.0}}]}
    for final in (None, squash):
        g = _guard_flame(bad, final)
        f = lr.flame.from_json(db, g)
        k = comp.get_flame_kernel(db, f)
        st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=4, count=20)
        r = k.bin(st, lr.bailout_args(iters=24, millis=0, quality=0))
        frac = r.draw_count / r.total_passes
        assert abs(frac - 0.5) < 0.005, (kind, final is not None, frac)
        dens = st.bins().cpu().numpy()[..., 3].astype(np.float64)
        assert abs(dens.sum() - r.draw_count) <= 1e-6 * r.draw_count + 1
        if final is None:
            # flat: every pixel hit, and each quadrant and the edge rows hold
            # their area's share of the draws
            assert np.all(dens > 0)
            q = dens.reshape(2, h // 2, 2, w // 2).sum(axis=(1, 3)) / dens.sum()
            np.testing.assert_allclose(q, 0.25, atol=0.01)
            edge = (dens[0].sum() + dens[-1].sum() + dens[:, 0].sum() + dens[:, -1].sum()) / dens.sum()
            assert abs(edge - 4 * 64 / 4096) < 0.01, edge
        else:
            # everything lands on the few pixels at the centre (screen jitter ~ 1/3 px)
            ys, xs = np.nonzero(dens)
            assert np.all(np.abs(ys - h // 2) <= 3) and np.all(np.abs(xs - w // 2) <= 3)


def test_rewarm_reuses_the_state(db, comp):
    """rfk_state_rewarm: warm-up into an existing state with new samples and
    seed renders exactly what a new state warmed up with them renders (same
    draws under a pass cap), restarts the quality at 0, and with clear=False
    keeps what the histogram held. Four passes keep the hottest pixels' sums
    far below 2^24, where FP32 additions stay exact enough to compare."""
    f1 = lr.flame.from_json(db, syn.plain_flame(4))
    k = comp.get_flame_kernel(db, f1)
    w, h = 96, 64
    s1 = f1.pack_samples(4, w, h)
    # samples of the kernel's structure with other values: every xform real scaled
    s2 = np.array(s1, dtype=np.float64).reshape(4, -1)
    s2[:, 13:f1.size_reals()] *= 0.97
    s2 = s2.ravel()
    st = k.warmup(s1, (w, h), seed=3, count=20)
    k.bin(st, lr.bailout_args(iters=4, millis=0, quality=0))
    ptr = st.bins_ptr()
    st.rewarm(s2, seed=9, count=20)
    assert st.quality == 0.0 and st.bins_ptr() == ptr
    assert float(st.bins().abs().sum().item()) == 0.0
    r = k.bin(st, lr.bailout_args(iters=4, millis=0, quality=0))
    fresh = k.warmup(s2, (w, h), seed=9, count=20)
    rf = k.bin(fresh, lr.bailout_args(iters=4, millis=0, quality=0))
    assert r.draw_count == rf.draw_count and r.quality == rf.quality
    a, b = st.bins().cpu().numpy(), fresh.bins().cpu().numpy()
    # the same draws; atomics may add them in another order (opacities are
    # not 1 here, so the sums round differently in the last bits)
    np.testing.assert_array_equal(a[..., 3] > 0, b[..., 3] > 0)
    np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)
    # without clearing, the next render draws on top: the same draws again
    # (each added to a sum that already holds the first render's). Every add
    # into a hot pixel now rounds at that pixel's doubled magnitude, and the
    # opacities are nearly constant, so the rounding errors add up with one
    # sign (measured 2e-4 of the total alpha); 1e-3 still separates the kept
    # histogram (2x the sums) from a cleared one (1x).
    st.rewarm(s2, seed=9, count=20, clear=False)
    r2 = k.bin(st, lr.bailout_args(iters=4, millis=0, quality=0))
    assert r2.draw_count == rf.draw_count
    c2 = st.bins().cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(c2.sum(axis=(0, 1)), 2 * b.astype(np.float64).sum(axis=(0, 1)), rtol=1e-3)
    np.testing.assert_array_equal(c2[..., 3] > 0, b[..., 3] > 0)
    # not while a bin call is pending
    k.bin_async(st, lr.bailout_args(iters=5, millis=0, quality=0))
    with pytest.raises(lr.RfkError):
        st.rewarm(s2, seed=1, count=20)
    st.wait()


def test_deterministic_with_pass_cap(db, comp):
    g = syn.plain_flame(4)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    outs = []
    for _ in range(2):
        st = k.warmup(f.pack_samples(4, 96, 96), (96, 96), seed=9, count=20)
        k.bin(st, lr.bailout_args(iters=40, millis=0, quality=0))
        outs.append(st.bins().cpu().numpy())
    # atomics reorder float sums: the counts (alpha, sums of 1.0) are exact, the
    # colour sums of hot pixels (1e5 terms) may differ in the last digits
    np.testing.assert_array_equal(outs[0][..., 3], outs[1][..., 3])
    np.testing.assert_allclose(outs[0], outs[1], rtol=1e-4, atol=1e-6)


def test_warmup_adopts_the_callers_histogram(db, comp):
    """warmup(samples, bins&&, ...) (flame_compiler.cpp:1037-1101): the state
    draws into the caller's image as it is, without clearing it."""
    g = syn.plain_flame(4)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    w, h = 96, 64
    samples = f.pack_samples(4, w, h)
    st = k.warmup(samples, (w, h), seed=9, count=20)
    r1 = k.bin(st, lr.bailout_args(iters=10, millis=0, quality=0))
    ref = st.bins().cpu().numpy().astype(np.float64)
    pre = torch.ones((h, w, 4), dtype=torch.float32, device="cuda")
    st2 = k.warmup(samples, pre, seed=9, count=20)
    assert st2.dims == (w, h) and st2.bins().data_ptr() == pre.data_ptr()
    r2 = k.bin(st2, lr.bailout_args(iters=10, millis=0, quality=0))
    assert r2.draw_count == r1.draw_count and r2.quality == r1.quality
    got = pre.cpu().numpy().astype(np.float64)
    np.testing.assert_array_equal(got[..., 3] - 1.0, ref[..., 3])  # same draws on top of the 1.0 already there
    np.testing.assert_allclose(got[..., :3] - 1.0, ref[..., :3], rtol=1e-4, atol=1e-5)
    del st2
    assert torch.all(pre[..., 3] >= 1.0).item()  # the caller's buffer outlives the state
    with pytest.raises(lr.RfkError):
        k.warmup(samples, torch.ones((h, w, 3), dtype=torch.float32, device="cuda"), seed=9, count=1)


def test_prepared_blocks_are_finite_and_repeatable(db, comp):
    """Every float of a prepared parameter block is defined: the padding after
    the reals (an odd count) and before the 16-byte aligned palette is 0, and
    two identical calls give the same bits (the blocks feed the bin kernels,
    the batch and the allocation-free entry point alike)."""
    g = syn.hd_flame(4)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    samples = f.pack_samples(4, 320, 180)
    seg, t = [0, 0, 0, 0], [0.0, 0.3, 0.6, 0.9]
    a = k.prepare_samples(samples, seg, t, seed=3)
    b = k.prepare_samples(samples, seg, t, seed=3)
    assert np.all(np.isfinite(a))
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    R = f.size_reals()
    pal0 = k.info["sample_floats"] - 1024
    if R % 2:
        assert np.all(a[:, R] == 0.0)
    # the floats between the pick tables and the palette (alignment padding)
    nx = k.info["num_xforms"]
    end_tables = (R + 1) // 2 * 2 + 2 * nx + (2 * nx * nx if k.info["chaos"] else 0)
    assert np.all(a[:, end_tables:pal0] == 0.0)


def test_prepared_flame_matches_oracle_interpolation(db, comp):
    """Row a3/a4: FP32 Catmull-Rom + polar affines + 8-bit palette vs FP64."""
    rng = np.random.default_rng(11)
    g = syn.hd_flame(3)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    w, h = 640, 360
    base = f.pack_sample(w, h)
    R = f.size_reals()
    keys = []
    for i in range(5):
        s = base.copy()
        s[13:R] += rng.normal(0, 0.05, R - 13)
        s[R:] = base[R:]
        keys.append(s)
    samples = np.concatenate(keys)
    seg = np.array([0, 0, 1, 1, 0, 1], dtype=np.uint32)
    t = np.array([0.0, 0.3, 0.5, 0.99, 0.75, 0.1], dtype=np.float32)
    got = k.prepare_samples(samples, seg, t)
    aff = set()
    for a in f.affine_indices():
        aff.update(range(a, a + 4))
    fixed = orc.fix_rotation(samples, R + 768, R, f.affine_indices()).reshape(5, -1)
    for i in range(len(seg)):
        p_ref, pal_ref = orc.prepared(g, w, h, t=float(t[i]), seg=int(seg[i]), samples=samples)
        p = got[i, :R].astype(np.float64)
        # weight sum slot, jitter-shifted screen translation and precalc slots are device-computed
        mask = np.ones(R, bool)
        mask[[4, 5, 12]] = False
        # interpolated reals: 4 FP32 ulps of the segment's largest knot (after the
        # angle / log-magnitude rewrite that the spline runs on)
        scale = np.max(np.abs(fixed[seg[i]:seg[i] + 4, :R]), axis=0)
        tol = 4 * np.spacing(scale.astype(np.float32)).astype(np.float64)
        for a in f.affine_indices():
            # affine columns are mag * (cos, sin) of interpolated (angle, log mag):
            # 8 ulps of the column magnitude
            for col in (0, 2):
                mag = np.hypot(p_ref[a + col], p_ref[a + col + 1])
                tol[a + col] = tol[a + col + 1] = 8 * np.spacing(np.float32(max(mag, 1e-30)))
        assert np.all((np.abs(p - p_ref) <= tol)[mask]), np.nonzero((np.abs(p - p_ref) > tol) & mask)
        # screen translation moved by the Gaussian(1/3 px) jitter
        assert abs(p[4] - p_ref[4]) < 3.0 and abs(p[5] - p_ref[5]) < 3.0
        pal = got[i, k.info["sample_floats"] - 1024:].reshape(256, 4)[:, :3]
        assert np.all(np.abs(pal - pal_ref) <= 1.0 / 255 + 1e-6)
        assert np.mean(np.abs(pal - pal_ref) < 1e-6) > 0.98


DETERMINISTIC = ["linear", "sinusoidal", "spherical", "swirl", "horseshoe", "polar", "handkerchief", "heart", "disc",
                 "spiral", "hyperbolic", "exponential", "power", "fisheye", "bubble", "diamond", "ex", "bent",
                 "cylinder", "exp", "eyefish", "cosine"]


def _ulp_errors(got, ref):
    """Error in FP32 ulps of the larger output component of each point."""
    scale = np.maximum(np.abs(ref[:, 0]), np.abs(ref[:, 1]))
    ulp = np.spacing(np.maximum(scale, 1e-30).astype(np.float32)).astype(np.float64)
    return np.max(np.abs(got[:, :2] - ref[:, :2]), axis=1) / ulp


def test_affine_step_exact_fma(db, comp):
    """The affine half of a map: x' = a x + b y + c as fma(a, x, fma(b, y, c))
    (flame.tpl:10-14), within 1 ulp of the largest term against FP64."""
    g = _one_variation_flame("linear", seed=3)
    g["xforms"][0]["vchain"][0]["variations"] = {"linear": 1.0}
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f, precise_math=1)
    prep = k.prepare_samples(f.pack_samples(4, 256, 256), [0], [0.0])[0]
    rng = np.random.default_rng(13)
    pts = np.stack([rng.uniform(-3, 3, 2048), rng.uniform(-3, 3, 2048), rng.uniform(0, 1, 2048)], 1).astype(np.float32)
    out = k.apply_xform(prep, 0, pts).astype(np.float64)
    a, d, b, e, c, ff = prep[17:23].astype(np.float64)
    x, y = pts[:, 0].astype(np.float64), pts[:, 1].astype(np.float64)
    # two roundings (inner and outer fma), each at most half an ulp of a partial
    # sum bounded by |a x| + |b y| + |c|
    for got, ref, terms in [(out[:, 0], a * x + b * y + c, abs(a * x) + abs(b * y) + abs(c)),
                            (out[:, 1], d * x + e * y + ff, abs(d * x) + abs(e * y) + abs(ff))]:
        assert np.all(np.abs(got - ref) <= np.spacing(terms.astype(np.float32)))


# Variations whose formula composes FP32-rounded angles of magnitude up to 2 pi
# with the radius (atan +- sqrt, sqrt * atan) or cancels (spiral: cosa + sin r,
# polar: sqrt - 1): the rounding of those intermediate arguments alone exceeds
# 4 ulp of the output for some inputs - even with every FP32 operation
# correctly rounded (tests/test_cpu_fp32_bounds.py) - so they are held to the
# measured distribution bounds of tests/fp32_ideal.py: forward-error median /
# 90th percentile in ulp, and the fraction of points whose backward error is
# within 4 ulp (GB300, 2048 points, |p| <= 1.5).
ANGLE_COMPOSED = fi.ANGLE_COMPOSED


@pytest.mark.parametrize("name", DETERMINISTIC)
def test_single_map_within_4_ulp(db, comp, name):
    """The variation half of a map in the precise-math build vs FP64
    evaluations of the reference formula (identity affine, so the FP32 input
    reaches the variation unrounded). Backward-error form: every FP32 result
    is within 4 ulp (of the larger output component) of the FP64 result at
    some input within 2 ulp of the given one - FP32 arguments such as
    sqrt * atan or (atan + sqrt) carry rounding that no FP32 evaluation can
    avoid. The forward error at the exact input is reported and bounded too:
    median <= 1 ulp, 90% <= 4 ulp."""
    g = _one_variation_flame(name, seed=zlib.crc32(name.encode()) % 1000)
    g["xforms"][0]["vchain"][0]["transform"] = [1.0, 0.0, 0.0, 1.0, 0.0, 0.0]
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f, precise_math=1)
    prep = k.prepare_samples(f.pack_samples(4, 256, 256), [0], [0.0])[0]
    rng = np.random.default_rng(12)
    n = 2048
    pts = np.stack([rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n), rng.uniform(0, 1, n)], 1).astype(np.float32)
    out = k.apply_xform(prep, 0, pts).astype(np.float64)
    P = prep[:f.size_reals()].astype(np.float64)
    ref = orc.apply_many(g, P, 0, pts)
    ok = np.all(np.isfinite(ref[:, :2]), axis=1) & (np.abs(ref[:, :2]).max(axis=1) < 1e6)
    scale = np.maximum(np.abs(ref[:, 0]), np.abs(ref[:, 1]))
    ulp = np.spacing(np.maximum(scale, 1e-30).astype(np.float32)).astype(np.float64)
    fwd = np.max(np.abs(out[:, :2] - ref[:, :2]), axis=1) / ulp
    # backward: nearest FP64 result over inputs perturbed by up to 2 ulps per coordinate
    best = fwd.copy()
    sx = np.spacing(pts[:, 0]).astype(np.float64)
    sy = np.spacing(pts[:, 1]).astype(np.float64)
    for i in range(-2, 3):
        for j in range(-2, 3):
            q = pts.astype(np.float64).copy()
            q[:, 0] += i * sx
            q[:, 1] += j * sy
            r2 = orc.apply_many(g, P, 0, q)
            best = np.minimum(best, np.max(np.abs(out[:, :2] - r2[:, :2]), axis=1) / ulp)
    print(name, "forward ulp p50/p90/p99/max", np.percentile(fwd[ok], [50, 90, 99, 100]).round(2),
          "backward max", float(best[ok].max()))
    if name in ANGLE_COMPOSED:
        p50, p90, frac = ANGLE_COMPOSED[name]
        assert np.median(fwd[ok]) <= p50 and np.percentile(fwd[ok], 90) <= p90, (name, np.percentile(fwd[ok], [50, 90]))
        assert np.mean(best[ok] <= 4) >= frac, (name, np.mean(best[ok] <= 4))
    else:
        assert np.all(best[ok] <= 4), (name, float(best[ok].max()))
        frac4 = fi.FORWARD_WITHIN_4.get(name, 0.99)
        assert np.median(fwd[ok]) <= 1.0 and np.mean(fwd[ok] <= 4) >= frac4, (name, np.percentile(fwd[ok], [50, 99]))
    np.testing.assert_allclose(out[:, 2], ref[:, 2], rtol=1e-6, atol=1e-7)  # colour blend
    assert np.all(out[:, 3] == 1.0)


def _density(hist):
    d = hist[..., 3].astype(np.float64)
    return d / d.sum()


def _render_parity(db, comp, g, w, h, spps, channels=(3,), threads=8):
    """GPU render vs two FP64 oracle renders fed with the same inputs: the
    device-prepared flame parameters and 8-bit palette (interpolation parity
    is tested on its own), the device's per-block screen jitters, and the same
    schedule - as many chains, Hammersley start points, 20 warm-up passes and
    the same number of drawing passes per chain."""
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    R = f.size_reals()
    p_ref, _ = orc.prepared(g, w, h)
    res = {}
    chains = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    for spp in spps:
        # a pass cap gives every chain the same number of passes, as the oracle
        # schedule; a quality target would let early blocks run extra passes
        passes = max(1, int(np.ceil(spp * w * h / chains)))
        st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=5, count=20)
        r = k.bin(st, lr.bailout_args(iters=passes, millis=0, quality=0))
        assert r.total_passes == passes * chains
        gpu = st.bins().cpu().numpy().astype(np.float64)
        samp = st.samples()
        params = samp[0, :R].astype(np.float64)
        params[4], params[5] = p_ref[4], p_ref[5]
        jit = np.stack([samp[:, 4] - p_ref[4], samp[:, 5] - p_ref[5]], 1)
        pal = samp[0, k.info["sample_floats"] - 1024:].reshape(256, 4)[:, :3].astype(np.float64)
        kw = dict(warmup=20, threads=threads, params=params, palette=pal, jitter=jit, hammersley=True)
        o1, _ = orc.render(g, w, h, chains, passes, seed=1, **kw)
        o2, _ = orc.render(g, w, h, chains, passes, seed=2, **kw)
        for c in channels:
            a = gpu[..., c] / gpu[..., c].sum()
            b1 = o1[..., c] / o1[..., c].sum()
            b2 = o2[..., c] / o2[..., c].sum()
            res[(spp, c)] = (float(np.abs(a - b1).sum()), float(np.abs(b1 - b2).sum()))
    return res


def test_render_matches_oracle_below_noise_floor(db, comp):
    """Converged-render parity: normalised density L1 between the GPU and the
    FP64 oracle at equal spp stays within 1.25x the L1 between two oracle
    seeds (the Monte-Carlo noise floor), and shrinks as spp grows (no bias
    floor). The oracle draws with the GPU's per-block screen jitters."""
    res = _render_parity(db, comp, syn.plain_flame(0), 128, 128, (16.0, 256.0))
    for (spp, c), (d, floor) in res.items():
        assert d < 1.25 * floor, (spp, d, floor)
    assert res[(256.0, 3)][0] < 0.5 * res[(16.0, 3)][0]


def test_hd_render_colour_matches_oracle(db, comp):
    """8 xforms + final xform, 14-variation set: density and colour channels."""
    res = _render_parity(db, comp, syn.hd_flame(0), 160, 90, (64.0,), channels=(0, 1, 2, 3))
    for (spp, c), (d, floor) in res.items():
        assert d < 1.25 * floor, (c, d, floor)


def test_pick_tables_encode_xform_weights(db, comp):
    """The alias tables of a prepared block pick xform k with probability
    weight_k / sum (zero weights never), and chaos row r with probability
    chaos[r][k] * weight_k / sum over k (flame.tpl:110-123, :170-177)."""
    g = syn.hd_flame(5)
    n = len(g["xforms"])
    g["xforms"][2]["weight"] = 0.0
    rng = np.random.default_rng(9)
    chaos = rng.uniform(0, 2, size=(n, n)) * (rng.uniform(size=(n, n)) < 0.7)
    chaos[3] = 0.0  # an all-zero row picks xform 0, as the reference's fallback
    g["chaos"] = chaos.tolist()
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    got = k.prepare_samples(f.pack_samples(4, 320, 240), [0], [0.0])[0]
    R = f.size_reals()
    wt = np.array([x["weight"] for x in g["xforms"]], dtype=np.float64)
    p = alias_distribution(got, R, n)
    np.testing.assert_allclose(p, wt / wt.sum(), atol=2e-6)
    assert p[2] == 0.0
    for r in range(n):
        row = chaos[r] * wt
        want = row / row.sum() if row.sum() > 0 else np.eye(n)[0]
        pr = alias_distribution(got, R, n, row=r)
        np.testing.assert_allclose(pr, want, atol=2e-6, err_msg=str(r))
        assert np.all(pr[row == 0] == 0.0) or row.sum() == 0


@pytest.mark.parametrize("sort", [2, 1, -1])
def test_chaos_rows_alternate(db, comp, sort):
    """Chaos rows [[0, 1], [1, 0]] on two near-constant maps (weights 0.9 /
    0.1): every chain alternates between the two points, so under a pass cap
    of an even number of passes both get exactly half of the draws, as in the
    oracle (tests/test_cpu_oracle.py)."""
    from tests.test_cpu_oracle import two_point_chaos_flame

    g = two_point_chaos_flame()
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f, sort=sort)
    assert k.info["chaos"] == 1
    st = k.warmup(f.pack_samples(4, 64, 64), (64, 64), seed=3, count=20)
    r = k.bin(st, lr.bailout_args(iters=20, millis=0, quality=0))
    d = st.bins().cpu().numpy()[..., 3].astype(np.float64)
    assert r.draw_count == r.total_passes and d.sum() == r.draw_count
    assert d[:, :32].sum() == d[:, 32:].sum() == r.draw_count / 2


def test_chaos_render_matches_oracle(db, comp):
    """A chaos flame (8 xforms + final, random chaos rows with zeros) against
    the FP64 oracle below the Monte-Carlo noise floor, density and colour."""
    # a seed whose chaos flame covers a third of the 160 x 90 frame (many
    # seeds collapse onto a few pixels, where FP32 pixel rounding outweighs
    # the Monte-Carlo noise)
    g = syn.hd_flame(21)
    rng = np.random.default_rng(121)
    n = len(g["xforms"])
    rows = rng.uniform(0.2, 1.5, size=(n, n)) * (rng.uniform(size=(n, n)) < 0.75)
    rows[np.arange(n), rng.integers(0, n, n)] += 0.5  # no all-zero row
    g["chaos"] = rows.tolist()
    res = _render_parity(db, comp, g, 160, 90, (64.0,), channels=(0, 1, 2, 3))
    for (spp, c), (d, floor) in res.items():
        assert d < 1.25 * floor, (c, d, floor)


@pytest.mark.parametrize("sort,flush", [(2, 0), (2, 1), (2, 2), (2, 3), (2, 4), (1, 2), (1, 4), (-1, 1), (-1, 4)])
def test_sort_and_flush_variants_agree(db, comp, sort, flush):
    """Every (sort, flush) variant the autotuner may pick renders the same
    flame: exact draw counts under a pass cap, the same density up to
    Monte-Carlo noise (L1 within 1.25x the noise floor of two oracle seeds
    against the default variant), and deterministic repeats."""
    g = syn.hd_flame(1)
    w, h = 160, 120
    f = lr.flame.from_json(db, g)
    base = comp.get_flame_kernel(db, f)
    k = comp.get_flame_kernel(db, f, sort=sort, flush=flush)
    chains_b = base.info["grid"] * base.info["block"] * base.info["chains_per_thread"]
    chains_k = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    passes = 64
    dens = []
    for kern, chains in ((base, chains_b), (k, chains_k), (k, chains_k)):
        st = kern.warmup(f.pack_samples(4, w, h), (w, h), seed=11, count=20)
        r = kern.bin(st, lr.bailout_args(iters=passes, millis=0, quality=0))
        assert r.total_passes == passes * chains
        b = st.bins().cpu().numpy().astype(np.float64)
        assert abs(b[..., 3].sum() - r.draw_count) <= 1e-4 * r.draw_count
        dens.append(b[..., 3])
    np.testing.assert_array_equal(dens[1], dens[2])  # same variant twice: identical counts
    a = dens[0] / dens[0].sum()
    c = dens[1] / dens[1].sum()
    # noise floor at this sample count from the oracle
    p_ref, pal = orc.prepared(g, w, h)
    o1, _ = orc.render(g, w, h, chains_k, passes, seed=1, threads=8, params=p_ref, palette=pal, hammersley=True)
    o2, _ = orc.render(g, w, h, chains_k, passes, seed=2, threads=8, params=p_ref, palette=pal, hammersley=True)
    floor = np.abs(o1[..., 3] / o1[..., 3].sum() - o2[..., 3] / o2[..., 3].sum()).sum()
    assert np.abs(a - c).sum() < 1.25 * floor + 0.002, (np.abs(a - c).sum(), floor)


@pytest.mark.parametrize("flush", [0, 1, 2, 4])
def test_hot_pixel_past_2_24_draws(db, comp, flush):
    """A flame whose one xform (x/2, y/2) pulls every chain onto the origin,
    framed at the centre of a 64 x 64 image, so that the warmed-up chains'
    draws all land on the (jittered) centre pixels, opacity 1, about 200 M
    draws: each of the few hot pixels passes 2^24 draws. With one red.v4 per
    draw (flush 0) a pixel that reaches 2^24 stays there - 2^24 + 1 is a tie
    that rounds to the even 2^24 - so the histogram loses most of the draws;
    this is why the autotuner never picks it. The aggregating strategies add
    warp or block sums, which keep counting: the density sum equals the draw
    count."""
    g = syn.plain_flame(3)
    g.update(center_x=0.0, center_y=0.0, scale=0.5, rotate=0.0)
    g["xforms"] = [{"weight": 1.0, "color": 0.5, "color_speed": 0.5, "opacity": 1.0,
                    "vchain": [{"transform": [0.5, 0.0, 0.0, 0.5, 0.0, 0.0], "mod_x": 0, "mod_y": 0, "mod_scale": 1,
                                "mod_rotate": 0, "variations": {"linear": 1.0}}]}]
    g.pop("final_xform", None)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f, sort=2, flush=flush)
    w = h = 64
    chains = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    passes = int(np.ceil(2.0e8 / chains))
    st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=4, count=40)
    r = k.bin(st, lr.bailout_args(iters=passes, millis=0, quality=0))
    assert r.draw_count == passes * chains  # every step draws, inside the image
    dens = st.bins().cpu().numpy().astype(np.float64)[..., 3]
    assert dens.max() > 2.0 ** 24 or flush == 0
    if flush == 0:
        assert dens.max() == 2.0 ** 24
        assert dens.sum() < 0.9 * r.draw_count
    else:
        assert abs(dens.sum() - r.draw_count) <= 1e-5 * r.draw_count, (dens.sum(), r.draw_count)


def test_autotune_picks_a_tested_variant_and_caches(db, comp):
    """rfk_autotune: its pick is one of the (sort, flush) variants that
    test_sort_and_flush_variants_agree renders against the default, with a
    launch shape that compiles and renders; a second call with the same flame,
    samples and size is answered from the cache (no candidate runs, same
    options), and another size is tuned again."""
    # aggregating strategies only: one red per draw stops counting at 2^24
    # (test_hot_pixel_past_2_24_draws)
    tested = {(2, 1), (2, 2), (2, 4), (1, 2), (1, 4), (-1, 1), (-1, 4)}
    f = lr.flame.from_json(db, syn.hd_flame(6))
    w, h = 320, 180
    samples = f.pack_samples(4, w, h)
    opts, rep = lr.autotune(db, f, samples, (w, h), passes=64)
    assert rep["candidates"] >= 8
    assert rep["best_iters_per_s"] >= rep["worst_iters_per_s"] > 0
    assert (opts["sort"], opts["flush"]) in tested
    k = comp.get_flame_kernel(db, f, **opts)
    assert (k.info["sort"], k.info["flush"]) == (opts["sort"], opts["flush"])
    st = k.warmup(samples, (w, h), seed=1, count=20)
    assert k.bin(st, lr.bailout_args(iters=0, millis=0, quality=8.0)).status & 1
    opts2, rep2 = lr.autotune(db, f, samples, (w, h), passes=64)
    assert rep2["candidates"] == 0 and opts2 == opts
    assert rep2["best_iters_per_s"] == rep["best_iters_per_s"]
    _, rep3 = lr.autotune(db, f, f.pack_samples(4, 256, 144), (256, 144), passes=64)
    assert rep3["candidates"] >= 8


def _schedule(S, nseg):
    """temporal_schedule of runtime.cpp (refactor.cu:266-270)."""
    size = S // nseg
    seg, t = [], []
    for s in range(S):
        sg, tt = s // size, (s % size) / float(S // nseg)
        if sg >= nseg:
            sg, tt = nseg - 1, 1.0
        seg.append(sg)
        t.append(tt)
    return seg, t


def test_temporal_multiplier_static_flame_matches_single_sample_render(db, comp):
    """temporal_multiplier T > 1 (flame_kernel::warmup / bin with T x grid
    temporal samples cycled by the persistent blocks): on a static genome the
    render matches the T = 1 render within the noise floor of two T = 1 seeds,
    the quality target is met (an equal share per block and sample), and the
    state holds T x grid prepared samples."""
    g = syn.hd_flame(2)
    f = lr.flame.from_json(db, g)
    k = comp.get_flame_kernel(db, f)
    # each (block, sample) share must span several check intervals of 1024
    # chains, or the first check already overshoots it (as in the reference)
    w, h = 320, 240
    samples = f.pack_samples(4, w, h)

    def render(T, seed):
        st = k.warmup(samples, (w, h), seed=seed, count=20, temporal_multiplier=T)
        r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=256.0, temporal_slicing=8))
        assert r.status & 1, r
        assert 256.0 <= r.quality <= 256.0 * 1.3, r.quality
        d = st.bins().cpu().numpy().astype(np.float64)[..., 3]
        return st, d / d.sum()

    st4, d4 = render(4, 5)
    assert st4.samples().shape[0] == 4 * k.info["grid"]
    _, d1 = render(1, 5)
    _, d1b = render(1, 6)
    assert np.abs(d4 - d1).sum() < 1.3 * np.abs(d1 - d1b).sum()


def test_temporal_multiplier_spreads_samples_over_the_segment(db, comp):
    """With T x grid temporal samples the prepared parameter blocks follow the
    reference schedule over the spline segments, T times finer: each equals
    rfk_prepare_samples at the same (segment, t) up to the screen jitter."""
    keys = lr.align_flames(db, [lr.flame.from_json(db, syn.hd_flame(40 + i, n_xforms=4, final=False)) for i in range(4)])
    k = comp.get_flame_kernel(db, keys[0])
    w, h = 96, 64
    samples = np.stack([f.pack_sample(w, h) for f in keys])
    T = 3
    st = k.warmup(samples, (w, h), seed=9, count=4, temporal_multiplier=T)
    got = st.samples().astype(np.float64)
    S = T * k.info["grid"]
    seg, t = _schedule(S, samples.shape[0] - 3)
    want = k.prepare_samples(samples, seg, t, seed=9).astype(np.float64)
    assert got.shape == want.shape
    pal0 = k.info["sample_floats"] - 1024
    R, nx = keys[0].size_reals(), k.info["num_xforms"]
    idx = np.r_[0:4, 6:R]
    ulp = np.spacing(np.maximum(np.abs(got), np.abs(want)).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(got - want)[:, idx] <= 4 * ulp[:, idx])
    assert np.all(np.abs(got - want)[:, pal0:] <= 1.0 / 255 + 1e-6)
    # weights a few ulps apart may give alias tables of another shape that
    # encode the same pick distribution
    for i in range(S):
        np.testing.assert_allclose(alias_distribution(got[i], R, nx), alias_distribution(want[i], R, nx), atol=1e-5)
