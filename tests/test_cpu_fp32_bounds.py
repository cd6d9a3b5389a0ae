"""Why some variations are held to distribution bounds instead of "every point
within 4 ulp" in the single-map GPU test: evaluated with every FP32 operation
of the formula correctly rounded (tests/fp32_ideal.py, the best any FP32
evaluation of the formula as written can do), they still miss the per-point
bound at some of that test's inputs, so the miss comes from the formula's
FP32 intermediates (angle sums rounded before a sine, cancellations), not from
the library's arithmetic. Variations whose correctly rounded evaluation meets
the bound are held to it on the GPU."""
import numpy as np
import pytest

from tests import fp32_ideal as fi


@pytest.mark.parametrize("name", fi.IDEAL)
def test_correctly_rounded_fp32_against_the_4_ulp_bound(name):
    w, pts = fi.single_map_points(name)
    out = fi.ideal(name, w, pts[:, 0], pts[:, 1])
    fwd, best, ok = fi.ulp_errors(name, w, pts, out)
    # the evaluation itself is sound: half the points are within an ulp or so
    assert np.median(fwd[ok]) <= 2.0
    if name in fi.ANGLE_COMPOSED:
        # some point misses 4 ulp however the FP32 arithmetic is done ...
        assert best[ok].max() > 4.0, (name, float(best[ok].max()))
        # ... and the GPU test's bound on the fraction is no stricter than
        # what correct rounding achieves
        assert np.mean(best[ok] <= 4.0) >= fi.ANGLE_COMPOSED[name][2], (name, np.mean(best[ok] <= 4.0))
    else:
        assert best[ok].max() <= 4.0, (name, float(best[ok].max()))
        # the forward fraction the GPU test asks for is reachable, and where
        # it is below the default 0.99, the default is not
        frac = float(np.mean(fwd[ok] <= 4.0))
        want = fi.FORWARD_WITHIN_4.get(name, 0.99)
        assert frac >= want, (name, frac)
        if name in fi.FORWARD_WITHIN_4:
            assert frac < 0.99, (name, frac)


def test_the_cancellation_and_angle_rounding_cases():
    """The worst inputs of two of them, which show the two mechanisms. polar
    near the unit circle (r = 0.9663): y = sqrt - 1 = -0.034 carries the
    rounding of sqrt, half an ulp of 1, which is about 4 ulp of the outputs
    near 0.03, and the atan part adds its own. handkerchief at r = 0.794, atan
    + sqrt = 3.14...: the angle sum rounded to FP32 (half an ulp of pi, 1.2e-7)
    moves the sine's argument near its zero by that much, while the output is
    0.005 (ulp 4.7e-10)."""
    for name, x, y, at_least in (("polar", -0.08807797729969025, 0.9622352123260498, 8.0),
                                 ("handkerchief", 0.5602803230285645, -0.5627108216285706, 30.0)):
        w, _ = fi.single_map_points(name)
        pts = np.array([[x, y]], dtype=np.float32)
        out = fi.ideal(name, w, pts[:, 0], pts[:, 1])
        fwd, best, ok = fi.ulp_errors(name, w, pts, out)
        assert ok.all() and best[0] > at_least, (name, float(best[0]))
