"""Converged renders of the reference's own chaos-game kernels
(assets/kernels/refactor.cu: warmup + bin, specialised per flame by
oracle/ref_flame.py from assets/templates/flame.tpl and compiled by
oracle/build_ref.py) against librfk's renders of the same flames at the
same spp.

The reference adds a draw to the histogram with a non-atomic load / add /
store (refactor.cu:361-383), which overwrites the updates other lanes and
blocks make to the same pixel in between: on these flames, which put most
draws on few pixels, most draws are lost (99.7% and 91.5% measured on a
GB300), and the surviving histogram is not an estimate of the flame's
density. The parity test therefore runs the reference module
whose only change is that update made atomic (refactor_<flame>_atomic):
normalised density and colour L1 against librfk within 1.25x the Monte-Carlo
noise floor (L1 between two seeds of the same renderer). The unchanged
module runs too, to measure the fraction it loses."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import ref_run, refkernels
from refraktor_gb300 import librefrakt as lr

pytestmark = pytest.mark.gpu

WARMUP = ref_run.WARMUP
reference_render = ref_run.reference_render


def librfk_render(tag: str, seed: int, spp: float) -> np.ndarray:
    m = refkernels.meta(f"refactor_{tag}")
    g, w, h = m["genome"], m["width"], m["height"]
    db = lr.flamedb()
    f = lr.flame.from_json(db, g)
    # the bench genome renders with the launch shape the bench uses (the
    # autotuner's pick for it); the small flames with warp aggregation
    opts = lr.autotune(db, f, f.pack_samples(4, w, h), (w, h))[0] if tag == "bench" else dict(flush=1)
    k = lr.flame_compiler().get_flame_kernel(db, f, **opts)
    st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=seed, count=WARMUP)
    r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=spp))
    assert r.status & 1, r
    return st.bins().cpu().numpy().astype(np.float64)


def _l1(a, b, c):
    return float(np.abs(a[..., c] / a[..., c].sum() - b[..., c] / b[..., c].sum()).sum())


# config 0 (512x512), a config-1 flame at 320x180, the 1080p bench genome at
# 1920x1080 (the configuration bench.py times), and the reference's own
# real-world genome (assets/flames_test/electricsheep.247.50049.flam3 at its
# size, 800x592: fisheye, bubble, julia, post affines)
CASES = [("c0", 32.0, (3,)), ("hd", 256.0, (0, 1, 2, 3)), ("bench", 32.0, (0, 1, 2, 3)),
         ("sheep", 64.0, (0, 1, 2, 3))]


@pytest.mark.parametrize("tag,spp,channels", CASES)
def test_reference_kernel_render_matches(tag, spp, channels):
    mod = f"refactor_{tag}_atomic"
    if not refkernels.available(mod) or not refkernels.available("catmull"):
        pytest.skip("reference kernels not built")
    r1, i1 = reference_render(mod, 11, spp)
    r2, i2 = reference_render(mod, 12, spp)
    for info in (i1, i2):
        assert info["quality"] >= spp, info  # reached the target (not the time bailout)
        assert abs(info["lost"]) < 1e-4, info  # atomic: every draw is in the histogram
    o1 = librfk_render(tag, 21, spp)
    o2 = librfk_render(tag, 22, spp)
    for c in channels:
        floor = max(_l1(r1, r2, c), _l1(o1, o2, c))
        d = _l1(r1, o1, c)
        assert d < 1.25 * floor, (tag, c, d, floor)


@pytest.mark.parametrize("tag,spp,channels", CASES)
def test_unchanged_reference_kernel_loses_draws(tag, spp, channels):
    """The reference module as it is reaches the quality target (its counter
    counts draws, not what the histogram kept) and loses a fraction of the
    draws to its non-atomic add."""
    mod = f"refactor_{tag}"
    if not refkernels.available(mod) or not refkernels.available("catmull"):
        pytest.skip("reference kernels not built")
    _, info = reference_render(mod, 11, spp)
    assert info["quality"] >= spp, info
    assert 0.0 <= info["lost"] < 1.0, info
