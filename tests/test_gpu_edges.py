"""Edge cases of the render path on the GPU: images of one pixel and ragged
sizes through warm-up + bin, the density blur and the tonemap; an empty
histogram; and the argument errors the C ABI reports instead of launching
(the reference exits the process on a CUDA error, util/cuda.h:16-25)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as orc
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

TINY = [(1, 1), (3, 1), (1, 5), (37, 23)]


@pytest.fixture(scope="module")
def kernel(db):
    f = lr.flame.from_json(db, syn.plain_flame(3))
    return f, lr.flame_compiler().get_flame_kernel(db, f)


@pytest.mark.parametrize("w,h", TINY)
def test_tiny_and_ragged_images_render(kernel, w, h):
    f, k = kernel
    st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=5, count=20)
    r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=2.0))
    assert r.status & 1, r
    assert r.quality >= 2.0
    bins = st.bins().cpu().numpy().astype(np.float64)
    assert bins.shape == (h, w, 4)
    assert np.all(np.isfinite(bins)) and bins.min() >= 0.0
    # opacity 1: every draw adds 1 to its pixel's density
    assert abs(bins[..., 3].sum() - r.draw_count) <= 1e-4 * r.draw_count


@pytest.mark.parametrize("w,h", TINY)
def test_density_blur_tiny_and_ragged(w, h):
    rng = np.random.default_rng(w * 100 + h)
    dens = rng.exponential(5.0, size=(h, w)).astype(np.float32)
    col = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    bins = np.ascontiguousarray(np.concatenate([col * dens[..., None], dens[..., None]], axis=-1), dtype=np.float32)
    d_in = torch.from_numpy(bins).cuda()
    d_out = torch.empty_like(d_in)
    lr.density_blur(d_in, d_out, (w, h), 9.0, 0.0, 0.5)
    got = d_out.cpu().numpy().astype(np.float64)
    ref = orc.density_blur(bins, 9.0, 0.0, 0.5)
    err = np.abs(got - ref)
    assert np.all(err <= 1e-5 * np.abs(ref) + 1e-6 * np.abs(ref).max()), float(err.max())


@pytest.mark.parametrize("w,h", TINY)
@pytest.mark.parametrize("fmt", [lr.HALF4, lr.FLOAT4])
def test_empty_histogram_tonemaps_to_zero(w, h, fmt):
    bins = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    out = torch.full((h, w, 4), 7.0, dtype=torch.float16 if fmt == lr.HALF4 else torch.float32, device="cuda")
    lr.tonemapper().run(bins, out, (w, h), 16.0, 2.2, 4.0, 1.0, fmt=fmt)
    assert torch.count_nonzero(out).item() == 0


def test_argument_errors_are_reported(kernel):
    f, k = kernel
    samples = f.pack_samples(4, 16, 16)
    with pytest.raises(lr.RfkError):
        k.warmup(samples, (0, 16), seed=1, count=1)  # empty image
    with pytest.raises(lr.RfkError):
        k.warmup(samples, (16, 0), seed=1, count=1)
    with pytest.raises(lr.RfkError):
        k.warmup(samples, (1 << 16, 1 << 16), seed=1, count=1)  # 2^32 pixels: beyond the 2^31 limit
    ss = k.info["size_reals"] + 768
    with pytest.raises(lr.RfkError):
        k.warmup(samples[: 3 * ss], (16, 16), seed=1, count=1)  # fewer than four samples
    with pytest.raises(lr.RfkError):
        k.warmup(samples, (16, 16), seed=1, count=1, temporal_multiplier=0)
    st = k.warmup(samples, (16, 16), seed=1, count=1)
    with pytest.raises(lr.RfkError):
        k.bin(st, lr.bailout_args(iters=0, millis=0, quality=0.0))  # no limit at all
    with pytest.raises(lr.RfkError):
        k.bin(st, lr.bailout_args(iters=0, millis=0, quality=-1.0))
    # the state stays usable after rejected calls
    r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=1.0))
    assert r.status & 1
    bins = st.bins()
    out = torch.empty_like(bins)
    with pytest.raises(lr.RfkError):
        lr.density_blur(bins, bins, (16, 16))  # in place
    with pytest.raises(lr.RfkError):
        lr.density_blur(bins, out, (16, 16), max_radius=10.0)  # beyond the radius cap
    with pytest.raises(lr.RfkError):
        lr.tonemapper().run(bins, out, (16, 16), 0.0, 2.2, 4.0, 1.0)  # quality must be positive
