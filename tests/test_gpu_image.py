"""GPU parity of the image steps: tonemap, density histogram, density blur,
Catmull-Rom coefficients - against the FP64 oracle and, where the reference
has the kernel, against the reference's own kernel run on the same data."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as orc
from refraktor_gb300 import librefrakt as lr

from oracle import refkernels

pytestmark = pytest.mark.gpu


def _histogram(h=123, w=217, seed=0, zero_frac=0.3):
    rng = np.random.default_rng(seed)
    dens = np.exp(rng.uniform(np.log(0.01), np.log(5e4), size=(h, w))).astype(np.float32)
    dens[rng.uniform(size=(h, w)) < zero_frac] = 0.0
    col = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    bins = np.concatenate([col * dens[..., None], dens[..., None]], axis=-1).astype(np.float32)
    bins[0, :5, 3] = [1.0, 0.5, 2.0, 4.0, 1e-30]  # edge values around the log2 bin boundaries
    return np.ascontiguousarray(bins)


TONEMAP_CASES = [(64.0, 2.2, 4.0, 1.0, -1.0), (3.0, 4.0, 64.08, 1.0, -1.0), (1024.0, 2.2, 4.0, 0.35, -1.0),
                 (16.0, 1.5, 8.0, 0.6, 1.0), (16.0, 2.2, 40.0, 1.0, 0.0)]


@pytest.mark.parametrize("q,gamma,bright,vib,hp", TONEMAP_CASES)
def test_tonemap_precise_matches_fp64_oracle(q, gamma, bright, vib, hp):
    bins = _histogram()
    h, w = bins.shape[:2]
    d_bins = torch.from_numpy(bins).cuda()
    out = torch.empty((h, w, 4), device="cuda")
    lr.tonemapper().run(d_bins, out, (w, h), q, gamma, bright, vib, highlight_power=hp, fmt=lr.FLOAT4, precise=True)
    got = out.cpu().numpy().astype(np.float64)
    ref = orc.tonemap(bins, q, gamma, bright, vib, hp)
    # tolerance from the acceptance criterion: 1e-5 relative, with an absolute
    # floor of 1e-7 (about one FP32 ulp at 1) for values near zero
    err = np.abs(got - ref)
    assert np.all(err <= 1e-5 * np.abs(ref) + 1e-7), float((err / (np.abs(ref) + 1e-7)).max())


@pytest.mark.parametrize("fmt,channels", [(lr.HALF3, 3), (lr.HALF4, 4), (lr.FLOAT3, 3)])
def test_tonemap_formats(fmt, channels):
    bins = _histogram(seed=2)
    h, w = bins.shape[:2]
    d_bins = torch.from_numpy(bins).cuda()
    dtype = torch.float16 if fmt in (lr.HALF3, lr.HALF4) else torch.float32
    out = torch.empty((h, w, channels), device="cuda", dtype=dtype)
    lr.tonemapper().run(d_bins, out, (w, h), 64.0, 2.2, 4.0, 1.0, fmt=fmt)
    ref = orc.tonemap(bins, 64.0, 2.2, 4.0, 1.0)[..., :channels]
    got = out.float().cpu().numpy()
    tol = 1e-3 if dtype == torch.float16 else 1e-5
    assert np.all(np.abs(got - ref) <= tol * np.abs(ref) + 1e-7)


@pytest.mark.skipif(not refkernels.available("tonemap"), reason="reference kernels not built")
@pytest.mark.parametrize("q,gamma,bright,vib", [c[:4] for c in TONEMAP_CASES if c[4] < 0])
def test_tonemap_fast_matches_reference_kernel(q, gamma, bright, vib):
    """The fast variant against assets/kernels/tonemap.cu itself (float4 output)."""
    bins = _histogram(seed=1)
    h, w = bins.shape[:2]
    n = h * w
    d_bins = torch.from_numpy(bins).cuda()
    mine = torch.empty((h, w, 4), device="cuda")
    lr.tonemapper().run(d_bins, mine, (w, h), q, gamma, bright, vib, fmt=lr.FLOAT4, precise=False)
    theirs = torch.zeros((h, w, 4), device="cuda")
    k = refkernels.kernel("tonemap", "tonemap<float4, 4>")
    scale_constant = np.float32(10.0) ** (-np.log10(np.float32(q)) - np.float32(0.5))
    args = [C.c_void_p(d_bins.data_ptr()), C.c_void_p(theirs.data_ptr()), C.c_uint(n), C.c_double(q), C.c_double(0.0),
            C.c_float(gamma), C.c_float(float(scale_constant)), C.c_float(bright), C.c_float(vib)]
    refkernels.launch(k, (n + 255) // 256, 256, args)
    torch.cuda.synchronize()
    a = mine.cpu().numpy()
    b = theirs.cpu().numpy()
    assert np.all(np.abs(a - b) <= 1e-5 * np.abs(b) + 1e-7), float(np.abs(a - b).max())
    # and the reference kernel itself against the FP64 restatement
    ref = orc.tonemap(bins, q, gamma, bright, vib)
    rel = np.abs(b - ref) / (np.abs(ref) + 1e-6)
    print("reference kernel vs FP64 oracle: max rel", float(rel.max()))


def test_density_histogram_matches_oracle():
    bins = _histogram(seed=3)
    n = bins.shape[0] * bins.shape[1]
    d = torch.from_numpy(bins).cuda()
    hist = torch.zeros(97, dtype=torch.int64, device="cuda")
    mx = torch.zeros(1, dtype=torch.int64, device="cuda")
    lr.density_histogram(d, n, hist, mx)
    h_ref, mx_ref = orc.density_histogram(bins)
    np.testing.assert_array_equal(hist.cpu().numpy().astype(np.uint64), h_ref)
    assert int(mx.item()) == mx_ref
    # the tonemap's fused histogram is the same
    hist2 = torch.zeros(97, dtype=torch.int64, device="cuda")
    mx2 = torch.zeros(1, dtype=torch.int64, device="cuda")
    out = torch.empty((bins.shape[0], bins.shape[1], 4), device="cuda")
    lr.tonemapper().run(d, out, (bins.shape[1], bins.shape[0]), 64, 2.2, 4, 1, histogram=hist2, max_density_out=mx2)
    np.testing.assert_array_equal(hist2.cpu().numpy(), hist.cpu().numpy())
    assert int(mx2.item()) == mx_ref


@pytest.mark.skipif(not refkernels.available("histogram"), reason="reference kernels not built")
def test_density_histogram_matches_reference_kernel():
    bins = _histogram(seed=4, h=300, w=301)
    n = bins.shape[0] * bins.shape[1]
    d = torch.from_numpy(bins).cuda()
    hist = torch.zeros(97, dtype=torch.int64, device="cuda")
    mx = torch.zeros(1, dtype=torch.int64, device="cuda")
    lr.density_histogram(d, n, hist, mx)
    rh = torch.zeros(97, dtype=torch.int64, device="cuda")
    rmx = torch.zeros(1, dtype=torch.int64, device="cuda")
    k = refkernels.kernel("histogram", "calculate_histogram<4>")
    refkernels.launch(k, n // 256 + 1, 256, [C.c_void_p(d.data_ptr()), C.c_int(n), C.c_void_p(rh.data_ptr()),
                                             C.c_void_p(rmx.data_ptr())])
    np.testing.assert_array_equal(hist.cpu().numpy(), rh.cpu().numpy())
    assert mx.item() == rmx.item()


@pytest.mark.parametrize("max_r,min_r,curve", [(9.0, 0.0, 0.5), (4.0, 0.5, 0.4), (0.0, 0.0, 0.5)])
def test_density_blur_matches_oracle(max_r, min_r, curve):
    rng = np.random.default_rng(5)
    h, w = 97, 131
    dens = np.where(rng.uniform(size=(h, w)) < 0.2, rng.exponential(20.0, size=(h, w)), 0.0).astype(np.float32)
    col = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    bins = np.ascontiguousarray(np.concatenate([col * dens[..., None], dens[..., None]], axis=-1), dtype=np.float32)
    d_in = torch.from_numpy(bins).cuda()
    d_out = torch.empty_like(d_in)
    lr.density_blur(d_in, d_out, (w, h), max_r, min_r, curve)
    got = d_out.cpu().numpy().astype(np.float64)
    ref = orc.density_blur(bins, max_r, min_r, curve)
    err = np.abs(got - ref)
    scale = np.abs(ref).max()
    assert np.all(err <= 1e-5 * np.abs(ref) + 1e-6 * scale), float(err.max())
    if max_r == 0.0:
        np.testing.assert_allclose(got, bins, rtol=1e-6)
    # energy: inside the image the blur conserves totals up to border losses
    assert got[..., 3].sum() <= bins[..., 3].sum() * (1 + 1e-5)


def test_density_blur_patchy_image_matches_oracle():
    """A render's usual layout: most tiles empty, dense regions (small blur
    radius), and isolated faint pixels (the full 9-pixel radius) near the
    edges of empty tiles. Each block loops only as far as the widest support
    of the sources in its tile and halo; the result must equal the scatter
    definition everywhere, also where a faint pixel's support reaches into an
    otherwise empty tile."""
    rng = np.random.default_rng(9)
    h, w = 150, 260
    dens = np.zeros((h, w), np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    for cy, cx, r in ((40, 60, 18), (110, 200, 12)):
        blob = (yy - cy) ** 2 + (xx - cx) ** 2 < r * r
        dens[blob] = rng.uniform(50, 400, size=blob.sum()).astype(np.float32)
    for _ in range(40):
        dens[rng.integers(0, h), rng.integers(0, w)] = rng.uniform(0.5, 2.0)
    col = rng.uniform(0, 1, size=(h, w, 3)).astype(np.float32)
    bins = np.ascontiguousarray(np.concatenate([col * dens[..., None], dens[..., None]], axis=-1), dtype=np.float32)
    d_in = torch.from_numpy(bins).cuda()
    d_out = torch.empty_like(d_in)
    lr.density_blur(d_in, d_out, (w, h), 9.0, 0.0, 0.5)
    got = d_out.cpu().numpy().astype(np.float64)
    ref = orc.density_blur(bins, 9.0, 0.0, 0.5)
    err = np.abs(got - ref)
    assert np.all(err <= 1e-5 * np.abs(ref) + 1e-6 * np.abs(ref).max()), float(err.max())
    # the empty tiles far from every source stay exactly 0
    far = np.ones((h, w), bool)
    for y, x in zip(*np.nonzero(dens)):
        far[max(0, y - 10):y + 11, max(0, x - 10):x + 11] = False
    assert far.any() and np.all(got[far] == 0.0)


T_VALUES = [0.0, 0.1, 0.25, 0.5, 0.77, 0.999, 1.0]


def _curve_scale(samples, n, nseg):
    p = samples.reshape(nseg + 3, n)
    return np.stack([np.abs(p[s:s + 4]).max(axis=0) for s in range(nseg)])


def test_catmull_segments_match_oracle():
    """FP32 Hermite segments evaluated at t vs the FP64 cubic of catmull.cu:
    within 4 FP32 ulps of the segment's largest control point."""
    rng = np.random.default_rng(6)
    n, nseg = 1000, 2
    samples = rng.uniform(-5, 5, size=(nseg + 3) * n)
    samples[:n] = samples[n:2 * n]  # flat start segment
    d_s = torch.from_numpy(samples).cuda()
    d_c = torch.empty((nseg, n, 4), device="cuda")
    lr.catmull_coefficients(d_s, n, nseg, d_c)
    got = d_c.cpu().numpy().astype(np.float64)
    ref = orc.catmull(samples, n)
    tol = 4 * np.spacing(_curve_scale(samples, n, nseg).astype(np.float32)).astype(np.float64)
    for t in T_VALUES:
        assert np.all(np.abs(orc.hermite_eval(got, t) - orc.cubic_eval(ref, t)) <= tol), t
    # knots are reproduced exactly (up to the FP32 rounding of the sample)
    p = samples.reshape(nseg + 3, n)
    np.testing.assert_array_equal(got[..., 0], p[1:nseg + 1].astype(np.float32))
    np.testing.assert_array_equal(got[..., 1], p[2:nseg + 2].astype(np.float32))


@pytest.mark.skipif(not refkernels.available("catmull"), reason="reference kernels not built")
def test_catmull_matches_reference_kernel():
    rng = np.random.default_rng(7)
    n, nseg = 777, 1
    samples = rng.uniform(-3, 3, size=(nseg + 3) * n)
    d_s = torch.from_numpy(samples).cuda()
    mine = torch.empty((nseg, n, 4), device="cuda")
    lr.catmull_coefficients(d_s, n, nseg, mine)
    theirs = torch.zeros((nseg, n, 4), device="cuda", dtype=torch.float64)
    k = refkernels.kernel("catmull", "generate_sample_coefficients")
    refkernels.launch(k, (n * nseg + 255) // 256, 256, [C.c_void_p(d_s.data_ptr()), C.c_uint(n), C.c_uint(nseg),
                                                        C.c_void_p(theirs.data_ptr())])
    a = mine.cpu().numpy().astype(np.float64)
    b = theirs.cpu().numpy()
    np.testing.assert_allclose(b, orc.catmull(samples, n), rtol=1e-12, atol=1e-12)  # reference kernel == oracle (FP64)
    tol = 4 * np.spacing(_curve_scale(samples, n, nseg).astype(np.float32)).astype(np.float64)
    for t in T_VALUES:
        assert np.all(np.abs(orc.hermite_eval(a, t) - orc.cubic_eval(b, t)) <= tol), t


def test_red_v4_probe_runs():
    ops = lr.probe_red_v4(4 << 20, 64)
    assert ops > 1e9


def test_pipe_probes_run():
    fma = lr.probe_pipe(0, 4096)
    sfu = lr.probe_pipe(1, 1024)
    assert 1e11 < sfu < fma  # the special-function unit has fewer lanes than the FMA pipe


def _convert_ref(img, cout, as_bytes, flip_y, swap):
    """numpy restatement of convert_to (assets/kernels/convert.cu:48-99)."""
    v = img.astype(np.float64)
    if v.shape[-1] == 3:
        v = np.concatenate([v, np.ones(v.shape[:-1] + (1,))], -1)
    if swap:
        v = v[..., [2, 1, 0, 3]]
    if flip_y:
        v = v[::-1]
    v = v[..., :cout]
    if as_bytes:
        return np.maximum(np.minimum(v * 255.0, 255.0), 0).astype(np.uint8)
    return v.astype(np.float32)


@pytest.mark.parametrize("cin", [3, 4])
@pytest.mark.parametrize("out_fmt", [lr.FLOAT3, lr.FLOAT4, lr.UCHAR3, lr.UCHAR4])
@pytest.mark.parametrize("flip,swap", [(False, False), (True, True), (True, False)])
def test_convert_matches_reference_restatement(cin, out_fmt, flip, swap):
    w, h = 37, 23
    rng = np.random.default_rng(cin * 10 + out_fmt)
    img = rng.uniform(-0.05, 1.05, size=(h, w, cin)).astype(np.float16)
    dev = torch.from_numpy(img).cuda()
    cout = 3 if out_fmt in (lr.FLOAT3, lr.UCHAR3) else 4
    as_bytes = out_fmt in (lr.UCHAR3, lr.UCHAR4)
    out = torch.empty((h, w, cout), dtype=torch.uint8 if as_bytes else torch.float32, device="cuda")
    lr.converter().run(dev, out, (w, h), lr.HALF3 if cin == 3 else lr.HALF4, out_fmt, flip_y=flip, swap_channels=swap)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), _convert_ref(img, cout, as_bytes, flip, swap))
