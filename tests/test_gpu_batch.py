"""Batched rendering (rfk_batch_*): many flames or frames of one structure in
one persistent launch. Each unit must render what an individual render of the
same genome renders (density and colour within the Monte-Carlo noise floor of
two individual renders), reach its own quality target, get the spline-prepared
parameters of the single-flame path, and the blur + tonemap of the
single-image calls; the CUDA-graph replay must give the same."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn
from tests.pick_tables import alias_distribution

pytestmark = pytest.mark.gpu

SIZES = [(96, 64), (128, 128), (160, 90)]


@pytest.fixture(scope="module")
def hetero(db):
    gs = [syn.hd_flame(21, n_xforms=3, final=False), syn.hd_flame(22, n_xforms=6, final=True),
          syn.hd_flame(23, n_xforms=9, final=False)]
    gs = [syn.frame_on_gpu(db, g, w, h, seed=1) for g, (w, h) in zip(gs, SIZES)]
    fs = [lr.flame.from_json(db, g) for g in gs]
    al = lr.align_flames(db, fs)
    k = lr.flame_compiler().get_flame_kernel(db, al[0])
    return al, k


def _units(al, spp):
    units, samples = [], []
    for i, (f, (w, h)) in enumerate(zip(al, SIZES)):
        tp = f.tonemap_params()
        units.append(lr.batch_unit(w, h, spp, segment=4 * i, t=0.0, gamma=tp["gamma"], brightness=tp["brightness"],
                                   vibrancy=tp["vibrancy"]))
        samples.append(f.pack_samples(4, w, h))
    return units, np.concatenate(samples)


def _l1(a, b):
    return float(np.abs(a / a.sum() - b / b.sum()).sum())


def _individual(k, f, w, h, spp, seed):
    st = k.warmup(f.pack_samples(4, w, h), (w, h), seed=seed, count=20)
    k.bin(st, lr.bailout_args(iters=0, millis=0, quality=spp))
    return st.bins().cpu().numpy().astype(np.float64)


def _batch_render(k, al, spp, seed):
    units, samples = _units(al, spp)
    b = lr.batch(k, units, samples.shape[0] // al[0].sample_size(), out_format=-1, seed=seed)
    b.set_samples(samples)
    b.run()
    tot, per = b.wait()
    return b, tot, per


def test_batch_units_match_individual_renders(hetero):
    """Per-flame parity of the batch with individual renders of the same
    genome: normalised density / colour L1 between the two stays within 1.3x
    the noise floor of the pair, sqrt((fb^2 + fi^2) / 2) from the L1 between
    two seeds of each renderer (fb batch, fi individual). A unit of a batch is
    worked on by few blocks whose chains run many passes, so at equal spp its
    Monte-Carlo noise can exceed that of the individual render, whose many
    chains run few passes each; the pair floor accounts for both."""
    al, k = hetero
    spp = 160.0
    b, tot, per = _batch_render(k, al, spp, seed=3)
    b2, _, _ = _batch_render(k, al, spp, seed=4)
    assert tot.status & 1
    for u, ((w, h), r) in enumerate(zip(SIZES, per)):
        assert r.status & 1
        # overshoot: the checks of every block working on the unit
        assert spp <= r.quality <= spp * 1.2, (u, r.quality)
        got = b.bins(u).cpu().numpy().astype(np.float64)
        got2 = b2.bins(u).cpu().numpy().astype(np.float64)
        assert got[..., 3].sum() == pytest.approx(r.draw_count, rel=1e-4)
        i1 = _individual(k, al[u], w, h, spp, seed=11)
        i2 = _individual(k, al[u], w, h, spp, seed=12)
        for c in (3, 0):
            fb, fi = _l1(got[..., c], got2[..., c]), _l1(i1[..., c], i2[..., c])
            floor = float(np.sqrt((fb * fb + fi * fi) / 2))
            d = _l1(got[..., c], i1[..., c])
            assert d < 1.3 * floor, (u, c, d, fb, fi)


def test_batch_graph_replay(hetero):
    al, k = hetero
    units, samples = _units(al, 16.0)
    b = lr.batch(k, units, samples.shape[0] // al[0].sample_size(), out_format=lr.HALF4, de=(4.0, 0.0, 0.5))
    b.set_samples(samples)
    s = torch.cuda.Stream()
    outs = []
    for _ in range(3):
        b.run(use_graph=True, stream=s)
        tot, per = b.wait()
        assert tot.status & 1
        assert all(r.status & 1 and r.quality < 16.0 * 1.5 + 8 for r in per)
        outs.append([b.bins(u).cpu().numpy().astype(np.float64) for u in range(len(units))])
    info = b.info()
    assert info["graph"] == 1
    # fix_rotation once per independent flame (their samples are joined by no
    # unit's segment), catmull, prepare, counter clear, iterate, then blur and
    # tonemap per unit
    assert info["launches_per_run"] == len(units) + 4 + 2 * len(units)
    # replays draw fresh random streams, and each starts from cleared histograms
    for u in range(len(units)):
        a, c = outs[0][u][..., 3], outs[1][u][..., 3]
        assert not np.array_equal(a, c)
        assert _l1(a, c) < 1.5 * _l1(outs[1][u][..., 3], outs[2][u][..., 3]) + 0.02


def test_independent_flames_prepare_bit_identically(db):
    """A batch of independent flames (each 4 copies of its own sample, unit i
    on segment 4 i, t = 0, as the heterogeneous workload): every unit's
    prepared parameter block equals, bit for bit, what the single-flame path
    prepares from that flame's 4 samples alone (the screen offsets aside,
    where the single-flame path adds its jitter). fix_rotation restarts its
    angle unwrapping between samples that no unit's segment joins; unwrapped
    across the flames, later flames' angles carried multiples of 2 pi into
    FP32 and their affines differed in the last bits, enough to move the
    render of a sensitive flame by more than its noise."""
    fl = lr.align_flames(db, [lr.flame.from_json(db, syn.hd_flame(70 + i, n_xforms=2 + 3 * i, final=False))
                              for i in range(4)])
    k = lr.flame_compiler().get_flame_kernel(db, fl[0])
    w, h = 96, 64
    samples = np.concatenate([f.pack_samples(4, w, h).reshape(4, -1) for f in fl])
    units = [lr.batch_unit(w, h, 1.0, segment=4 * i, t=0.0) for i in range(len(fl))]
    b = lr.batch(k, units, samples.shape[0], out_format=-1)
    b.set_samples(samples)
    b.run()
    b.wait()
    R = fl[0].size_reals()
    for u in range(len(fl)):
        got = b.params(u).cpu().numpy()
        want = k.prepare_samples(samples[4 * u:4 * u + 4], [0], [0.0])[0]
        idx = np.r_[0:4, 6:got.size]
        np.testing.assert_array_equal(got[idx], want[idx], err_msg=f"unit {u}")
        assert R > 6


def test_batch_prepare_matches_single_flame_prepare(db):
    """Animation frames: Catmull-Rom over 4 aligned keyframes (first and last
    repeated) evaluated on the device per frame, as rfk_prepare_samples does
    (screen jitter aside: the batch jitters per queue item instead)."""
    keys = [lr.flame.from_json(db, syn.hd_flame(30 + i, n_xforms=6, final=False)) for i in range(4)]
    keys = lr.align_flames(db, keys)
    k = lr.flame_compiler().get_flame_kernel(db, keys[0])
    w, h = 128, 72
    ks = [f.pack_sample(w, h) for f in keys]
    samples = np.stack([ks[0], ks[0], ks[1], ks[2], ks[3], ks[3]])
    frames = 9
    seg, t = [], []
    for i in range(frames):
        x = 3.0 * i / (frames - 1)
        s_ = min(int(x), 2)
        seg.append(s_)
        t.append(float(x - s_))
    units = [lr.batch_unit(w, h, 1.0, segment=s_, t=tt) for s_, tt in zip(seg, t)]
    b = lr.batch(k, units, samples.shape[0], out_format=-1)
    b.set_samples(samples)
    b.run()
    b.wait()
    want = k.prepare_samples(samples, seg, t, seed=1)
    R, nx = keys[0].size_reals(), k.info["num_xforms"]
    sf = k.info["sample_floats"]
    pal0 = sf - 1024
    for u in range(frames):
        got = b.params(u).cpu().numpy().astype(np.float64)
        ref = want[u].astype(np.float64)
        ulp = np.spacing(np.maximum(np.abs(got), np.abs(ref)).astype(np.float32)).astype(np.float64)
        d = np.abs(got - ref)
        idx = np.r_[0:4, 6:R]
        assert np.all(d[idx] <= 4 * ulp[idx]), (u, float((d[idx] / np.maximum(ulp[idx], 1e-45)).max()))
        # pick tables: weights a few ulps apart may give alias tables of another
        # shape; the xform distributions they encode agree
        np.testing.assert_allclose(alias_distribution(b.params(u).cpu().numpy(), R, nx),
                                   alias_distribution(want[u], R, nx), atol=1e-5)
        assert np.all(d[pal0:] <= 1.0 / 255 + 1e-6)
        # the single-flame path adds its jitter here, the batch per item
        assert np.all(d[4:6] < 2.0)


def test_batch_blur_and_tonemap_match_single_image_calls(hetero):
    al, k = hetero
    units, samples = _units(al, 8.0)
    de = (6.0, 0.5, 0.4)
    b = lr.batch(k, units, samples.shape[0] // al[0].sample_size(), out_format=lr.FLOAT4, de=de)
    b.set_samples(samples)
    b.run()
    _, per = b.wait()
    for u, ((w, h), U, r) in enumerate(zip(SIZES, units, per)):
        bins = b.bins(u)
        blurred = torch.empty_like(bins)
        lr.density_blur(bins, blurred, (w, h), *de)
        want = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
        lr.tonemapper().run(blurred, want, (w, h), r.quality, U.gamma, U.brightness, U.vibrancy, fmt=lr.FLOAT4)
        got = b.image(u)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-5, atol=1e-6)


def test_batch_rejects_bad_units(hetero):
    al, k = hetero
    units, samples = _units(al, 8.0)
    n = samples.shape[0] // al[0].sample_size()
    bad = list(units)
    bad[1] = lr.batch_unit(0, 10, 8.0)
    with pytest.raises(lr.RfkError):
        lr.batch(k, bad, n)
    bad[1] = lr.batch_unit(10, 10, 8.0, segment=n - 3)
    with pytest.raises(lr.RfkError):
        lr.batch(k, bad, n)
    b = lr.batch(k, units, n)
    with pytest.raises(lr.RfkError):
        b.run()  # samples not set
