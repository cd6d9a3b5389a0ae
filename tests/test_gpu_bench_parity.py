"""Parity at the benchmarked configurations.

- The 1080p single flame (refraktor_gb300/workloads/hd_1080p.json, 8 xforms +
  final xform, 14-variation set) at 1920x1080, rendered with the launch shape
  the autotuner picks for it, against two FP64 oracle renders fed the same
  prepared flame, palette, jitters and schedule: normalised density and
  colour L1 within 1.25x the L1 between the two oracle seeds.
- The 64-flame heterogeneous batch (hetero_64.json: 256^2 .. 2048x1152,
  2-12 xforms, 64/256/1024 spp, one union-of-variations kernel, the
  autotuner's launch shape) and the 120-frame 720p animation (anim_720p.json:
  Catmull-Rom over 4 keyframes): every unit reaches its target, and at least
  eight units per workload, among them the 1920x1080 and 2048x1152 flames,
  match individual plain renders of the same genome within 1.3x the pair's
  noise floor (the criterion of tests/test_gpu_batch.py).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bench
from oracle import oracle as orc
from refraktor_gb300 import librefrakt as lr

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8


def _l1(a, b):
    return float(np.abs(a / a.sum() - b / b.sum()).sum())


def test_bench_genome_at_1080p_matches_oracle(db):
    g = bench.load_workload()
    w, h, spp = bench.W, bench.H, 32.0
    f = lr.flame.from_json(db, g)
    samples = f.pack_samples(4, w, h)
    opts, _ = lr.autotune(db, f, samples, (w, h))
    k = lr.flame_compiler().get_flame_kernel(db, f, **opts)
    R = f.size_reals()
    chains = k.info["grid"] * k.info["block"] * k.info["chains_per_thread"]
    # a pass cap gives every chain the same number of passes, as the oracle's schedule
    passes = int(np.ceil(spp * w * h / chains))
    st = k.warmup(samples, (w, h), seed=5, count=bench.WARMUP_PASSES)
    r = k.bin(st, lr.bailout_args(iters=passes, millis=0, quality=0))
    assert r.total_passes == passes * chains
    assert r.draw_count > 0.95 * r.total_passes  # the framed bench genome draws almost every step
    gpu = st.bins().cpu().numpy().astype(np.float64)
    p_ref, _ = orc.prepared(g, w, h)
    samp = st.samples()
    params = samp[0, :R].astype(np.float64)
    params[4], params[5] = p_ref[4], p_ref[5]
    jit = np.stack([samp[:, 4] - p_ref[4], samp[:, 5] - p_ref[5]], 1)
    pal = samp[0, k.info["sample_floats"] - 1024:].reshape(256, 4)[:, :3].astype(np.float64)
    kw = dict(warmup=bench.WARMUP_PASSES, threads=THREADS, params=params, palette=pal, jitter=jit, hammersley=True)
    o1, _ = orc.render(g, w, h, chains, passes, seed=1, **kw)
    o2, _ = orc.render(g, w, h, chains, passes, seed=2, **kw)
    for c in (3, 0, 1, 2):
        d, floor = _l1(gpu[..., c], o1[..., c]), _l1(o1[..., c], o2[..., c])
        assert d < 1.25 * floor, (c, d, floor)


def _check_units(k, units, al_of, samples_of, b1, b2, per, picks, seeds=(11, 12, 13, 14)):
    """Per unit: batch renders b1, b2 against individual plain renders of the
    same genome with `seeds`. The single-flame path keeps one antialiasing
    jitter per block for a whole render, so on flames with a few hot points
    its seed-to-seed distance is dominated by a handful of random sub-pixel
    shifts and varies a lot from pair to pair; distances are therefore means
    over all pairs: fi over the individual pairs, d over (b1, individual)."""
    import itertools

    for u in picks:
        U = units[u]
        w, h, spp = U.width, U.height, U.quality
        assert per[u].status & 1 and per[u].quality >= spp, (u, per[u])
        got = b1.bins(u).cpu().numpy().astype(np.float64)
        got2 = b2.bins(u).cpu().numpy().astype(np.float64)
        ind = []
        for s in seeds:
            st = k.warmup(samples_of(u), (w, h), seed=s, count=bench.WARMUP_PASSES)
            r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=spp))
            assert r.status & 1
            ind.append(st.bins().cpu().numpy().astype(np.float64))
            del st
        for c in (3, 0):
            fb = _l1(got[..., c], got2[..., c])
            fi = float(np.mean([_l1(a[..., c], b[..., c]) for a, b in itertools.combinations(ind, 2)]))
            floor = float(np.sqrt((fb * fb + fi * fi) / 2))
            d = float(np.mean([_l1(got[..., c], a[..., c]) for a in ind]))
            assert d < 1.3 * floor, (u, (w, h, spp), c, d, fb, fi)


def _run_batch(k, units, samples, seed):
    b = lr.batch(k, units, samples.shape[0], passes_per_item=256, warmup=bench.WARMUP_PASSES, seed=seed, out_format=-1)
    b.set_samples(samples)
    b.run()
    tot, per = b.wait()
    assert tot.status & 1
    return b, per


def test_hetero_64_units_match_individual_renders(db):
    kf, samples, units, _, (tf, tsamples, tdims) = bench.batch_workload(lr, db, "hetero")
    opts, _ = lr.autotune(db, tf, tsamples, tdims)
    k = lr.flame_compiler().get_flame_kernel(db, kf, **opts)
    samples = samples.reshape(-1, kf.sample_size())
    b1, per = _run_batch(k, units, samples, seed=3)
    b2, _ = _run_batch(k, units, samples, seed=4)
    for u, r in enumerate(per):
        assert r.status & 1 and r.quality >= units[u].quality, (u, r)
    sizes = [(U.width, U.height) for U in units]
    picks = sorted({sizes.index((1920, 1080)), sizes.index((2048, 1152)), 0, 2, 3, 4, 6, 8, 17, 30, 43})
    assert len(picks) >= 8
    _check_units(k, units, None, lambda u: samples[4 * u:4 * u + 4], b1, b2, per, picks)


def _frame_samples(fixed, ss, R, aff, seg, t):
    """The genome of one animation frame as 4 identical packed samples: the
    FP64 Catmull-Rom of the rotation-fixed keyframe samples at (seg, t),
    with every affine's (angle, log magnitude) columns turned back into
    Cartesian ones, so that the single-flame path's own fix_rotation and
    spline reproduce the frame."""
    coeff = orc.catmull(fixed, ss)
    v = orc.cubic_eval(coeff[seg], t)
    out = v.copy()
    for a in aff:
        ax, ay, mx, my = v[a], v[a + 1], np.exp(v[a + 2]), np.exp(v[a + 3])
        out[a], out[a + 1], out[a + 2], out[a + 3] = mx * np.cos(ax), mx * np.sin(ax), my * np.cos(ay), my * np.sin(ay)
    return np.tile(out, 4)


def test_anim_720p_frames_match_individual_renders(db):
    kf, samples, units, _, (tf, tsamples, tdims) = bench.batch_workload(lr, db, "anim")
    opts, _ = lr.autotune(db, tf, tsamples, tdims)
    k = lr.flame_compiler().get_flame_kernel(db, kf, **opts)
    ss = kf.sample_size()
    R = kf.size_reals()
    aff = kf.affine_indices()
    samples = np.asarray(samples, dtype=np.float64).reshape(-1, ss)
    fixed = lr.fix_rotation(samples, ss, R, aff)
    b1, per = _run_batch(k, units, samples, seed=5)
    b2, _ = _run_batch(k, units, samples, seed=6)
    for u, r in enumerate(per):
        assert r.status & 1 and r.quality >= units[u].quality, (u, r)
    picks = [0, 17, 34, 51, 68, 85, 102, 119]
    _check_units(k, units, None, lambda u: _frame_samples(fixed, ss, R, aff, units[u].segment, units[u].t), b1, b2,
                 per, picks)
