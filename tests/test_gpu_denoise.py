"""The learned denoiser through its C ABI (include/rfk_denoise.h): forward
pass, loss and parameter gradients against the float64 CPU restatement of the
same network (oracle/unet.py) with the GPU's bf16 storage points, training
reducing the loss, and the denoise call's output."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import unet as oref
from refraktor_gb300 import _lib
from refraktor_gb300 import denoise as dn

pytestmark = pytest.mark.gpu


def _make(seed=1):
    L = _lib.lib()
    h = C.c_void_p()
    assert L.rfk_denoiser_create(seed, C.byref(h)) == 0, L.rfk_last_error()
    return L, h


def _params(L, h):
    n = L.rfk_denoiser_param_count(h)
    assert n == oref.param_count()
    out = np.zeros(n, dtype=np.float32)
    assert L.rfk_denoiser_get_params(h, out.ctypes.data, n) == 0
    return out


def _batch(n, hh, ww, seed):
    """Random sparse histograms (density with a heavy tail, colour below it),
    random base images and random RGB targets."""
    rng = np.random.default_rng(seed)
    d = rng.exponential(4.0, size=(n, hh, ww)) * (rng.uniform(size=(n, hh, ww)) < 0.7)
    rgb = rng.uniform(0, 1, size=(n, hh, ww, 3)) * d[..., None]
    bins = np.concatenate([rgb, d[..., None]], -1).astype(np.float32)
    base = np.concatenate([rng.uniform(0, 1, size=(n, hh, ww, 3)), np.ones((n, hh, ww, 1))], -1).astype(np.float32)
    tgt = np.concatenate([rng.uniform(0, 1, size=(n, hh, ww, 3)), np.ones((n, hh, ww, 1))], -1).astype(np.float32)
    return bins, base, tgt


def test_gradients_match_float64_oracle():
    L, h = _make(3)
    try:
        n, hh, ww, spp = 2, 16, 512, 32.0
        bins, base, tgt = _batch(n, hh, ww, 5)
        flat = _params(L, h)
        db = torch.from_numpy(bins).cuda()
        dbase = torch.from_numpy(base).cuda()
        dt = torch.from_numpy(tgt).cuda()
        g = np.zeros_like(flat)
        assert L.rfk_denoiser_gradients(h, db.data_ptr(), dbase.data_ptr(), n, ww, hh, spp, dt.data_ptr(), g.ctypes.data,
                                        g.size, None) == 0, L.rfk_last_error()
        loss = C.c_double()
        assert L.rfk_denoiser_loss(h, db.data_ptr(), dbase.data_ptr(), n, ww, hh, spp, dt.data_ptr(), C.byref(loss),
                                   None) == 0
        ref_loss, ref = oref.loss_and_gradients(flat, bins, base, spp, tgt)
        assert loss.value == pytest.approx(ref_loss, rel=2e-3)
        # bf16 storage of activations and gradients (rounded at the same
        # points in the oracle) leaves a few % of relative noise per layer
        for li, ((gw, gb), (rw, rb)) in enumerate(zip(oref.unpack(g), oref.unpack(ref))):
            for got, want in ((gw, rw), (gb, rb)):
                nrm = np.linalg.norm(want)
                assert nrm > 0, li
                rel = np.linalg.norm(got - want) / nrm
                cos = float(np.dot(got.ravel(), want.ravel()) / (np.linalg.norm(got) * nrm))
                assert rel < 0.05 and cos > 0.998, (li, rel, cos)
    finally:
        L.rfk_denoiser_destroy(h)


def test_forward_matches_float64_oracle():
    L, h = _make(4)
    try:
        bins, base, _ = _batch(1, 72, 136, 6)
        flat = _params(L, h)
        # output weights of a trained network's size (they start near zero)
        (w_out, _) = oref.unpack(flat)[oref.L_OUT]
        w_out *= 10.0
        assert L.rfk_denoiser_set_params(h, flat.ctypes.data, flat.size) == 0
        db = torch.from_numpy(bins[0]).cuda()
        dbase = torch.from_numpy(base[0]).cuda()
        out = torch.empty(72, 136, 4, dtype=torch.float32, device="cuda")
        assert L.rfk_denoise(h, db.data_ptr(), dbase.data_ptr(), 136, 72, 32.0, out.data_ptr(), 3, None) == 0, \
            L.rfk_last_error()
        ref = oref.denoise(flat, bins, base, 32.0)[0]
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[..., :3], ref, atol=2e-3 + 0.02 * float(np.abs(ref).max()))
        assert np.all((got[..., 3] >= 0) & (got[..., 3] <= 1))
    finally:
        L.rfk_denoiser_destroy(h)


def test_training_reduces_loss():
    L, h = _make(5)
    try:
        n, hh, ww = 2, 32, 512
        bins, _, _ = _batch(n, hh, ww, 7)
        # a learnable target: the mean colour of the histogram, seen through a
        # noisy base image
        d = bins[..., 3:4]
        tgt = np.concatenate([np.where(d > 0, bins[..., :3] / np.maximum(d, 1e-9), 0), np.ones_like(d)], -1)
        noise = np.random.default_rng(8).uniform(-0.3, 0.3, size=tgt.shape)
        base = np.clip(tgt + noise, 0, 1).astype(np.float32)
        db = torch.from_numpy(bins).cuda()
        dbase = torch.from_numpy(base).cuda()
        dt = torch.from_numpy(tgt.astype(np.float32)).cuda()
        losses = []
        for _ in range(80):
            loss = C.c_double()
            assert L.rfk_denoiser_train_step(h, db.data_ptr(), dbase.data_ptr(), n, ww, hh, 32.0, dt.data_ptr(), 1e-3,
                                             C.byref(loss), None) == 0, L.rfk_last_error()
            losses.append(loss.value)
        assert np.mean(losses[-10:]) < 0.8 * np.mean(losses[:5]), losses[::10]
    finally:
        L.rfk_denoiser_destroy(h)


def test_rejects_bad_sizes():
    L, h = _make(6)
    try:
        x = torch.zeros(8, 8, 4, device="cuda")
        loss = C.c_double()
        assert L.rfk_denoiser_train_step(h, x.data_ptr(), x.data_ptr(), 1, 8, 8, 32.0, x.data_ptr(), 1e-3, C.byref(loss),
                                         None) == 1
        assert b"512" in L.rfk_last_error()
        out = torch.zeros(8, 12, 4, device="cuda")
        assert L.rfk_denoise(h, x.data_ptr(), x.data_ptr(), 12, 8, 32.0, out.data_ptr(), 3, None) == 1
    finally:
        L.rfk_denoiser_destroy(h)


def test_trained_network_beats_the_plain_low_spp_image():
    """What the learned part gains over the method without it: a denoiser
    trained for a short while on the renderer's own 32-spp / 4096-spp pairs of
    seeded flames raises the PSNR of held-out 32-spp renders against their
    4096-spp renders (the plain path at 32 spp is the baseline)."""
    from refraktor_gb300 import denoise as dn
    from refraktor_gb300 import librefrakt as lr
    from refraktor_gb300 import synthetic as syn

    db = lr.flamedb()
    gs = dn.visible_set(db, syn.hd_flame, list(range(5000, 5000 + 400)), 72, 512, 256, min_coverage=0.2)
    bins, base = dn.render_set(db, gs, 512, 256, 32.0, seed=1, both=True)
    tgt = dn.render_set(db, gs, 512, 256, 1024.0, seed=2, tonemap=True)
    net = dn.denoiser(seed=2)
    dn.train(net, bins[8:], base[8:], tgt[8:], 32.0, steps=200, batch=16)
    out = torch.empty(256, 512, 4, device="cuda")
    gains = []
    for i in range(8):
        net.denoise(bins[i], base[i], out, 32.0)
        gains.append(dn.psnr(out, tgt[i]) - dn.psnr(base[i], tgt[i]))
    assert np.mean(gains) > 2.0 and min(gains) > 0.0, gains


def test_factory_makes_the_trained_network():
    path = Path(dn.__file__).resolve().parent / "workloads" / "denoiser_weights.npz"
    d = dn.denoiser.make("rfkt::gb300_unet_denoiser", path)
    np.testing.assert_array_equal(d.params(), dn.read_params(path))
    fresh = dn.denoiser.make("rfkt::gb300_unet_denoiser")
    assert fresh.param_count() == d.param_count()

