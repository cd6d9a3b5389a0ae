"""The device fix_rotation (the batch path and the no-alloc preparation run it
on the GPU) against the host fix_rotation (flame_compiler.cpp:957-1035
restated in genome.cpp), on noisy samples whose affine angles and palette
hues cross the +-pi / +-180 degree wraps between samples."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from refraktor_gb300 import _lib
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _device_fix_rotation(samples, ss, fs, aff):
    L = _lib.lib()
    fn = L.rfk_launch_fix_rotation
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_void_p, C.c_uint, C.c_void_p]
    d = torch.from_numpy(samples.copy()).cuda()
    a = torch.tensor(np.asarray(aff, dtype=np.uint32).view(np.int32), device="cuda")
    rc = fn(d.data_ptr(), samples.size // ss, ss, fs, a.data_ptr(), len(aff), None)
    assert rc == 0
    torch.cuda.synchronize()
    return d.cpu().numpy()


def test_device_fix_rotation_matches_host():
    db = lr.flamedb()
    f = lr.flame.from_json(db, syn.hd_flame(2))
    R = f.size_reals()
    ss = R + 768
    aff = f.affine_indices()
    rng = np.random.default_rng(11)
    base = f.pack_sample(320, 180)
    keys = []
    for k in range(6):
        s = base.copy()
        for a in aff:
            # rotate each column by a growing angle so consecutive samples wrap
            for c in (0, 2):
                ang = rng.uniform(-np.pi, np.pi) + 2.9 * k
                mag = rng.uniform(0.05, 2.0)
                s[a + c], s[a + c + 1] = mag * np.cos(ang), mag * np.sin(ang)
        hues = s[R::3]
        hues[:] = np.where(np.arange(256) % 2 == 0, 179.5 + 0.4 * k, -179.5 - 0.4 * k) + rng.normal(0, 0.05, 256)
        hues[:] = (hues + 180.0) % 360.0 - 180.0
        keys.append(s)
    # one affine with a zero column: its angle follows the other column
    keys[3][aff[0]] = keys[3][aff[0] + 1] = 0.0
    samples = np.concatenate(keys)
    want = lr.fix_rotation(samples, ss, R, aff)
    got = _device_fix_rotation(samples, ss, R, aff)
    # angles (atan2) and log-magnitudes (log) come from the device's and the
    # host's libm, each within an ulp or so of the exact value; the unwrap then
    # adds whole turns (2 pi) after the same comparisons, which keeps the
    # absolute difference, so the bound is in ulps of the values before the
    # unwrap (|angle| <= 2 pi, |log magnitude| < 2 pi here); hues are plain
    # additions of 360
    cols = np.zeros(ss, dtype=bool)
    for a in aff:
        cols[a:a + 4] = True
    w2, g2 = want.reshape(-1, ss), got.reshape(-1, ss)
    wa, ga = w2[:, cols], g2[:, cols]
    same = wa == ga  # includes log(0) = -inf of the zero column
    wa, ga = wa[~same], ga[~same]
    assert np.all(np.isfinite(wa) & np.isfinite(ga)), "a non-finite value differs"
    ulp = np.spacing(np.maximum(np.maximum(np.abs(wa), np.abs(ga)), 2 * np.pi))
    d = np.abs(wa - ga)
    assert np.all(d <= 4 * ulp), float((d / ulp).max())
    # the unwrap took the same branch everywhere: no sample differs by a turn
    assert np.all(d < 1e-9)
    # everything else (other reals, palette hue / saturation / value) is bit-exact
    np.testing.assert_array_equal(g2[:, ~cols], w2[:, ~cols])
