"""rfk_prepare_samples_noalloc: the genome-preparation step for callers that
cannot allocate device memory (their memory belongs to their own pool, or a
cudaMalloc / cudaFree stall is not acceptable in their loop). It must give
what rfk_prepare_samples gives, call after call, through the C ABI.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from refraktor_gb300 import _lib
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _prepare(fn, k, samples, seg, t, seed):
    L = _lib.lib()
    out = np.zeros((len(seg), k.info["sample_floats"]), dtype=np.float32)
    s = np.ascontiguousarray(samples, dtype=np.float64)
    sg = np.ascontiguousarray(seg, dtype=np.uint32)
    tt = np.ascontiguousarray(t, dtype=np.float32)
    ss = k.info["size_reals"] + 768
    rc = getattr(L, fn)(k._h, s.ctypes.data, s.size // ss, sg.ctypes.data, tt.ctypes.data, sg.size, seed, out.ctypes.data)
    assert rc == 0, L.rfk_last_error().decode()
    return out


def _close(a, b, k):
    """The interpolation tolerance of the parity tests: 4 FP32 ulps of the
    larger value for the parameters, one 8-bit step for the palette."""
    pal0 = k.info["sample_floats"] - 1024
    ulp = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32)).astype(np.float64)
    d = np.abs(a.astype(np.float64) - b.astype(np.float64))
    assert np.all(d[:, :pal0] <= 4 * ulp[:, :pal0]), float((d[:, :pal0] / np.maximum(ulp[:, :pal0], 1e-45)).max())
    assert np.all(d[:, pal0:] <= 1.0 / 255 + 1e-6)


def test_no_alloc_prepare_matches_allocating_entry_point():
    db = lr.flamedb()
    rng = np.random.default_rng(3)
    g = syn.hd_flame(4)
    f = lr.flame.from_json(db, g)
    k = lr.flame_compiler().get_flame_kernel(db, f)
    base = f.pack_sample(640, 360)
    R = f.size_reals()
    keys = []
    for _ in range(5):
        s = base.copy()
        s[13:R] += rng.normal(0, 0.05, R - 13)
        keys.append(s)
    samples = np.concatenate(keys)
    # two calls in a row with different schedules: the second must not see the first's data
    for seg, t in [([0, 1, 1, 0], [0.0, 0.5, 0.99, 0.25]), ([1, 0, 1], [0.75, 0.1, 0.0])]:
        want = _prepare("rfk_prepare_samples", k, samples, seg, t, 7)
        got = _prepare("rfk_prepare_samples_noalloc", k, samples, seg, t, 7)
        _close(got, want, k)


def test_no_alloc_rejects_requests_beyond_the_scratch():
    db = lr.flamedb()
    f = lr.flame.from_json(db, syn.plain_flame(1))
    k = lr.flame_compiler().get_flame_kernel(db, f)
    samples = f.pack_samples(4, 64, 64)
    n = (4 << 20) // (k.info["sample_floats"] * 4) + 1  # output blocks alone exceed 4 MiB
    L = _lib.lib()
    out = np.zeros((n, k.info["sample_floats"]), dtype=np.float32)
    seg = np.zeros(n, dtype=np.uint32)
    t = np.zeros(n, dtype=np.float32)
    rc = L.rfk_prepare_samples_noalloc(k._h, samples.ctypes.data, 4, seg.ctypes.data, t.ctypes.data, n, 0, out.ctypes.data)
    assert rc == 1
    assert b"scratch" in L.rfk_last_error()
