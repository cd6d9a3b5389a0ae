"""The learned denoiser: Python mirror of the reference's denoiser interface
(src/librefrakt/include/librefrakt/interface/denoiser.h:21-39) over
include/rfk_denoise.h, plus the renderer-driven training data, training loop
and PSNR evaluation of the denoised low-spp path against the plain path.
Device memory is torch CUDA memory; all compute is librfk's kernels.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import librefrakt as lr
from ._lib import check, lib


def _ptr(t) -> int:
    return int(t.data_ptr())


def _stream(s) -> Optional[int]:
    return lr._stream_ptr(s)


class denoiser:
    """A U-Net denoiser (interface::denoiser): denoise(bins, base, out) maps
    the histogram of a low-spp render and its tonemapped image (base) to the
    tonemapped image of a converged render, as base + a learned correction."""

    def __init__(self, seed: int = 1, params: Optional[np.ndarray] = None):
        h = C.c_void_p()
        check(lib().rfk_denoiser_create(seed, C.byref(h)))
        self._h = h
        if params is not None:
            self.set_params(params)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_denoiser_destroy(self._h)
            self._h = None

    @classmethod
    def make(cls, name: str, weights_path: str | Path | None = None) -> "denoiser":
        """denoiser::make by registered name (factory.h:71-98); raises
        RfkError for an unknown name."""
        h = C.c_void_p()
        check(lib().rfk_denoiser_make(name.encode(), str(weights_path).encode() if weights_path else None, C.byref(h)))
        d = cls.__new__(cls)
        d._h = h
        return d

    def param_count(self) -> int:
        return int(lib().rfk_denoiser_param_count(self._h))

    def params(self) -> np.ndarray:
        out = np.zeros(self.param_count(), dtype=np.float32)
        check(lib().rfk_denoiser_get_params(self._h, out.ctypes.data, out.size))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().rfk_denoiser_set_params(self._h, p.ctypes.data, p.size))

    def save(self, path: str | Path) -> None:
        np.savez_compressed(path, params=self.params().astype(np.float16))

    @classmethod
    def load(cls, path: str | Path) -> "denoiser":
        return cls(params=np.load(path)["params"].astype(np.float32))

    def train_step(self, bins, base, spp: float, targets, lr_: float = 1e-3, stream=None) -> float:
        """bins (n, h, w, 4) f32 histograms, base (n, h, w, 4) their tonemapped
        images, targets (n, h, w, 4) f32 RGBA (CUDA tensors)."""
        n, h, w, _ = bins.shape
        loss = C.c_double()
        check(lib().rfk_denoiser_train_step(self._h, _ptr(bins), _ptr(base), n, w, h, float(spp), _ptr(targets),
                                            float(lr_), C.byref(loss), _stream(stream)))
        return loss.value

    def loss(self, bins, base, spp: float, targets, stream=None) -> float:
        n, h, w, _ = bins.shape
        loss = C.c_double()
        check(lib().rfk_denoiser_loss(self._h, _ptr(bins), _ptr(base), n, w, h, float(spp), _ptr(targets), C.byref(loss),
                                      _stream(stream)))
        return loss.value

    def denoise(self, bins, base, out, spp: float, fmt: int = lr.FLOAT4, stream=None) -> None:
        """bins (h, w, 4) histogram, base (h, w, 4) its tonemapped image, out
        (h, w, channels of fmt) CUDA tensors."""
        h, w, _ = bins.shape
        check(lib().rfk_denoise(self._h, _ptr(bins), _ptr(base), w, h, float(spp), _ptr(out), fmt, _stream(stream)))


# ------------------------------------------------------------------ data ----
def frame_set(db, genomes: Sequence[dict], w: int, h: int, preview: int = 256, chunk: int = 128) -> list[tuple[dict, float]]:
    """Camera fit of many genomes at once, the batched form of
    synthetic.frame_on_gpu: a wide preview render locates the 1%..99% box of
    the drawn points, a second render at that box refines it, a third gives
    the lit fraction. The genomes must share one structure (align_flames).
    Returns (framed genome, lit fraction) pairs."""
    from . import synthetic as syn

    rw = preview
    rh = max(16, int(round(rw * h / w)))
    gs = [dict(g, center_x=0.0, center_y=0.0, scale=1.0 / 40.0) for g in genomes]
    cov = [0.0] * len(gs)
    for it in range(3):
        dens = render_set(db, gs, rw, rh, 16.0, seed=11 + it, chunk=chunk)[..., 3].cpu().numpy()
        if it == 2:
            cov = [float((d > 0).mean()) for d in dens]
            break
        nxt = []
        for g, d in zip(gs, dens):
            box = syn._quantile_box(d, g, rw, rh)
            if box is None:
                nxt.append(g)
                continue
            x0, x1, y0, y1 = box
            sx, sy = max(x1 - x0, 1e-4), max(y1 - y0, 1e-4)
            nxt.append(dict(g, center_x=float((x0 + x1) / 2), center_y=float((y0 + y1) / 2),
                            scale=float(min(rw / (sx * rh), 1.0 / sy) * 0.95)))
        gs = nxt
    return [(dict(g0, center_x=g["center_x"], center_y=g["center_y"], scale=float(g["scale"]) * (rh / rw) / (h / w)), c)
            for g0, g, c in zip(genomes, gs, cov)]


def visible_set(db, make, seeds: Sequence[int], count: int, w: int, h: int, min_coverage: float = 0.25) -> list[dict]:
    """The first `count` genomes make(seed) (in seed order) whose framed preview
    lights at least `min_coverage` of its pixels, aligned to one structure and
    framed for w x h (synthetic.visible_flame's rejection, batched)."""
    al = aligned_genomes(db, [make(s) for s in seeds])
    framed = frame_set(db, al, w, h)
    keep = [g for g, c in framed if c >= min_coverage]
    if len(keep) < count:
        raise RuntimeError(f"only {len(keep)} of {len(seeds)} candidates are visible; need {count}")
    return keep[:count]


def render_set(db, genomes: Sequence[dict], w: int, h: int, spp: float, seed: int = 1, tonemap: bool = False,
               chunk: int = 64, kernel=None, both: bool = False):
    """Renders genomes of one structure (align_flames first) at w x h to spp
    with the batch renderer; returns (N, h, w, 4) f32 histograms, or the
    tonemapped RGBA images when `tonemap`, or (histograms, images) when
    `both`."""
    import torch

    fs = [lr.flame.from_json(db, g) for g in genomes]
    k = kernel or lr.flame_compiler().get_flame_kernel(db, fs[0])
    hist = torch.empty((len(fs), h, w, 4), dtype=torch.float32, device="cuda") if (both or not tonemap) else None
    imgs = torch.empty((len(fs), h, w, 4), dtype=torch.float32, device="cuda") if (both or tonemap) else None
    for c0 in range(0, len(fs), chunk):
        part = fs[c0:c0 + chunk]
        units, samples = [], []
        for i, f in enumerate(part):
            tp = f.tonemap_params()
            units.append(lr.batch_unit(w, h, spp, segment=4 * i, t=0.0, gamma=tp["gamma"], brightness=tp["brightness"],
                                       vibrancy=tp["vibrancy"]))
            samples.append(f.pack_samples(4, w, h).reshape(4, -1))
        b = lr.batch(k, units, 4 * len(part), seed=seed + c0, out_format=lr.FLOAT4 if imgs is not None else -1)
        b.set_samples(np.concatenate(samples))
        b.run()
        b.wait()
        for i in range(len(part)):
            if hist is not None:
                hist[c0 + i].copy_(b.bins(i))
            if imgs is not None:
                imgs[c0 + i].copy_(b.image(i))
        torch.cuda.synchronize()
        del b
    if both:
        return hist, imgs
    return imgs if tonemap else hist


def aligned_genomes(db, genomes: Sequence[dict]) -> list[dict]:
    """Genomes given one structure (align_flames), as JSON dicts."""
    al = lr.align_flames(db, [lr.flame.from_json(db, g) for g in genomes])
    return [f.serialize() for f in al]


def psnr(a, b) -> float:
    """PSNR (peak 1) over the RGB channels of two (h, w, >=3) images."""
    import torch

    mse = torch.mean((a[..., :3].float() - b[..., :3].float()) ** 2).item()
    return float("inf") if mse == 0 else 10.0 * np.log10(1.0 / mse)


# ----------------------------------------------------------------- train ----
@dataclass
class train_report:
    steps: int
    seconds: float
    first_loss: float
    last_loss: float
    val_loss: float
    ms_per_step: float


def train(net: denoiser, bins, base, targets, spp, steps: int, batch: int = 16, lr_: float = 1e-3,
          val: Optional[tuple] = None, seed: int = 0, log=None, augment: bool = True) -> train_report:
    """Adam on random mini-batches of the (N, h, w, 4) training tensors,
    randomly mirrored; cosine-decayed learning rate. val: (bins, base,
    targets). Several input sample counts: `bins`, `base` and `spp` are lists
    (one histogram / image set per spp, of the same flames and targets), and
    the steps take them in turn, so that the network's log-spp input channel
    sees every count; val then holds one (bins, base) per spp and the
    validation loss is their mean."""
    import torch

    sets = list(zip(bins, base, spp)) if isinstance(spp, (list, tuple)) else [(bins, base, spp)]
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = sets[0][0].shape[0]
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        sb, sbase, sspp = sets[s % len(sets)]
        idx = torch.randint(0, n, (batch,), generator=g).cuda()
        lr_s = lr_ * 0.5 * (1.0 + np.cos(np.pi * s / max(steps, 1)))
        b, bb, tt = sb.index_select(0, idx), sbase.index_select(0, idx), targets.index_select(0, idx)
        if augment:
            # mirror images: the chaos game's statistics do not depend on orientation
            flips = [d for d, bit in ((1, 1), (2, 2)) if int(torch.randint(0, 4, (1,), generator=g)) & bit]
            if flips:
                b, bb, tt = b.flip(flips), bb.flip(flips), tt.flip(flips)
        l = net.train_step(b.contiguous(), bb.contiguous(), sspp, tt.contiguous(), max(lr_s, lr_ * 0.02))
        losses.append(l)
        if log and (s % 100 == 0 or s == steps - 1):
            log(f"step {s} loss {l:.6f}")
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    vl = float("nan")
    if val is not None:
        vt = val[2]
        vsets = list(zip(val[0], val[1], spp)) if isinstance(spp, (list, tuple)) else [(val[0], val[1], spp)]
        vl = float(np.mean([net.loss(vb[i:i + 4].contiguous(), vbase[i:i + 4].contiguous(), vs, vt[i:i + 4].contiguous())
                            for vb, vbase, vs in vsets for i in range(0, vb.shape[0], 4)]))
    return train_report(steps, dt, losses[0], float(np.mean(losses[-20:])), vl, 1e3 * dt / max(steps, 1))


def _profile_case(argv=None) -> None:
    """Fixed workloads for timing and profiler captures, with random inputs:
    `infer` runs the U-Net on a 1920 x 1080 histogram, `train` runs training
    steps on 16 x 512 x 512."""
    import argparse

    import torch

    from . import build

    ap = argparse.ArgumentParser(prog="python -m refraktor_gb300.denoise")
    ap.add_argument("--case", choices=["infer", "train"], default="infer")
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    build.build()
    net = denoiser.load(Path(__file__).resolve().parent / "workloads" / "denoiser_weights.npz")
    g = torch.Generator(device="cuda").manual_seed(1)
    if a.case == "infer":
        bins = torch.rand(1080, 1920, 4, device="cuda", generator=g) * 8
        base = torch.rand(1080, 1920, 4, device="cuda", generator=g)
        out = torch.empty(1080, 1920, 4, device="cuda")
        for _ in range(a.reps):
            net.denoise(bins, base, out, 32.0)
    else:
        bins = torch.rand(16, 512, 512, 4, device="cuda", generator=g) * 8
        base = torch.rand(16, 512, 512, 4, device="cuda", generator=g)
        tgt = torch.rand(16, 512, 512, 4, device="cuda", generator=g)
        for _ in range(a.reps):
            net.train_step(bins, base, 32.0, tgt, 1e-4)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        if a.case == "infer":
            net.denoise(bins, base, out, 32.0)
        else:
            net.train_step(bins, base, 32.0, tgt, 1e-4)
    e1.record()
    torch.cuda.synchronize()
    print(f"{a.case}: {e0.elapsed_time(e1) / a.reps:.3f} ms per call")


def names() -> list[str]:
    """The registered denoiser names."""
    out, buf = [], C.create_string_buffer(256)
    while lib().rfk_denoiser_name(len(out), buf, 256) == 0:
        out.append(buf.value.decode())
    return out


def read_params(path: str | Path) -> np.ndarray:
    """The parameters of a weight file through the library's own reader
    (rfk_denoiser_read_params), as a C or C++ caller loads them."""
    n = C.c_size_t()
    check(lib().rfk_denoiser_read_params(str(path).encode(), None, 0, C.byref(n)))
    out = np.empty(n.value, dtype=np.float32)
    check(lib().rfk_denoiser_read_params(str(path).encode(), out.ctypes.data, out.size, C.byref(n)))
    return out


if __name__ == "__main__":
    _profile_case()
