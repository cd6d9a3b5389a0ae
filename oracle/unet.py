"""Oracle of the learned denoiser: a CPU restatement in float64 (torch on the
CPU) of the network of refraktor_gb300/csrc/host/denoiser.cpp - the same
layers, channel layout, input features and loss - for checking the GPU
forward pass and gradients. Test infrastructure: only tests import it.

bf16=True rounds every tensor the GPU stores in bf16 (weights, activations,
and - through a custom autograd function - the gradients flowing back through
those tensors) at the same points, so that the comparison measures the
kernels rather than the storage precision.
"""
from __future__ import annotations

import numpy as np
import torch

F = torch.nn.functional

# (cin, cout, live_in, live_out) as kLayers in denoiser.cpp
LAYERS = [(32, 32, 9, 32), (32, 32, 32, 32), (32, 64, 32, 64), (64, 64, 64, 64), (64, 128, 64, 128),
          (128, 128, 128, 128), (128, 256, 128, 256), (256, 256, 256, 256), (384, 128, 384, 128),
          (128, 128, 128, 128), (192, 64, 192, 64), (64, 64, 64, 64), (96, 32, 96, 32), (32, 32, 32, 32),
          (32, 32, 32, 3)]
L_IN, E1B, E2A, E2B, E3A, E3B, B1, B2, D3A, D3B, D2A, D2B, D1A, D1B, L_OUT = range(15)


def param_count() -> int:
    return sum(co * 9 * ci + co for ci, co, _, _ in LAYERS)


def unpack(params: np.ndarray) -> list[tuple[np.ndarray, np.ndarray]]:
    """Flat parameter array (per layer: weights [cout][9][cin], bias [cout])."""
    out, o = [], 0
    for ci, co, _, _ in LAYERS:
        w = params[o:o + co * 9 * ci].reshape(co, 9, ci)
        o += co * 9 * ci
        b = params[o:o + co]
        o += co
        out.append((w, b))
    return out


def pack(layers: list[tuple[np.ndarray, np.ndarray]]) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)]) for w, b in layers])


def _bf16(x: np.ndarray) -> np.ndarray:
    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()


def features(bins: np.ndarray, base: np.ndarray, spp: float, bf16: bool = True) -> np.ndarray:
    """Input channels of histograms (..., h, w, 4) and their tonemapped images
    (base, ..., h, w, 4): log1p(density) / 8, mean colour, alpha as the
    tonemapper's, ln(spp) / 8, base RGB, zeros to 32 channels."""
    b = np.asarray(bins, dtype=np.float64)
    d = b[..., 3]
    f = np.zeros(b.shape[:-1] + (32,))
    f[..., 0] = np.log1p(np.maximum(d, 0)) / 8
    nz = d > 0
    for j in range(3):
        f[..., 1 + j] = np.where(nz, b[..., j] / np.where(nz, d, 1), 0)
    with np.errstate(divide="ignore"):
        f[..., 4] = np.where(d >= 1, np.clip(np.log(np.maximum(d, 1e-30)) * (4 / np.log(2)) / 96, 0, 1), 0)
    f[..., 5] = np.log(max(spp, 1.0)) / 8
    f[..., 6:9] = np.asarray(base, dtype=np.float64)[..., :3]
    return _bf16(f) if bf16 else f


class _Round(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        return x.to(torch.bfloat16).to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        return g.to(torch.bfloat16).to(g.dtype)


def forward(x: torch.Tensor, params: list[tuple[torch.Tensor, torch.Tensor]], bf16: bool = True) -> torch.Tensor:
    """x: (n, 32, h, w); returns the (n, 3, h, w) network output (f32 on the
    GPU), the correction that is added to the base image."""
    r = _Round.apply if bf16 else (lambda t: t)

    def conv(l, t, relu=True):
        w, b = params[l]
        y = F.conv2d(t, w, b, padding=1)
        return r(torch.relu(y)) if relu else y

    def up(t):
        return F.interpolate(t, scale_factor=2, mode="nearest")

    a1 = conv(L_IN, x)
    s1 = conv(E1B, a1)
    p1 = r(F.avg_pool2d(s1, 2))
    a2 = conv(E2A, p1)
    s2 = conv(E2B, a2)
    p2 = r(F.avg_pool2d(s2, 2))
    a3 = conv(E3A, p2)
    s3 = conv(E3B, a3)
    p3 = r(F.avg_pool2d(s3, 2))
    b1 = conv(B1, p3)
    b2 = conv(B2, b1)
    e3 = conv(D3A, torch.cat([up(b2), s3], 1))
    d3 = conv(D3B, e3)
    e2 = conv(D2A, torch.cat([up(d3), s2], 1))
    d2 = conv(D2B, e2)
    e1 = conv(D1A, torch.cat([up(d2), s1], 1))
    d1 = conv(D1B, e1)
    out = conv(L_OUT, d1, relu=False)
    return out[:, :3]


def torch_params(flat: np.ndarray, bf16: bool = True, requires_grad: bool = False):
    ps = []
    for w, b in unpack(flat):
        co, _, ci = w.shape
        wt = _bf16(w) if bf16 else np.asarray(w, dtype=np.float64)
        wt = torch.from_numpy(wt.reshape(co, 3, 3, ci).transpose(0, 3, 1, 2).copy())
        bt = torch.from_numpy(np.asarray(b, dtype=np.float64).copy())
        wt.requires_grad_(requires_grad)
        bt.requires_grad_(requires_grad)
        ps.append((wt, bt))
    return ps


def _nchw(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.asarray(a, dtype=np.float64)[..., :3].transpose(0, 3, 1, 2).copy())


def loss_and_gradients(flat: np.ndarray, bins: np.ndarray, base: np.ndarray, spp: float, targets: np.ndarray,
                       bf16: bool = True):
    """MSE over RGB of base + output and its gradients in the flat parameter layout."""
    ps = torch_params(flat, bf16=bf16, requires_grad=True)
    x = torch.from_numpy(features(bins, base, spp, bf16).transpose(0, 3, 1, 2).copy())
    out = forward(x, ps, bf16=bf16) + _nchw(base)
    loss = ((out - _nchw(targets)) ** 2).mean()
    loss.backward()
    grads = []
    for w, b in ps:
        g = w.grad.permute(0, 2, 3, 1).reshape(w.shape[0], 9, w.shape[1]).numpy()
        grads.append((g, b.grad.numpy()))
    return float(loss.item()), pack(grads)


def denoise(flat: np.ndarray, bins: np.ndarray, base: np.ndarray, spp: float, bf16: bool = True) -> np.ndarray:
    """base + network output clamped to [0, 1], (n, h, w, 3)."""
    ps = torch_params(flat, bf16=bf16)
    x = torch.from_numpy(features(bins, base, spp, bf16).transpose(0, 3, 1, 2).copy())
    with torch.no_grad():
        out = forward(x, ps, bf16=bf16) + _nchw(base)
    return np.clip(out.numpy().transpose(0, 2, 3, 1), 0, 1)
