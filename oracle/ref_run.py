"""Runs the reference's own chaos-game module (assets/kernels/refactor.cu,
specialised per flame by oracle/ref_flame.py and compiled by
oracle/build_ref.py into oracle/_ref/) the way flame_kernel::warmup + bin
drive it: the parity tests compare its renders with librfk's, and the bench's
reference arm times it. Test infrastructure only."""
import ctypes as C

import numpy as np
import torch

from oracle import oracle as orc
from oracle import refkernels
from refraktor_gb300 import librefrakt as lr

WARMUP = 20


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def reference_render(mod: str, seed: int, spp: float, timing=None) -> tuple[np.ndarray, dict]:
    """flame_kernel::warmup + bin (flame_compiler.cpp:866-955, :1037-1108) on
    the reference's module: 4 packed samples, fix_rotation, Catmull-Rom
    segments from the reference's own kernel, shuffle buffers of random
    permutations, one temporal sample per block. `timing`: a (start, end)
    pair of CUDA events recorded around the bin launch."""
    m = refkernels.meta(mod)
    g, w, h = m["genome"], m["width"], m["height"]
    tpb, grid, R = m["threads_per_block"], m["grid"], m["size_reals"]
    ss = R + 768
    db = lr.flamedb()
    f = lr.flame.from_json(db, g)
    assert f.size_reals() == R
    samples = np.asarray(f.pack_samples(4, w, h), dtype=np.float64)
    fixed = np.ascontiguousarray(orc.fix_rotation(samples, ss, R, f.affine_indices()), dtype=np.float64)
    d_samples = torch.from_numpy(fixed).cuda()
    segments = torch.zeros((1, ss, 4), dtype=torch.float64, device="cuda")
    refkernels.launch(refkernels.kernel("catmull", "generate_sample_coefficients"), (ss + 255) // 256, 256,
                      [_ptr(d_samples), C.c_uint(ss), C.c_uint(1), _ptr(segments)])
    size = torch.zeros(1, dtype=torch.int64, device="cuda")
    refkernels.launch(refkernels.kernel(mod, "get_sample_state_size"), 1, 1, [_ptr(size)])
    state_bytes = int(size.item())
    assert 0 < state_bytes < (1 << 20) and state_bytes % 16 == 0
    # shuffle buffers: NUM_SHUF_BUFS permutations of the block's lanes
    shuf_ptr, shuf_size = refkernels.global_symbol(mod, "shuf_bufs")
    nbuf = m["num_shuf_bufs"]
    assert shuf_size == 2 * tpb * nbuf
    rng = np.random.default_rng(seed)
    perms = np.stack([rng.permutation(tpb) for _ in range(nbuf)]).astype(np.uint16)
    assert perms.max() < tpb
    host = np.ascontiguousarray(perms)
    rt = refkernels._rt()
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    assert rt.cudaMemcpy(C.c_void_p(shuf_ptr), host.ctypes.data, shuf_size, 1) == 0
    state = torch.zeros(grid * state_bytes, dtype=torch.uint8, device="cuda")
    warm_hits = torch.zeros(1, dtype=torch.int64, device="cuda")
    refkernels.launch(refkernels.kernel(mod, "warmup"), grid, tpb,
                      [C.c_uint(1), _ptr(segments), C.c_uint(seed), C.c_uint(WARMUP), C.c_uint(w), C.c_uint(h),
                       _ptr(state), C.c_int(1), _ptr(warm_hits)])
    bins = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    counters = torch.zeros(5, dtype=torch.int64, device="cuda")  # quality, passes, -, earliest, latest
    counters[3] = -1  # atomicMin start
    stop = torch.zeros(1, dtype=torch.uint8, device="cuda")
    indices = torch.arange(grid, dtype=torch.int32, device="cuda")
    target = int(spp * w * h * 255.0)
    time_ns = 5_000_000_000
    cp = counters.data_ptr()
    if timing:
        timing[0].record()
    refkernels.launch(refkernels.kernel(mod, "bin"), grid, tpb,
                      [_ptr(state), C.c_uint64(target), C.c_uint(0xFFFFFFFF), C.c_uint64(time_ns), _ptr(bins),
                       C.c_uint(w), C.c_uint(h), C.c_void_p(cp), C.c_void_p(cp + 8), _ptr(stop), C.c_int(1),
                       C.c_int(100), _ptr(warm_hits), C.c_void_p(cp + 24), C.c_void_p(cp + 32), _ptr(indices)])
    if timing:
        timing[1].record()
        torch.cuda.synchronize()
    c = counters.cpu().numpy()
    out = bins.cpu().numpy().astype(np.float64)
    return out, {"quality": c[0] / (w * h * 255.0), "passes": int(c[1]), "draws": c[0] / 255.0,
                 "lost": 1.0 - out[..., 3].sum() / max(c[0] / 255.0, 1.0)}
