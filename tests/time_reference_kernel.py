"""Times the reference's own chaos-game kernels (oracle/_ref/refactor_<flame>
and its atomic-draw variant, see tests/test_gpu_refrender.py) beside librfk's
autotuned kernel on the same flame, size and spp: chain steps per second of
the bin launch (CUDA events), and the fraction of draws each histogram kept.
Test infrastructure, run by hand on a GPU:

    python tests/time_reference_kernel.py --flame bench --spp 1024
"""
import argparse
import json
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import torch  # noqa: E402

from refraktor_gb300 import librefrakt as lr  # noqa: E402
from tests import refkernels  # noqa: E402
from tests import test_gpu_refrender as rr  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--flame", default="bench")
    ap.add_argument("--spp", type=float, default=1024.0)
    args = ap.parse_args()
    out = {}
    for mod in (f"refactor_{args.flame}", f"refactor_{args.flame}_atomic"):
        rr.reference_render(mod, 1, min(args.spp, 16.0))  # load and warm the module
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        rr.TIMING = (e0, e1)
        _, info = rr.reference_render(mod, 2, args.spp)
        rr.TIMING = None
        ms = e0.elapsed_time(e1)
        out[mod] = {"iterations_per_s": info["passes"] / (ms * 1e-3), "bin_ms": ms, "kept": 1.0 - info["lost"],
                    "quality": info["quality"]}
    m = refkernels.meta(f"refactor_{args.flame}")
    db = lr.flamedb()
    f = lr.flame.from_json(db, m["genome"])
    w, h = m["width"], m["height"]
    samples = f.pack_samples(4, w, h)
    opts, _ = lr.autotune(db, f, samples, (w, h))
    k = lr.flame_compiler().get_flame_kernel(db, f, **opts)
    st = k.warmup(samples, (w, h), seed=2, count=rr.WARMUP)
    r0 = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=min(args.spp, 16.0)))
    r = k.bin(st, lr.bailout_args(iters=0, millis=0, quality=args.spp))
    kept = float(st.bins()[..., 3].double().sum().item()) / max(r0.draw_count + r.draw_count, 1)
    out["librfk"] = {"iterations_per_s": r.total_passes / (r.elapsed_ms * 1e-3), "bin_ms": r.elapsed_ms,
                     "kept": kept, "opts": opts}
    print(json.dumps({"flame": args.flame, "width": w, "height": h, "spp": args.spp, **out}))


if __name__ == "__main__":
    main()
