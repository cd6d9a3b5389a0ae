"""Generates the seeded benchmark genomes of this directory (needs a GPU for
the camera fit; run once, the JSON files are committed):

  plain_512.json   plain single flame: 3 xforms 0.5/0.3/0.2 from
                   {linear, sinusoidal, spherical}, framed for 512x512
  hd_1080p.json    8 xforms (Dirichlet(1) weights) + final xform, 1-3
                   variations each from the 14-variation set, framed for
                   1920x1080
  anim_720p.json   4 keyframes of one structure (6 xforms, variation sets
                   shared, affines and weights per keyframe), framed for
                   1280x720: the batched-animation workload (120 frames)
  hetero_64.json   64 independent flames with their sizes and spp targets:
                   the heterogeneous-batch workload

Each is the first candidate of its seed that passes the visibility rejection
of synthetic.visible_flame (at least 25% of a 256-pixel preview lit).
Run: python -m refraktor_gb300.workloads.make_workloads [file names]
"""
import json
from pathlib import Path

from refraktor_gb300 import build
from refraktor_gb300 import librefrakt as lr
from refraktor_gb300 import synthetic as syn

HERE = Path(__file__).resolve().parent


def main(only: list[str] | None = None) -> None:
    build.build()
    db = lr.flamedb()
    makers = {
        "plain_512.json": lambda: syn.visible_flame(db, syn.plain_flame, 0, 512, 512),
        "hd_1080p.json": lambda: syn.visible_flame(db, syn.hd_flame, 0, 1920, 1080),
        "anim_720p.json": lambda: {"keyframes": syn.animation_keyframes(db, 0, 1280, 720), "width": 1280, "height": 720,
                                   "frames": 120, "spp": 256},
        "hetero_64.json": lambda: {"flames": syn.hetero_batch(db, 0)},
    }
    for name, make in makers.items():
        if only and name not in only:
            continue
        g = make()
        (HERE / name).write_text(json.dumps(g, indent=1))
        print("wrote", HERE / name, g.get("name", ""))


if __name__ == "__main__":
    import sys

    main(sys.argv[1:] or None)
