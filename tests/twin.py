"""FP64 host twin of a generated flame (test infrastructure).

The flame compiler's output - the device prelude (csrc/jit/rfk_device.cuh)
and the generated per-flame code - also compiles as plain C++ when
RFK_HOST_TWIN is defined; with RFK_REAL=double and RFK_PARAM_T=double every
variation formula is evaluated in FP64. The twin's random draws come from the
same Philox4x32-10 streams as the device's rfk_apply (point index, sub-stream
0xFFFC, pass 0, key (seed, 0)), and a uniform draw is the same FP32 value on
both sides, so stochastic variations compare point by point too."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import numpy as np

from refraktor_gb300 import build
from refraktor_gb300 import librefrakt as lr

ITERATE_MARK = "// Chaos-game kernels, specialised per flame structure by NVRTC."

MAIN = r"""
#include <cstdio>
#include <vector>
int main() {
    unsigned n = 0, np = 0, seed = 0;
    int xf = 0;
    if (std::scanf("%u %u %d %u", &n, &np, &xf, &seed) != 4) return 2;
    std::vector<double> P(np);
    for (unsigned i = 0; i < np; i++)
        if (std::scanf("%lf", &P[i]) != 1) return 3;
    for (unsigned j = 0; j < n; j++) {
        unsigned idx = 0;
        double x = 0, y = 0, c = 0;
        if (std::scanf("%u %lf %lf %lf", &idx, &x, &y, &c) != 4) return 4;
        Rng rng;
        rng.start(idx, 0xFFFCu, 0ull, seed, 0u);
        V2 p = fl_vec2(x, y);
        R col = c;
        R op = 0;
#if RFK_HAS_FINAL
        if (xf < 0) op = rfk_final(p, col, P.data(), rng);
        else
#endif
        op = rfk_dispatch(xf, p, col, P.data(), rng);
        std::printf("%.17g %.17g %.17g %.17g\n", (double)p.x, (double)p.y, (double)col, (double)op);
    }
    return 0;
}
"""


class Twin:
    """The compiled FP64 twin of one flame."""

    def __init__(self, db: lr.flamedb, f: lr.flame, workdir: Path):
        cxx = shutil.which("g++")
        if not cxx:
            raise RuntimeError("no C++ compiler")
        src = lr.generate_source(db, f)
        cut = src.index(ITERATE_MARK)
        workdir.mkdir(parents=True, exist_ok=True)
        cpp = workdir / "twin.cpp"
        cpp.write_text("#define RFK_HOST_TWIN 1\n#define RFK_REAL double\n#define RFK_PARAM_T double\n" + src[:cut] + MAIN)
        self.exe = workdir / "twin"
        r = subprocess.run([cxx, "-std=c++17", "-O1", "-ffp-contract=off", "-w", str(cpp), "-o", str(self.exe)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(r.stderr[-4000:])

    def apply(self, params: np.ndarray, xform: int, pts: np.ndarray, idx: np.ndarray, seed: int = 0) -> np.ndarray:
        """(n, 4) = (x, y, colour, opacity) of xform `xform` at points (n, 3),
        point i drawing from Philox stream idx[i]."""
        P = np.asarray(params, dtype=np.float64)
        head = f"{len(pts)} {P.size} {xform} {seed}\n" + " ".join(repr(float(v)) for v in P) + "\n"
        body = "".join(f"{int(i)} {float(x)!r} {float(y)!r} {float(c)!r}\n" for i, (x, y, c) in zip(idx, pts))
        r = subprocess.run([str(self.exe)], input=head + body, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(f"twin exited {r.returncode}: {r.stderr[-2000:]}")
        return np.array([[float(v) for v in line.split()] for line in r.stdout.strip().split("\n")])


def variation_params(yaml_text: str) -> dict[str, list[tuple[str, float | None]]]:
    """Parameter names of every variation of a variations_new.yml text, with
    their defaults (None when there is none), leaving out precalc ones."""
    out: dict[str, list] = {}
    name = None
    in_param = False
    cur = None
    for line in yaml_text.splitlines():
        if not line.strip() or line.lstrip().startswith("#"):
            continue
        m = re.match(r"^([A-Za-z_]\w*):", line)
        if m:
            name = m.group(1)
            out[name] = []
            in_param = False
            continue
        if name is None:
            continue
        if re.match(r"^  param:", line):
            in_param = True
            continue
        if re.match(r"^  \S", line):
            in_param = False
            continue
        if in_param:
            m = re.match(r"^    ([A-Za-z_]\w*):(.*)$", line)
            if m:
                rest = m.group(2)
                d = re.search(r"default:\s*([-+0-9.eE]+)", rest)
                cur = [m.group(1), float(d.group(1)) if d else None, "precalc" in rest]
                out[name].append(cur)
            elif cur is not None and "precalc" in line:
                cur[2] = True
    return {k: [(n, d) for n, d, pre in v if not pre] for k, v in out.items()}
