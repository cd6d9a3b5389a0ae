"""Compiles the reference's own flame-independent CUDA kernels with NVRTC for
sm_103a into oracle/_ref/ (test infrastructure: the parity tests run them on
the GPU beside librfk's kernels).

Sources are read where they lie in the reference tree; nothing is copied into
the repository. Flags follow the reference's host code:
  tonemap.cu        tonemap<half3|half4|float3|float4, 4>; -use_fast_math,
                    -default-device, extra device vectorization
                    (src/librefrakt/src/image/tonemapper.cpp:10-22)
  catmull.cu        generate_sample_coefficients; -default-device
                    (src/librefrakt/src/flame_compiler.cpp:760-766)
  density_histo.cu  calculate_histogram<4>; -default-device
                    (src/librefrakt/src/flame_compiler.cpp:773-780)
Each module is written as <name>.cubin with <name>.json holding the lowered
kernel names.

The reference's chaos-game module (refactor.cu) is specialised per flame: for
each flame of REF_FLAMES its flame_generated.h is produced by
oracle/ref_flame.py (flame.tpl + the flang rule table) and the module is
compiled with the reference's options (flame_compiler.cpp:600-620, :834-860:
-extra-device-vectorization, -default-device, -lineinfo, -use_fast_math,
NUM_SHUF_BUFS 512 and the launch-shape defines, refrakt/random.h and
refrakt/flamelib.h as headers) into refactor_<flame>.cubin; its json also
holds the genome, the launch shape and the flame's real count. A second
module, refactor_<flame>_atomic, differs in one place: the histogram update
of pass_and_draw (refactor.cu:374-381), a non-atomic load / add / store that
loses the draws of lanes and blocks hitting the same pixel at once, becomes
four atomic adds of the same contribution (ATOMIC_DRAW below), so that the
reference's sampling (warp vote, iterator shuffle, xoroshiro64) can be
compared with librfk's apart from the lost draws.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout this recipe reads (absent on machines that only run
# the prebuilt files); RFK_REFERENCE_ROOT overrides it
REFERENCE_ROOT = Path(os.environ.get("RFK_REFERENCE_ROOT", "/root/reference"))
CUDA = Path("/usr/local/cuda")

MODULES = {
    "tonemap": ("assets/kernels/tonemap.cu", ["tonemap<half3, 4>", "tonemap<half4, 4>", "tonemap<float3, 4>",
                                              "tonemap<float4, 4>"],
                ["-use_fast_math", "-default-device", "-extra-device-vectorization"]),
    "catmull": ("assets/kernels/catmull.cu", ["generate_sample_coefficients"],
                ["-default-device", "-extra-device-vectorization"]),
    "histogram": ("assets/kernels/density_histo.cu", ["calculate_histogram<4>"],
                  ["-default-device", "-extra-device-vectorization"]),
}


def _nvrtc() -> C.CDLL:
    L = C.CDLL(str(CUDA / "lib64" / "libnvrtc.so"))
    L.nvrtcGetErrorString.restype = C.c_char_p
    return L


def compile_module(src: str, name: str, kernels: list[str], flags: list[str], arch: str = "sm_103a",
                   headers: dict[str, str] | None = None) -> tuple[bytes, dict]:
    L = _nvrtc()
    prog = C.c_void_p()
    headers = headers or {}
    hsrc = (C.c_char_p * max(1, len(headers)))(*[v.encode() for v in headers.values()])
    hname = (C.c_char_p * max(1, len(headers)))(*[k.encode() for k in headers])
    r = L.nvrtcCreateProgram(C.byref(prog), src.encode(), f"{name}.cu".encode(), len(headers),
                             hsrc if headers else None, hname if headers else None)
    if r:
        raise RuntimeError(f"nvrtcCreateProgram: {L.nvrtcGetErrorString(r).decode()}")
    for k in kernels:
        L.nvrtcAddNameExpression(prog, k.encode())
    opts = [f"--gpu-architecture={arch}", "--std=c++20", "-DROCCU_CUDA", *flags]
    arr = (C.c_char_p * len(opts))(*[o.encode() for o in opts])
    r = L.nvrtcCompileProgram(prog, len(opts), arr)
    n = C.c_size_t(0)
    L.nvrtcGetProgramLogSize(prog, C.byref(n))
    log = C.create_string_buffer(n.value + 1)
    L.nvrtcGetProgramLog(prog, log)
    if r:
        raise RuntimeError(f"NVRTC failed for {name}: {L.nvrtcGetErrorString(r).decode()}\n{log.value.decode()}")
    lowered = {}
    for k in kernels:
        p = C.c_char_p()
        L.nvrtcGetLoweredName(prog, k.encode(), C.byref(p))
        lowered[k] = p.value.decode()
    L.nvrtcGetCUBINSize(prog, C.byref(n))
    buf = C.create_string_buffer(n.value)
    L.nvrtcGetCUBIN(prog, buf)
    L.nvrtcDestroyProgram(C.byref(prog))
    return buf.raw, lowered


# Flames whose reference chaos-game module is built: genome maker (seeded),
# image size, threads per block and blocks per SM (the grid is blocks per SM
# x the 152 SMs of a GB300, fixed at compile time through TOTAL_THREADS).
# The reference's only real-world genome, assets/flames_test/electricsheep.247.50049.flam3
# (fisheye, bubble, julia, post affines, gamma 4), imported with the library's
# flam3 reader (flame_types.cpp:131-239 restated) and rendered at its own size.
SHEEP = "assets/flames_test/electricsheep.247.50049.flam3"


def _ref_flames(ref_root: Path) -> dict:
    sys.path.insert(0, str(HERE.parent))
    from refraktor_gb300 import librefrakt as lr
    from refraktor_gb300 import synthetic as syn

    bench = json.loads((HERE.parent / "refraktor_gb300" / "workloads" / "hd_1080p.json").read_text())
    sheep = lr.flame.import_flam3(lr.flamedb(), (Path(ref_root) / SHEEP).read_text()).serialize()
    return {
        "c0": (syn.plain_flame(0), 512, 512, 128, 8),
        "hd": (syn.hd_flame(21), 320, 180, 128, 8),
        "bench": (bench, 1920, 1080, 128, 8),
        "sheep": (sheep, 800, 592, 128, 8),
    }


REF_SMS = 152

# refactor.cu:374 and :381, and their replacements in the atomic variant
ATOMIC_DRAW = [("float4 new_bin = bin;", "float4 new_bin = make_float4(0.0f, 0.0f, 0.0f, 0.0f);"),
               ("bin = new_bin;", "atomicAdd(&bin.x, new_bin.x); atomicAdd(&bin.y, new_bin.y); "
                                  "atomicAdd(&bin.z, new_bin.z); atomicAdd(&bin.w, new_bin.w);")]


def _atomic_draw(src: str) -> str:
    for old, new in ATOMIC_DRAW:
        if src.count(old) != 1:
            raise RuntimeError(f"refactor.cu: expected one '{old}'")
        src = src.replace(old, new)
    return src


def build_flames(ref_root: Path) -> None:
    from oracle import oracle as orc
    from oracle import ref_flame

    rel = "assets/kernels/refactor.cu"
    inc = Path(ref_root) / "assets" / "kernels" / "include" / "refrakt"
    for tag, (g, w, h, tpb, bpmp) in _ref_flames(ref_root).items():
        R = orc.size_reals(g)
        header = ref_flame.flame_header(Path(ref_root), g, orc.affine_indices(g))
        grid = bpmp * REF_SMS
        flags = ["-extra-device-vectorization", "-default-device", "-lineinfo", "-use_fast_math",
                 "-DNUM_SHUF_BUFS=512", f"-DTHREADS_PER_BLOCK={tpb}", f"-DBLOCKS_PER_MP={bpmp}",
                 f"-DFLAME_SIZE_REALS={R}", f"-DFLAME_SIZE_BYTES={4 * R}", f"-DTOTAL_THREADS={grid * tpb}",
                 "-DFLAMEDB_HASH=rfkharness"]
        if "chaos" in g:
            flags.append("-DUSE_CHAOS")
        headers = {"flame_generated.h": header, "refrakt/random.h": (inc / "random.h").read_text(),
                   "refrakt/flamelib.h": (inc / "flamelib.h").read_text()}
        names = ["warmup", "bin", "get_sample_state_size", "shuf_bufs"]
        src = (Path(ref_root) / rel).read_text()
        for suffix, text in (("", src), ("_atomic", _atomic_draw(src))):
            cubin, lowered = compile_module(text, f"refactor_{tag}{suffix}", names, flags, headers=headers)
            (OUT / f"refactor_{tag}{suffix}.cubin").write_bytes(cubin)
            (OUT / f"refactor_{tag}{suffix}.json").write_text(json.dumps(
                {"source": rel, "atomic_draw": bool(suffix), "kernels": lowered, "flags": flags, "genome": g,
                 "width": w, "height": h, "threads_per_block": tpb, "blocks_per_sm": bpmp, "grid": grid,
                 "size_reals": R, "num_shuf_bufs": 512}, indent=1))


def build(ref_root: Path) -> None:
    OUT.mkdir(exist_ok=True)
    for name, (rel, kernels, flags) in MODULES.items():
        src_path = Path(ref_root) / rel
        cubin, lowered = compile_module(src_path.read_text(), name, kernels, flags)
        (OUT / f"{name}.cubin").write_bytes(cubin)
        (OUT / f"{name}.json").write_text(json.dumps({"source": rel, "kernels": lowered, "flags": flags}, indent=1))
    build_flames(ref_root)
    print(f"reference kernels built into {OUT}")


if __name__ == "__main__":
    build(Path(sys.argv[1]) if len(sys.argv) > 1 else REFERENCE_ROOT)
