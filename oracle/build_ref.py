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
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
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


def compile_module(src: str, name: str, kernels: list[str], flags: list[str], arch: str = "sm_103a") -> tuple[bytes, dict]:
    L = _nvrtc()
    prog = C.c_void_p()
    r = L.nvrtcCreateProgram(C.byref(prog), src.encode(), f"{name}.cu".encode(), 0, None, None)
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


def build(ref_root: Path) -> None:
    OUT.mkdir(exist_ok=True)
    for name, (rel, kernels, flags) in MODULES.items():
        src_path = Path(ref_root) / rel
        cubin, lowered = compile_module(src_path.read_text(), name, kernels, flags)
        (OUT / f"{name}.cubin").write_bytes(cubin)
        (OUT / f"{name}.json").write_text(json.dumps({"source": rel, "kernels": lowered, "flags": flags}, indent=1))
    print(f"reference kernels built into {OUT}")


if __name__ == "__main__":
    build(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
