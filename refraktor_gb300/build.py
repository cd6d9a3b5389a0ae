"""Builds librfk.so in-tree (refraktor_gb300/_build/) for sm_103a.

Host C++ is compiled with g++, the flame-independent kernels with nvcc
(-gencode arch=compute_103a,code=sm_103a), and the NVRTC kernel texts
(csrc/jit/*.cuh) are embedded as string literals. Translation units are
compiled in parallel and skipped when their object is newer than every input.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "librfk.so"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SOURCES = ["dsl.cpp", "value.cpp", "inflate.cpp", "flamedb.cpp", "genome.cpp", "align.cpp", "flam3.cpp", "codegen.cpp",
                "runtime.cpp", "batch.cpp", "denoiser.cpp", "image_io.cpp",
                "weights_io.cpp"]
CUDA_SOURCES = {"image.cu": [], "tonemap_fast.cu": ["--use_fast_math"], "noalloc.cu": ["--fmad=false"], "unet_tc.cu": [],
                "unet_ops.cu": []}
JIT_TEXTS = {"rfk_src_device": "rfk_device.cuh", "rfk_src_iterate": "rfk_iterate.cuh"}


def _headers() -> list[Path]:
    hs = list((CSRC / "host").glob("*.h")) + list((CSRC / "kernels").glob("*.h")) + list((CSRC / "kernels").glob("*.cuh"))
    hs.append(PKG.parent / "include" / "rfk.h")
    return hs


def _stale(obj: Path, inputs: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _embed_jit() -> Path:
    out = BUILD / "jit_sources.cpp"
    parts = ["// generated by build.py from csrc/jit/*.cuh\n"]
    for sym, fname in JIT_TEXTS.items():
        text = (CSRC / "jit" / fname).read_text()
        delim = "rfk_src_delim"
        assert f"){delim}\"" not in text
        parts.append(f'extern const char* const {sym};\nconst char* const {sym} = R"{delim}({text}){delim}";\n')
    content = "".join(parts)
    if not out.exists() or out.read_text() != content:
        out.write_text(content)
    return out


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    jit = _embed_jit()
    headers = _headers()
    jobs: list[tuple[Path, list[str], list[Path]]] = []
    inc = [f"-I{CUDA / 'include'}", f"-I{PKG.parent / 'include'}"]
    cxx = os.environ.get("CXX", "g++")
    # no FMA contraction: host arithmetic gives the same bits on x86-64 and aarch64
    cflags = ["-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function"] + inc
    for src in HOST_SOURCES:
        s = CSRC / "host" / src
        o = BUILD / (src + ".o")
        jobs.append((o, [cxx, *cflags, "-c", str(s), "-o", str(o)], [s, *headers, Path(__file__)]))
    o = BUILD / "jit_sources.o"
    jobs.append((o, [cxx, "-std=c++20", "-O1", "-fPIC", "-c", str(jit), "-o", str(o)], [jit]))
    nvcc = str(CUDA / "bin" / "nvcc")
    for src, extra in CUDA_SOURCES.items():
        s = CSRC / "kernels" / src
        o = BUILD / (src + ".o")
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", *extra, "-Xcompiler", "-fPIC", *inc, "-c", str(s), "-o", str(o)]
        jobs.append((o, cmd, [s, *headers]))

    todo = [(o, cmd) for o, cmd, ins in jobs if _stale(o, ins)]
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(_run, cmd) for _, cmd in todo]
            for f in futs:
                f.result()
    objs = [o for o, _, _ in jobs]
    if todo or _stale(LIB, objs):
        link = [cxx, "-shared", "-o", str(LIB), *map(str, objs), f"-L{CUDA / 'lib64'}",
                "-lcudart", "-lnvrtc", f"-Wl,-rpath,{CUDA / 'lib64'}"]
        _run(link)
    if verbose:
        print(f"built {LIB}")
    return LIB


def clean() -> None:
    if BUILD.exists():
        shutil.rmtree(BUILD)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
