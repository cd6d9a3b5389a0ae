"""Loads the reference's own kernels (built by oracle/build_ref.py into
oracle/_ref/) and launches them on torch CUDA tensors: the parity tests and
the bench's reference arm run them. Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

REF = Path(__file__).resolve().parent / "_ref"
_cudart = None
_libs: dict = {}


def available(name: str) -> bool:
    return (REF / f"{name}.cubin").exists() and (REF / f"{name}.json").exists()


def _rt() -> C.CDLL:
    global _cudart
    if _cudart is None:
        for cand in ["/usr/local/cuda/lib64/libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so", "libcudart.so.13"]:
            try:
                _cudart = C.CDLL(cand)
                break
            except OSError:
                continue
        if _cudart is None:
            raise RuntimeError("libcudart not found")
        _cudart.cudaGetErrorString.restype = C.c_char_p
    return _cudart


def _check(r: int, what: str) -> None:
    if r != 0:
        raise RuntimeError(f"{what}: {_rt().cudaGetErrorString(r).decode()}")


def meta(module: str) -> dict:
    return json.loads((REF / f"{module}.json").read_text())


def _library(module: str) -> C.c_void_p:
    key = ("lib", module)
    if key not in _libs:
        data = (REF / f"{module}.cubin").read_bytes()
        buf = C.create_string_buffer(data, len(data))
        lib = C.c_void_p()
        _check(_rt().cudaLibraryLoadData(C.byref(lib), buf, None, None, 0, None, None, 0), "cudaLibraryLoadData")
        _libs[key] = lib
        _libs[("buf", module)] = buf
    return _libs[key]


def kernel(module: str, name: str) -> C.c_void_p:
    key = (module, name)
    if key in _libs:
        return _libs[key]
    k = C.c_void_p()
    _check(_rt().cudaLibraryGetKernel(C.byref(k), _library(module), meta(module)["kernels"][name].encode()),
           "cudaLibraryGetKernel")
    _libs[key] = k
    return k


def global_symbol(module: str, name: str) -> tuple[int, int]:
    """Device address and size in bytes of a __device__ variable of a module."""
    ptr, size = C.c_void_p(), C.c_size_t(0)
    _check(_rt().cudaLibraryGetGlobal(C.byref(ptr), C.byref(size), _library(module), meta(module)["kernels"][name].encode()),
           "cudaLibraryGetGlobal")
    return int(ptr.value), int(size.value)


class Dim3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def launch(k: C.c_void_p, grid: int, block: int, args: list, stream: int = 0) -> None:
    ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
    rt = _rt()
    rt.cudaLaunchKernel.argtypes = [C.c_void_p, Dim3, Dim3, C.c_void_p, C.c_size_t, C.c_void_p]
    _check(rt.cudaLaunchKernel(k, Dim3(grid, 1, 1), Dim3(block, 1, 1), ptrs, 0, C.c_void_p(stream)), "cudaLaunchKernel")
    _check(rt.cudaDeviceSynchronize(), "sync")
