"""Python mirror of librefrakt's hot-path interface over librfk.so.

Names, argument meaning and failure behaviour follow the reference C++ API:
  rfkt::flamedb / rfkt::initialize        src/librefrakt/include/librefrakt/flame_info.h:18-159
  rfkt::flame (+ import_flam3, JSON)      src/librefrakt/include/librefrakt/flame_types.h:552-807
  rfkt::flame_compiler::get_flame_kernel  src/librefrakt/include/librefrakt/flame_compiler.h:153-229
  rfkt::flame_kernel::warmup / bin        flame_compiler.h:22-149
  rfkt::tonemapper::run                   src/librefrakt/include/librefrakt/image/tonemapper.h:6-35
The reference reports failures as std::optional / empty results plus a log;
here they raise RfkError with the library's message. Device memory is torch
CUDA memory; the compute is librfk's CUDA kernels (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
import json as _json
from dataclasses import dataclass
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (Bailout, BatchInfo, BatchOpts, BatchUnit, BinResult, CompileOpts, DEArgs, KernelInfo, RfkError, TonemapArgs,
                   TuneReport, check, lib, text_out)

DEFAULT_CONFIG = Path(__file__).resolve().parent / "config"

HALF3, HALF4, FLOAT3, FLOAT4 = 0, 1, 2, 3
HISTOGRAM_BINS = 97


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)  # torch.cuda.Stream


def _dev_ptr(t) -> int:
    if isinstance(t, int):
        return t
    return int(t.data_ptr())


def _device_view(ptr: int, shape: tuple, typestr: str):
    """A torch CUDA tensor viewing library-owned device memory."""
    import torch

    class _View:
        __cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3,
                                    "strides": None}

    return torch.as_tensor(_View(), device="cuda")


class flamedb:
    """Variation database (flame_info.h:18-157)."""

    def __init__(self, config_dir: str | Path | None = None):
        self._h = C.c_void_p()
        check(lib().rfk_db_load(str(config_dir or DEFAULT_CONFIG).encode(), C.byref(self._h)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_db_destroy(self._h)
            self._h = None

    def variations(self) -> list[str]:
        out = []
        buf = C.create_string_buffer(256)
        for i in range(lib().rfk_db_variation_count(self._h)):
            check(lib().rfk_db_variation_name(self._h, i, buf, 256))
            out.append(buf.value.decode())
        return out

    def is_variation(self, name: str) -> bool:
        return lib().rfk_db_is_variation(self._h, name.encode()) == 1

    def is_parameter(self, vname: str, pname: str) -> bool:
        return lib().rfk_db_is_parameter(self._h, vname.encode(), pname.encode()) == 1

    def is_common(self, name: str) -> bool:
        return lib().rfk_db_is_common(self._h, name.encode()) == 1

    def add_or_update_variations(self, yaml_text: str) -> None:
        """flamedb::add_or_update_variation for every entry of a document in
        variations_new.yml format; raises RfkError on the first invalid one."""
        check(lib().rfk_db_add_variations(self._h, yaml_text.encode()))

    def add_or_update_common(self, name: str, code: str) -> None:
        check(lib().rfk_db_add_common(self._h, name.encode(), code.encode()))

    def remove_variation(self, name: str) -> bool:
        return lib().rfk_db_remove_variation(self._h, name.encode()) == 1

    def remove_common(self, name: str) -> bool:
        return lib().rfk_db_remove_common(self._h, name.encode()) == 1

    def hash(self) -> int:
        return lib().rfk_db_hash(self._h)

    def variation_source(self, name: str) -> str:
        return text_out(lib().rfk_db_variation_source, self._h, name.encode())


def initialize(fdb_or_path=None) -> flamedb:
    """rfkt::initialize(fdb, config_path): returns a loaded database."""
    return flamedb(fdb_or_path)


class flame:
    """Genome (flame_types.h:552-807); construct with from_json / import_flam3."""

    def __init__(self, handle: C.c_void_p, db: flamedb):
        self._h = handle
        self._db = db

    @classmethod
    def from_json(cls, db: flamedb, js: str | dict) -> "flame":
        text = js if isinstance(js, str) else _json.dumps(js)
        h = C.c_void_p()
        check(lib().rfk_flame_from_json(db._h, text.encode(), C.byref(h)))
        return cls(h, db)

    @classmethod
    def import_flam3(cls, db: flamedb, xml: str) -> "flame":
        h = C.c_void_p()
        check(lib().rfk_flame_from_flam3(db._h, xml.encode(), C.byref(h)))
        return cls(h, db)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_flame_destroy(self._h)
            self._h = None

    def serialize(self) -> dict:
        return _json.loads(text_out(lib().rfk_flame_to_json, self._h))

    def size_reals(self) -> int:
        return lib().rfk_flame_size_reals(self._h)

    def sample_size(self) -> int:
        return self.size_reals() + 256 * 3

    def pack_sample(self, w: int, h: int) -> np.ndarray:
        n = self.sample_size()
        out = np.zeros(n, dtype=np.float64)
        check(lib().rfk_flame_pack_sample(self._h, w, h, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out

    def pack_samples(self, count: int, w: int, h: int) -> np.ndarray:
        """pack_samples(packer, invoker, start, offset, count, w, h): a static genome repeats t0."""
        return np.tile(self.pack_sample(w, h), count)

    def affine_indices(self) -> list[int]:
        n = C.c_size_t(0)
        check(lib().rfk_flame_affine_indices(self._h, None, 0, C.byref(n)))
        arr = (C.c_size_t * n.value)()
        check(lib().rfk_flame_affine_indices(self._h, arr, n.value, C.byref(n)))
        return list(arr)

    def tonemap_params(self) -> dict:
        out = (C.c_double * 4)()
        check(lib().rfk_flame_tonemap_params(self._h, out))
        return {"gamma": out[0], "brightness": out[1], "vibrancy": out[2], "highlight_power": out[3]}

    def structure_hash(self) -> int:
        return lib().rfk_flame_structure_hash(self._h)


@dataclass
class bailout_args:
    """flame_compiler.h:92-96 (iters is a per-chain pass cap here), plus the
    temporal slicing of flame_kernel::bin (0 = 100 passes)."""
    iters: int = 0
    millis: int = 1000
    quality: float = 128.0
    temporal_slicing: int = 0


@dataclass
class bin_result:
    """flame_compiler.h:27-35 plus draw_count and the bailout status bits."""
    quality: float
    elapsed_ms: float
    total_passes: int
    total_draws: int
    total_bins: int
    passes_per_thread: float
    max_density: float
    draw_count: int
    status: int


def compile_check(db: flamedb, f: flame, arch: str = "sm_103a", **opts) -> str:
    """NVRTC-compiles the flame's kernels for `arch` without a device; returns the NVRTC log."""
    o = CompileOpts(**opts)
    log = C.create_string_buffer(1 << 16)
    check(lib().rfk_compile_check(db._h, f._h, C.byref(o), arch.encode(), log, len(log)))
    return log.value.decode()


def generate_source(db: flamedb, f: flame) -> str:
    return text_out(lib().rfk_generate_source, db._h, f._h)


class flame_kernel:
    """A compiled chaos-game module (flame_compiler.h:22-149)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        info = KernelInfo()
        check(lib().rfk_kernel_get_info(self._h, C.byref(info)))
        self.info = {k: getattr(info, k) for k, _ in KernelInfo._fields_}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_kernel_destroy(self._h)
            self._h = None

    def valid(self) -> bool:
        return bool(self._h)

    def source(self) -> str:
        return text_out(lib().rfk_kernel_source, self._h)

    def warmup(self, samples: np.ndarray, dims, seed: int, count: int, temporal_multiplier: int = 1,
               stream=None) -> "saved_state":
        """flame_kernel::warmup(stream, samples, dims | bins, seed, count,
        temporal_multiplier) (flame_compiler.h:99-100). `dims` is (w, h) for
        a new cleared histogram, or a float32 CUDA tensor (h, w, 4) that the
        state adopts as it is, without clearing (flame_compiler.cpp:1037);
        the state keeps a reference to the tensor."""
        s = np.ascontiguousarray(samples, dtype=np.float64)
        ss = self.info["size_reals"] + 768
        if s.size % ss != 0:
            raise RfkError(1, f"samples length {s.size} is not a multiple of the sample size {ss}")
        h = C.c_void_p()
        sp = s.ctypes.data_as(C.POINTER(C.c_double))
        if hasattr(dims, "data_ptr"):
            bins = dims
            if (bins.dim() != 3 or bins.shape[2] != 4 or not bins.is_contiguous() or str(bins.dtype) != "torch.float32"
                    or not bins.is_cuda):
                raise RfkError(1, "an adopted histogram is a contiguous (h, w, 4) float32 CUDA tensor")
            w, hh = int(bins.shape[1]), int(bins.shape[0])
            check(lib().rfk_warmup_adopt(self._h, sp, s.size // ss, C.c_void_p(bins.data_ptr()), w, hh, seed & 0xFFFFFFFF,
                                         count, temporal_multiplier, _stream_ptr(stream), C.byref(h)))
            st = saved_state(h, self, (w, hh))
            st._adopted = bins
            return st
        check(lib().rfk_warmup(self._h, sp, s.size // ss, int(dims[0]), int(dims[1]),
                               seed & 0xFFFFFFFF, count, temporal_multiplier, _stream_ptr(stream), C.byref(h)))
        return saved_state(h, self, (int(dims[0]), int(dims[1])))

    def bin(self, state: "saved_state", bo: bailout_args, stream=None) -> bin_result:
        """flame_kernel::bin(stream, state, bailout) (waits for the result)."""
        b = Bailout(bo.iters, bo.millis, bo.quality, bo.temporal_slicing)
        r = BinResult()
        check(lib().rfk_bin(state._h, C.byref(b), _stream_ptr(stream), C.byref(r)))
        return bin_result(**r.as_dict())

    def bin_async(self, state: "saved_state", bo: bailout_args, stream=None) -> None:
        b = Bailout(bo.iters, bo.millis, bo.quality, bo.temporal_slicing)
        check(lib().rfk_bin_async(state._h, C.byref(b), _stream_ptr(stream)))

    def apply_xform(self, params: np.ndarray, xform: int, points: np.ndarray, seed: int = 0) -> np.ndarray:
        """Single map application: points (n, 3) -> (n, 4) = (x, y, colour, opacity)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        pts = np.ascontiguousarray(points, dtype=np.float32)
        out = np.zeros((pts.shape[0], 4), dtype=np.float32)
        check(lib().rfk_apply_xform(self._h, p.ctypes.data, xform, pts.ctypes.data, pts.shape[0], out.ctypes.data, seed))
        return out

    def prepare_samples(self, samples: np.ndarray, seg: Sequence[int], t: Sequence[float], seed: int = 0) -> np.ndarray:
        s = np.ascontiguousarray(samples, dtype=np.float64)
        ss = self.info["size_reals"] + 768
        sg = np.ascontiguousarray(seg, dtype=np.uint32)
        tt = np.ascontiguousarray(t, dtype=np.float32)
        out = np.zeros((sg.size, self.info["sample_floats"]), dtype=np.float32)
        check(lib().rfk_prepare_samples(self._h, s.ctypes.data, s.size // ss, sg.ctypes.data, tt.ctypes.data, sg.size,
                                        seed, out.ctypes.data))
        return out


class saved_state:
    """flame_kernel::saved_state (flame_compiler.h:37-90)."""

    def __init__(self, handle: C.c_void_p, kernel: flame_kernel, dims: tuple[int, int]):
        self._h = handle
        self.kernel = kernel
        self.dims = dims

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_state_destroy(self._h)
            self._h = None

    @property
    def quality(self) -> float:
        return lib().rfk_state_quality(self._h)

    def abort_binning(self) -> None:
        check(lib().rfk_state_abort(self._h))

    def rewarm(self, samples: np.ndarray, seed: int, count: int, clear: bool = True, stream=None) -> None:
        """warmup into this state's buffers (rfk_state_rewarm): new samples,
        same kernel and size, fresh chains and counters, histogram cleared
        unless `clear` is False; allocates nothing."""
        s = np.ascontiguousarray(samples, dtype=np.float64)
        ss = self.kernel.info["size_reals"] + 768
        check(lib().rfk_state_rewarm(self._h, s.ctypes.data, s.size // ss, seed & 0xFFFFFFFF, count, 1 if clear else 0,
                                     _stream_ptr(stream)))

    def bins_ptr(self) -> int:
        return lib().rfk_state_bins(self._h)

    def bins(self):
        """The float4 histogram as a torch CUDA tensor (h, w, 4) viewing state memory."""
        w, h = self.dims
        return _device_view(self.bins_ptr(), (h, w, 4), "<f4")

    def wait(self) -> bin_result:
        r = BinResult()
        check(lib().rfk_bin_wait(self._h, C.byref(r)))
        return bin_result(**r.as_dict())

    def chains(self) -> np.ndarray:
        n = C.c_size_t(0)
        check(lib().rfk_state_chains(self._h, None, None, None, 0, C.byref(n)))
        out = np.zeros((3, n.value), dtype=np.float32)
        check(lib().rfk_state_chains(self._h, out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data, n.value, C.byref(n)))
        return out

    def samples(self) -> np.ndarray:
        n = C.c_size_t(0)
        check(lib().rfk_state_samples(self._h, None, 0, C.byref(n)))
        out = np.zeros(n.value, dtype=np.float32)
        check(lib().rfk_state_samples(self._h, out.ctypes.data, n.value, C.byref(n)))
        return out.reshape(-1, self.kernel.info["sample_floats"])


class flame_compiler:
    """flame_compiler::get_flame_kernel (flame_compiler.h:153-229). Kernels are
    cached per (database, structure, options) inside the library."""

    def __init__(self, **default_opts):
        self.default_opts = default_opts

    def get_flame_kernel(self, db: flamedb, f: flame, **opts) -> flame_kernel:
        o = CompileOpts(**{**self.default_opts, **opts})
        h = C.c_void_p()
        log = C.create_string_buffer(1 << 16)
        check(lib().rfk_compile(db._h, f._h, C.byref(o), C.byref(h), log, len(log)))
        k = flame_kernel(h)
        k.log = log.value.decode()
        return k


def autotune(db: flamedb, f: flame, samples: np.ndarray, dims: Sequence[int], passes: int = 256) -> tuple[dict, dict]:
    """Times launch shapes and flush strategies on this flame; returns
    (compile options, report)."""
    s = np.ascontiguousarray(samples, dtype=np.float64)
    o = CompileOpts()
    rep = TuneReport()
    check(lib().rfk_autotune(db._h, f._h, s.ctypes.data, s.size // f.sample_size(), int(dims[0]), int(dims[1]), passes,
                             C.byref(o), C.byref(rep)))
    opts = {k: getattr(o, k) for k, _ in CompileOpts._fields_}
    return opts, {k: getattr(rep, k) for k, _ in TuneReport._fields_}


class tonemapper:
    """tonemapper::run (image/tonemapper.h:6-35)."""

    def run(self, bins, out, dims: Sequence[int], quality: float, gamma: float, brightness: float, vibrancy: float,
            max_density: float = 0.0, highlight_power: float = -1.0, fmt: int = FLOAT4, precise: bool = True,
            histogram=None, max_density_out=None, stream=None) -> None:
        a = TonemapArgs(quality, gamma, brightness, vibrancy, max_density, highlight_power, 1 if precise else 0)
        check(lib().rfk_tonemap(_dev_ptr(bins), int(dims[0]), int(dims[1]), _dev_ptr(out), fmt, C.byref(a),
                                None if histogram is None else _dev_ptr(histogram),
                                None if max_density_out is None else _dev_ptr(max_density_out), _stream_ptr(stream)))


def density_histogram(bins, count: int, histogram, max_density, stream=None) -> None:
    check(lib().rfk_density_histogram(_dev_ptr(bins), count, _dev_ptr(histogram), _dev_ptr(max_density), _stream_ptr(stream)))


def density_blur(bins_in, bins_out, dims: Sequence[int], max_radius: float = 9.0, min_radius: float = 0.0,
                 curve: float = 0.5, stream=None) -> None:
    a = DEArgs(max_radius, min_radius, curve)
    check(lib().rfk_density_blur(_dev_ptr(bins_in), _dev_ptr(bins_out), int(dims[0]), int(dims[1]), C.byref(a),
                                 _stream_ptr(stream)))


def catmull_coefficients(samples_dev, sample_size: int, nseg: int, coeff_dev, stream=None) -> None:
    check(lib().rfk_catmull_coefficients(_dev_ptr(samples_dev), sample_size, nseg, _dev_ptr(coeff_dev), _stream_ptr(stream)))


def fix_rotation(samples: np.ndarray, sample_size: int, flame_size: int, affine_indices: Sequence[int]) -> np.ndarray:
    s = np.ascontiguousarray(samples, dtype=np.float64).copy()
    idx = (C.c_size_t * len(affine_indices))(*affine_indices)
    check(lib().rfk_fix_rotation(s.ctypes.data, s.size // sample_size, sample_size, flame_size, idx, len(affine_indices)))
    return s


def probe_red_v4(nbytes: int, iters: int = 256) -> float:
    out = C.c_double(0)
    check(lib().rfk_probe_red_v4(nbytes, iters, C.byref(out)))
    return out.value


def probe_pipe(pipe: int, iters: int = 4096) -> float:
    """Lane operations per second of one arithmetic pipe (0 = FP32 FMA, 1 = SFU)."""
    out = C.c_double(0)
    check(lib().rfk_probe_pipe(pipe, iters, C.byref(out)))
    return out.value


def sm_count() -> int:
    return lib().rfk_device_sm_count()


def align_flames(db: flamedb, flames: Sequence[flame], by_weight: bool = False) -> list[flame]:
    """Gives the genomes one structure without changing what each renders (the
    reference interpolator's alignment, src/refraktor/src/refraktor.cpp:117-191,
    for any number of genomes); returns new flames."""
    n = len(flames)
    ins = (C.c_void_p * n)(*[f._h for f in flames])
    outs = (C.c_void_p * n)()
    check(lib().rfk_flames_align(db._h, ins, n, 1 if by_weight else 0, outs))
    return [flame(C.c_void_p(outs[i]), db) for i in range(n)]


@dataclass
class batch_unit:
    """One flame or frame of a batch: image size, spp target, spline position
    (segment, t) in the batch's samples, tonemap parameters."""
    width: int
    height: int
    quality: float
    segment: int = 0
    t: float = 0.0
    gamma: float = 4.0
    brightness: float = 1.0
    vibrancy: float = 1.0
    highlight_power: float = -1.0


_PIXEL = {HALF3: (3, "<f2"), HALF4: (4, "<f2"), FLOAT3: (3, "<f4"), FLOAT4: (4, "<f4")}


class batch:
    """Many units of one flame structure in one persistent launch, then blur and
    tonemap per unit, optionally replayed as one CUDA graph. No reference
    counterpart (the reference renders one flame per flame_kernel::bin)."""

    def __init__(self, kernel: flame_kernel, units: Sequence[batch_unit], nsamples: int, *, passes_per_item: int = 256,
                 warmup: int = 20, seed: int = 1, millis: int = 0, de: Optional[Sequence[float]] = None,
                 out_format: int = HALF4, precise_tonemap: bool = True, item_factor: int = 3):
        self.kernel = kernel
        self.units = list(units)
        arr = (BatchUnit * len(self.units))()
        for i, u in enumerate(self.units):
            arr[i] = BatchUnit(u.width, u.height, u.quality, u.segment, u.t, u.gamma, u.brightness, u.vibrancy,
                               u.highlight_power)
        de = tuple(de) if de else (0.0, 0.0, 0.0)
        o = BatchOpts(passes_per_item, warmup, seed, millis, de[0], de[1], de[2], out_format, 1 if precise_tonemap else 0,
                      item_factor)
        self.out_format = out_format
        self.nsamples = int(nsamples)
        h = C.c_void_p()
        check(lib().rfk_batch_create(kernel._h, arr, len(self.units), nsamples, C.byref(o), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().rfk_batch_destroy(self._h)
            self._h = None

    def set_samples(self, samples: np.ndarray) -> None:
        """nsamples packed samples (any shape holding nsamples x (size_reals + 768) doubles)."""
        s = np.ascontiguousarray(samples, dtype=np.float64)
        need = self.nsamples * (self.kernel.info["size_reals"] + 768)
        if s.size != need:
            raise RfkError(1, f"samples hold {s.size} values; the batch was created for {need}")
        check(lib().rfk_batch_set_samples(self._h, s.ctypes.data))

    def run(self, use_graph: bool = False, stream=None) -> None:
        check(lib().rfk_batch_run(self._h, 1 if use_graph else 0, _stream_ptr(stream)))

    def wait(self) -> tuple[bin_result, list[bin_result]]:
        tot = BinResult()
        per = (BinResult * len(self.units))()
        check(lib().rfk_batch_wait(self._h, C.byref(tot), per))
        return bin_result(**tot.as_dict()), [bin_result(**per[i].as_dict()) for i in range(len(self.units))]

    def bins(self, u: int):
        U = self.units[u]
        return _device_view(lib().rfk_batch_bins(self._h, u), (U.height, U.width, 4), "<f4")

    def image(self, u: int):
        if self.out_format < 0:
            raise RfkError(1, "batch has no tonemapped images (out_format < 0)")
        U = self.units[u]
        ch, ts = _PIXEL[self.out_format]
        return _device_view(lib().rfk_batch_image(self._h, u), (U.height, U.width, ch), ts)

    def params(self, u: int):
        return _device_view(lib().rfk_batch_params(self._h, u), (self.kernel.info["sample_floats"],), "<f4")

    def info(self) -> dict:
        i = BatchInfo()
        check(lib().rfk_batch_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in BatchInfo._fields_}


UCHAR3, UCHAR4 = 4, 5


class converter:
    """convert_to<In, Out> (assets/kernels/convert.cu:70-99): a half3 / half4
    image to float3 / float4 / uchar3 / uchar4, optionally flipped bottom-up
    and with R and B swapped."""

    def run(self, img, out, dims: Sequence[int], in_fmt: int, out_fmt: int, flip_y: bool = False,
            swap_channels: bool = False, stream=None) -> None:
        check(lib().rfk_convert(_dev_ptr(img), in_fmt, _dev_ptr(out), out_fmt, int(dims[0]), int(dims[1]),
                                1 if flip_y else 0, 1 if swap_channels else 0, _stream_ptr(stream)))


def write_png(path: str | Path, pixels: np.ndarray) -> None:
    """8-bit (h, w, 3 | 4) host pixels to a PNG file."""
    p = np.ascontiguousarray(pixels, dtype=np.uint8)
    h, w, c = p.shape
    check(lib().rfk_write_png(str(path).encode(), p.ctypes.data, w, h, c))
