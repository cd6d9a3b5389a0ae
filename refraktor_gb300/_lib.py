"""ctypes bindings of librfk.so (include/rfk.h).

The library is built in-tree by refraktor_gb300.build; loading fails loudly
when it is missing, there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "librfk.so"

c_size_p = C.POINTER(C.c_size_t)


class CompileOpts(C.Structure):
    _fields_ = [("precise_math", C.c_int), ("block", C.c_int), ("chains_per_thread", C.c_int), ("flush", C.c_int),
                ("blocks_per_sm", C.c_int), ("sort", C.c_int)]


class KernelInfo(C.Structure):
    _fields_ = [("grid", C.c_int), ("block", C.c_int), ("chains_per_thread", C.c_int), ("flush", C.c_int),
                ("sort", C.c_int), ("registers", C.c_int), ("num_xforms", C.c_int), ("has_final", C.c_int), ("chaos", C.c_int),
                ("size_reals", C.c_size_t), ("sample_floats", C.c_size_t), ("compile_ms", C.c_double),
                ("sfu_per_iter", C.c_double), ("fma_per_iter", C.c_double)]


class Bailout(C.Structure):
    _fields_ = [("iters", C.c_uint32), ("millis", C.c_uint32), ("quality", C.c_double), ("temporal_slicing", C.c_uint32)]


class BinResult(C.Structure):
    _fields_ = [("quality", C.c_double), ("elapsed_ms", C.c_double), ("total_passes", C.c_uint64),
                ("total_draws", C.c_uint64), ("total_bins", C.c_uint64), ("passes_per_thread", C.c_double),
                ("max_density", C.c_double), ("draw_count", C.c_uint64), ("status", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneReport(C.Structure):
    _fields_ = [("candidates", C.c_int), ("best_iters_per_s", C.c_double), ("worst_iters_per_s", C.c_double)]


class TonemapArgs(C.Structure):
    _fields_ = [("quality", C.c_double), ("gamma", C.c_double), ("brightness", C.c_double), ("vibrancy", C.c_double),
                ("max_density", C.c_double), ("highlight_power", C.c_double), ("precise", C.c_int)]


class DEArgs(C.Structure):
    _fields_ = [("max_radius", C.c_double), ("min_radius", C.c_double), ("curve", C.c_double)]


class BatchUnit(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("quality", C.c_double), ("segment", C.c_uint32),
                ("t", C.c_float), ("gamma", C.c_float), ("brightness", C.c_float), ("vibrancy", C.c_float),
                ("highlight_power", C.c_float)]


class BatchOpts(C.Structure):
    _fields_ = [("passes_per_item", C.c_uint32), ("warmup", C.c_uint32), ("seed", C.c_uint32), ("millis", C.c_uint32),
                ("de_max_radius", C.c_float), ("de_min_radius", C.c_float), ("de_curve", C.c_float),
                ("out_format", C.c_int), ("precise_tonemap", C.c_int), ("item_factor", C.c_uint32)]


class BatchInfo(C.Structure):
    _fields_ = [("units", C.c_size_t), ("items", C.c_uint64), ("hist_bytes", C.c_size_t), ("image_bytes", C.c_size_t),
                ("launches_per_run", C.c_int), ("graph", C.c_int)]


# name -> (restype, argtypes)
SIGNATURES = {
    "rfk_last_error": (C.c_char_p, []),
    "rfk_version": (C.c_int, []),
    "rfk_db_load": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    "rfk_db_destroy": (None, [C.c_void_p]),
    "rfk_db_variation_count": (C.c_int, [C.c_void_p]),
    "rfk_db_variation_name": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_size_t]),
    "rfk_db_hash": (C.c_uint64, [C.c_void_p]),
    "rfk_db_add_variations": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rfk_db_add_common": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "rfk_db_remove_variation": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rfk_db_remove_common": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rfk_db_is_variation": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rfk_db_is_parameter": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "rfk_db_is_common": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rfk_db_variation_source": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_size_t, c_size_p]),
    "rfk_flame_from_json": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "rfk_flame_from_flam3": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "rfk_flame_to_json": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t, c_size_p]),
    "rfk_flame_destroy": (None, [C.c_void_p]),
    "rfk_flame_size_reals": (C.c_size_t, [C.c_void_p]),
    "rfk_flame_pack_sample": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_size_t]),
    "rfk_flame_affine_indices": (C.c_int, [C.c_void_p, c_size_p, C.c_size_t, c_size_p]),
    "rfk_flame_tonemap_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "rfk_flame_structure_hash": (C.c_uint64, [C.c_void_p]),
    "rfk_compile": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CompileOpts), C.POINTER(C.c_void_p), C.c_char_p, C.c_size_t]),
    "rfk_kernel_destroy": (None, [C.c_void_p]),
    "rfk_kernel_get_info": (C.c_int, [C.c_void_p, C.POINTER(KernelInfo)]),
    "rfk_generate_source": (C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t, c_size_p]),
    "rfk_compile_check": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CompileOpts), C.c_char_p, C.c_char_p, C.c_size_t]),
    "rfk_kernel_source": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t, c_size_p]),
    "rfk_warmup": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                             C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "rfk_warmup_adopt": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t, C.c_void_p, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "rfk_state_destroy": (None, [C.c_void_p]),
    "rfk_state_rewarm": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_int, C.c_void_p]),
    "rfk_bin": (C.c_int, [C.c_void_p, C.POINTER(Bailout), C.c_void_p, C.POINTER(BinResult)]),
    "rfk_bin_async": (C.c_int, [C.c_void_p, C.POINTER(Bailout), C.c_void_p]),
    "rfk_bin_wait": (C.c_int, [C.c_void_p, C.POINTER(BinResult)]),
    "rfk_state_abort": (C.c_int, [C.c_void_p]),
    "rfk_state_bins": (C.c_void_p, [C.c_void_p]),
    "rfk_state_quality": (C.c_double, [C.c_void_p]),
    "rfk_state_chains": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, c_size_p]),
    "rfk_state_samples": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, c_size_p]),
    "rfk_apply_xform": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_uint32]),
    "rfk_prepare_samples": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32,
                                      C.c_void_p]),
    "rfk_prepare_samples_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t,
                                              C.c_uint32, C.c_void_p]),
    "rfk_tonemap": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_int, C.POINTER(TonemapArgs), C.c_void_p,
                              C.c_void_p, C.c_void_p]),
    "rfk_density_histogram": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rfk_density_blur": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(DEArgs), C.c_void_p]),
    "rfk_catmull_coefficients": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]),
    "rfk_fix_rotation": (C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t]),
    "rfk_probe_red_v4": (C.c_int, [C.c_size_t, C.c_uint32, C.POINTER(C.c_double)]),
    "rfk_probe_pipe": (C.c_int, [C.c_int, C.c_uint32, C.POINTER(C.c_double)]),
    "rfk_device_sm_count": (C.c_int, []),
    "rfk_autotune": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_uint32, C.c_uint32, C.c_uint32,
                               C.POINTER(CompileOpts), C.POINTER(TuneReport)]),
    "rfk_flames_align": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "rfk_batch_create": (C.c_int, [C.c_void_p, C.POINTER(BatchUnit), C.c_size_t, C.c_size_t, C.POINTER(BatchOpts),
                                   C.POINTER(C.c_void_p)]),
    "rfk_batch_destroy": (None, [C.c_void_p]),
    "rfk_batch_set_samples": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rfk_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "rfk_batch_wait": (C.c_int, [C.c_void_p, C.POINTER(BinResult), C.POINTER(BinResult)]),
    "rfk_batch_bins": (C.c_void_p, [C.c_void_p, C.c_size_t]),
    "rfk_batch_image": (C.c_void_p, [C.c_void_p, C.c_size_t]),
    "rfk_batch_params": (C.c_void_p, [C.c_void_p, C.c_size_t]),
    "rfk_batch_get_info": (C.c_int, [C.c_void_p, C.POINTER(BatchInfo)]),
    "rfk_convert": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int,
                              C.c_void_p]),
    "rfk_write_png": (C.c_int, [C.c_char_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int]),
    # rfk_denoise.h
    "rfk_denoiser_create": (C.c_int, [C.c_uint64, C.POINTER(C.c_void_p)]),
    "rfk_denoiser_make": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "rfk_denoiser_name": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t]),
    "rfk_denoiser_destroy": (None, [C.c_void_p]),
    "rfk_denoiser_param_count": (C.c_size_t, [C.c_void_p]),
    "rfk_denoiser_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "rfk_denoiser_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "rfk_denoiser_read_params": (C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "rfk_denoiser_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p,
                                        C.c_void_p]),
    "rfk_denoiser_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                          C.c_double, C.c_void_p, C.c_float, C.POINTER(C.c_double), C.c_void_p]),
    "rfk_denoiser_loss": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_double,
                                    C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "rfk_denoiser_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32,
                                         C.c_double, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "rfk_denoise": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p,
                              C.c_int, C.c_void_p]),
}


class RfkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rfk error {code}: {msg}")
        self.code = code


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise RuntimeError(f"librfk.so is not built ({_LIB_PATH}); run refraktor_gb300.build.build()")
        L = C.CDLL(str(_LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != 0:
        raise RfkError(code, lib().rfk_last_error().decode(errors="replace"))


def text_out(fn, *args, cap: int = 1 << 16) -> str:
    """Calls an entry point of the (..., char* buf, size_t cap, size_t* len) form."""
    n = C.c_size_t(0)
    check(fn(*args, None, 0, C.byref(n)))
    buf = C.create_string_buffer(n.value + 1)
    check(fn(*args, buf, n.value + 1, C.byref(n)))
    return buf.value.decode()
