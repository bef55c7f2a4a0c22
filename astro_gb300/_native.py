"""ctypes binding of libastro_cuda.so (include/astro_cuda.h).

The library is built in-tree by astro_gb300.build. Loading fails loudly when
it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_size_t, c_uint32, c_uint64, c_void_p
from pathlib import Path

from .layouts import Params

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libastro_cuda.so"

STATUS = {
    0: "ASTRO_OK",
    -1: "ASTRO_ERR_INVALID_ARGUMENT",
    -2: "ASTRO_ERR_CAPACITY",
    -3: "ASTRO_ERR_CUDA",
    -4: "ASTRO_ERR_OUT_OF_MEMORY",
    -5: "ASTRO_ERR_STATE",
    -6: "ASTRO_ERR_DEVICE_TIMEOUT",
    -7: "ASTRO_ERR_NOT_SUPPORTED",
    -8: "ASTRO_ERR_DEVICE_OVERFLOW",
}


class AstroError(RuntimeError):
    """A libastro_cuda call returned a negative status."""

    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


# Every exported symbol with (restype, argtypes); also the list the ABI
# tests check against include/astro_cuda.h.
SIGNATURES = {
    "astro_params_default": (c_int, [c_uint32, POINTER(Params)]),
    "astro_create": (c_int, [POINTER(Params), c_uint32, c_uint32, POINTER(c_void_p)]),
    "astro_destroy": (c_int, [c_void_p]),
    "astro_set_params": (c_int, [c_void_p, POINTER(Params)]),
    "astro_get_params": (c_int, [c_void_p, POINTER(Params)]),
    "astro_upload": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_uint32]),
    "astro_upload_systems": (c_int, [c_void_p, c_void_p, c_void_p, POINTER(c_uint32), c_uint32]),
    "astro_download": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "astro_encode": (c_int, [c_void_p]),
    "astro_sort": (c_int, [c_void_p]),
    "astro_build": (c_int, [c_void_p]),
    "astro_traverse": (c_int, [c_void_p]),
    "astro_integrate": (c_int, [c_void_p, c_float]),
    "astro_step": (c_int, [c_void_p, c_float, c_uint32]),
    "astro_synchronize": (c_int, [c_void_p]),
    "astro_read_keys": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32]),
    "astro_read_tree_info": (c_int, [c_void_p, POINTER(c_uint32), c_void_p, c_void_p, c_void_p,
                                     c_uint32]),
    "astro_read_nodes": (c_int, [c_void_p, c_void_p, c_uint64, c_uint64]),
    "astro_read_accel": (c_int, [c_void_p, c_void_p, c_uint32]),
    "astro_read_stats": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64),
                                 POINTER(c_uint64)]),
    "astro_read_far_stats": (c_int, [c_void_p, POINTER(c_uint64), POINTER(c_uint64)]),
    "astro_read_traverse_times": (c_int, [c_void_p, POINTER(c_float), POINTER(c_float)]),
    "astro_step_batched": (c_int, [c_void_p, c_void_p, c_uint32, c_float, c_uint32]),
    "astro_autotune": (c_int, [c_void_p, c_char_p]),
    "astro_autotune_ex": (c_int, [c_void_p, c_char_p, c_float, c_uint32]),
    "astro_autotune_keep": (c_int, [c_void_p, c_char_p, c_float, c_uint32, c_uint32]),
    "astro_direct_accel_f64": (c_int, [c_void_p, c_void_p, c_uint32, c_void_p]),
    "astro_lighting": (c_int, [c_void_p, c_uint32]),
    "astro_splat": (c_int, [c_void_p, c_void_p, c_uint32, c_uint32, c_void_p, c_void_p, c_void_p]),
    "astro_read_colors": (c_int, [c_void_p, c_void_p, c_uint32]),
    "astro_save_state": (c_int, [c_void_p, c_char_p, c_uint64, c_double]),
    "astro_load_state": (c_int, [c_char_p, c_uint32, POINTER(c_void_p), POINTER(c_uint64),
                                 POINTER(c_double)]),
    "astro_get_stream": (c_int, [c_void_p, POINTER(c_void_p)]),
    "astro_last_error": (c_char_p, [c_void_p]),
    "astro_version": (c_char_p, []),
    "astro_status_string": (c_char_p, [c_int]),
    "astro_radix_sort_temp_bytes": (c_int, [c_uint32, c_uint32, POINTER(c_size_t)]),
    "astro_radix_sort": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32, c_void_p,
                                 c_uint32, c_void_p, c_size_t, c_void_p]),
    "astro_radix_sort_status": (c_int, [c_void_p, c_void_p]),
    "astro_radix_sort_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_uint32,
                                         c_void_p, c_uint32, c_void_p]),
    "astro_radix_sort_noalloc_status": (c_int, [c_void_p]),
    "astro_test_sort_lookback_timeout": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32,
                                                 c_uint32, c_uint32, c_void_p, c_size_t,
                                                 c_void_p]),
    "astro_upload_async": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "astro_download_async": (c_int, [c_void_p, c_void_p, c_void_p, c_uint32]),
    "astro_test_walk_capacity": (c_int, [c_void_p, c_uint64, c_uint32]),
    "astro_read_walk_buffers": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "astro_generate_ic": (c_int, [c_uint32, c_uint64, c_uint32, c_uint32, c_double, c_double,
                                  c_void_p, c_void_p, c_void_p]),
    "astro_generate_system_sizes": (c_int, [c_uint64, c_uint32, c_uint32, c_uint32, c_double,
                                            c_double, c_void_p, c_void_p]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load libastro_cuda.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m astro_gb300.build` "
                "(there is no CPU fallback)")
        l = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(status: int, ctx=None) -> None:
    if status != 0:
        msg = ""
        if ctx:
            raw = lib().astro_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise AstroError(status, msg)


def ptr(a) -> c_void_p:
    """Address of a numpy array or a torch tensor (None passes NULL)."""
    if a is None:
        return c_void_p(0)
    if hasattr(a, "data_ptr"):
        return c_void_p(a.data_ptr())
    return c_void_p(a.ctypes.data)
