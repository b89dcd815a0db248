"""ctypes binding of libpa_gb300.so (the C ABI declared in include/pa_gpu.h).

The library is loaded from this package directory.  There is no fallback:
if it is missing or cannot be loaded, `lib()` raises, and so does every
operation that needs it.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpa_gb300.so"

PA_OK, PA_ERR_ARG, PA_ERR_OOM, PA_ERR_CUDA, PA_ERR_TIMEOUT, PA_ERR_NO_DEVICE = range(6)


class PaOpts(ctypes.Structure):
    _fields_ = [("stream", ctypes.c_void_p), ("async_device", ctypes.c_int), ("digit_bits", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


class SegSortConfig(ctypes.Structure):
    _fields_ = [("small_cutoff", ctypes.c_int), ("tile_keys", ctypes.c_int), ("digit_bits", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("reserved", ctypes.c_int * 4)]


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_U = ctypes.c_uint
_O = ctypes.POINTER(PaOpts)

# name -> argtypes; every entry point returns int (pa_status)
SIGNATURES: dict[str, list] = {
    "pa_sort_u32": [_P, _P, _SZ, _O],
    "pa_sort_u32_inplace": [_P, _SZ, _SZ, _O],
    "pa_sort_u64": [_P, _P, _SZ, _O],
    "pa_sort_f32": [_P, _P, _SZ, _O],
    "pa_sort_kv_u32": [_P, _P, _P, _P, _SZ, _O],
    "pa_sort_kv_u64": [_P, _P, _P, _P, _SZ, _O],
    "pa_sort_kv_f32": [_P, _P, _P, _P, _SZ, _O],
    "pa_sort_two_phase_u32": [_P, _P, _SZ, _O],
    "pa_sort_timed": [ctypes.c_int, _P, _P, _P, _P, _SZ, _P, ctypes.c_int, _O],
    "pa_sort_u32_noalloc": [_P, _P, _SZ, _O],
    "pa_hist_byte_components_u32": [_P, _SZ, _P, _O],
    "pa_hist_one_byte_u32": [_P, _SZ, _U, _P, _O],
    "pa_hist_u8": [_P, _SZ, _P, _O],
    "pa_counting_sort_u8": [_P, _SZ, _O],
    "pa_partition_radix_u32": [_P, _SZ, _P, _SZ, _O],
    "pa_sort_copy_u32": [_P, _P, _SZ, _O],
    "pa_hist_quanta_u32": [_P, _SZ, _SZ, _SZ, _SZ, _U, _P, _O],
    "pa_start_of_bins_u32": [_P, _SZ, _SZ, _SZ, _U, _P, _O],
    "pa_select_u32": [_P, _SZ, _SZ, _P, _O],
    "pa_select_u64": [_P, _SZ, _SZ, _P, _O],
    "pa_select_radix_u32": [_P, _SZ, _SZ, _SZ, _P, _O],
    "pa_sum_u32": [_P, _SZ, _P, _O],
    "pa_sum_u64": [_P, _SZ, _P, _O],
    "pa_sum_typed": [_P, _SZ, ctypes.c_int, _P, _O],
    "pa_sum_chunked": [_P, _SZ, ctypes.c_int, _SZ, _P, _P, _O],
    "pa_segsort_plan_create": [_P, _SZ, ctypes.POINTER(SegSortConfig), ctypes.POINTER(ctypes.c_void_p)],
    "pa_segsort_plan_run": [_P, _P, _P, _O],
    "pa_segsort_plan_sync": [_P, _P],
    "pa_segsort_plan_info": [_P, _P, _P, _P],
    "pa_segsort_plan_destroy": [_P],
    "pa_segmented_sort_u32": [_P, _P, _SZ, ctypes.POINTER(SegSortConfig), _O],
    "pa_server_create": [_P, ctypes.POINTER(ctypes.c_void_p)],
    "pa_server_submit": [_P, _P],
    "pa_server_wait": [_P, _P],
    "pa_server_drain": [_P],
    "pa_server_stats": [_P, _P, ctypes.c_int],
    "pa_server_destroy": [_P],
    "pa_hist_one_byte_u64": [_P, _SZ, _U, _P, _O],
    "pa_selftest_wait_expiry": [_U],
    "pa_stream_check": [_P],
    "pa_device_available": [],
    "pa_release_workspaces": [],
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class PaError(RuntimeError):
    """A pa_* call returned a status other than PA_OK."""

    def __init__(self, name: str, status: int, detail: str):
        self.status = status
        super().__init__(f"{name} failed with {status_name(status)}: {detail}")


def lib() -> ctypes.CDLL:
    """Loads libpa_gb300.so once; raises if it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                    "(there is no CPU fallback)")
            h = ctypes.CDLL(str(LIB_PATH))
            for name, args in SIGNATURES.items():
                fn = getattr(h, name)
                fn.argtypes = args
                fn.restype = ctypes.c_int
            h.pa_status_string.argtypes = [ctypes.c_int]
            h.pa_status_string.restype = ctypes.c_char_p
            h.pa_last_error_message.argtypes = []
            h.pa_last_error_message.restype = ctypes.c_char_p
            _lib = h
    return _lib


def status_name(status: int) -> str:
    return lib().pa_status_string(status).decode()


def call(name: str, *args) -> None:
    """Calls a pa_* entry point and raises PaError on failure."""
    rc = getattr(lib(), name)(*args)
    if rc != PA_OK:
        raise PaError(name, rc, lib().pa_last_error_message().decode())


def opts(stream: int | None = None, async_device: bool = False, digit_bits: int = 0) -> ctypes.POINTER(PaOpts) | None:
    if stream is None and not async_device and not digit_bits:
        return None
    o = PaOpts()
    o.stream = stream or None
    o.async_device = 1 if async_device else 0
    o.digit_bits = digit_bits
    return ctypes.pointer(o)
