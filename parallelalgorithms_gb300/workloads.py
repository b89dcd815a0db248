"""Seeded synthetic inputs (host numpy arrays) for tests and benchmarks.

The generators are native (pa_workloads.cpp in libpa_gb300.so) so that every
machine produces identical bytes.  The uniform 32-bit recipe is the
reference's own (ParallelAlgorithms.cpp:91, 112-115: std::mt19937_64(1234),
key = low 32 bits of each draw).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._native import lib

SEED_UNIFORM_U32 = 1234   # ParallelAlgorithms.cpp:91
SEED_UNIFORM_U64 = 1235
SEED_ZIPF_U64 = 1236
SEED_NORMAL_F32 = 1237
SEED_SEGMENT_SIZES = 1238
SEED_SERVING = 1239


def _l():
    h = lib()
    if not getattr(h, "_pa_gen_typed", False):
        h.pa_gen_uniform_u32.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
        h.pa_gen_uniform_u64.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_void_p]
        h.pa_gen_zipf_u64.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double, ctypes.c_uint32,
                                      ctypes.c_void_p]
        h.pa_gen_normal_specials_f32.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p]
        h.pa_gen_log_uniform_sizes.argtypes = [ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_void_p]
        for f in ("pa_gen_uniform_u32", "pa_gen_uniform_u64", "pa_gen_zipf_u64", "pa_gen_normal_specials_f32",
                  "pa_gen_log_uniform_sizes"):
            getattr(h, f).restype = None
        h._pa_gen_typed = True
    return h


def _empty(n: int, dtype, pinned: bool):
    if pinned:
        import torch
        t = torch.empty(n * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dtype), t
    return np.empty(n, dtype), None


def uniform_u32(n: int, seed: int = SEED_UNIFORM_U32, pinned: bool = False) -> np.ndarray:
    """Keys (uint32)mt19937_64(seed)() -- the reference's input recipe."""
    a, keep = _empty(n, np.uint32, pinned)
    _l().pa_gen_uniform_u32(seed, n, a.ctypes.data)
    return _hold(a, keep)


def uniform_u64(n: int, seed: int = SEED_UNIFORM_U64, pinned: bool = False) -> np.ndarray:
    a, keep = _empty(n, np.uint64, pinned)
    _l().pa_gen_uniform_u64(seed, n, a.ctypes.data)
    return _hold(a, keep)


def zipf_u64(n: int, s: float = 1.1, ranks: int = 1 << 20, seed: int = SEED_ZIPF_U64,
             pinned: bool = False) -> np.ndarray:
    """Zipf(s) ranks over `ranks` values, each mapped to splitmix64(rank)."""
    a, keep = _empty(n, np.uint64, pinned)
    _l().pa_gen_zipf_u64(seed, n, s, ranks, a.ctypes.data)
    return _hold(a, keep)


def normal_specials_f32(n: int, frac: float = 0.01, seed: int = SEED_NORMAL_F32, pinned: bool = False) -> np.ndarray:
    """N(0,1) float32 with `frac` each of +0.0, -0.0, +inf, -inf and denormals."""
    a, keep = _empty(n, np.float32, pinned)
    _l().pa_gen_normal_specials_f32(seed, n, frac, a.ctypes.data)
    return _hold(a, keep)


def presorted_u32(n: int) -> np.ndarray:
    """0, 1, ..., n-1."""
    return np.arange(n, dtype=np.uint32)


def constant_u32(n: int, value: int = 42) -> np.ndarray:
    return np.full(n, value, dtype=np.uint32)


def log_uniform_sizes(count: int, lo: float, hi: float, seed: int = SEED_SEGMENT_SIZES) -> np.ndarray:
    """count sizes round(exp(U(ln lo, ln hi)))."""
    a = np.empty(count, np.uint64)
    _l().pa_gen_log_uniform_sizes(seed, count, lo, hi, a.ctypes.data)
    return a


class _Pinned(np.ndarray):
    """numpy view that keeps its pinned torch storage alive."""


def _hold(a: np.ndarray, keep):
    if keep is None:
        return a
    v = a.view(_Pinned)
    v._pa_keep = keep
    return v
