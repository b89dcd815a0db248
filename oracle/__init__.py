"""CPU checkers for the GB300 radix hot path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
arm may import this package, and only to check results or as the timed CPU
baseline.  The product path (parallelalgorithms_gb300) never imports it.

Two checkers:
  * `port`: the project's plain-C restatement of the reference algorithm
    (oracle/pa_oracle.c, every function citing the reference file:line it
    restates), built into oracle/libpa_oracle.so;
  * `ref`: the reference's own CPU code compiled unchanged
    (oracle/_ref/libpa_ref.so, see oracle/build.py), present where the
    reference sources were available to build it.
The restatement is pinned against the compiled reference and against the
golden fixtures in tests/golden/ (produced by the compiled reference).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

_P = ctypes.c_void_p
_SZ = ctypes.c_size_t


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


class _Port:
    def __init__(self, path: Path):
        h = ctypes.CDLL(str(path))
        h.pa_oracle_lsd_sort.argtypes = [_P, _P, _P, _P, _SZ, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        h.pa_oracle_lsd_sort.restype = ctypes.c_int
        h.pa_oracle_hist_byte_components_u32.argtypes = [_P, _SZ, _SZ, _P]
        h.pa_oracle_hist_one_byte_u32.argtypes = [_P, _SZ, _SZ, ctypes.c_uint, _P]
        h.pa_oracle_hist_u8.argtypes = [_P, _SZ, _SZ, _P]
        h.pa_oracle_hist_digits.argtypes = [_P, _SZ, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
        h.pa_oracle_hist_qc_u32.argtypes = [_P, _SZ, _SZ, _SZ, _SZ, ctypes.c_uint, _P]
        h.pa_oracle_start_of_bins_u32.argtypes = [_P, _SZ, _SZ, _SZ, ctypes.c_uint, _P]
        h.pa_oracle_select_u32.argtypes = [_P, _SZ, _SZ, _SZ]
        h.pa_oracle_select_u32.restype = ctypes.c_uint32
        h.pa_oracle_select_u64.argtypes = [_P, _SZ, _SZ, _SZ]
        h.pa_oracle_select_u64.restype = ctypes.c_uint64
        h.pa_oracle_sum_u32.argtypes = [_P, _SZ, _SZ]
        h.pa_oracle_sum_u32.restype = ctypes.c_uint64
        h.pa_oracle_sum_u64.argtypes = [_P, _SZ, _SZ]
        h.pa_oracle_sum_u64.restype = ctypes.c_uint64
        h.pa_oracle_counting_sort_u8.argtypes = [_P, _SZ, _SZ]
        h.pa_oracle_partition_radix_u32.argtypes = [_P, _SZ, _P, _SZ]
        h.pa_oracle_gen_uniform_u32.argtypes = [ctypes.c_uint64, _SZ, _P]
        h.pa_oracle_gen_uniform_u32.restype = None
        self.h = h

    def gen_uniform_u32(self, n: int, seed: int = 1234) -> np.ndarray:
        """The reference benchmark's keys: (uint32)std::mt19937_64(seed)()."""
        a = np.empty(n, np.uint32)
        self.h.pa_oracle_gen_uniform_u32(seed, n, _p(a))
        return a

    def sort(self, keys: np.ndarray, vals: np.ndarray | None = None, digit_bits: int = 8):
        """Returns sorted copies (keys, vals) -- SortRadixPar widened to
        uint64 / float32 keys and a uint32 payload."""
        k = np.ascontiguousarray(keys).copy()
        is_float = k.dtype == np.float32
        kb = k.dtype.itemsize
        tmp = np.empty_like(k)
        v = tv = None
        if vals is not None:
            v = np.ascontiguousarray(vals, dtype=np.uint32).copy()
            tv = np.empty_like(v)
        rc = self.h.pa_oracle_lsd_sort(_p(k), _p(tmp), _p(v) if v is not None else None,
                                       _p(tv) if tv is not None else None, k.size, kb, digit_bits, int(is_float))
        if rc:
            raise RuntimeError(f"oracle sort failed ({rc})")
        return k, v

    def hist_byte_components(self, a: np.ndarray, l: int, r: int) -> np.ndarray:
        out = np.zeros((8, 256), np.uint64)
        self.h.pa_oracle_hist_byte_components_u32(_p(a), l, r, _p(out))
        return out

    def hist_one_byte(self, a: np.ndarray, l: int, r: int, shift: int) -> np.ndarray:
        out = np.zeros(256, np.uint64)
        self.h.pa_oracle_hist_one_byte_u32(_p(a), l, r, shift, _p(out))
        return out

    def hist_u8(self, a: np.ndarray, l: int, r: int) -> np.ndarray:
        out = np.zeros(256, np.uint64)
        self.h.pa_oracle_hist_u8(_p(a), l, r, _p(out))
        return out

    def hist_digits(self, a: np.ndarray, digit_bits: int = 8) -> np.ndarray:
        kb = a.dtype.itemsize
        passes = (8 * kb + digit_bits - 1) // digit_bits
        out = np.zeros((passes, 1 << digit_bits), np.uint64)
        self.h.pa_oracle_hist_digits(_p(a), a.size, kb, digit_bits, int(a.dtype == np.float32), _p(out))
        return out

    def hist_qc(self, a, l, r, work_quanta, quanta, which_byte) -> np.ndarray:
        out = np.zeros((quanta, 256), np.uint64)
        self.h.pa_oracle_hist_qc_u32(_p(a), l, r, work_quanta, quanta, which_byte, _p(out))
        return out

    def start_of_bins(self, a, n, work_quanta, quanta, digit) -> np.ndarray:
        out = np.zeros((quanta, 256), np.uint64)
        self.h.pa_oracle_start_of_bins_u32(_p(a), n, work_quanta, quanta, digit, _p(out))
        return out

    def select(self, a: np.ndarray, k: int, start: int = 0, length: int | None = None) -> int:
        """k-th smallest (k absolute) of a[start, start+length), on a copy
        (the restated algorithm is destructive, like the reference)."""
        c = np.ascontiguousarray(a).copy()
        length = c.size - start if length is None else length
        if c.dtype == np.uint64:
            return int(self.h.pa_oracle_select_u64(_p(c), start, length, k))
        return int(self.h.pa_oracle_select_u32(_p(c), start, length, k))

    def sum(self, a: np.ndarray, l: int = 0, r: int | None = None) -> int:
        r = a.size if r is None else r
        if a.dtype == np.uint64:
            return int(self.h.pa_oracle_sum_u64(_p(a), l, r))
        return int(self.h.pa_oracle_sum_u32(_p(a), l, r))

    def counting_sort_u8(self, a: np.ndarray, l: int = 0, r: int | None = None) -> np.ndarray:
        """Sorted copy of a byte array (counting sort of a[l, r))."""
        c = np.ascontiguousarray(a).copy()
        self.h.pa_oracle_counting_sort_u8(_p(c), l, c.size if r is None else r)
        return c

    def partition_radix(self, a: np.ndarray, ks) -> np.ndarray:
        """PartitionRadix(a, n, k[], kLength) on a copy; ks ascending."""
        c = np.ascontiguousarray(a, dtype=np.uint32).copy()
        k = np.ascontiguousarray(ks, dtype=np.uint64)
        self.h.pa_oracle_partition_radix_u32(_p(c), c.size, _p(k), k.size)
        return c


class _Ref:
    """The reference's own code (compiled unchanged) behind extern "C"."""

    def __init__(self, path: Path):
        h = ctypes.CDLL(str(path))
        h.pa_ref_hardware_concurrency.restype = ctypes.c_int
        for f in ("pa_ref_sort_radix_par_u32", "pa_ref_sort_two_phase_par_u32", "pa_ref_sort_two_phase_serial_u32"):
            getattr(h, f).argtypes = [_P, _P, _SZ]
        h.pa_ref_sort_radix_par_alloc_u32.argtypes = [_P, _SZ]
        h.pa_ref_hist_byte_components_par_u32.argtypes = [_P, _SZ, _SZ, _P]
        h.pa_ref_hist_one_byte_par_u32.argtypes = [_P, _SZ, _SZ, ctypes.c_ulong, _P]
        h.pa_ref_hist_u8_par.argtypes = [_P, _SZ, _SZ, _P]
        h.pa_ref_hist_qc_par_u32.argtypes = [_P, _SZ, _SZ, _SZ, _SZ, ctypes.c_uint, _P]
        h.pa_ref_compute_start_of_bins_par_u32.argtypes = [_P, _SZ, _SZ, _SZ, ctypes.c_uint, _P]
        h.pa_ref_select_radix_u32.argtypes = [_P, _SZ, _SZ]
        h.pa_ref_select_radix_u32.restype = ctypes.c_uint
        h.pa_ref_select_radix_range_u32.argtypes = [_P, _SZ, _SZ, _SZ]
        h.pa_ref_select_radix_range_u32.restype = ctypes.c_uint
        for f in ("pa_ref_sum_par_nonrec_u32", "pa_ref_sum_par_nonrec_u64", "pa_ref_sum_par_u64"):
            getattr(h, f).argtypes = [_P, _SZ, _SZ]
            getattr(h, f).restype = ctypes.c_ulonglong
        for f in ("pa_ref_sum_par_template_u32", "pa_ref_sum_par_template_u8", "pa_ref_sum_par_template_i32",
                  "pa_ref_sum_par_template_f32"):
            getattr(h, f).argtypes = [_P, _SZ, _SZ]
            getattr(h, f).restype = ctypes.c_longlong
        h.pa_ref_sum_par_nonrec_array_u32.argtypes = [_P, _SZ, _SZ, _P, _SZ]
        h.pa_ref_sum_par_nonrec_array_u32.restype = ctypes.c_ulonglong
        h.pa_ref_std_stable_sort_u64.argtypes = [_P, _SZ]
        h.pa_ref_std_stable_sort_f32_bits.argtypes = [_P, _SZ]
        h.pa_ref_std_stable_sort_kv_u64.argtypes = [_P, _P, _SZ]
        h.pa_ref_counting_sort_par_u8.argtypes = [_P, _SZ]
        h.pa_ref_partition_radix_u32.argtypes = [_P, _SZ, _P, _SZ]
        h.pa_ref_merge_sort_hybrid_radix_u32.argtypes = [_P, _SZ, _SZ, _P, ctypes.c_int]
        h.pa_ref_preventative_adaptive_sort_u32.argtypes = [_P, _SZ]
        h.pa_ref_msd_radix_sort_u32.argtypes = [_P, _SZ]
        h.pa_ref_gen_uniform_u32.argtypes = [ctypes.c_uint64, _SZ, _P]
        h.pa_ref_gen_uniform_u32.restype = None
        self.h = h

    def gen_uniform_u32(self, n: int, seed: int = 1234) -> np.ndarray:
        """The reference benchmark's keys: (uint32)std::mt19937_64(seed)()."""
        a = np.empty(n, np.uint32)
        self.h.pa_ref_gen_uniform_u32(seed, n, _p(a))
        return a

    def threads(self) -> int:
        return int(self.h.pa_ref_hardware_concurrency())

    def sort_radix_par(self, a: np.ndarray, tmp: np.ndarray | None = None) -> np.ndarray:
        """SortRadixPar(a, tmp, n) in place on `a` (uint32)."""
        if tmp is None:
            tmp = np.empty_like(a)
        self.h.pa_ref_sort_radix_par_u32(_p(a), _p(tmp), a.size)
        return a

    def sort_radix_par_alloc(self, a: np.ndarray) -> np.ndarray:
        self.h.pa_ref_sort_radix_par_alloc_u32(_p(a), a.size)
        return a

    def sort_two_phase_par(self, a: np.ndarray, b: np.ndarray) -> None:
        self.h.pa_ref_sort_two_phase_par_u32(_p(a), _p(b), a.size)

    def sort_two_phase_serial(self, a: np.ndarray, b: np.ndarray) -> None:
        self.h.pa_ref_sort_two_phase_serial_u32(_p(a), _p(b), a.size)

    def hist_byte_components(self, a, l, r) -> np.ndarray:
        out = np.zeros((8, 256), np.uint64)
        self.h.pa_ref_hist_byte_components_par_u32(_p(a), l, r, _p(out))
        return out

    def hist_one_byte(self, a, l, r, shift) -> np.ndarray:
        out = np.zeros(256, np.uint64)
        self.h.pa_ref_hist_one_byte_par_u32(_p(a), l, r, shift, _p(out))
        return out

    def hist_u8(self, a, l, r) -> np.ndarray:
        out = np.zeros(256, np.uint64)
        self.h.pa_ref_hist_u8_par(_p(a), l, r, _p(out))
        return out

    def hist_qc(self, a, l, r, work_quanta, quanta, which_byte) -> np.ndarray:
        out = np.zeros((quanta, 256), np.uint64)
        self.h.pa_ref_hist_qc_par_u32(_p(a), l, r, work_quanta, quanta, which_byte, _p(out))
        return out

    def start_of_bins(self, a, n, work_quanta, quanta, digit) -> np.ndarray:
        out = np.zeros((quanta, 256), np.uint64)
        self.h.pa_ref_compute_start_of_bins_par_u32(_p(a), n, work_quanta, quanta, digit, _p(out))
        return out

    def select(self, a: np.ndarray, k: int, start: int = 0, length: int | None = None) -> int:
        """SelectRadix on a copy with one spare element (the reference reads
        one past the range, RadixSelect.h:112)."""
        length = a.size - start if length is None else length
        c = np.zeros(a.size + 1, np.uint32)
        c[:a.size] = a
        if start == 0 and length == a.size:
            return int(self.h.pa_ref_select_radix_u32(_p(c), length, k))
        return int(self.h.pa_ref_select_radix_range_u32(_p(c), start, length, k))

    def sum_nonrec(self, a, l=0, r=None) -> int:
        r = a.size if r is None else r
        f = self.h.pa_ref_sum_par_nonrec_u64 if a.dtype == np.uint64 else self.h.pa_ref_sum_par_nonrec_u32
        return int(f(_p(a), l, r))

    def sum_recursive_u64(self, a, l=0, r=None) -> int:
        return int(self.h.pa_ref_sum_par_u64(_p(a), l, a.size if r is None else r))

    def sum_template_u32(self, a, l=0, r=None) -> int:
        return int(self.h.pa_ref_sum_par_template_u32(_p(a), l, a.size if r is None else r))

    def sum_template(self, a, l=0, r=None) -> int:
        """template SumParallel<_Type> (SumParallel.h:207) for uint8 / uint32 /
        int32 / float32 arrays."""
        f = {np.dtype(np.uint8): self.h.pa_ref_sum_par_template_u8, np.dtype(np.uint32): self.h.pa_ref_sum_par_template_u32,
             np.dtype(np.int32): self.h.pa_ref_sum_par_template_i32,
             np.dtype(np.float32): self.h.pa_ref_sum_par_template_f32}[a.dtype]
        return int(f(_p(a), l, a.size if r is None else r))

    def sum_nonrec_array(self, a, l, r, threshold):
        """SumParallelNonRecursive(a, l, r, sum_array, threshold): (total, sum_array)."""
        tasks = (r - l + threshold - 1) // threshold
        arr = np.zeros(max(tasks, 1), np.uint64)
        total = int(self.h.pa_ref_sum_par_nonrec_array_u32(_p(a), l, r, _p(arr), threshold))
        return total, arr[:tasks]

    def counting_sort_u8(self, a: np.ndarray) -> np.ndarray:
        c = np.ascontiguousarray(a).copy()
        self.h.pa_ref_counting_sort_par_u8(_p(c), c.size)
        return c

    def partition_radix(self, a: np.ndarray, ks) -> np.ndarray:
        c = np.ascontiguousarray(a, dtype=np.uint32).copy()
        k = np.ascontiguousarray(ks, dtype=np.uint64)
        self.h.pa_ref_partition_radix_u32(_p(c), c.size, _p(k), k.size)
        return c

    def merge_sort_hybrid_radix(self, src: np.ndarray, l: int, r: int, dst: np.ndarray, src_to_dst: bool) -> None:
        """In place on src / dst, as the reference (r inclusive)."""
        self.h.pa_ref_merge_sort_hybrid_radix_u32(_p(src), l, r, _p(dst), int(src_to_dst))

    def msd_radix_sort(self, a: np.ndarray) -> None:
        self.h.pa_ref_msd_radix_sort_u32(_p(a), a.size)

    def preventative_adaptive_sort(self, a: np.ndarray) -> None:
        self.h.pa_ref_preventative_adaptive_sort_u32(_p(a), a.size)

    def std_stable_sort_u64(self, a):
        self.h.pa_ref_std_stable_sort_u64(_p(a), a.size)

    def std_stable_sort_f32(self, a):
        self.h.pa_ref_std_stable_sort_f32_bits(_p(a.view(np.uint32)), a.size)

    def std_stable_sort_kv_u64(self, k, v):
        self.h.pa_ref_std_stable_sort_kv_u64(_p(k), _p(v), k.size)


_port: _Port | None = None
_ref: _Ref | None = None


def port() -> _Port:
    """The plain-C restatement (built on demand)."""
    global _port
    if _port is None:
        _port = _Port(_build.build_oracle())
    return _port


def ref() -> _Ref | None:
    """The compiled reference, or None where its sources are unavailable."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not path.exists():
            return None
        _ref = _Ref(path)
    return _ref
