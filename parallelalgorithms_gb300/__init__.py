"""GB300-native radix hot path of ParallelAlgorithms.

Host-side mirror of the reference's C++ interface for the path: the same
function names, argument meaning (index conventions, inclusive/exclusive
ends, default thresholds) and in-place/result semantics, running on one GPU
through the C ABI in include/pa_gpu.h.  Buffers may be numpy arrays (host
memory; copied to the GPU and back) or CUDA torch tensors (used in place on
torch's current stream).  There is no CPU fallback: without the native
library or a GPU every call raises.

Reference entry points mirrored here (file:line within the reference):
  SortRadixPar                 RadixSortLsdParallel.h:340, :367
  SortRadixInnerPar            RadixSortLsdParallel.h:215
  RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase  RadixSortLsdParallel.h:86
  HistogramByteComponentsParallel      HistogramParallel.h:249
  HistogramOneByteComponentParallel    HistogramParallel.h:535 (uint32), :17 (uint8)
  HistogramByteComponentsQCPar         HistogramParallel.h:444
  ComputeStartOfBinsPar                RadixSortLsdParallel.h:108
  SelectRadix                          RadixSelect.h:139, :157
  SumParallelNonRecursive              SumParallel.h:261, :285, :419, :442
  SumParallel                          SumParallel.h:162, :207
  SumParallelNonRecursiveBuffered(Locally), SumNonRecursive  SumParallel.h:309-416, :240
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import PaError, call, lib

__all__ = [
    "SortRadixPar", "SortRadixInnerPar", "RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase",
    "RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize",
    "HistogramByteComponentsParallel", "HistogramOneByteComponentParallel", "HistogramByteComponentsQCPar",
    "ComputeStartOfBinsPar", "SelectRadix", "SumParallelNonRecursive", "SumParallel",
    "SumParallelNonRecursiveBufferedLocally", "SumParallelNonRecursiveBuffered", "SumNonRecursive",
    "counting_sort_parallel", "counting_sort_parallel_inner", "PartitionRadix",
    "parallel_merge_sort_hybrid_radix", "parallel_linear_in_place_preventative_adaptive_sort",
    "parallel_hybrid_inplace_msd_radix_sort",
    "sort", "select", "sum_u64", "histogram_digit", "PaError", "lib",
]


# ---------------------------------------------------------------------------
# buffer plumbing
# ---------------------------------------------------------------------------
def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _info(x):
    """(pointer, element count, numpy dtype, stream or None) of a buffer."""
    if _is_torch(x):
        import torch
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        dt = {torch.int32: np.uint32, torch.int64: np.uint64, torch.uint8: np.uint8,
              torch.float32: np.float32, torch.int8: np.int8, torch.int16: np.int16,
              torch.float64: np.float64}.get(x.dtype)
        if hasattr(torch, "uint32") and x.dtype == torch.uint32:
            dt = np.uint32
        if hasattr(torch, "uint64") and x.dtype == torch.uint64:
            dt = np.uint64
        if dt is None:
            raise TypeError(f"unsupported tensor dtype {x.dtype}")
        stream = torch.cuda.current_stream(x.device).cuda_stream if x.is_cuda else None
        return x.data_ptr(), x.numel(), np.dtype(dt), stream
    if isinstance(x, np.ndarray):
        if not x.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data, x.size, x.dtype, None
    raise TypeError(f"unsupported buffer type {type(x)}")


def _ptr(x):
    return ctypes.c_void_p(_info(x)[0]) if x is not None else None


def _opts(*bufs, digit_bits: int = 0):
    stream = None
    for b in bufs:
        if b is not None and _is_torch(b):
            s = _info(b)[3]
            if s is not None:
                stream = s
    return _native.opts(stream, digit_bits=digit_bits)


def _offset(x, elems: int, itemsize: int):
    p = _info(x)[0]
    return ctypes.c_void_p(p + elems * itemsize)


def _kind(dt: np.dtype) -> str:
    if dt == np.uint32 or dt == np.int32:
        return "u32"
    if dt == np.uint64 or dt == np.int64:
        return "u64"
    if dt == np.float32:
        return "f32"
    if dt == np.uint8:
        return "u8"
    raise TypeError(f"unsupported dtype {dt}")


# ---------------------------------------------------------------------------
# sort
# ---------------------------------------------------------------------------
def sort(keys, values=None, tmp_keys=None, tmp_values=None, n: int | None = None, digit_bits: int = 8) -> None:
    """Stable ascending LSD radix sort of keys[:n] in place (uint32, uint64 or
    float32 keys, float32 by IEEE total order), moving an optional uint32
    payload with its key.  digit_bits: 8 (one pass per key byte, the
    reference's radix) or 11 (2048 bins, fewer passes; same result)."""
    ptr, size, dt, _ = _info(keys)
    n = size if n is None else n
    if n > size:
        raise ValueError("n exceeds the key buffer")
    k = _kind(dt)
    o = _opts(keys, values, tmp_keys, tmp_values, digit_bits=0 if digit_bits == 8 else digit_bits)
    if values is None:
        call(f"pa_sort_{k}", ctypes.c_void_p(ptr), _ptr(tmp_keys), n, o)
    else:
        if _info(values)[1] < n:
            raise ValueError("values shorter than n")
        call(f"pa_sort_kv_{k}", ctypes.c_void_p(ptr), _ptr(values), _ptr(tmp_keys), _ptr(tmp_values), n, o)


def SortRadixPar(a, tmp_work_buff=None, a_size: int | None = None, parallelThreshold: int = 512 * 1024) -> None:
    """RadixSortLsdParallel.h:367 SortRadixPar(a, tmp_work_buff, a_size) and
    :340 SortRadixPar(a, a_size): stable LSD sort of unsigned 32-bit a[0, a_size)
    in place; tmp_work_buff is scratch (contents clobbered).  As in the
    reference, SortRadixPar(a, n) -- an int in the second position -- is the
    allocating overload.  parallelThreshold is accepted and has no effect."""
    if isinstance(tmp_work_buff, (int, np.integer)) and a_size is None:
        a_size, tmp_work_buff = int(tmp_work_buff), None
    _require_u32(a)
    sort(a, tmp_keys=tmp_work_buff, n=a_size)


def SortRadixInnerPar(inputArray, workArray, inputSize: int, ParallelWorkQuantum: int = 64 * 1024) -> None:
    """RadixSortLsdParallel.h:215 SortRadixInnerPar<256,8>: result in inputArray."""
    _require_u32(inputArray)
    sort(inputArray, tmp_keys=workArray, n=inputSize)


def RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(a, b, a_size: int) -> None:
    """RadixSortLsdParallel.h:86: afterwards both a and b hold the sorted keys."""
    _require_u32(a)
    call("pa_sort_two_phase_u32", _ptr(a), _ptr(b), a_size, _opts(a, b))


def RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize(a, b, a_size: int) -> None:
    """RadixSortLsdParallel.h:491.  The reference's body is commented out for
    a_size >= 100 (:503) and leaves b untouched; this implements the intended
    result, the same as the two-phase sort: sorted keys in a and b."""
    RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(a, b, a_size)


def _require_u32(a):
    if _info(a)[2] not in (np.dtype(np.uint32), np.dtype(np.int32)):
        raise TypeError("the reference entry point sorts unsigned 32-bit keys; use sort() for other key types")


# ---------------------------------------------------------------------------
# histograms
# ---------------------------------------------------------------------------
def HistogramByteComponentsParallel(inArray, l: int, r: int, parallelThreshold: int = 64 * 1024,
                                    PowerOfTwoRadix: int = 256, Log2ofPowerOfTwoRadix: int = 8) -> np.ndarray:
    """HistogramParallel.h:249 HistogramByteComponentsParallel<256,8>(a, l, r),
    r inclusive.  Returns the reference's Log2ofPowerOfTwoRadix = 8 rows of 256
    counts: rows 0-3 are the four byte digits, rows 4-7 are zero, as the
    reference allocates them (:252, :260-293)."""
    if (PowerOfTwoRadix, Log2ofPowerOfTwoRadix) != (256, 8):
        raise ValueError("only <256, 8> is defined (the reference's loop is hard-wired to 4 byte digits)")
    out = np.zeros((8, 256), np.uint64)
    n = r - l + 1 if l <= r else 0
    body = np.zeros(4 * 256, np.uint64)
    call("pa_hist_byte_components_u32", _offset(inArray, l, 4), n, ctypes.c_void_p(body.ctypes.data),
         _opts(inArray))
    out[:4] = body.reshape(4, 256)
    return out


def HistogramOneByteComponentParallel(inArray, l: int, r: int, shiftRight: int | None = None,
                                      parallelThreshold: int = 64 * 1024) -> np.ndarray:
    """uint32 input: HistogramParallel.h:535 HistogramOneByteComponentParallel
    <256,8>(a, l, r, shiftRight), r INCLUSIVE, counts of (a[i] >> shiftRight) & 255.
    uint8 input: HistogramParallel.h:17 HistogramOneByteComponentParallel<256>
    (a, l, r), r EXCLUSIVE, byte counts."""
    out = np.zeros(256, np.uint64)
    k = _kind(_info(inArray)[2])
    if k == "u8":
        n = max(0, r - l)
        call("pa_hist_u8", _offset(inArray, l, 1), n, ctypes.c_void_p(out.ctypes.data), _opts(inArray))
    else:
        if shiftRight is None:
            raise TypeError("shiftRight is required for 32-bit input")
        n = r - l + 1 if l <= r else 0
        call("pa_hist_one_byte_u32", _offset(inArray, l, 4), n, int(shiftRight), ctypes.c_void_p(out.ctypes.data),
             _opts(inArray))
    return out


def histogram_digit(a, shift: int = 0) -> np.ndarray:
    """256 counts of ((key >> shift) & 255) over the whole uint32 array."""
    n = _info(a)[1]
    return HistogramOneByteComponentParallel(a, 0, n - 1, shift)


def HistogramByteComponentsQCPar(inArray, l: int, r: int, workQuanta: int, numberOfQuantas: int, whichByte: int,
                                 parallelThreshold: int = 16 * 1024) -> np.ndarray:
    """HistogramParallel.h:444: counts of byte whichByte per work quantum
    (quantum = index // workQuanta) over a[l..r], r inclusive; shape
    (numberOfQuantas, 256)."""
    out = np.zeros((numberOfQuantas, 256), np.uint64)
    call("pa_hist_quanta_u32", _ptr(inArray), l, r, workQuanta, numberOfQuantas, whichByte,
         ctypes.c_void_p(out.ctypes.data), _opts(inArray))
    return out


def ComputeStartOfBinsPar(inArray, size: int, workQuanta: int, numberOfQuantas: int, digit: int,
                          parallelThreshold: int = 16 * 1024) -> np.ndarray:
    """RadixSortLsdParallel.h:108: startOfBin[q][b], shape (numberOfQuantas, 256)."""
    out = np.zeros((numberOfQuantas, 256), np.uint64)
    call("pa_start_of_bins_u32", _ptr(inArray), size, workQuanta, numberOfQuantas, digit,
         ctypes.c_void_p(out.ctypes.data), _opts(inArray))
    return out


# ---------------------------------------------------------------------------
# select
# ---------------------------------------------------------------------------
def SelectRadix(a, *args) -> int:
    """RadixSelect.h:157 SelectRadix(a, length, k) and :139 SelectRadix(a,
    start, length, k): the k-th smallest (k absolute, 0-based) of
    a[start, start + length); like the reference it leaves the result at
    a[k], by swapping a[k] with the first element of the range that holds
    it, so `a` stays a permutation of its input."""
    if len(args) == 2:
        start, (length, k) = 0, args
    elif len(args) == 3:
        start, length, k = args
    else:
        raise TypeError("SelectRadix(a, length, k) or SelectRadix(a, start, length, k)")
    _require_u32(a)
    out = np.zeros(1, np.uint32)
    call("pa_select_radix_u32", _ptr(a), start, length, k, ctypes.c_void_p(out.ctypes.data), _opts(a))
    return int(out[0])


def select(a, k: int) -> int:
    """k-th smallest (0-based) of a uint32 or uint64 array; a is not modified."""
    ptr, n, dt, _ = _info(a)
    kind = _kind(dt)
    out = np.zeros(1, np.uint64 if kind == "u64" else np.uint32)
    call(f"pa_select_{kind}", ctypes.c_void_p(ptr), n, k, ctypes.c_void_p(out.ctypes.data), _opts(a))
    return int(out[0])


# ---------------------------------------------------------------------------
# sum
# ---------------------------------------------------------------------------
def _sum(in_array, l: int, r: int) -> int:
    dt = _info(in_array)[2]
    kind = _kind(dt)
    if kind not in ("u32", "u64"):
        raise TypeError("sum is defined for unsigned 32- and 64-bit arrays")
    out = np.zeros(1, np.uint64)
    isz = 4 if kind == "u32" else 8
    call(f"pa_sum_{kind}", _offset(in_array, l, isz), max(0, r - l), ctypes.c_void_p(out.ctypes.data),
         _opts(in_array))
    return int(out[0])


# element kinds of pa_sum_typed (PA_ELEM_* in include/pa_gpu.h)
_ELEM_KIND = {np.dtype(np.uint8): 0, np.dtype(np.int8): 1, np.dtype(np.uint16): 2, np.dtype(np.int16): 3,
              np.dtype(np.uint32): 4, np.dtype(np.int32): 5, np.dtype(np.uint64): 6, np.dtype(np.int64): 7,
              np.dtype(np.float32): 8, np.dtype(np.float64): 9}


def _elem(in_array) -> tuple[int, int]:
    dt = _info(in_array)[2]
    if dt not in _ELEM_KIND:
        raise TypeError(f"no sum for element type {dt}")
    return _ELEM_KIND[dt], dt.itemsize


def _signed64(v: int) -> int:
    return v - (1 << 64) if v >= (1 << 63) else v


def SumParallelNonRecursive(in_array, l: int, r: int, sum_array=None, parallelThreshold: int = 16 * 1024) -> int:
    """SumParallel.h:261 (unsigned[]) and :285 (unsigned long long[]): sum of
    in_array[l, r), r exclusive, modulo 2^64, as an unsigned 64-bit value.
    With `sum_array` (a uint64 array of ceil((r - l) / parallelThreshold)
    entries, or an int in its place, which is then taken as the threshold),
    the caller-buffer overloads :419, :442: sum_array[i] receives the sum of
    the i-th parallelThreshold-element chunk."""
    if isinstance(sum_array, (int, np.integer)):
        sum_array, parallelThreshold = None, int(sum_array)
    if sum_array is None:
        return _sum(in_array, l, r)
    kind, isz = _elem(in_array)
    n = max(0, r - l)
    need = -(-n // parallelThreshold)
    if _info(sum_array)[1] < need:
        raise ValueError(f"sum_array holds fewer than the {need} chunk sums")
    out = np.zeros(1, np.uint64)
    call("pa_sum_chunked", _offset(in_array, l, isz), n, kind, parallelThreshold, _ptr(sum_array),
         ctypes.c_void_p(out.ctypes.data), _opts(in_array, sum_array))
    return int(out[0])


def SumParallel(in_array, l: int, r: int, parallelThreshold: int = 16 * 1024) -> int:
    """SumParallel.h:162 (unsigned long long[] -> unsigned long long) and the
    template :207 (any other element type -> long long): every element is
    converted to a 64-bit integer (floats truncated toward zero) and summed
    modulo 2^64; the template's result is those 64 bits read as signed.
    Tensors of torch.int32 / int64 hold unsigned keys in this package and are
    summed as such."""
    kind, isz = _elem(in_array)
    out = np.zeros(1, np.uint64)
    call("pa_sum_typed", _offset(in_array, l, isz), max(0, r - l), kind, ctypes.c_void_p(out.ctypes.data),
         _opts(in_array))
    v = int(out[0])
    return v if kind == _ELEM_KIND[np.dtype(np.uint64)] else _signed64(v)


def SumParallelNonRecursiveBufferedLocally(in_array, l: int, r: int, parallelThreshold: int = 16 * 1024) -> int:
    """SumParallel.h:309, :337: the same sum as SumParallelNonRecursive (the
    reference's variant differs only in how each CPU task reads its chunk)."""
    return _sum(in_array, l, r)


def SumParallelNonRecursiveBuffered(in_array, l: int, r: int, parallelThreshold: int = 16 * 1024) -> int:
    """SumParallel.h:366, :393: the same sum as SumParallelNonRecursive."""
    return _sum(in_array, l, r)


def SumNonRecursive(in_array, l: int, r: int, parallelThreshold: int = 128 * 1024) -> int:
    """SumParallel.h:240 (unsigned long long[]): the same sum."""
    return _sum(in_array, l, r)


def sum_u64(a) -> int:
    """Sum of a whole uint32/uint64 array modulo 2^64."""
    return _sum(a, 0, _info(a)[1])


# ---------------------------------------------------------------------------
# byte counting sort
# ---------------------------------------------------------------------------
def counting_sort_parallel_inner(array_to_sort, l: int, r: int, threshold_count: int = 64 * 1024,
                                 threshold_fill: int = 64 * 1024) -> None:
    """CountingSortParallel.h:29 counting_sort_parallel_inner<256>(a, l, r):
    sorts the bytes a[l, r) (r EXCLUSIVE) in place.  The thresholds are
    accepted and have no effect."""
    if _kind(_info(array_to_sort)[2]) != "u8":
        raise TypeError("counting sort takes a uint8 array")
    n = max(0, r - l)
    call("pa_counting_sort_u8", _offset(array_to_sort, l, 1), n, _opts(array_to_sort))


def counting_sort_parallel(a, a_size: int | None = None) -> None:
    """CountingSortParallel.h:81 counting_sort_parallel(a, a_size): sorts the
    bytes a[0, a_size) in place."""
    counting_sort_parallel_inner(a, 0, _info(a)[1] if a_size is None else a_size)


# ---------------------------------------------------------------------------
# radix partition
# ---------------------------------------------------------------------------
def PartitionRadix(a, *args):
    """RadixPartition.h forms, in place on a uint32 array:
      PartitionRadix(a, aLength, k) -> a[k]                       (:92)
      PartitionRadix(a, aStart, aLength, k) -> a[k], k absolute   (:124)
      PartitionRadix(a, aLength, k_list)                          (:152)
      PartitionRadix(a, aStart, aLength, k_list, kStart, kLength) (:165)
    Afterwards every listed a[k] is the k-th smallest of the (sub)range and
    the range is partitioned around it."""
    _require_u32(a)
    if len(args) == 2 and np.ndim(args[1]) == 0:
        length, k = int(args[0]), int(args[1])
        _partition(a, 0, length, [k])
        return int(np.asarray(_fetch(a, k)))
    if len(args) == 3 and np.ndim(args[2]) == 0:
        start, length, k = int(args[0]), int(args[1]), int(args[2])
        _partition(a, start, length, [k])
        return int(np.asarray(_fetch(a, k)))
    if len(args) == 2:
        _partition(a, 0, int(args[0]), list(np.asarray(args[1]).ravel()))
        return None
    if len(args) == 5:
        start, length, ks, kstart, klen = args
        _partition(a, int(start), int(length), list(np.asarray(ks).ravel()[int(kstart):int(kstart) + int(klen)]))
        return None
    raise TypeError("PartitionRadix: unsupported argument list")


def _fetch(a, i: int):
    if _is_torch(a):
        return int(a[i].item()) & 0xFFFFFFFF
    return a[i]


def _partition(a, start: int, length: int, ks) -> None:
    """ks: absolute indices inside [start, start + length), ascending."""
    rel = np.ascontiguousarray([int(k) - start for k in ks], dtype=np.uint64)
    call("pa_partition_radix_u32", _offset(a, start, 4), length, ctypes.c_void_p(rel.ctypes.data), rel.size,
         _opts(a))


# ---------------------------------------------------------------------------
# callers that use LSD radix sort as their leaf
# ---------------------------------------------------------------------------
def parallel_merge_sort_hybrid_radix(src, l: int, r: int, dst, srcToDst: bool = True,
                                     parallelThreshold: int = 24 * 1024) -> None:
    """ParallelMergeSort.h:287: sorts src[l, r] (r INCLUSIVE); the result is
    in dst[l, r] when srcToDst (src then holds scratch), else in src."""
    _require_u32(src)
    n = r - l + 1 if r >= l else 0
    if n == 0:
        return
    if srcToDst:
        _require_u32(dst)
        call("pa_sort_copy_u32", _offset(src, l, 4), _offset(dst, l, 4), n, _opts(src, dst))
    else:
        call("pa_sort_u32", _offset(src, l, 4), _offset(dst, l, 4) if dst is not None else None, n, _opts(src, dst))


def parallel_linear_in_place_preventative_adaptive_sort(src, src_size: int | None = None, stable: bool = True,
                                                        physical_memory_threshold_post: float = 0.75,
                                                        parallelThreshold: int = 24 * 1024) -> None:
    """ParallelMergeSort.h:549: sorts src in place (the GPU's radix sort needs
    no memory-pressure fallback: device scratch is taken from HBM)."""
    _require_u32(src)
    sort(src, n=src_size)


def parallel_hybrid_inplace_msd_radix_sort(a, a_size: int | None = None, scratch_keys: int = 0) -> None:
    """RadixSortMsdParallel.h:291: sorts a[0, a_size) in place holding a
    bounded device scratch (scratch_keys keys, 0 = 2^24) instead of a second
    array of a_size keys (pa_sort_u32_inplace).  For keys alone the unstable
    MSD sort gives the same array as any sort."""
    _require_u32(a)
    n = _info(a)[1] if a_size is None else a_size
    if n >= 2:
        call("pa_sort_u32_inplace", _ptr(a), n, scratch_keys, _opts(a))
