"""Batched segmented sort and its autotuner.

Many uint32 arrays of uneven size, stored back to back in one device buffer
and described by offsets, are sorted independently in ONE persistent kernel
launch (pa_segsort_plan_* in include/pa_gpu.h): segments up to a cutoff are
sorted inside one CTA's shared memory, longer ones by the onesweep passes.
A plan is built once per segmentation and replayed through a captured CUDA
graph.

The autotuner times every candidate configuration (small/large cutoff and
digit width; the onesweep tile of 11-bit plans) on the caller's own data and
remembers the fastest per (GPU, workload shape) in a JSON file, so later
plans for the same shape start from the tuned choice without measuring
again.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import time
from dataclasses import asdict, dataclass
from pathlib import Path

import numpy as np

from . import _native
from ._native import SegSortConfig, call

P = ctypes.c_void_p


@dataclass(frozen=True)
class SegSortChoice:
    small_cutoff: int = 4096
    tile_keys: int = 8192
    digit_bits: int = 8

    def config(self, use_graph: bool = True) -> SegSortConfig:
        c = SegSortConfig()
        c.small_cutoff = self.small_cutoff
        c.tile_keys = self.tile_keys
        c.digit_bits = self.digit_bits
        c.use_graph = 1 if use_graph else 0
        return c


# the small/large cutoff with 8-bit digits (whose passes use the plain
# sort's tile), and 11-bit digits (three passes of 2048 bins) at the default
# cutoff with either tile
CANDIDATES = ([SegSortChoice(c, 8192) for c in (2048, 4096, 8192)] +
              [SegSortChoice(4096, t, 11) for t in (4096, 8192)])


def _ptr(x) -> int:
    return x.data_ptr() if hasattr(x, "data_ptr") else x.ctypes.data


class SegmentedSortPlan:
    """A plan for one segmentation (offsets: num_segments + 1 non-decreasing
    uint64 values).  run() sorts every segment of a device key buffer in place."""

    def __init__(self, offsets: np.ndarray, choice: SegSortChoice | None = None, use_graph: bool = True):
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.choice = choice or SegSortChoice()
        self.total = int(self.offsets[-1]) if self.offsets.size else 0
        cfg = self.choice.config(use_graph)
        h = ctypes.c_void_p()
        call("pa_segsort_plan_create", P(self.offsets.ctypes.data), self.offsets.size - 1, ctypes.byref(cfg),
             ctypes.byref(h))
        self._h = h

    def info(self) -> dict:
        s, l, i = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        call("pa_segsort_plan_info", self._h, ctypes.byref(s), ctypes.byref(l), ctypes.byref(i))
        return {"small_segments": s.value, "large_segments": l.value, "work_items": i.value}

    def run(self, keys, tmp, stream: int | None = None, sync: bool = True) -> None:
        """keys, tmp: CUDA tensors (or device pointers) of the plan's total length."""
        o = _native.opts(stream, async_device=not sync)
        call("pa_segsort_plan_run", self._h, P(_ptr(keys)), P(_ptr(tmp)), o)

    def sync(self, stream: int | None = None) -> None:
        call("pa_segsort_plan_sync", self._h, P(stream or 0))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().pa_segsort_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def segmented_sort(keys, offsets: np.ndarray, choice: SegSortChoice | None = None) -> None:
    """One-shot batched sort of a host (numpy) or device (CUDA tensor) uint32 buffer."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    cfg = (choice or SegSortChoice()).config(use_graph=False)
    stream = None
    if hasattr(keys, "data_ptr"):
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    call("pa_segmented_sort_u32", P(_ptr(keys)), P(off.ctypes.data), off.size - 1, ctypes.byref(cfg),
         _native.opts(stream))


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
def _cache_file() -> Path:
    env = os.environ.get("PA_AUTOTUNE_FILE")
    if env:
        return Path(env)
    return Path.home() / ".cache" / "parallelalgorithms_gb300" / "autotune.json"


def shape_key(offsets: np.ndarray) -> str:
    """GPU name + workload shape bucket (total keys and segment count, powers of 2,
    and the median segment length)."""
    import torch
    sizes = np.diff(offsets.astype(np.int64))
    total = int(sizes.sum())
    med = int(np.median(sizes)) if sizes.size else 0
    b = lambda x: int(round(math.log2(max(x, 1))))  # noqa: E731
    return f"{torch.cuda.get_device_name()}|segsort_u32|n2^{b(total)}|s2^{b(sizes.size)}|m2^{b(med)}"


def load_choice(offsets: np.ndarray) -> SegSortChoice | None:
    f = _cache_file()
    if not f.exists():
        return None
    try:
        table = json.loads(f.read_text())
        e = table.get(shape_key(offsets))
        return SegSortChoice(**e["choice"]) if e else None
    except Exception:
        return None


def autotune(offsets: np.ndarray, keys, tmp, candidates=None, reps: int = 3, persist: bool = True) -> dict:
    """Times each candidate on (a copy of) the caller's device keys and returns
    {"choice": best, "ms": {candidate: median ms}}; persists the winner."""
    import torch
    cands = list(candidates or CANDIDATES)
    pristine = keys.clone()
    stream = torch.cuda.current_stream()
    results = {}
    for c in cands:
        plan = SegmentedSortPlan(offsets, c, use_graph=True)
        times = []
        for r in range(reps + 1):
            keys.copy_(pristine)
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record(stream)
            plan.run(keys, tmp, stream.cuda_stream, sync=False)
            e.record(stream)
            plan.sync(stream.cuda_stream)
            if r:
                times.append(s.elapsed_time(e))
        plan.close()
        results[c] = float(np.median(times))
    keys.copy_(pristine)
    best = min(results, key=results.get)
    out = {"choice": best, "ms": {f"cutoff={c.small_cutoff},tile={c.tile_keys},bits={c.digit_bits}": v
                                  for c, v in results.items()}}
    if persist:
        f = _cache_file()
        f.parent.mkdir(parents=True, exist_ok=True)
        table = {}
        if f.exists():
            try:
                table = json.loads(f.read_text())
            except Exception:
                table = {}
        table[shape_key(offsets)] = {"choice": asdict(best), "ms": out["ms"], "when": time.time()}
        tmpf = f.with_suffix(".tmp")
        tmpf.write_text(json.dumps(table, indent=1))
        os.replace(tmpf, f)
    return out
