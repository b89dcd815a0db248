"""Serving loop: a Server takes sort / select / histogram requests as they
arrive (pa_server_* in include/pa_gpu.h; the scheduler runs on its own native
thread), admits them against an HBM budget, overlaps them on several streams
and coalesces waiting uint32 sorts into one batched launch.

Also the C5 request stream (Poisson arrivals; 70 % sort, 20 % select at a
random k, 10 % 256-bin histogram; sizes log-uniform in [1e4, 5e7]; uint32 or
uint64 keys 50/50) and the two ways of serving it that the benchmark
compares: through the Server, and one plain call per request.
"""
from __future__ import annotations

import ctypes
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _native
from ._native import call

P = ctypes.c_void_p
REQ_SORT, REQ_SELECT, REQ_HISTOGRAM = 0, 1, 2
KEY_U32, KEY_U64 = 0, 1


class PaRequest(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int), ("key_kind", ctypes.c_int), ("keys", ctypes.c_void_p),
                ("n", ctypes.c_size_t), ("k", ctypes.c_uint64), ("shift", ctypes.c_uint),
                ("result", ctypes.c_void_p), ("status", ctypes.c_int), ("unit_size", ctypes.c_int),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double),
                ("internal_device", ctypes.c_int)]


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int),
                ("max_batch_requests", ctypes.c_int), ("no_coalesce", ctypes.c_int),
                ("num_streams", ctypes.c_int), ("reserve_mib", ctypes.c_int),
                ("join_max_keys_log2", ctypes.c_int), ("unit_max_keys_log2", ctypes.c_int),
                ("reserved", ctypes.c_int * 1)]


@dataclass
class Request:
    """One request; `keys` is a numpy array (host; pinned for overlap) or a CUDA
    tensor.  A sort leaves the keys sorted in place; select / histogram results
    land in `result` (1 or 256 uint64 words)."""
    op: int
    keys: object
    k: int = 0
    shift: int = 0
    result: np.ndarray = field(default=None)
    c: PaRequest = field(default=None)

    def __post_init__(self):
        dt = getattr(self.keys, "dtype", None)
        name = str(dt)
        self.key_kind = KEY_U64 if ("64" in name) else KEY_U32
        n = self.keys.numel() if hasattr(self.keys, "numel") else self.keys.size
        ptr = self.keys.data_ptr() if hasattr(self.keys, "data_ptr") else self.keys.ctypes.data
        if self.result is None:
            self.result = np.zeros(256 if self.op == REQ_HISTOGRAM else 1, np.uint64)
        self.c = PaRequest(op=self.op, key_kind=self.key_kind, keys=ptr, n=n, k=self.k, shift=self.shift,
                           result=self.result.ctypes.data, status=-1)

    @property
    def n(self) -> int:
        return int(self.c.n)

    @property
    def latency(self) -> float:
        return self.c.t_done - self.c.t_submit


class Server:
    def __init__(self, budget_bytes: int = 64 << 30, max_inflight: int = 4, max_batch_requests: int = 256,
                 coalesce: bool = True, num_streams: int = 4, reserve_bytes: int = 0,
                 join_max_keys_log2: int = 0, unit_max_keys_log2: int = 0):
        cfg = ServeConfig(hbm_budget_bytes=budget_bytes, max_inflight=max_inflight,
                          max_batch_requests=max_batch_requests, no_coalesce=0 if coalesce else 1,
                          num_streams=num_streams, reserve_mib=(reserve_bytes + (1 << 20) - 1) >> 20,
                          join_max_keys_log2=join_max_keys_log2, unit_max_keys_log2=unit_max_keys_log2)
        h = ctypes.c_void_p()
        call("pa_server_create", ctypes.byref(cfg), ctypes.byref(h))
        self._h = h

    def submit(self, req: Request) -> None:
        call("pa_server_submit", self._h, ctypes.byref(req.c))

    def wait(self, req: Request) -> int:
        return _native.lib().pa_server_wait(self._h, ctypes.byref(req.c))

    def drain(self) -> None:
        call("pa_server_drain", self._h)

    def stats(self) -> dict:
        out = (ctypes.c_uint64 * 9)()
        call("pa_server_stats", self._h, out, 9)
        keys = ["submitted", "completed", "rejected", "units", "batched_units", "coalesced_requests", "peak_bytes",
                "launch_us", "finish_us"]
        return dict(zip(keys, list(out)))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _native.lib().pa_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------
# the C5 request stream
# ---------------------------------------------------------------------------
@dataclass
class Spec:
    op: int
    key_kind: int
    n: int
    k: int
    seed: int


def make_specs(count: int, seed: int = 1239, lo: float = 1e4, hi: float = 5e7) -> list[Spec]:
    """count requests: 70 % sort, 20 % select (random k), 10 % histogram; sizes
    log-uniform in [lo, hi]; uint32 / uint64 keys 50/50."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        u = rng.random()
        op = REQ_SORT if u < 0.7 else REQ_SELECT if u < 0.9 else REQ_HISTOGRAM
        kind = KEY_U32 if rng.random() < 0.5 else KEY_U64
        n = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        k = int(rng.integers(0, n))
        specs.append(Spec(op, kind, n, k, seed * 100003 + i))
    return specs


def _pinned(n: int, dtype):
    import torch
    t = torch.empty(n * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
    return t.numpy().view(dtype), t


def materialize(specs: list[Spec], pinned: bool = True):
    """Host key buffers for each spec (pinned so copies overlap) and pristine copies."""
    from . import workloads
    bufs = []
    for s in specs:
        src = workloads.uniform_u32(s.n, seed=s.seed) if s.key_kind == KEY_U32 else \
            workloads.uniform_u64(s.n, seed=s.seed)
        if pinned:
            dst, keep = _pinned(s.n, src.dtype)
            np.copyto(dst, src)
            bufs.append((dst, keep, src))
        else:
            bufs.append((src.copy(), None, src))
    return bufs


def run_served(server: Server, specs: list[Spec], bufs, rate: float | None, seed: int = 7) -> list[Request]:
    """Submits the requests with Poisson inter-arrival times (rate requests/s;
    None = all at once) and waits for all of them.  The inputs are restored
    before the first submission."""
    rng = np.random.default_rng(seed)
    reqs = []
    for s, (buf, _, src) in zip(specs, bufs):
        np.copyto(buf, src)
        reqs.append(Request(s.op, buf, k=s.k))
    t_next = time.perf_counter()
    for r in reqs:
        if rate:
            t_next += rng.exponential(1.0 / rate)
            while time.perf_counter() < t_next:
                pass
        server.submit(r)
    server.drain()
    return reqs


def run_plain(specs: list[Spec], bufs, per_call: list | None = None) -> tuple[list, float]:
    """One plain synchronous call per request (the per-request form), one
    after another.  Returns the results and the total wall time of the calls
    (restoring each input before its call is not timed); per_call, if given,
    receives each call's own duration."""
    results = []
    total = 0.0
    for s, (buf, _, src) in zip(specs, bufs):
        np.copyto(buf, src)
        kk = "u32" if s.key_kind == KEY_U32 else "u64"
        t0 = time.perf_counter()
        if s.op == REQ_SORT:
            call(f"pa_sort_{kk}", P(buf.ctypes.data), None, s.n, None)
            results.append(None)
        elif s.op == REQ_SELECT:
            out = np.zeros(1, np.uint64)
            call(f"pa_select_{kk}", P(buf.ctypes.data), s.n, s.k, P(out.ctypes.data), None)
            results.append(out)
        else:
            out = np.zeros(256, np.uint64)
            call(f"pa_hist_one_byte_{kk}", P(buf.ctypes.data), s.n, 0, P(out.ctypes.data), None)
            results.append(out)
        dt = time.perf_counter() - t0
        total += dt
        if per_call is not None:
            per_call.append(dt)
    return results, total


def device_copies(bufs) -> list:
    """(work, pristine) CUDA tensor pairs holding each request's keys in HBM,
    for the device-resident forms of the stream."""
    import torch
    out = []
    for (_, _, src) in bufs:
        t = torch.from_numpy(src.view(np.int32 if src.dtype == np.uint32 else np.int64)).cuda()
        out.append((torch.empty_like(t), t))
    torch.cuda.synchronize()
    return out


def run_served_device(server: Server, specs: list[Spec], dev, rate: float | None, seed: int = 7) -> list[Request]:
    """run_served with the keys already in HBM (restored before the first submission)."""
    import torch
    rng = np.random.default_rng(seed)
    for work, src in dev:
        work.copy_(src)
    torch.cuda.synchronize()
    reqs = [Request(s.op, work, k=s.k) for s, (work, _) in zip(specs, dev)]
    t_next = time.perf_counter()
    for r in reqs:
        if rate:
            t_next += rng.exponential(1.0 / rate)
            while time.perf_counter() < t_next:
                pass
        server.submit(r)
    server.drain()
    return reqs


def run_plain_device(specs: list[Spec], dev, per_call: list | None = None) -> tuple[list, float]:
    """run_plain with the keys already in HBM: one synchronous call per request
    on the device buffer (restoring it is not timed)."""
    import torch
    results = []
    total = 0.0
    for s, (work, src) in zip(specs, dev):
        work.copy_(src)
        torch.cuda.synchronize()
        kk = "u32" if s.key_kind == KEY_U32 else "u64"
        ptr = P(work.data_ptr())
        t0 = time.perf_counter()
        if s.op == REQ_SORT:
            call(f"pa_sort_{kk}", ptr, None, s.n, None)
            results.append(None)
        elif s.op == REQ_SELECT:
            out = np.zeros(1, np.uint64)
            call(f"pa_select_{kk}", ptr, s.n, s.k, P(out.ctypes.data), None)
            results.append(out)
        else:
            out = np.zeros(256, np.uint64)
            call(f"pa_hist_one_byte_{kk}", ptr, s.n, 0, P(out.ctypes.data), None)
            results.append(out)
        dt = time.perf_counter() - t0
        total += dt
        if per_call is not None:
            per_call.append(dt)
    return results, total


def latency_stats(reqs: list[Request]) -> dict:
    lat = np.array([r.latency for r in reqs]) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max())}
