#!/usr/bin/env python3
"""Benchmark of the GB300 radix hot path.

Headline workload: stable LSD radix sort of 100,000,000 uniform uint32 keys
((uint32)std::mt19937_64(1234)(), the reference's recipe) on one GPU, 8-bit
digits (4 passes).  One step = one sort of the whole array with the keys
already resident in HBM; the input is restored from a pristine device copy
before each step, outside the step's CUDA events.  The 400 MB input is
larger than the 129 MB L2, so no L2 flush is needed between steps.

Printed as one JSON line (rank 0):
  value       keys/s over the device-resident sort (CUDA events per step)
  e2e         keys/s through the reference-facing C ABI (pa_sort_u32) with
              pinned HOST buffers: host->device copy, sort, device->host copy
  roofline    the dominant kernel (one onesweep digit pass): algorithmic
              bytes per launch (8 bytes/key: read + write each key once)
              over its CUDA-event duration, against the measured HBM copy
              bandwidth in MEASURED_PEAKS.json
  cpu_baseline the reference's own SortRadixPar (compiled unchanged, TBB
              stand-in thread pool) on this host's cores, same input
  extras      presorted / constant sorts, 64-bit key+payload and float32
              sorts, low-digit histogram, select k = n/2 and 64-bit sum at
              100M, each with its own bytes-moved roofline fraction; byte
              counting sort, PartitionRadix, the bounded-scratch in-place
              sort, the batched segmented sort and the serving stream

--impl reference times the reference's CPU SortRadixPar on the same
workload (rank 0 only under torchrun; other ranks exit without work).
With --gpus N > 1 every rank sorts its own replica (the path does not
shard): value = all keys sorted / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "uint32 keys/s sorted at 100M vs HBM roofline; batched/served keys/s + p99 latency"
UNIT = "keys/s"
# The reference's published figure for this metric: parallel LSD radix sort of
# 100,000,000 random uint32 keys, 2865 M keys/s on a 48-core AWS c7a.24xlarge
# (the reference README's table, its fastest published machine).
PUBLISHED_KEYS_PER_S = 2.865e9
PUBLISHED_SOURCE = "reference README: parallel LSD radix sort, 100M random uint32, 48-core AWS c7a.24xlarge"
PROFILE_TRAFFIC = ROOT / "profiles" / "onesweep_pass_u32_100m_traffic.txt"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--n", type=int, default=100_000_000)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--cpu-steps", type=int, default=5)
    p.add_argument("--no-extras", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    # profiling driver: runs one operation `--reps` times on device-resident
    # seeded input and prints no JSON line (the commands in profiles/ use it)
    p.add_argument("--profile-op", default=None,
                   choices=["sort_u32", "sort_u32_host", "sort_u64", "sort_kv_u64", "sort_f32", "hist_u32",
                            "select_u32", "sum_u32", "sort_u32_inplace", "partition_u32", "batched_c4"])
    p.add_argument("--reps", type=int, default=2)
    # the serving stream alone (the default run measures it in a child
    # process of its own, started this way)
    p.add_argument("--serving-only", action="store_true")
    p.add_argument("--dist", default="uniform", choices=["uniform", "presorted", "constant"])
    return p.parse_args()


def profile_op(a) -> None:
    """Runs one operation of the path `a.reps` times with nothing else on the
    GPU, so that an ncu launch filter (-k regex:... -s <skip> -c <count>)
    lands on known launches.  The seeded input is generated once and kept
    device-resident.  Per sort: the workspace memset, one digit histogram,
    one scan, one onesweep launch per key byte, one final copy.
    `sort_u32_host` sorts a page-locked host copy through the C ABI instead
    (the pipelined host-buffer path); `sort_u32_inplace` is the bounded-scratch
    in-place sort, `partition_u32` PartitionRadix around k = n/2 and n - 21,
    `batched_c4` one run of the batched segmented sort on the C4 arrays."""
    import torch

    from parallelalgorithms_gb300 import _native, build, workloads
    build.build()
    P = ctypes.c_void_p
    n = a.n
    if a.profile_op in ("sort_kv_u64", "sort_u64"):
        keys = workloads.uniform_u64(n)
    elif a.profile_op == "sort_f32":
        keys = workloads.normal_specials_f32(n).view(np.uint32)
    elif a.dist == "presorted":
        keys = workloads.presorted_u32(n)
    elif a.dist == "constant":
        keys = workloads.constant_u32(n)
    else:
        keys = workloads.uniform_u32(n)
    src = torch.from_numpy(keys.view({4: np.int32, 8: np.int64}[keys.dtype.itemsize])).cuda()
    k = torch.empty_like(src)
    t = torch.empty_like(src)
    v = tv = None
    if a.profile_op == "sort_kv_u64":
        v = torch.arange(n, dtype=torch.int32, device="cuda")
        tv = torch.empty_like(v)
    out = torch.zeros(256, dtype=torch.int64, device="cuda")
    o = _native.opts(torch.cuda.current_stream().cuda_stream)
    host_t = host = None
    if a.profile_op == "sort_u32_host":
        host_t = torch.empty(n, dtype=torch.int32, pin_memory=True)  # (kept alive for the view below)
        host = host_t.numpy().view(np.uint32)
    op = a.profile_op
    if op == "batched_c4":  # the C4 segmentation (4096 arrays, 2.0 G keys), default plan; --n is not used
        from parallelalgorithms_gb300 import batched
        del src, k, t
        sizes = workloads.log_uniform_sizes(4096, 1e3, 4e6)
        off = np.zeros(sizes.size + 1, np.uint64)
        off[1:] = np.cumsum(sizes)
        c4_src = torch.from_numpy(workloads.uniform_u32(int(off[-1]), seed=workloads.SEED_SEGMENT_SIZES)
                                  .view(np.int32)).cuda()
        c4_keys = c4_src.clone()
        c4_tmp = torch.empty_like(c4_src)
        c4_plan = batched.SegmentedSortPlan(off, use_graph=False)
        k = c4_keys
        src = c4_src
    for _ in range(a.reps):
        k.copy_(src)
        if op == "sort_u32_host":
            np.copyto(host, keys)
            _native.call("pa_sort_u32", P(host.ctypes.data), None, n, None)
        elif op == "sort_u32":
            _native.call("pa_sort_u32", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif op == "sort_f32":
            _native.call("pa_sort_f32", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif op == "sort_u64":
            _native.call("pa_sort_u64", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif op == "sort_kv_u64":
            _native.call("pa_sort_kv_u64", P(k.data_ptr()), P(v.data_ptr()), P(t.data_ptr()), P(tv.data_ptr()), n, o)
        elif op == "hist_u32":
            _native.call("pa_hist_byte_components_u32", P(k.data_ptr()), n, P(out.data_ptr()), o)
        elif op == "select_u32":
            _native.call("pa_select_u32", P(k.data_ptr()), n, n // 2, P(out.data_ptr()), o)
        elif op == "sum_u32":
            _native.call("pa_sum_u32", P(k.data_ptr()), n, P(out.data_ptr()), o)
        elif op == "sort_u32_inplace":
            _native.call("pa_sort_u32_inplace", P(k.data_ptr()), n, 0, o)
        elif op == "batched_c4":
            c4_plan.run(c4_keys, c4_tmp, torch.cuda.current_stream().cuda_stream)
        elif op == "partition_u32":
            ks = np.array([n // 2, n - 21], np.uint64)
            _native.call("pa_partition_radix_u32", P(k.data_ptr()), n, P(ks.ctypes.data), ks.size, o)
    torch.cuda.synchronize()
    print(f"profile driver done: op={op} n={n} reps={a.reps}")


# ---------------------------------------------------------------------------
# clocks: NVML read through ctypes (settings are only read, never changed)
# ---------------------------------------------------------------------------
REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
           0x80: "hw_power_brake_slowdown", 0x2: "applications_clocks_setting"}


class ClockSampler:
    def __init__(self, cuda_index: int, period_s: float = 0.005):
        self.samples: list[tuple[int, int]] = []
        self.max_mhz = None
        self.period = period_s
        self._stop = threading.Event()
        self._thread = None
        self.nvml = None
        self.handle = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit failed")
            h = ctypes.c_void_p()
            bus = None
            try:
                import torch
                pr = torch.cuda.get_device_properties(cuda_index)
                bus = f"{pr.pci_domain_id:08x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0".encode()
            except Exception:
                bus = None
            ok = bus is not None and nv.nvmlDeviceGetHandleByPciBusId_v2(bus, ctypes.byref(h)) == 0
            if not ok and nv.nvmlDeviceGetHandleByIndex_v2(cuda_index, ctypes.byref(h)) != 0:
                raise OSError("no NVML handle")
            self.nvml, self.handle = nv, h
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = mx.value
        except OSError:
            self.nvml = None

    def _read(self):
        mhz = ctypes.c_uint()
        rs = ctypes.c_ulonglong()
        self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(mhz))
        self.nvml.nvmlDeviceGetCurrentClocksEventReasons(self.handle, ctypes.byref(rs))
        return mhz.value, rs.value

    def _loop(self):
        while not self._stop.is_set():
            self.samples.append(self._read())
            time.sleep(self.period)

    def __enter__(self):
        if self.nvml is not None:
            self._thread = threading.Thread(target=self._loop, daemon=True)
            self._thread.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._thread:
            self._thread.join()

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["nvml unavailable"], "samples": 0}
        mhz = [m for m, _ in self.samples]
        seen = 0
        for _, r in self.samples:
            seen |= r
        return {"sm_mhz": statistics.median(mhz), "sm_max_mhz": self.max_mhz,
                "reasons": sorted(v for k, v in REASONS.items() if seen & k), "samples": len(self.samples)}


# ---------------------------------------------------------------------------
def measured_peak_gbs() -> tuple[float, str]:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_traffic_per_launch() -> float | None:
    """dram read+write bytes per onesweep launch from the committed ncu summary."""
    if not PROFILE_TRAFFIC.exists():
        return None
    for line in PROFILE_TRAFFIC.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, dist=None) -> float:
    """The largest x over all ranks (x itself without a process group).  The
    reduction tensor lives where the backend wants it: host memory for gloo,
    the current GPU for nccl."""
    if dist is None:
        return float(x)
    import torch
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: int, world: int, slowest_seconds: float) -> float:
    """Units all ranks processed per second of the slowest rank (replicas: every
    rank processes the same number of units)."""
    return units_per_rank * world / slowest_seconds


def cpu_reference_sort(keys: np.ndarray, steps: int, warmup: int) -> dict:
    """The reference's SortRadixPar(a, tmp, n) on this host; median of steps."""
    import oracle
    from oracle import build as obuild
    obuild.build_ref()
    ref = oracle.ref()
    n = keys.size
    a = np.empty_like(keys)
    tmp = np.empty_like(keys)
    if ref is not None:
        kind, cores = "reference", ref.threads()
        run = lambda: ref.sort_radix_par(a, tmp)  # noqa: E731
        what = "SortRadixPar(a, tmp, n) compiled from the reference headers with a thread-pool TBB stand-in"
    else:
        port = oracle.port()
        kind, cores = "port", 1
        run = lambda: port.sort(a)  # noqa: E731
        what = "oracle restatement (single thread)"
    times = []
    for i in range(warmup + steps):
        np.copyto(a, keys)
        tmp[:] = 0  # page in the scratch buffer as the reference benchmark does
        t0 = time.perf_counter()
        run()
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
    med = statistics.median(times)
    return {"value": n / med, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{what}; {n} uniform uint32 keys (mt19937_64 seed 1234); median of {steps} after {warmup} "
                      f"warm-up; {med * 1e3:.1f} ms per sort",
            "ms": [t * 1e3 for t in times]}


def workload_config(n: int, world: int) -> dict:
    """The `config` both arms print (same workload, same keys)."""
    return {"workload": f"LSD radix sort of {n} uniform uint32 keys (mt19937_64 seed 1234), 8-bit digits, 4 passes",
            "keys_per_gpu": n, "key_type": "uint32", "distribution": "uniform mt19937_64(1234)", "digit_bits": 8,
            "l2": "inputs (400 MB) larger than L2; no flush",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def reference_arm(args) -> None:
    """The reference's own SortRadixPar on this host's cores.  Loads only the
    CPU checkers under oracle/ (the compiled reference, or the restatement
    where the reference could not be built); the GPU library is never
    loaded, and the keys come from the reference benchmark's own recipe."""
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    import oracle
    from oracle import build as obuild
    obuild.build_ref()
    ref = oracle.ref()
    keys = (ref if ref is not None else oracle.port()).gen_uniform_u32(args.n, 1234)
    cb = cpu_reference_sort(keys, args.steps, args.warmup)
    med_s = args.n / cb["value"]
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": med_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": cb["value"] / PUBLISHED_KEYS_PER_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u32", "data": "synthetic",
            "config": workload_config(args.n, world),
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def gb300_arm(args) -> None:
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from parallelalgorithms_gb300 import build as pabuild
    pabuild.build()
    import parallelalgorithms_gb300 as pa
    from parallelalgorithms_gb300 import _native, workloads

    lib = pa.lib()
    n = args.n
    keys = workloads.uniform_u32(n)
    src = torch.from_numpy(keys.view(np.int32)).cuda()
    d_keys = torch.empty_like(src)
    d_tmp = torch.empty_like(src)
    stream = torch.cuda.current_stream()
    opts = _native.opts(stream.cuda_stream, async_device=True)
    P = ctypes.c_void_p

    def sort_once():
        rc = lib.pa_sort_u32(P(d_keys.data_ptr()), P(d_tmp.data_ptr()), n, opts)
        if rc:
            raise RuntimeError(f"pa_sort_u32 failed: {lib.pa_last_error_message().decode()}")

    for _ in range(args.warmup):
        d_keys.copy_(src)
        sort_once()
    _native.call("pa_stream_check", P(stream.cuda_stream))
    flipped = d_keys ^ torch.tensor(-2147483648, dtype=torch.int32, device=d_keys.device)
    if not bool(torch.all(flipped[1:] >= flipped[:-1])):
        raise RuntimeError("warm-up sort result is not sorted")
    del flipped

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    with sampler:
        t0 = time.perf_counter()
        for i in range(args.steps):
            d_keys.copy_(src)
            starts[i].record(stream)
            sort_once()
            ends[i].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    _native.call("pa_stream_check", P(stream.cuda_stream))
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = statistics.mean(step_ms)
    ms_max = max_over_ranks(ms, dist)
    value = whole_job_rate(n, world, ms_max / 1e3)

    # per-kernel device times (same stream, CUDA events between launches)
    phases = np.zeros(16, np.float32)
    reps = 10
    acc = np.zeros(16, np.float64)
    for _ in range(reps):
        d_keys.copy_(src)
        _native.call("pa_sort_timed", 0, P(d_keys.data_ptr()), P(d_tmp.data_ptr()), None, None, n,
                     P(phases.ctypes.data), 16, _native.opts(stream.cuda_stream))
        acc += phases
    acc /= reps
    hist_ms, scan_ms = float(acc[0]), float(acc[1])
    pass_ms = [float(x) for x in acc[2:6]]
    copy_ms = float(acc[6])
    peak, peak_kind = measured_peak_gbs()
    pass_avg = statistics.mean(pass_ms)
    achieved = 8.0 * n / (pass_avg / 1e3) / 1e9
    traffic = profiled_traffic_per_launch()
    roofline = {"bound": "hbm", "kernel": "onesweep digit pass (uint32 keys, 8-bit digit)", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                else "fallback 6800 GB/s",
                "bytes_per_launch": 8 * n, "launch_ms": pass_avg}
    sort_bytes = 36.0 * n
    whole = {"bytes_per_key": 36, "achieved_gbs": sort_bytes / (ms / 1e3) / 1e9,
             "frac": sort_bytes / (ms / 1e3) / 1e9 / peak,
             "phase_ms": {"histogram": hist_ms, "scan": scan_ms, "passes": pass_ms, "final_copy": copy_ms}}

    # end to end through the C ABI with pinned host buffers
    h_src = workloads.uniform_u32(n, pinned=True)
    h_buf = torch.empty(n, dtype=torch.int32, pin_memory=True)
    h_keys = h_buf.numpy().view(np.uint32)
    e2e_times = []
    if dist:
        dist.barrier()
    for i in range(args.e2e_steps + 1):
        np.copyto(h_keys, h_src)
        t0 = time.perf_counter()
        _native.call("pa_sort_u32", P(h_keys.ctypes.data), None, n, None)
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_times.append(dt)
    if not np.all(h_keys[1:] >= h_keys[:-1]):
        raise RuntimeError("end-to-end sort result is not sorted")
    e2e_med = max_over_ranks(statistics.median(e2e_times), dist)
    e2e = {"value": whole_job_rate(n, world, e2e_med), "unit": UNIT, "h2d_bytes_per_step": 4 * n,
           "d2h_bytes_per_step": 4 * n, "ms_per_step": e2e_med * 1e3,
           "api": "pa_sort_u32 (C ABI) on pinned host buffers, synchronous; copies pipelined with the sort "
                  "(chunked copy-in, bucket groups copied out while the next group sorts)"}

    # other workloads of the path: on a single GPU only (replica runs measure the headline)
    extras = {} if (args.no_extras or world > 1) else run_extras(pa, lib, _native, workloads, n, stream, peak)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_reference_sort(keys, args.cpu_steps, 1)
        cpu = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}

    launches_per_step = 1 + 1 + 4 + 1  # histogram, scan, 4 digit passes, final copy
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / PUBLISHED_KEYS_PER_S, "vs_baseline_source": PUBLISHED_SOURCE,
            "dtype": "u32", "data": "synthetic",
            "config": workload_config(n, world),
            "step_timing": {"how": "CUDA events around each device-resident sort; input restored from a pristine "
                                   "device copy before each step, outside the events",
                            "wall_ms_per_step_incl_restore": wall * 1e3 / args.steps},
            "roofline": roofline, "sort_roofline": whole, "e2e": e2e, "cpu_baseline": cpu,
            "gpu_launches": launches_per_step * args.steps, "clocks": sampler.summary(), "extras": extras,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _time_device(fn, reps: int, stream, restore=None) -> float:
    import torch
    ts = []
    for _ in range(reps):
        if restore:
            restore()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        torch.cuda.synchronize()
        ts.append(s.elapsed_time(e))
    return statistics.median(ts)


def batched_extra(lib, _native, workloads, stream, peak) -> dict:
    """4096 uint32 arrays, sizes log-uniform in [1e3, 4e6] (seed 1238; 2.0 G keys
    in total): one batched plan (autotuned, CUDA graph) vs one pa_sort_u32 per
    array."""
    import torch

    from parallelalgorithms_gb300 import batched
    P = ctypes.c_void_p
    sizes = workloads.log_uniform_sizes(4096, 1e3, 4e6)
    off = np.zeros(sizes.size + 1, np.uint64)
    off[1:] = np.cumsum(sizes)
    total = int(off[-1])
    keys = workloads.uniform_u32(total, seed=workloads.SEED_SEGMENT_SIZES)
    src = torch.from_numpy(keys.view(np.int32)).cuda()
    d = src.clone()
    t = torch.empty_like(src)
    tune = batched.autotune(off, d, t, reps=2)
    choice = tune["choice"]
    plan = batched.SegmentedSortPlan(off, choice, use_graph=True)
    info = plan.info()
    times = []
    for r in range(6):
        d.copy_(src)
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record(stream)
        plan.run(d, t, stream.cuda_stream, sync=False)
        e.record(stream)
        plan.sync(stream.cuda_stream)
        if r:
            times.append(s.elapsed_time(e))
    ms = statistics.median(times)
    # sorted within every segment (order-preserving int32 view: flip the sign bit)
    f = d ^ torch.tensor(-2147483648, dtype=torch.int32, device=d.device)
    ok = f[1:] >= f[:-1]
    bounds = torch.from_numpy(off[1:-1].astype(np.int64) - 1).cuda()
    ok[bounds[(bounds >= 0) & (bounds < ok.numel())]] = True
    sorted_ok = bool(torch.all(ok))
    del f, ok
    # the same arrays, one plain sort call per array
    o = _native.opts(stream.cuda_stream, async_device=True)
    d.copy_(src)
    torch.cuda.synchronize()
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    s.record(stream)
    base = d.data_ptr()
    tbase = t.data_ptr()
    for i in range(sizes.size):
        a = int(off[i])
        _native.call("pa_sort_u32", P(base + 4 * a), P(tbase + 4 * a), int(sizes[i]), o)
    e.record(stream)
    torch.cuda.synchronize()
    wall_plain = (time.perf_counter() - t0) * 1e3
    _native.call("pa_stream_check", P(stream.cuda_stream))
    plain_ms = s.elapsed_time(e)
    small = sizes <= choice.small_cutoff
    model_bytes = float(8 * sizes[small].sum() + 36 * sizes[~small].sum())
    plan.close()
    del src, d, t
    torch.cuda.empty_cache()
    return {"segments": int(sizes.size), "keys": total, "ms": ms, "keys_per_s": total / (ms / 1e3),
            "sorted_within_segments": sorted_ok,
            "choice": {"small_cutoff": choice.small_cutoff, "tile_keys": choice.tile_keys,
                       "digit_bits": choice.digit_bits},
            "autotune_ms": tune["ms"], "plan": info, "graph": True,
            "plain_per_array_ms": plain_ms, "plain_per_array_wall_ms": wall_plain,
            "speedup_vs_plain_per_array": plain_ms / ms,
            "bytes_model": "8 B/key for shared-memory segments, 36 B/key for onesweep segments",
            "achieved_gbs": model_bytes / (ms / 1e3) / 1e9, "frac": model_bytes / (ms / 1e3) / 1e9 / peak}


def serving_extra(count: int = 120) -> dict:
    """C5: `count` requests (70 % sort, 20 % select at random k, 10 % 256-bin
    histogram; sizes log-uniform in [1e4, 5e7]; uint32 / uint64 keys 50/50;
    seed 1239), pinned host buffers, 64 GiB budget.  The plain per-request
    form (one synchronous call after another) against the server at several
    Poisson arrival rates; every served result is checked against the plain
    one."""
    from parallelalgorithms_gb300 import serving
    specs = serving.make_specs(count)
    bufs = serving.materialize(specs)
    total = sum(s.n for s in specs)
    serving.run_plain(specs[:8], bufs[:8])  # warm the plain path's workspace
    plain_runs = []
    for _ in range(3):  # median of three, like the saturating server runs
        per_call: list = []
        res, secs = serving.run_plain(specs, bufs, per_call)
        plain_runs.append((secs, res, per_call))
    plain_runs.sort(key=lambda x: x[0])
    plain_s, plain_res, per_call = plain_runs[1]
    plain_sorted = {i: b[0].copy() for i, (s, b) in enumerate(zip(specs, bufs)) if s.op == serving.REQ_SORT and
                    i % 10 == 0}
    lat = np.array(per_call) * 1e3
    out = {"requests": count, "keys": int(total),
           "mix": "70% sort / 20% select / 10% histogram, sizes log-uniform [1e4, 5e7], u32/u64 50/50, seed 1239",
           "budget_bytes": 64 << 30,
           "plain_per_request": {"keys_per_s": total / plain_s, "seconds": plain_s,
                                 "seconds_all": [x[0] for x in plain_runs],
                                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                 "latency": "each call's own duration (no queueing)"}}
    # 24 GiB pre-mapped (peak use is ~6 GB): a block freed by a unit still in
    # flight on its stream cannot serve another stream, and with 8 GiB the
    # pool mapped new memory under load, stalling launches for up to 9 ms
    kw = dict(budget_bytes=64 << 30, max_inflight=32, num_streams=32, reserve_bytes=24 << 30)

    def check(reqs) -> bool:
        ok = all(r.c.status == 0 for r in reqs)
        for i, (s, r, (buf, _, _)) in enumerate(zip(specs, reqs, bufs)):
            if s.op == serving.REQ_SORT:
                ok = ok and bool(np.all(buf[1:] >= buf[:-1]))
                if i in plain_sorted:
                    ok = ok and np.array_equal(buf, plain_sorted[i])
            else:
                ok = ok and np.array_equal(r.result, plain_res[i])
        return ok

    def span_of(reqs) -> float:
        return max(r.c.t_done for r in reqs) - min(r.c.t_submit for r in reqs)

    # all requests waiting at once (the throughput comparison): one measured
    # run on each of five servers created one after another, median reported
    sat = []
    import torch
    sampler = ClockSampler(torch.cuda.current_device())
    with sampler:  # SM clocks and throttle reasons while the servers run
        for _ in range(5):
            with serving.Server(**kw) as srv:
                serving.run_served(srv, specs, bufs, None)  # warm the server's pinned staging blocks
                reqs = serving.run_served(srv, specs, bufs, None)
                sat.append((span_of(reqs), reqs, srv.stats()))
    in_order = [x[0] for x in sat]
    sat.sort(key=lambda x: x[0])
    span, reqs, sat_stats = sat[len(sat) // 2]
    spans = [x[0] for x in sat]
    out["served_saturating"] = {"keys_per_s": total / span, "makespan_s": span, "results_match_plain": check(reqs),
                                **serving.latency_stats(reqs), "latency": "submit to completion (includes queueing)",
                                "speedup_vs_plain_per_request": plain_s / span,
                                "speedup_all_servers": sorted(plain_s / x for x in spans),
                                "makespans_s": spans, "makespans_s_in_creation_order": in_order,
                                "servers": len(sat),
                                "server_stats": sat_stats, "clocks": sampler.summary(),
                                "shared_unit_requests_share": sat_stats["coalesced_requests"] / max(1, sat_stats["completed"])}
    with serving.Server(**kw) as srv:
        serving.run_served(srv, specs, bufs, None)  # warm the server's pinned staging blocks
        for rate in (400.0, 200.0, 100.0):
            reqs = serving.run_served(srv, specs, bufs, rate)
            span = span_of(reqs)
            # arrivals pace the stream: keys/s is the offered load, latency is the result
            out[f"served_poisson_{int(rate)}_per_s"] = {
                "keys_per_s": total / span, "makespan_s": span, "results_match_plain": check(reqs),
                **serving.latency_stats(reqs), "latency": "submit to completion (includes queueing)",
                "offered_requests_per_s": rate}
        out["server_stats"] = srv.stats()
        # the same stream with every request's keys already in HBM: no copies,
        # so this pair isolates what overlapping and coalescing save on the device
        dev = serving.device_copies(bufs)
        serving.run_plain_device(specs[:8], dev[:8])
        dplain_res, dplain_s = serving.run_plain_device(specs, dev)
        serving.run_served_device(srv, specs, dev, None)
        reqs = serving.run_served_device(srv, specs, dev, None)
        ok = all(r.c.status == 0 for r in reqs)
        for i, (s, r, (work, _)) in enumerate(zip(specs, reqs, dev)):
            if s.op == serving.REQ_SORT and i in plain_sorted:
                got = work.cpu().numpy().view(plain_sorted[i].dtype)
                ok = ok and np.array_equal(got, plain_sorted[i])
            elif s.op != serving.REQ_SORT:
                ok = ok and np.array_equal(r.result, dplain_res[i]) and np.array_equal(r.result, plain_res[i])
        span = max(r.c.t_done for r in reqs) - min(r.c.t_submit for r in reqs)
        out["device_resident"] = {"plain_keys_per_s": total / dplain_s, "plain_seconds": dplain_s,
                                  "served_keys_per_s": total / span, "served_makespan_s": span,
                                  "speedup_vs_plain_per_request": dplain_s / span, "results_match_plain": ok,
                                  **serving.latency_stats(reqs)}
        del dev
    # what the host-buffer form must move over the host link
    h2d = sum(s.n * (4 if s.key_kind == serving.KEY_U32 else 8) for s in specs)
    d2h = sum(s.n * (4 if s.key_kind == serving.KEY_U32 else 8) for s in specs if s.op == serving.REQ_SORT)
    out["host_link_bytes"] = {"h2d": h2d, "d2h": d2h}
    out["host_link_gbs"] = host_link_gbs()
    out["host_buffers_page_locked"] = all(keep is not None and keep.is_pinned() for _, keep, _ in bufs)
    return out


def host_link_gbs() -> dict:
    """Copy-engine bandwidth of this GPU's host link, GB/s: eight 256 MB
    page-locked copies on eight streams, host to device, device to host, and
    half each way at once (the overlap the server's streams rely on)."""
    import torch
    nbytes = 256 << 20
    hs = [torch.empty(nbytes, dtype=torch.uint8, pin_memory=True) for _ in range(8)]
    ds = [torch.empty(nbytes, dtype=torch.uint8, device="cuda") for _ in range(8)]
    streams = [torch.cuda.Stream() for _ in range(8)]
    res = {}
    for mode in ("h2d", "d2h", "both_ways"):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in range(8):
            with torch.cuda.stream(streams[i]):
                if mode == "h2d" or (mode == "both_ways" and i % 2 == 0):
                    ds[i].copy_(hs[i], non_blocking=True)
                else:
                    hs[i].copy_(ds[i], non_blocking=True)
        torch.cuda.synchronize()
        res[mode] = round(8 * nbytes / (time.perf_counter() - t) / 1e9, 1)
    return res


def run_extras(pa, lib, _native, workloads, n, stream, peak) -> dict:
    """Other 100M workloads of the same path, device-resident, median of 5."""
    import torch
    P = ctypes.c_void_p
    o = _native.opts(stream.cuda_stream, async_device=True)
    out = {}
    # the serving stream first, on a GPU not just loaded by the batched and
    # 100M workloads below (after those, the servers' overlapped copies run
    # in a slower mode; it is measured again at the end)
    out["serving_c5"] = serving_in_own_process()

    def dev(a):
        return torch.from_numpy(a.view({4: np.int32, 8: np.int64}[a.dtype.itemsize])).cuda()

    def sort_case(name, keys, vals=None, fn="pa_sort_u32", bytes_per_key=36):
        src = dev(keys)
        k = torch.empty_like(src)
        tk = torch.empty_like(src)
        v = tv = vsrc = None
        if vals is not None:
            vsrc = dev(vals)
            v = torch.empty_like(vsrc)
            tv = torch.empty_like(vsrc)

        def restore():
            k.copy_(src)
            if vals is not None:
                v.copy_(vsrc)

        if vals is None:
            f = lambda: _native.call(fn, P(k.data_ptr()), P(tk.data_ptr()), n, o)  # noqa: E731
        else:
            f = lambda: _native.call(fn, P(k.data_ptr()), P(v.data_ptr()), P(tk.data_ptr()),  # noqa: E731
                                     P(tv.data_ptr()), n, o)
        restore()
        f()
        ms = _time_device(f, 5, stream, restore)
        _native.call("pa_stream_check", P(stream.cuda_stream))
        gbs = bytes_per_key * n / (ms / 1e3) / 1e9
        out[name] = {"ms": ms, "keys_per_s": n / (ms / 1e3), "bytes_per_key": bytes_per_key,
                     "achieved_gbs": gbs, "frac": gbs / peak}
        del src, k, tk, v, tv, vsrc
        torch.cuda.empty_cache()

    sort_case("sort_u32_presorted", workloads.presorted_u32(n))
    sort_case("sort_u32_constant42", workloads.constant_u32(n, 42))
    sort_case("sort_kv_u64_uniform_u32payload", workloads.uniform_u64(n), np.arange(n, dtype=np.uint32),
              "pa_sort_kv_u64", 200)
    sort_case("sort_kv_u64_zipf_u32payload", workloads.zipf_u64(n), np.arange(n, dtype=np.uint32),
              "pa_sort_kv_u64", 200)
    sort_case("sort_f32_normal_specials", workloads.normal_specials_f32(n).view(np.uint32), None, "pa_sort_f32", 36)

    for dname, keys in (("uniform", workloads.uniform_u32(n)), ("presorted", workloads.presorted_u32(n)),
                        ("constant42", workloads.constant_u32(n, 42))):
        d = dev(keys)
        hist = torch.zeros(256, dtype=torch.int64, device="cuda")
        res = torch.zeros(1, dtype=torch.int64, device="cuda")
        ms = _time_device(lambda: _native.call("pa_hist_one_byte_u32", P(d.data_ptr()), n, 0, P(hist.data_ptr()),
                                               o), 5, stream)
        out[f"histogram_low_digit_{dname}"] = {"ms": ms, "achieved_gbs": 4 * n / (ms / 1e3) / 1e9,
                                               "frac": 4 * n / (ms / 1e3) / 1e9 / peak}
        ms = _time_device(lambda: _native.call("pa_select_u32", P(d.data_ptr()), n, n // 2, P(res.data_ptr()), o),
                          5, stream)
        out[f"select_k_half_{dname}"] = {"ms": ms, "achieved_gbs_one_read": 4 * n / (ms / 1e3) / 1e9,
                                         "frac_one_read": 4 * n / (ms / 1e3) / 1e9 / peak}
        ms = _time_device(lambda: _native.call("pa_sum_u32", P(d.data_ptr()), n, P(res.data_ptr()), o), 5, stream)
        out[f"sum_u64_{dname}"] = {"ms": ms, "achieved_gbs": 4 * n / (ms / 1e3) / 1e9,
                                   "frac": 4 * n / (ms / 1e3) / 1e9 / peak}
        _native.call("pa_stream_check", P(stream.cuda_stream))
        del d
    # byte counting sort (CountingSortParallel.h:81), 400 MB of uniform bytes:
    # one histogram read + one fill write = 2 B/byte
    nb = 4 * n
    bsrc = torch.randint(0, 256, (nb,), dtype=torch.uint8, device="cuda",
                         generator=torch.Generator(device="cuda").manual_seed(1241))
    bw = torch.empty_like(bsrc)
    ms = _time_device(lambda: _native.call("pa_counting_sort_u8", P(bw.data_ptr()), nb, o), 5, stream,
                      lambda: bw.copy_(bsrc))
    ok = bool(torch.all(bw[1:] >= bw[:-1]))
    out["counting_sort_u8_400MB"] = {"ms": ms, "bytes_per_s_sorted": nb / (ms / 1e3), "bytes_per_key": 2,
                                     "achieved_gbs": 2 * nb / (ms / 1e3) / 1e9,
                                     "frac": 2 * nb / (ms / 1e3) / 1e9 / peak, "sorted": ok}
    del bsrc, bw
    # PartitionRadix around k = n/2 and n - 21 (RadixPartition.h:152), 100M uniform keys
    d = dev(workloads.uniform_u32(n))
    pw = torch.empty_like(d)
    kk = np.array([n - 21, n // 2], np.uint64)
    kk.sort()
    ms = _time_device(lambda: _native.call("pa_partition_radix_u32", P(pw.data_ptr()), n, P(kk.ctypes.data), kk.size,
                                           o), 5, stream, lambda: pw.copy_(d))
    out["partition_radix_2k_uniform"] = {"ms": ms, "keys_per_s": n / (ms / 1e3),
                                         "how": "one select per k, then one bucket pass (count, scan, write) and a copy back",
                                         "bytes_per_key": 4 * 2 + 4 + 8 + 8}
    # in-place MSD sort (RadixSortMsdParallel.h:291) holding the default
    # bounded scratch (2^24 keys) instead of a second array of n keys
    ms = _time_device(lambda: _native.call("pa_sort_u32_inplace", P(pw.data_ptr()), n, 0, o), 5, stream,
                      lambda: pw.copy_(d))
    ref_sorted = d.clone()
    _native.call("pa_sort_u32", P(ref_sorted.data_ptr()), None, n, o)
    torch.cuda.synchronize()
    out["sort_u32_inplace_bounded_scratch"] = {
        "ms": ms, "keys_per_s": n / (ms / 1e3), "scratch_bytes": 4 << 24, "plain_sort_second_buffer_bytes": 4 * n,
        "same_as_plain_sort": bool(torch.equal(pw, ref_sorted)),
        "how": "top digit partitioned in place in rounds through two 2^23-key scratch halves, bucket groups "
               "sorted by the batched segmented sort on the low three digits; includes the host's wait for "
               "the top digit's counts",
        "bytes_per_key": 4 + 16 + 4 + 3 * 8 + 8}
    del d, pw, ref_sorted
    out["batched_segmented_sort_4096_arrays"] = batched_extra(lib, _native, workloads, stream, peak)
    late = serving_in_own_process()
    sat = late["served_saturating"]
    out["serving_c5_after_other_workloads"] = {
        "when": "after the batched and 100M workloads above (the serving stream's slow mode)",
        "speedup_vs_plain_per_request": sat["speedup_vs_plain_per_request"], "makespan_s": sat["makespan_s"],
        "makespans_s_in_creation_order": sat["makespans_s_in_creation_order"], "p99_ms": sat["p99_ms"],
        "poisson_400_per_s_p99_ms": late["served_poisson_400_per_s"]["p99_ms"],
        "plain_seconds": late["plain_per_request"]["seconds"], "clocks": sat["clocks"],
        "host_link_gbs": late["host_link_gbs"]}
    return out


def serving_in_own_process() -> dict:
    """The C5 serving stream measured in a fresh process, as a serving
    process runs: in the bench process, after the other workloads, the
    servers' host-buffer makespans varied 36-96 ms from server to server
    while the same stream in a process of its own measured 37-61 ms."""
    import subprocess
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--serving-only"], capture_output=True, text=True,
                       timeout=900)
    if r.returncode != 0:
        raise RuntimeError(f"serving child failed ({r.returncode}): {r.stderr[-2000:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["process"] = "a child process of its own (bench.py --serving-only)"
    return out


def main():
    args = parse_args()
    if args.serving_only:
        from parallelalgorithms_gb300 import build
        build.build()
        print(json.dumps(serving_extra()))
    elif args.profile_op:
        profile_op(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gb300_arm(args)


if __name__ == "__main__":
    main()
