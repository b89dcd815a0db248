"""Minimal driver for profiling one operation of the radix path under ncu.

    python -m parallelalgorithms_gb300.profile --op sort_u32 --n 50000000 --reps 2

Generates the seeded input once, keeps it device-resident, and runs the
operation `reps` times with nothing else on the GPU, so that an ncu launch
filter (-k regex:onesweep -s <skip> -c <count>) lands on known launches.
Per sort: one digit histogram, one scan, one onesweep launch per key byte,
one final copy (plus the workspace memset).  `sort_u32_host` sorts a
page-locked host copy of the keys through the C ABI instead (the pipelined
host-buffer path: chunk passes, bucket bounds and totals, group sorts, with
the copies between them).
"""
from __future__ import annotations

import argparse
import ctypes

import numpy as np


def main() -> None:
    p = argparse.ArgumentParser()
    p.add_argument("--op", default="sort_u32",
                   choices=["sort_u32", "sort_u32_host", "sort_u64", "sort_kv_u64", "sort_f32", "hist_u32", "select_u32",
                            "sum_u32"])
    p.add_argument("--n", type=int, default=50_000_000)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--dist", default="uniform", choices=["uniform", "presorted", "constant"])
    a = p.parse_args()

    import torch

    from . import _native, build, workloads
    build.build()
    lib = _native.lib()
    P = ctypes.c_void_p
    n = a.n
    if a.op in ("sort_kv_u64", "sort_u64"):
        keys = workloads.uniform_u64(n)
    elif a.op == "sort_f32":
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
    if a.op == "sort_kv_u64":
        v = torch.arange(n, dtype=torch.int32, device="cuda")
        tv = torch.empty_like(v)
    out = torch.zeros(256, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    o = _native.opts(stream.cuda_stream)
    host_t = host = None
    if a.op == "sort_u32_host":
        host_t = torch.empty(n, dtype=torch.int32, pin_memory=True)  # (kept alive for the view below)
        host = host_t.numpy().view(np.uint32)
    for _ in range(a.reps):
        k.copy_(src)
        if a.op == "sort_u32_host":
            np.copyto(host, keys)
            _native.call("pa_sort_u32", P(host.ctypes.data), None, n, None)
        elif a.op == "sort_u32":
            _native.call("pa_sort_u32", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif a.op == "sort_f32":
            _native.call("pa_sort_f32", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif a.op == "sort_u64":
            _native.call("pa_sort_u64", P(k.data_ptr()), P(t.data_ptr()), n, o)
        elif a.op == "sort_kv_u64":
            _native.call("pa_sort_kv_u64", P(k.data_ptr()), P(v.data_ptr()), P(t.data_ptr()), P(tv.data_ptr()), n, o)
        elif a.op == "hist_u32":
            _native.call("pa_hist_byte_components_u32", P(k.data_ptr()), n, P(out.data_ptr()), o)
        elif a.op == "select_u32":
            _native.call("pa_select_u32", P(k.data_ptr()), n, n // 2, P(out.data_ptr()), o)
        elif a.op == "sum_u32":
            _native.call("pa_sum_u32", P(k.data_ptr()), n, P(out.data_ptr()), o)
    torch.cuda.synchronize()
    print(f"profile driver done: op={a.op} n={n} reps={a.reps}")


if __name__ == "__main__":
    main()
