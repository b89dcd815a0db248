"""Sizes past 2^30 keys, where the look-back status words switch from
32-bit (2-bit flag + 30-bit count) to 64-bit: sort, select and sum of
2^30 + 4099 device-resident uint32 keys, checked with independent torch
computations (sortedness, every byte's histogram, the sum, the k-th value
by counting)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = (1 << 30) + 4099


def _u32(t):
    """int32 tensor holding uint32 bits -> int64 tensor of the unsigned values."""
    return t.to(__import__("torch").int64) & 0xFFFFFFFF


def test_sort_select_sum_past_2_30(pa, torch_cuda):
    torch = torch_cuda
    g = torch.Generator(device="cuda")
    g.manual_seed(1240)
    src = torch.randint(-(2 ** 31), 2 ** 31, (N,), dtype=torch.int32, device="cuda", generator=g)
    want_sum = int(_u32(src).sum().item())
    hist_before = [torch.bincount((_u32(src) >> (8 * b)) & 255, minlength=256) for b in range(4)]

    # select k = n/2 and k = n - 21 (non-destructive on device memory)
    for k in (N // 2, N - 21):
        got = pa.select(src, k)
        v = got
        below = int((_u32(src) < v).sum().item())
        equal = int((_u32(src) == v).sum().item())
        assert below <= k < below + equal, (k, v, below, equal)
    assert pa.SumParallelNonRecursive(src, 0, N) == want_sum

    keys = src.clone()
    del src
    pa.sort(keys)
    u = _u32(keys)
    assert bool(torch.all(u[1:] >= u[:-1]))
    for b in range(4):
        assert torch.equal(torch.bincount((u >> (8 * b)) & 255, minlength=256), hist_before[b])
    assert int(u.sum().item()) == want_sum
