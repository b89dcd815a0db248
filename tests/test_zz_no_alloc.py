"""pa_sort_u32_noalloc, the sort entry point for callers that cannot
allocate GPU memory (a framework's caching allocator owns all of it, or a
cudaMalloc's device-wide synchronisation is not acceptable), checked
through the C ABI against pa_sort_u32 and the oracle restatement on the
same inputs.

Kept in a file of its own that pytest collects last.  Calls in a row show
that a call is unaffected by what the previous call left in the shared
scratch array."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_KEYS = 1 << 22


def _sort_both(lib, torch, a: np.ndarray):
    P = ctypes.c_void_p
    want = torch.from_numpy(a.view(np.int32).copy()).cuda()
    wtmp = torch.empty_like(want)
    assert lib.pa_sort_u32(P(want.data_ptr()), P(wtmp.data_ptr()), a.size, None) == 0
    got = torch.from_numpy(a.view(np.int32).copy()).cuda()
    gtmp = torch.empty_like(got)
    rc = lib.pa_sort_u32_noalloc(P(got.data_ptr()), P(gtmp.data_ptr()), a.size, None)
    assert rc == 0, lib.pa_last_error_message()
    torch.cuda.synchronize()
    return got.cpu().numpy().view(np.uint32), want.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_pa_sort_u32_two_calls_in_a_row(pa, port, torch_cuda):
    from parallelalgorithms_gb300 import workloads
    lib = pa.lib()
    first = workloads.uniform_u32(MAX_KEYS)                                   # the largest size allowed
    second = np.random.default_rng(5).integers(0, 1000, 1_000_003, dtype=np.uint32)  # smaller, many ties
    for a in (first, second):
        got, want = _sort_both(lib, torch_cuda, a)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(got, port.sort(a)[0])


@pytest.mark.parametrize("n", [1, 2, 6143, 6144, 8192, 8193, 12289])
def test_noalloc_sort_small_and_one_tile_sizes(pa, port, torch_cuda, n):
    """Sizes around the one-CTA shared-memory sort's limit (8192 keys) and the
    onesweep tile (6144 keys): the same result as pa_sort_u32 and the oracle."""
    lib = pa.lib()
    for seed in (n, n + 1):  # two calls in a row
        a = np.random.default_rng(seed).integers(0, 2**32, n, dtype=np.uint32)
        got, want = _sort_both(lib, torch_cuda, a)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(got, port.sort(a)[0])


def test_noalloc_sort_rejects_what_it_cannot_do_without_allocating(pa, torch_cuda):
    lib = pa.lib()
    P = ctypes.c_void_p
    host = np.zeros(16, np.uint32)
    dev = torch_cuda.zeros(16, dtype=torch_cuda.int32, device="cuda")
    # host buffers would need staging memory
    assert lib.pa_sort_u32_noalloc(P(host.ctypes.data), P(dev.data_ptr()), 16, None) == 1
    # above the fixed scratch's limit (checked before any device work)
    assert lib.pa_sort_u32_noalloc(P(dev.data_ptr()), P(dev.data_ptr()), MAX_KEYS + 1, None) == 1
    assert b"4,194,304" in lib.pa_last_error_message()
