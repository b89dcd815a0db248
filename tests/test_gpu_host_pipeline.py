"""Host-buffer sorts of 2^24 keys or more take the pipelined path (chunked
copy-in with top-digit counts, one top-digit pass, bucket groups sorted and
copied out in turn).  Its result must equal the oracle's bit for bit, for
inputs that exercise the grouping: uniform, presorted, constant (one bucket
holds every key: the top-digit pass is skipped), two buckets only, a
heavy bucket beside light ones, and 64-bit keys."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = (1 << 24) + 12345  # above the pipeline threshold, not a multiple of the chunking


def _inputs():
    from parallelalgorithms_gb300 import workloads
    u = workloads.uniform_u32(N)
    two = np.where(u & 1, np.uint32(0x7F000000), np.uint32(0x01000000)) | (u & 0xFFFF)
    heavy = u.copy()
    heavy[: N // 2] &= 0x00FFFFFF  # half the keys in bucket 0
    return {"uniform": u, "presorted": workloads.presorted_u32(N), "constant": workloads.constant_u32(N, 42),
            "two_buckets": two.astype(np.uint32), "heavy_bucket": heavy}


@pytest.mark.parametrize("name", ["uniform", "presorted", "constant", "two_buckets", "heavy_bucket"])
def test_pipelined_host_sort_u32(pa, port, name):
    a = _inputs()[name]
    want, _ = port.sort(a)
    got = a.copy()
    pa.sort(got)
    np.testing.assert_array_equal(got, want)
    # the same call with a reference-style host scratch buffer
    got2, tmp = a.copy(), np.zeros_like(a)
    pa.SortRadixPar(got2, tmp, a.size)
    np.testing.assert_array_equal(got2, want)


def test_pipelined_host_sort_u64(pa, port):
    from parallelalgorithms_gb300 import workloads
    for a in (workloads.uniform_u64(N), workloads.zipf_u64(N)):
        want, _ = port.sort(a)
        got = a.copy()
        pa.sort(got)
        np.testing.assert_array_equal(got, want)


def test_pipelined_equals_device_sort_100m(pa, torch_cuda):
    from parallelalgorithms_gb300 import workloads
    a = workloads.uniform_u32(100_000_000)
    d = torch_cuda.from_numpy(a.view(np.int32)).cuda()
    pa.sort(d)
    host = a.copy()
    pa.sort(host)
    np.testing.assert_array_equal(host, d.cpu().numpy().view(np.uint32))
