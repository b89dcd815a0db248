"""Host-buffer sorts of 2^24 keys or more take the pipelined path (chunked
copy-in; each chunk sorted on its top 16 bits (32-bit keys) or split on its
top byte (64-bit keys) as it arrives; groups of top-byte buckets finished and
copied out in turn).  Its result must equal the oracle's bit for bit, for
inputs that exercise the grouping and both ways a 32-bit group is finished:
uniform, presorted, constant, two buckets only, a heavy bucket beside light
ones, buckets at the shared-memory sort's size limits, and 64-bit keys."""
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


def test_pipelined_bucket_sizes_at_the_shared_memory_limits(pa, port):
    """32-bit groups whose 16-bit buckets (keys sharing their top 16 bits)
    all hold at most 8192 keys are sorted bucket by bucket in shared memory,
    by a 2048-, 4096- or 8192-key tile picked from the group's largest
    bucket; a group with a larger bucket falls back to the batched sort.
    Buckets of exactly 2048, 2049, 4096, 4097, 8192 and 8193 keys, each in a
    top byte of its own, exercise every boundary."""
    from parallelalgorithms_gb300 import workloads
    u = workloads.uniform_u32(N)
    rng = np.random.default_rng(3)
    donors = np.flatnonzero((u >> np.uint32(24)) >= 0x80)  # keys moved into the buckets below
    used = 0
    for top16, size in ((0x1100, 2048), (0x2200, 2049), (0x3300, 4096), (0x4400, 4097), (0x5500, 8192),
                        (0x6600, 8193)):
        need = size - int(np.count_nonzero((u >> np.uint32(16)) == top16))
        pick = donors[used:used + need]
        used += need
        u[pick] = (np.uint32(top16) << np.uint32(16)) | rng.integers(0, 1 << 16, need, dtype=np.uint32)
        assert int(np.count_nonzero((u >> np.uint32(16)) == top16)) == size
    want, _ = port.sort(u)
    got = u.copy()
    pa.sort(got)
    np.testing.assert_array_equal(got, want)


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


def test_pipeline_out_of_memory_falls_back_to_the_plain_host_sort(tmp_path):
    """With the pipeline's allocation failing (host-side fault injection),
    the same call still sorts through the two-buffer host path."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    script = tmp_path / "oom_fallback.py"
    script.write_text(
        "import sys\n"
        f"sys.path.insert(0, {str(root)!r})\n"
        "import numpy as np\n"
        "import parallelalgorithms_gb300 as pa\n"
        "from parallelalgorithms_gb300 import workloads\n"
        f"a = workloads.uniform_u32({N})\n"
        "got = a.copy()\n"
        "pa.sort(got)\n"
        "assert np.array_equal(got, np.sort(a))\n"
        "print('fallback ok')\n")
    env = dict(os.environ, PA_FAULT_PIPELINE_OOM="1")
    r = subprocess.run([sys.executable, str(script)], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fallback ok" in r.stdout
