"""GPU path vs the CPU oracle, bit-exact, through the C ABI.

Inputs are seeded and sized so the oracle finishes in seconds; sizes sit on
both sides of every tile boundary the kernels use (8192 keys for 32-bit
keys, 6144 for 32-bit key+payload and 64-bit keys, 4096 for 64-bit
key+payload) and below the reference's insertion-sort cutoff (100).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 7, 99, 100, 101, 1000, 4095, 4096, 4097, 6143, 6144, 6145, 8191, 8192, 8193, 16385, 65536,
         100003, 1 << 20, 3_000_017]


def u32_inputs(n: int) -> dict[str, np.ndarray]:
    from parallelalgorithms_gb300 import workloads
    rng = np.random.default_rng(n)
    nearly = np.arange(n, dtype=np.uint32)
    nearly[::100] = 0x1010
    return {
        "uniform": workloads.uniform_u32(n),
        "presorted": np.arange(n, dtype=np.uint32),
        "descending": np.arange(n, dtype=np.uint32)[::-1].copy(),
        "constant": np.full(n, 42, np.uint32),
        "nearly": nearly,
        "few": rng.integers(0, 16, n, dtype=np.uint32),
        "high_byte": (rng.integers(0, 256, n, dtype=np.uint32) << np.uint32(24)),
        "max": np.full(n, 0xFFFFFFFF, np.uint32),
    }


def to_dev(torch, a: np.ndarray):
    view = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64, np.dtype(np.float32): np.float32,
            np.dtype(np.uint8): np.uint8}[a.dtype]
    return torch.from_numpy(a.view(view).copy()).cuda()


def from_dev(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(dtype)


@pytest.mark.parametrize("n", SIZES)
def test_sort_u32_host_and_device_match_oracle(pa, port, torch_cuda, n):
    for name, a in u32_inputs(n).items():
        want, _ = port.sort(a)
        h = a.copy()
        pa.SortRadixPar(h, np.empty_like(h), n)
        np.testing.assert_array_equal(h, want, err_msg=f"host {name} n={n}")
        d = to_dev(torch_cuda, a)
        pa.sort(d)
        torch_cuda.cuda.synchronize()
        np.testing.assert_array_equal(from_dev(d, np.uint32), want, err_msg=f"device {name} n={n}")


@pytest.mark.parametrize("n", [1, 100, 4097, 6144, 6145, 8192, 8193, 65537, 1 << 20])
def test_sort_kv_u32_stable(pa, port, n):
    for name, a in u32_inputs(n).items():
        vals = np.arange(n, dtype=np.uint32)
        wk, wv = port.sort(a, vals)
        k, v = a.copy(), vals.copy()
        pa.sort(k, v)
        np.testing.assert_array_equal(k, wk, err_msg=name)
        np.testing.assert_array_equal(v, wv, err_msg=name)


@pytest.mark.parametrize("n", [1, 99, 4096, 4097, 6143, 6144, 6145, 100003, 1 << 20])
def test_sort_u64_and_kv_u64(pa, port, n):
    from parallelalgorithms_gb300 import workloads
    rng = np.random.default_rng(7 + n)
    cases = {
        "uniform": workloads.uniform_u64(n),
        "zipf": workloads.zipf_u64(n),
        "top_byte": rng.integers(0, 256, n, dtype=np.uint64) << np.uint64(56),
        "constant": np.full(n, 0xDEADBEEFCAFEF00D, np.uint64),
        "small": rng.integers(0, 1000, n, dtype=np.uint64),
    }
    for name, a in cases.items():
        want, _ = port.sort(a)
        k = a.copy()
        pa.sort(k)
        np.testing.assert_array_equal(k, want, err_msg=name)
        vals = np.arange(n, dtype=np.uint32)
        wk, wv = port.sort(a, vals)
        k, v = a.copy(), vals.copy()
        pa.sort(k, v)
        np.testing.assert_array_equal(k, wk, err_msg=name)
        np.testing.assert_array_equal(v, wv, err_msg=name)


@pytest.mark.parametrize("n", [1, 2, 100, 8192, 8193, 100003, 1 << 20])
def test_sort_f32_total_order_and_payload(pa, port, torch_cuda, n):
    from parallelalgorithms_gb300 import workloads
    a = workloads.normal_specials_f32(n)
    want, _ = port.sort(a)
    k = a.copy()
    pa.sort(k)
    np.testing.assert_array_equal(k.view(np.uint32), want.view(np.uint32))
    vals = np.arange(n, dtype=np.uint32)
    wk, wv = port.sort(a, vals)
    k, v = a.copy(), vals.copy()
    pa.sort(k, v)
    np.testing.assert_array_equal(k.view(np.uint32), wk.view(np.uint32))
    np.testing.assert_array_equal(v, wv)
    d = to_dev(torch_cuda, a)
    pa.sort(d)
    np.testing.assert_array_equal(from_dev(d, np.float32).view(np.uint32), want.view(np.uint32))


def test_sort_f32_all_equal_digits_skips_passes(pa, port):
    # constant float keys: every pass is trivial, the transform must not leak
    for v in (-0.0, 0.0, -1.5, np.inf):
        a = np.full(10001, v, np.float32)
        k = a.copy()
        pa.sort(k)
        np.testing.assert_array_equal(k.view(np.uint32), a.view(np.uint32))
    # one non-trivial pass only (low byte differs), negative numbers
    base = np.float32(-1.0).view(np.uint32)
    a = (base + np.random.default_rng(1).integers(0, 200, 50000, dtype=np.uint32)).view(np.float32)
    want, _ = port.sort(a)
    k = a.copy()
    pa.sort(k)
    np.testing.assert_array_equal(k.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("n", [1, 99, 8192, 8193, 100003, 1 << 20])
def test_histograms_match_oracle(pa, port, n):
    for name, a in u32_inputs(n).items():
        np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(a, 0, n - 1),
                                      port.hist_byte_components(a, 0, n - 1), err_msg=name)
        for sh in (0, 5, 8, 16, 24, 31):
            np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(a, 0, n - 1, sh),
                                          port.hist_one_byte(a, 0, n - 1, sh), err_msg=f"{name} shift {sh}")
        if n > 10:
            l, r = 3, n - 5
            np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(a, l, r),
                                          port.hist_byte_components(a, l, r), err_msg=name)
        u8 = (a & np.uint32(0xFF)).astype(np.uint8)
        np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(u8, 0, n), port.hist_u8(u8, 0, n))
        if n > 20:
            np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(u8, 7, n - 3),
                                          port.hist_u8(u8, 7, n - 3))


@pytest.mark.parametrize("n", [1, 1000, 100003])
def test_quanta_histogram_and_start_of_bins(pa, port, n):
    a = u32_inputs(n)["uniform"]
    for wq in (1, 7, 4096, max(1, n // 3), n):
        q = (n - 1) // wq + 1
        for byte in range(4):
            np.testing.assert_array_equal(pa.HistogramByteComponentsQCPar(a, 0, n - 1, wq, q, byte),
                                          port.hist_qc(a, 0, n - 1, wq, q, byte))
            np.testing.assert_array_equal(pa.ComputeStartOfBinsPar(a, n, wq, q, byte),
                                          port.start_of_bins(a, n, wq, q, byte))
        if n > 10:
            np.testing.assert_array_equal(pa.HistogramByteComponentsQCPar(a, 2, n - 3, wq, q, 1),
                                          port.hist_qc(a, 2, n - 3, wq, q, 1))


@pytest.mark.parametrize("n", [1, 2, 99, 100, 8193, 100003, 1 << 20, 3_000_017])
def test_select_matches_oracle(pa, port, n):
    for name, a in u32_inputs(n).items():
        for k in sorted({0, n // 2, max(0, n - 21), n - 1}):
            want = port.select(a, k)
            assert pa.select(a, k) == want, (name, k)
            c = a.copy()
            assert pa.SelectRadix(c, n, k) == want
            assert c[k] == want  # the reference leaves the k-th element at a[k]
            # only a[k] and the first element holding the answer may trade places
            np.testing.assert_array_equal(np.sort(c), np.sort(a))
            assert np.count_nonzero(c != a) in (0, 2)
    if n > 100:
        a = u32_inputs(n)["uniform"]
        start, length = 17, n - 40
        k = start + length // 3
        c = a.copy()
        assert pa.SelectRadix(c, start, length, k) == port.select(a, k, start=start, length=length)
        np.testing.assert_array_equal(np.sort(c), np.sort(a))
        np.testing.assert_array_equal(c[:start], a[:start])
        np.testing.assert_array_equal(c[start + length:], a[start + length:])


@pytest.mark.parametrize("n", [1, 1000, 1 << 20])
def test_select_radix_device_array_stays_a_permutation(pa, port, torch_cuda, n):
    """SelectRadix on a device array: a[k] holds the answer, a[k] and the
    first element holding the answer traded places, nothing else moved."""
    for name, a in u32_inputs(n).items():
        k = n // 3
        want = port.select(a, k)
        d = torch_cuda.from_numpy(a.view(np.int32).copy()).cuda()
        assert pa.SelectRadix(d, n, k) == want
        c = d.cpu().numpy().view(np.uint32)
        assert c[k] == want, name
        diff = np.flatnonzero(c != a)
        assert diff.size in (0, 2), name
        if diff.size:
            j = diff[diff != k][0]
            assert a[j] == want and c[j] == a[k]
            assert not np.any(a[:j] == want)  # the first place that held it


def test_select_sample_bracket_paths(pa, port):
    """Select reads the input once against a bracket [lo, hi] taken from 8192
    keys at even strides (position (j n + n / 2) / 8192).  Inputs here put
    rank k at lo or hi, between them, outside them (the strided sample sees
    only one value), and make the keys between them overflow the candidate
    buffer; every case must give the oracle's answer."""
    rng = np.random.default_rng(77)
    n = 8192 * 4  # sampled positions are 2 (mod 4)
    sampled = np.zeros(n, bool)
    sampled[2::4] = True
    # the sample sees only zeros: the bracket collapses to [0, 0] and rank n/2 lies above it
    a = rng.integers(1 << 20, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    a[sampled] = 0
    # the sample spreads over all 32 bits, the other keys crowd the middle: the
    # keys strictly inside the bracket outnumber the candidate buffer
    b = rng.integers((1 << 31) - (1 << 26) + 1, (1 << 31) + (1 << 26), n, dtype=np.uint64).astype(np.uint32)
    b[sampled] = np.arange(8192, dtype=np.uint32) << np.uint32(19)
    # a handful of values: rank k usually falls on lo or hi themselves
    c = rng.integers(0, 5, n, dtype=np.uint32) * np.uint32(1000)
    # 60 % zeros then 40 % 77s in every ten keys: rank 0.61 n is the bracket's hi
    d = (np.arange(n) % 10 >= 6).astype(np.uint32) * np.uint32(77)
    for name, x in (("sample_zeros", a), ("overflow", b), ("five_values", c), ("two_values", d)):
        for k in sorted({0, 1, n // 4, n // 2, n // 2 + 1, int(n * 0.61), 3 * n // 4, n - 2, n - 1}):
            assert pa.select(x, k) == port.select(x, k), (name, k)
    for m in (100003, 1 << 20):  # many ranks of a uniform and a Zipf input
        u = u32_inputs(m)["uniform"]
        z = np.minimum(rng.zipf(1.3, m), 1 << 31).astype(np.uint32)
        for k in rng.integers(0, m, 12):
            assert pa.select(u, int(k)) == port.select(u, int(k)), ("uniform", m, k)
            assert pa.select(z, int(k)) == port.select(z, int(k)), ("zipf", m, k)
    a64 = a.astype(np.uint64) << np.uint64(31)
    for k in (0, n // 2, n - 1):
        assert pa.select(a64, k) == port.select(a64, k), ("sample_zeros_u64", k)


@pytest.mark.parametrize("n", [1, 99, 100003, 1 << 20])
def test_select_u64(pa, port, n):
    from parallelalgorithms_gb300 import workloads
    for a in (workloads.uniform_u64(n), workloads.zipf_u64(n), np.full(n, 7, np.uint64)):
        for k in sorted({0, n // 3, n - 1}):
            assert pa.select(a, k) == port.select(a, k)


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 17, 100003, 1 << 20, 3_000_017])
def test_sum_matches_oracle(pa, port, torch_cuda, n):
    a = u32_inputs(max(n, 1))["uniform"][:n]
    assert pa.SumParallelNonRecursive(a, 0, n) == port.sum(a)
    m = np.full(n, 0xFFFFFFFF, np.uint32)
    assert pa.SumParallelNonRecursive(m, 0, n) == port.sum(m)
    w = np.full(n, 0xFFFFFFFFFFFFFFFF, np.uint64)  # wraps modulo 2^64
    assert pa.SumParallel(w, 0, n) == port.sum(w)
    if n > 10:
        assert pa.SumParallelNonRecursive(a, 3, n - 2) == port.sum(a, 3, n - 2)
        s = pa.SumParallel(a, 0, n)
        assert s == np.int64(np.uint64(port.sum(a)))
        d = to_dev(torch_cuda, a)
        assert pa.sum_u64(d) == port.sum(a)
        assert pa.sum_u64(d[1:]) == port.sum(a, 1, n)  # unaligned start


def test_two_phase_leaves_result_in_both(pa, port):
    a = u32_inputs(50001)["uniform"]
    want, _ = port.sort(a)
    x, b = a.copy(), np.zeros_like(a)
    pa.RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(x, b, a.size)
    np.testing.assert_array_equal(x, want)
    np.testing.assert_array_equal(b, want)


def test_unaligned_device_buffers(pa, port, torch_cuda):
    # tiles of a buffer that does not start on 16 bytes take the plain-load path
    a = u32_inputs(100003)["uniform"]
    want, _ = port.sort(a[1:])
    base = to_dev(torch_cuda, a)
    view = base[1:]
    pa.sort(view)
    np.testing.assert_array_equal(from_dev(view, np.uint32), want)


def test_select_unaligned_device_buffers(pa, port, torch_cuda):
    # a device view that does not start on 16 bytes: its head and tail are read
    # with plain loads, the rest with 16-byte vectors
    for n in (5, 100003, 1 << 20):
        a = u32_inputs(n + 3)["uniform"]
        base = to_dev(torch_cuda, a)
        for off in (1, 2, 3):
            m = n + 3 - off
            view = base[off:]
            for k in sorted({0, m // 2, m - 1}):
                assert pa.select(view, k) == port.select(a[off:], k), (n, off, k)
        a64 = np.arange(n + 1, dtype=np.uint64)[::-1].copy()
        v64 = torch_cuda.from_numpy(a64.view(np.int64)).cuda()[1:]
        assert pa.select(v64, n // 3) == port.select(a64[1:], n // 3)


def test_repeated_calls_reuse_workspace(pa, port):
    for n in (100003, 5, 1 << 20, 100003, 3):
        a = u32_inputs(n)["uniform"]
        want, _ = port.sort(a)
        k = a.copy()
        pa.sort(k)
        np.testing.assert_array_equal(k, want)


@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 4099, 100003, 1 << 20, 10_000_019])
def test_counting_sort_u8(pa, port, torch_cuda, n):
    """counting_sort_parallel (CountingSortParallel.h:81) against the oracle:
    host arrays, uniform / skewed / single-value bytes, and device views that
    start off a 16-byte boundary (the fill's head and tail bytes)."""
    rng = np.random.default_rng(4100 + n)
    cases = {"uniform": rng.integers(0, 256, n, dtype=np.uint8),
             "skewed": np.minimum(rng.geometric(0.05, n), 255).astype(np.uint8),
             "single": np.full(n, 77, np.uint8)}
    for name, a in cases.items():
        want = port.counting_sort_u8(a)
        got = a.copy()
        pa.counting_sort_parallel(got)
        np.testing.assert_array_equal(got, want, err_msg=name)
    a = cases["uniform"]
    if n > 40:
        l, r = 5, n - 3
        got = a.copy()
        pa.counting_sort_parallel_inner(got, l, r)
        want = a.copy()
        want[l:r] = port.counting_sort_u8(a[l:r])
        np.testing.assert_array_equal(got, want)
        base = torch_cuda.from_numpy(a.copy()).cuda()
        for off in (1, 7):
            view = base[off:]
            pa.counting_sort_parallel(view)
            np.testing.assert_array_equal(view.cpu().numpy(), port.counting_sort_u8(base.cpu().numpy()[off:]))


@pytest.mark.parametrize("n", [1, 2, 48, 100003, 1 << 20])
def test_partition_radix(pa, port, ref, n):
    """PartitionRadix (RadixPartition.h:92, :124, :152, :165): every listed
    a[k] equals the reference's (the k-th smallest), nothing before it is
    larger and nothing after it is smaller, and the keys are a permutation
    of the input."""
    rng = np.random.default_rng(4200 + n)
    a = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    ks = sorted({0, n // 3, n // 2, n - 1})
    got = a.copy()
    pa.PartitionRadix(got, n, np.array(ks, np.uint64))
    want = port.partition_radix(a, ks)
    if ref is not None:
        np.testing.assert_array_equal(want, ref.partition_radix(a, ks))
    for k in ks:
        assert got[k] == want[k]
        assert np.all(got[:k] <= got[k]) and np.all(got[k + 1:] >= got[k])
    np.testing.assert_array_equal(np.sort(got), np.sort(a))
    k = n // 2
    assert pa.PartitionRadix(a.copy(), n, k) == int(np.sort(a)[k])
    if n > 10:
        start, length = 3, n - 5
        c = a.copy()
        v = pa.PartitionRadix(c, start, length, start + length // 2)
        assert v == int(np.sort(a[start:start + length])[length // 2])
        np.testing.assert_array_equal(c[:start], a[:start])
        np.testing.assert_array_equal(c[start + length:], a[start + length:])


@pytest.mark.parametrize("nk", [1, 2, 3, 6, 7, 12])
@pytest.mark.parametrize("dist", ["uniform", "few", "presorted", "constant"])
def test_partition_radix_select_and_sort_paths(pa, port, torch_cuda, nk, dist):
    """Up to six k go through one select per k and a bucket pass, more k
    through a sort: either way every listed a[k] is the oracle's, the parts
    hold, and the keys are a permutation of the input (host and device)."""
    n = 300_007
    rng = np.random.default_rng(nk)
    a = {"uniform": rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32),
         "few": rng.integers(0, 5, n, dtype=np.uint32),
         "presorted": np.arange(n, dtype=np.uint32),
         "constant": np.full(n, 42, np.uint32)}[dist]
    ks = np.unique(rng.integers(0, n, nk)).astype(np.uint64)
    if ks.size < nk:  # keep exactly nk distinct k (repeats are allowed by the contract, but test the count)
        ks = np.linspace(0, n - 1, nk).astype(np.uint64)
    srt = np.sort(a)
    for dev in (False, True):
        got = a.copy()
        if dev:
            t = torch_cuda.from_numpy(got.view(np.int32)).cuda()
            pa.PartitionRadix(t, n, ks)
            got = t.cpu().numpy().view(np.uint32)
        else:
            pa.PartitionRadix(got, n, ks)
        for k in ks.tolist():
            assert got[k] == srt[k], (dev, k)
            assert np.all(got[:k] <= got[k]) and np.all(got[k + 1:] >= got[k])
        np.testing.assert_array_equal(np.sort(got), srt)
    want = port.partition_radix(a, ks)
    for k in ks.tolist():
        assert want[k] == srt[k]


@pytest.mark.parametrize("n", [1, 2, 100003, 1 << 20])
def test_radix_leaf_merge_sorts(pa, ref, torch_cuda, n):
    """parallel_merge_sort_hybrid_radix (ParallelMergeSort.h:287) with the
    result in dst or in src, on a sub-range, and
    parallel_linear_in_place_preventative_adaptive_sort (:549): the same
    sorted keys as the compiled reference."""
    rng = np.random.default_rng(4400 + n)
    a = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    want = np.sort(a)
    if ref is not None:
        s_ref, d_ref = a.copy(), np.zeros_like(a)
        ref.merge_sort_hybrid_radix(s_ref, 0, n - 1, d_ref, True)
        np.testing.assert_array_equal(d_ref, want)
    src, dst = a.copy(), np.zeros_like(a)
    pa.parallel_merge_sort_hybrid_radix(src, 0, n - 1, dst, True)
    np.testing.assert_array_equal(dst, want)
    src, work = a.copy(), np.zeros_like(a)
    pa.parallel_merge_sort_hybrid_radix(src, 0, n - 1, work, False)
    np.testing.assert_array_equal(src, want)
    c = a.copy()
    pa.parallel_linear_in_place_preventative_adaptive_sort(c)
    np.testing.assert_array_equal(c, want)
    c = a.copy()
    pa.parallel_hybrid_inplace_msd_radix_sort(c)
    np.testing.assert_array_equal(c, want)
    if ref is not None:
        m = a.copy()
        ref.msd_radix_sort(m)
        np.testing.assert_array_equal(m, want)
    if n > 10:  # sub-range [l, r] inclusive, device buffers
        l, r = 3, n - 4
        ds = torch_cuda.from_numpy(a.view(np.int32).copy()).cuda()
        dd = torch_cuda.zeros_like(ds)
        pa.parallel_merge_sort_hybrid_radix(ds, l, r, dd, True)
        got = dd.cpu().numpy().view(np.uint32)
        np.testing.assert_array_equal(got[l:r + 1], np.sort(a[l:r + 1]))
        assert not got[:l].any() and not got[r + 1:].any()


TYPED = [np.uint8, np.int8, np.uint16, np.int16, np.uint32, np.int32, np.uint64, np.int64, np.float32, np.float64]


def _typed_input(dtype, n, seed):
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.floating):
        a = (rng.standard_normal(n) * 1e6).astype(dtype)
        if n > 10:
            a[3], a[7] = dtype(-0.0), dtype(2.5e9)
        return a
    info = np.iinfo(dtype)
    return rng.integers(info.min, info.max, n, dtype=dtype, endpoint=True)


def _template_sum(a) -> int:
    """template SumParallel<_Type> (SumParallel.h:207-237): each element cast
    to long long (floats truncated toward zero), summed modulo 2^64, read as
    signed; the unsigned long long overload (:162) returns the unsigned sum."""
    if a.dtype == np.uint64:
        return int(np.sum(a, dtype=np.uint64))
    w = np.trunc(a).astype(np.int64) if np.issubdtype(a.dtype, np.floating) else a.astype(np.int64)
    return int(np.sum(w, dtype=np.int64))


@pytest.mark.parametrize("dtype", TYPED)
@pytest.mark.parametrize("n", [0, 1, 17, 4097, 1_000_003])
def test_typed_sum_is_the_template_sum(pa, dtype, n):
    a = _typed_input(dtype, n, n + 7)
    assert pa.SumParallel(a, 0, n) == _template_sum(a)
    if n > 10:
        assert pa.SumParallel(a, 3, n - 2) == _template_sum(a[3:n - 2])  # unaligned start


def test_typed_sum_against_the_compiled_reference(pa, ref):
    for dtype in (np.uint8, np.uint32, np.int32, np.float32):
        for n in (1, 1000, 1_000_003):
            a = _typed_input(dtype, n, n)
            assert pa.SumParallel(a, 0, n) == ref.sum_template(a), (dtype, n)


@pytest.mark.parametrize("n,threshold", [(1, 16384), (100_000, 16384), (1_000_003, 1000), (65536, 16384),
                                         (5, 1)])
def test_chunked_sums_fill_the_callers_sum_array(pa, ref, n, threshold):
    a = workloads_u32(n)
    l, r = (2, n - 1) if n > 4 else (0, n)
    tasks = -(-(r - l) // threshold)
    arr = np.zeros(tasks, np.uint64)
    total = pa.SumParallelNonRecursive(a, l, r, arr, threshold)
    want_total, want_arr = ref.sum_nonrec_array(a, l, r, threshold)
    assert total == want_total
    np.testing.assert_array_equal(arr, want_arr)


def workloads_u32(n):
    from parallelalgorithms_gb300 import workloads
    return workloads.uniform_u32(n)


@pytest.mark.parametrize("n", [8193, 100_003, 1 << 20, 3_000_017])
def test_sort_11bit_digits(pa, port, torch_cuda, n):
    """11-bit digits (2048 bins; three passes for 32-bit keys, six for 64-bit):
    the same stable result as the oracle's 11-bit restatement and as the 8-bit
    sort, for every key type, with a payload, on host and device buffers."""
    rng = np.random.default_rng(n)
    u32 = u32_inputs(n)
    for name in ("uniform", "presorted", "few", "high_byte", "max"):
        a = u32[name]
        got = a.copy()
        pa.sort(got, digit_bits=11)
        want = port.sort(a, digit_bits=11)[0]
        np.testing.assert_array_equal(got, want, err_msg=name)
        np.testing.assert_array_equal(want, port.sort(a)[0])
    k64 = rng.integers(0, 2 ** 64, n, dtype=np.uint64)
    k64[::7] = k64[3]  # ties for stability
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = k64.copy(), vals.copy()
    pa.sort(gk, gv, digit_bits=11)
    wk, wv = port.sort(k64, vals, digit_bits=11)
    np.testing.assert_array_equal(gk, wk)
    np.testing.assert_array_equal(gv, wv)
    f = (rng.standard_normal(n) * 1e3).astype(np.float32)
    f[::11] = -0.0
    f[5::13] = 0.0
    gf, gfv = f.copy(), vals.copy()
    pa.sort(gf, gfv, digit_bits=11)
    wf, wfv = port.sort(f, vals, digit_bits=11)
    np.testing.assert_array_equal(gf.view(np.uint32), wf.view(np.uint32))
    np.testing.assert_array_equal(gfv, wfv)
    d = to_dev(torch_cuda, u32["uniform"])
    pa.sort(d, digit_bits=11)
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), port.sort(u32["uniform"])[0])
