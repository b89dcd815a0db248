"""The 100M-key workloads (uniform, presorted 0..n-1, constant 42; 64-bit
keys with payload; float32 with specials) on the GPU, checked bit-exact
against the reference's own code compiled unchanged (SortRadixPar,
HistogramOneByteComponentParallel, HistogramByteComponentsParallel,
SelectRadix and SumParallelNonRecursive on this host's cores, tens of ms
each at this size), against the oracle restatement, against numpy's stable
argsort for the key + index payload case, and through size-independent
properties: sortedness, histogram and sum invariance under the permutation,
stability of the index payload."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 100_000_000


@pytest.fixture(scope="module")
def inputs():
    from parallelalgorithms_gb300 import workloads
    return {"uniform": workloads.uniform_u32(N), "presorted": workloads.presorted_u32(N),
            "constant": workloads.constant_u32(N, 42)}


@pytest.mark.parametrize("dist", ["uniform", "presorted", "constant"])
def test_u32_100m_sort_histogram_select_sum(pa, port, torch_cuda, inputs, dist):
    a = inputs[dist]
    d = torch_cuda.from_numpy(a.view(np.int32)).cuda()
    pa.sort(d)
    got = d.cpu().numpy().view(np.uint32)
    assert np.all(got[1:] >= got[:-1])
    want, _ = port.sort(a)
    np.testing.assert_array_equal(got, want)
    # the permutation preserves every digit histogram and the sum
    np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(got, 0, N - 1),
                                  pa.HistogramByteComponentsParallel(a, 0, N - 1))
    np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(a, 0, N - 1, 0),
                                  port.hist_one_byte(a, 0, N - 1, 0))
    assert pa.SumParallelNonRecursive(a, 0, N) == port.sum(a) == pa.SumParallelNonRecursive(got, 0, N)
    for k in (N // 2, N - 21):
        assert pa.select(a, k) == int(want[k])


@pytest.mark.parametrize("dist", ["uniform", "presorted", "constant"])
def test_u32_100m_against_the_compiled_reference(pa, ref, torch_cuda, inputs, dist):
    """The C2 calls on each 100M array, the GPU against the reference's own
    code (RadixSortLsdBenchmark.cpp:95-110, RadixSelectBenchmark.cpp:51-66,
    SumBenchmark.cpp:135-160 make the same calls)."""
    a = inputs[dist]
    want = ref.sort_radix_par(a.copy())
    d = torch_cuda.from_numpy(a.view(np.int32)).cuda()
    pa.SortRadixPar(d, torch_cuda.empty_like(d), N)
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want)
    # the in-place MSD sort (bounded scratch: partition rounds, then bucket groups)
    d.copy_(torch_cuda.from_numpy(a.view(np.int32)))
    pa.parallel_hybrid_inplace_msd_radix_sort(d)
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want)
    del d
    np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(a, 0, N - 1, 0),
                                  ref.hist_one_byte(a, 0, N - 1, 0))
    np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(a, 0, N - 1),
                                  ref.hist_byte_components(a, 0, N - 1))
    for k in (N // 2, N - 21):
        v = ref.select(a, k)
        assert v == int(want[k])
        c = a.copy()
        assert pa.SelectRadix(c, N, k) == v
        assert c[k] == v
    assert pa.SumParallelNonRecursive(a, 0, N) == ref.sum_nonrec(a)


def test_u64_kv_100m_stable(pa, port):
    from parallelalgorithms_gb300 import workloads
    for keys in (workloads.uniform_u64(N), workloads.zipf_u64(N)):
        vals = np.arange(N, dtype=np.uint32)
        k, v = keys.copy(), vals.copy()
        pa.sort(k, v)
        assert np.all(k[1:] >= k[:-1])
        np.testing.assert_array_equal(keys[v], k)  # payload = original index
        same = k[1:] == k[:-1]
        assert np.all(v[1:][same] > v[:-1][same])  # stable: equal keys keep input order
        wk, wv = port.sort(keys, vals)
        np.testing.assert_array_equal(k, wk)
        np.testing.assert_array_equal(v, wv)
        # independent of the restatement: numpy's stable argsort gives the payload
        np.testing.assert_array_equal(v, np.argsort(keys, kind="stable").astype(np.uint32))


def test_f32_100m_total_order(pa, port):
    from parallelalgorithms_gb300 import workloads
    a = workloads.normal_specials_f32(N)
    vals = np.arange(N, dtype=np.uint32)
    k, v = a.copy(), vals.copy()
    pa.sort(k, v)
    wk, wv = port.sort(a, vals)
    np.testing.assert_array_equal(k.view(np.uint32), wk.view(np.uint32))
    np.testing.assert_array_equal(v, wv)


def test_batched_4096_arrays_200m(pa, port, torch_cuda):
    """4096 arrays, sizes log-uniform in [1e3, 4e6] (~200M keys), one plan,
    bit-exact per segment against the oracle."""
    from parallelalgorithms_gb300 import batched, workloads
    torch = torch_cuda
    sizes = workloads.log_uniform_sizes(4096, 1e3, 4e6)
    off = np.zeros(sizes.size + 1, np.uint64)
    off[1:] = np.cumsum(sizes)
    keys = workloads.uniform_u32(int(off[-1]), seed=workloads.SEED_SEGMENT_SIZES)
    d = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    t = torch.empty_like(d)
    plan = batched.SegmentedSortPlan(off)
    plan.run(d, t)
    got = d.cpu().numpy().view(np.uint32)
    for i in range(sizes.size):
        a, b = int(off[i]), int(off[i + 1])
        want, _ = port.sort(keys[a:b])
        np.testing.assert_array_equal(got[a:b], want, err_msg=f"segment {i}")
    plan.close()


def test_u32_above_2_30_keys_plain_and_inplace(pa, torch_cuda):
    """2^30 + 3 keys: the sorts' 64-bit look-back words (the plain sort's and
    the in-place sort's scatter passes) and 64-bit positions, checked through
    size-independent properties on the device: sorted, and every byte
    histogram unchanged by the permutation."""
    import ctypes
    torch = torch_cuda
    n = (1 << 30) + 3
    P = ctypes.c_void_p
    g = torch.Generator(device="cuda").manual_seed(1301)
    src = torch.randint(-2 ** 31, 2 ** 31, (n,), dtype=torch.int32, device="cuda", generator=g)
    hist = torch.zeros(1024, dtype=torch.int64, device="cuda")
    pa.call("pa_hist_byte_components_u32", P(src.data_ptr()), n, P(hist.data_ptr()), None)
    want_hist = hist.clone()
    flip = torch.tensor(-2 ** 31, dtype=torch.int32, device="cuda")  # order-preserving signed view

    def check(d):
        f = d ^ flip
        assert bool(torch.all(f[1:] >= f[:-1]))
        hist.zero_()
        pa.call("pa_hist_byte_components_u32", P(d.data_ptr()), n, P(hist.data_ptr()), None)
        assert torch.equal(hist, want_hist)

    d = src.clone()
    tmp = torch.empty_like(d)
    pa.call("pa_sort_u32", P(d.data_ptr()), P(tmp.data_ptr()), n, None)
    check(d)
    del tmp
    d.copy_(src)
    pa.call("pa_sort_u32_inplace", P(d.data_ptr()), n, 0, None)
    check(d)
