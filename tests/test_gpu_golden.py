"""GPU path vs the golden fixtures recorded from the reference's own code
(tests/golden/make_golden.py), through the C ABI, bit-exact."""
import numpy as np
import pytest

from golden.make_golden import SIZES

pytestmark = pytest.mark.gpu

DISTS = ["uniform", "nearly", "constant", "c42"]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dist", DISTS)
def test_gpu_matches_reference_golden(pa, golden, n, dist):
    key = f"{dist}_{n}"
    a = golden[f"in_{key}"]
    s = a.copy()
    pa.SortRadixPar(s, np.empty_like(s), n)
    np.testing.assert_array_equal(s, golden[f"sort_{key}"])
    s2 = a.copy()
    pa.SortRadixPar(s2, n)  # allocating overload
    np.testing.assert_array_equal(s2, golden[f"sort_{key}"])
    assert pa.SumParallelNonRecursive(a, 0, n) == int(golden[f"sum32_{key}"][0])
    assert pa.SumParallel(a, 0, n) == int(golden[f"sumtpl_{key}"][0])
    a64 = a.astype(np.uint64) * np.uint64(0x100000001)
    assert pa.SumParallelNonRecursive(a64, 0, n) == int(golden[f"sum64_{key}"][0])
    assert pa.SumParallel(a64, 0, n) == int(golden[f"sum64r_{key}"][0])
    if n == 0:
        return
    x, b = a.copy(), np.zeros_like(a)
    pa.RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(x, b, n)
    np.testing.assert_array_equal(x, golden[f"twophase_a_{key}"])
    np.testing.assert_array_equal(b, golden[f"twophase_b_{key}"])
    np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(a, 0, n - 1), golden[f"histbc_{key}"])
    for sh in (0, 8, 13, 24, 31):
        np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(a, 0, n - 1, sh),
                                      golden[f"hist1_s{sh}_{key}"])
    for k, v in zip(golden[f"selk_{key}"], golden[f"selv_{key}"]):
        c = a.copy()
        assert pa.SelectRadix(c, n, int(k)) == int(v)
        assert c[int(k)] == v
    wq = max(1, n // 5)
    q = (n - 1) // wq + 1
    np.testing.assert_array_equal(pa.HistogramByteComponentsQCPar(a, 0, n - 1, wq, q, 1), golden[f"qc_{key}"])
    np.testing.assert_array_equal(pa.ComputeStartOfBinsPar(a, n, wq, q, 0), golden[f"sob_{key}"])


def test_gpu_subranges_match_golden(pa, golden):
    a = golden["sub_in"]
    np.testing.assert_array_equal(pa.HistogramByteComponentsParallel(a, 17, 4321), golden["sub_histbc"])
    np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(a, 5, 4999, 16), golden["sub_hist1"])
    np.testing.assert_array_equal(pa.HistogramByteComponentsQCPar(a, 123, 4444, 1000, 5, 2), golden["sub_qc"])
    assert pa.SumParallelNonRecursive(a, 10, 4990) == int(golden["sub_sum"][0])
    assert pa.SelectRadix(a.copy(), 1000, 3000, 2600) == int(golden["sub_sel"][0])
    u8 = golden["u8_in"]
    np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(u8, 0, u8.size), golden["u8_hist"])
    np.testing.assert_array_equal(pa.HistogramOneByteComponentParallel(u8, 3, 9000), golden["u8_hist_sub"])
