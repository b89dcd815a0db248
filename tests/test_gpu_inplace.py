"""In-place MSD sort with bounded scratch (pa_sort_u32_inplace, the
parallel_hybrid_inplace_msd_radix_sort drop-in) against the oracle and the
compiled reference: small scratch sizes force many partition rounds, the
recursion into buckets larger than the scratch, groups of buckets, and the
plain path for inputs that fit the scratch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH = 1 << 16  # the smallest scratch: the most rounds and levels


def make(dist: str, n: int, seed: int = 77) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = lambda m: rng.integers(0, 2 ** 32, m, dtype=np.uint64).astype(np.uint32)  # noqa: E731
    if dist == "uniform":
        return u(n)
    if dist == "zipf":
        return (rng.zipf(1.2, n) % (2 ** 32)).astype(np.uint32)
    if dist == "presorted":
        return np.sort(u(n))
    if dist == "reversed":
        return np.sort(u(n))[::-1].copy()
    if dist == "constant":
        return np.full(n, 0xDEADBEEF, np.uint32)
    if dist == "two_values":
        return rng.choice(np.array([0x01000000, 0xFE0000FF], np.uint32), n)
    if dist == "top_byte_constant":  # one top-digit bucket: the next digit partitions
        return (u(n) & 0x00FFFFFF) | 0x7F000000
    if dist == "top_two_bytes_constant":
        return (u(n) & 0x0000FFFF) | 0x12340000
    if dist == "one_big_bucket":  # 90 % in one bucket larger than the scratch, the rest spread
        a = u(n)
        big = rng.random(n) < 0.9
        a[big] = (a[big] & 0x00FFFFFF) | 0x80000000
        return a
    if dist == "low_entropy":
        return u(n) & u(n) & u(n)
    if dist == "few_low_values":  # all keys below 2^8: top three digits constant
        return rng.integers(0, 256, n, dtype=np.uint32)
    raise ValueError(dist)


DISTS = ["uniform", "zipf", "presorted", "reversed", "constant", "two_values", "top_byte_constant",
         "top_two_bytes_constant", "one_big_bucket", "low_entropy", "few_low_values"]


def run_device(pa, torch, a: np.ndarray, scratch: int) -> np.ndarray:
    d = torch.from_numpy(a.view(np.int32).copy()).cuda()
    pa.call("pa_sort_u32_inplace", d.data_ptr(), a.size, scratch, pa._opts(d))
    return d.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("dist", DISTS)
@pytest.mark.parametrize("n", [65537, 300_001, 1_000_003])
def test_matches_oracle_small_scratch(pa, port, torch_cuda, dist, n):
    a = make(dist, n)
    want, _ = port.sort(a)
    np.testing.assert_array_equal(run_device(pa, torch_cuda, a, SCRATCH), want)


@pytest.mark.parametrize("n", [2, 3, 100, 8191, 8193, 65535, 65536])
def test_fits_the_scratch(pa, port, torch_cuda, n):
    for dist in ("uniform", "zipf", "reversed"):
        a = make(dist, n, seed=n)
        want, _ = port.sort(a)
        np.testing.assert_array_equal(run_device(pa, torch_cuda, a, SCRATCH), want)


@pytest.mark.parametrize("scratch", [1 << 17, (1 << 18) + 2, 1 << 20, 0])
def test_scratch_sizes(pa, port, torch_cuda, scratch):
    a = make("uniform", 2_500_017, seed=scratch)
    want, _ = port.sort(a)
    np.testing.assert_array_equal(run_device(pa, torch_cuda, a, scratch), want)


def test_host_buffer_and_dropin(pa, ref, torch_cuda):
    """Host numpy input through the Python mirror of the drop-in, and the
    compiled reference's own in-place MSD sort on the same keys."""
    for dist in ("uniform", "one_big_bucket"):
        a = make(dist, 3_000_001, seed=5)
        m = a.copy()
        ref.msd_radix_sort(m)
        h = a.copy()
        pa.parallel_hybrid_inplace_msd_radix_sort(h, scratch_keys=SCRATCH)
        np.testing.assert_array_equal(h, m)
        h = a.copy()
        pa.parallel_hybrid_inplace_msd_radix_sort(h)  # default scratch: the plain path at this size
        np.testing.assert_array_equal(h, m)


def test_subrange_leaves_the_rest(pa, port, torch_cuda):
    a = make("uniform", 1_000_000, seed=9)
    d = torch_cuda.from_numpy(a.view(np.int32).copy()).cuda()
    lo, hi = 1001, 900_001  # a start that is not 16-byte aligned
    pa.call("pa_sort_u32_inplace", d.data_ptr() + 4 * lo, hi - lo, SCRATCH, pa._opts(d))
    got = d.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(got[lo:hi], port.sort(a[lo:hi])[0])
    np.testing.assert_array_equal(got[:lo], a[:lo])
    np.testing.assert_array_equal(got[hi:], a[hi:])


def test_errors(pa):
    with pytest.raises(pa.PaError):
        pa.call("pa_sort_u32_inplace", None, 10, 0, None)
    pa.call("pa_sort_u32_inplace", None, 0, 0, None)  # nothing to sort
