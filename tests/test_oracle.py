"""The CPU oracle restatement (oracle/pa_oracle.c) pinned against the
reference: the golden fixtures produced by the reference's own code, the
compiled reference itself where it can be built, and std::stable_sort
semantics (numpy stable argsort) for the key types the reference lacks."""
import numpy as np
import pytest

from golden.make_golden import SIZES

DISTS = ["uniform", "nearly", "constant", "c42"]


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dist", DISTS)
def test_port_sort_matches_reference_golden(golden, port, n, dist):
    key = f"{dist}_{n}"
    a = golden[f"in_{key}"]
    got, _ = port.sort(a)
    np.testing.assert_array_equal(got, golden[f"sort_{key}"])


@pytest.mark.parametrize("n", [s for s in SIZES if s])
@pytest.mark.parametrize("dist", DISTS)
def test_port_histograms_select_sum_match_golden(golden, port, n, dist):
    key = f"{dist}_{n}"
    a = golden[f"in_{key}"]
    np.testing.assert_array_equal(port.hist_byte_components(a, 0, n - 1), golden[f"histbc_{key}"])
    for sh in (0, 8, 13, 24, 31):
        np.testing.assert_array_equal(port.hist_one_byte(a, 0, n - 1, sh), golden[f"hist1_s{sh}_{key}"])
    for k, v in zip(golden[f"selk_{key}"], golden[f"selv_{key}"]):
        assert port.select(a, int(k)) == int(v)
    wq = max(1, n // 5)
    q = (n - 1) // wq + 1
    np.testing.assert_array_equal(port.hist_qc(a, 0, n - 1, wq, q, 1), golden[f"qc_{key}"])
    np.testing.assert_array_equal(port.start_of_bins(a, n, wq, q, 0), golden[f"sob_{key}"])
    assert port.sum(a) == int(golden[f"sum32_{key}"][0])
    assert np.int64(np.uint64(port.sum(a))) == golden[f"sumtpl_{key}"][0]
    a64 = a.astype(np.uint64) * np.uint64(0x100000001)
    assert port.sum(a64) == int(golden[f"sum64_{key}"][0]) == int(golden[f"sum64r_{key}"][0])


def test_port_subranges_match_golden(golden, port):
    a = golden["sub_in"]
    np.testing.assert_array_equal(port.hist_byte_components(a, 17, 4321), golden["sub_histbc"])
    np.testing.assert_array_equal(port.hist_one_byte(a, 5, 4999, 16), golden["sub_hist1"])
    np.testing.assert_array_equal(port.hist_qc(a, 123, 4444, 1000, 5, 2), golden["sub_qc"])
    assert port.sum(a, 10, 4990) == int(golden["sub_sum"][0])
    assert port.select(a, 2600, start=1000, length=3000) == int(golden["sub_sel"][0])
    u8 = golden["u8_in"]
    np.testing.assert_array_equal(port.hist_u8(u8, 0, u8.size), golden["u8_hist"])
    np.testing.assert_array_equal(port.hist_u8(u8, 3, 9000), golden["u8_hist_sub"])


def test_two_phase_golden_leaves_sorted_keys_in_both_buffers(golden):
    # RadixSortLsdParallel.h:77-82 copies the result into b; a also ends sorted.
    for n in [s for s in SIZES if s]:
        for dist in DISTS:
            key = f"{dist}_{n}"
            np.testing.assert_array_equal(golden[f"twophase_a_{key}"], golden[f"sort_{key}"])
            np.testing.assert_array_equal(golden[f"twophase_b_{key}"], golden[f"sort_{key}"])


# ---- the compiled reference itself -----------------------------------------
def test_reference_build_reproduces_golden(golden, ref):
    for n in SIZES:
        for dist in DISTS:
            key = f"{dist}_{n}"
            s = golden[f"in_{key}"].copy()
            ref.sort_radix_par(s)
            np.testing.assert_array_equal(s, golden[f"sort_{key}"])


@pytest.mark.parametrize("n", [1, 99, 100, 4097, 300001, 1000003])
def test_port_matches_reference_on_larger_inputs(port, ref, n):
    rng = np.random.default_rng(n)
    for a in (rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32),
              rng.integers(0, 1000, n, dtype=np.uint32),
              np.arange(n, dtype=np.uint32)[::-1].copy()):
        got, _ = port.sort(a)
        np.testing.assert_array_equal(got, ref.sort_radix_par(a.copy()))
        np.testing.assert_array_equal(port.hist_byte_components(a, 0, n - 1), ref.hist_byte_components(a, 0, n - 1))
        np.testing.assert_array_equal(port.hist_one_byte(a, 0, n - 1, 7), ref.hist_one_byte(a, 0, n - 1, 7))
        for k in {0, n // 2, n - 1}:
            assert port.select(a, k) == ref.select(a, k)
        assert port.sum(a) == ref.sum_nonrec(a)


def test_reference_two_phase_and_serial_sorts(ref):
    a = np.random.default_rng(5).integers(0, 2**32, 70001, dtype=np.uint64).astype(np.uint32)
    want = np.sort(a, kind="stable")
    x, b = a.copy(), np.zeros_like(a)
    ref.sort_two_phase_par(x, b)
    np.testing.assert_array_equal(x, want)
    np.testing.assert_array_equal(b, want)
    y, t = a.copy(), np.zeros_like(a)
    ref.sort_two_phase_serial(y, t)
    np.testing.assert_array_equal(y, want)


# ---- widened restatement: u64, float32, payloads, 11-bit digits ----------
def _stable_ref(keys, vals):
    order = np.argsort(keys, kind="stable")
    return keys[order], vals[order]


def _f32_order(bits: np.ndarray) -> np.ndarray:
    b = bits.view(np.uint32)
    return np.where(b >> 31 == 1, ~b, b | np.uint32(0x80000000)).astype(np.uint32)


@pytest.mark.parametrize("digit_bits", [8, 11])
@pytest.mark.parametrize("n", [0, 1, 5, 1000, 65537])
def test_port_kv_u32_u64_stable(port, n, digit_bits):
    rng = np.random.default_rng(10 + n)
    for keys in (rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32),
                 rng.integers(0, 50, n, dtype=np.uint32),
                 rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True),
                 rng.integers(0, 7, n, dtype=np.uint64) << np.uint64(40)):
        vals = np.arange(n, dtype=np.uint32)
        gk, gv = port.sort(keys, vals, digit_bits=digit_bits)
        wk, wv = _stable_ref(keys, vals)
        np.testing.assert_array_equal(gk, wk)
        np.testing.assert_array_equal(gv, wv)


@pytest.mark.parametrize("digit_bits", [8, 11])
def test_port_f32_total_order(port, digit_bits):
    specials = np.array([0.0, -0.0, np.inf, -np.inf, 1e-45, -1e-45, 1.0, -1.0, 3.4e38, -3.4e38], np.float32)
    rng = np.random.default_rng(3)
    keys = np.concatenate([rng.standard_normal(5000).astype(np.float32), np.repeat(specials, 7)])
    rng.shuffle(keys)
    vals = np.arange(keys.size, dtype=np.uint32)
    gk, gv = port.sort(keys, vals, digit_bits=digit_bits)
    order = np.argsort(_f32_order(keys), kind="stable")
    np.testing.assert_array_equal(gk.view(np.uint32), keys[order].view(np.uint32))
    np.testing.assert_array_equal(gv, vals[order])
    neg0 = np.flatnonzero(gk.view(np.uint32) == 0x80000000)
    pos0 = np.flatnonzero(gk.view(np.uint32) == 0)
    assert neg0.max() < pos0.min()


def test_port_hist_digits_is_every_digit(port):
    a = np.random.default_rng(2).integers(0, 2**64 - 1, 3001, dtype=np.uint64, endpoint=True)
    h = port.hist_digits(a)
    for d in range(8):
        np.testing.assert_array_equal(h[d], np.bincount(((a >> np.uint64(8 * d)) & np.uint64(255)).astype(np.int64),
                                                        minlength=256))


def test_port_select_u64(port):
    a = np.random.default_rng(4).integers(0, 2**64 - 1, 10001, dtype=np.uint64, endpoint=True)
    s = np.sort(a)
    for k in (0, 17, 5000, 10000):
        assert port.select(a, k) == int(s[k])


@pytest.mark.parametrize("n", [0, 1, 2, 15, 16, 17, 47, 48, 49, 1000, 4099, 100003])
def test_counting_sort_and_partition_restatements_match_reference(port, ref, n):
    """CountingSortParallel.h:29-79 and RadixPartition.h:30-79 restated in C
    give the compiled reference's result (the partition's exact in-place
    permutation included)."""
    rng = np.random.default_rng(4000 + n)
    b = rng.integers(0, 256, n, dtype=np.uint8)
    np.testing.assert_array_equal(port.counting_sort_u8(b), np.sort(b))
    if ref is not None:
        np.testing.assert_array_equal(ref.counting_sort_u8(b), np.sort(b))
    u = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    skew = ((rng.integers(0, 4, n, dtype=np.uint64) << 24) | rng.integers(0, 100, n, dtype=np.uint64)).astype(np.uint32)
    for a in (u, skew):
        s = np.sort(a)
        for ks in ([0], [n // 2], [n - 1], sorted({0, n // 3, n // 2, n - 1})):
            ks = [k for k in ks if 0 <= k < n]
            if not ks:
                continue
            got = port.partition_radix(a, ks)
            for k in ks:
                assert got[k] == s[k]
                assert np.all(got[:k] <= got[k]) and np.all(got[k + 1:] >= got[k])
            if ref is not None:
                np.testing.assert_array_equal(got, ref.partition_radix(a, ks))


@pytest.mark.parametrize("n", [1, 2, 100, 100003])
def test_reference_merge_sorts_sort(ref, n):
    """The reference's radix-leaf merge sorts, compiled unchanged, sort (the
    GPU drop-ins are checked against the same sorted result)."""
    if ref is None:
        pytest.skip("reference not built")
    rng = np.random.default_rng(4300 + n)
    a = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    src, dst = a.copy(), np.zeros_like(a)
    ref.merge_sort_hybrid_radix(src, 0, n - 1, dst, True)
    np.testing.assert_array_equal(dst, np.sort(a))
    src, work = a.copy(), np.zeros_like(a)
    ref.merge_sort_hybrid_radix(src, 0, n - 1, work, False)
    np.testing.assert_array_equal(src, np.sort(a))
    c = a.copy()
    ref.preventative_adaptive_sort(c)
    np.testing.assert_array_equal(c, np.sort(a))
    c = a.copy()
    ref.msd_radix_sort(c)
    np.testing.assert_array_equal(c, np.sort(a))


def test_restatement_generator_is_the_reference_recipe(golden, port):
    """The oracle's MT19937-64 gives the reference benchmark's keys (the golden
    inputs were drawn by the compiled reference's std::mt19937_64(1234))."""
    np.testing.assert_array_equal(port.gen_uniform_u32(8191, 1234), golden["in_uniform_8191"])


def test_compiled_reference_generator_matches_the_restatement(ref, port):
    for seed in (1, 1234, 2**63 + 5):
        np.testing.assert_array_equal(ref.gen_uniform_u32(100_003, seed), port.gen_uniform_u32(100_003, seed))
