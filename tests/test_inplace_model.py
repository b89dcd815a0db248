"""CPU model of the in-place partition's rounds (the plan arithmetic of
csrc/pa_inplace.cu: top-up from the tops of the unread parts, the runs in
the way copied out, the keys in hand scattered at the cursors), checked on
the invariants the device code relies on: every key ends in its bucket's
region, the cursors end at the regions' ends, and ceil(n / H) + 1 rounds
always suffice.  No GPU; the device kernels themselves are checked against
the oracle in tests/test_gpu_inplace.py."""
import numpy as np
import pytest


def partition_rounds(a: np.ndarray, shift: int, half: int) -> int:
    """Partitions a in place by (a >> shift) & 255 as the device rounds do;
    returns the rounds that moved keys."""
    d = (a >> shift) & 255
    cnt = np.bincount(d, minlength=256).astype(np.int64)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    end = start + cnt
    w, r = start.copy(), end.copy()      # write cursors, ends of the unread parts
    hand = np.empty(0, a.dtype)          # keys in the scratch half
    rounds = 0
    for _ in range(-(-a.size // half) + 1 if a.size else 0):
        # 1. top-up: the first half - |hand| unread keys, bucket by bucket from the tops
        want = half - hand.size
        unread = r - w
        before = np.concatenate([[0], np.cumsum(unread)[:-1]])
        g = np.clip(want - before, 0, unread)
        tops = [a[r[b] - g[b]:r[b]] for b in range(256) if g[b]]
        r = r - g
        if tops:
            hand = np.concatenate([hand] + tops)
        if hand.size == 0:
            break
        rounds += 1
        # 2. the unread keys in the way of the keys in hand are copied out
        need = np.bincount((hand >> shift) & 255, minlength=256).astype(np.int64)
        stop = np.minimum(w + need, r)
        x = np.maximum(stop - w, 0)
        nxt = np.concatenate([a[w[b]:w[b] + x[b]] for b in range(256)] + [np.empty(0, a.dtype)])
        base = w.copy()
        w = w + need
        r = np.maximum(r, w)
        # 3. the keys in hand go to [old cursor, old cursor + need) (any order within a bucket)
        dh = (hand >> shift) & 255
        order = np.argsort(dh, kind="stable")
        sorted_hand = hand[order]
        off = np.concatenate([[0], np.cumsum(need)[:-1]])
        for b in np.nonzero(need)[0]:
            a[base[b]:base[b] + need[b]] = sorted_hand[off[b]:off[b] + need[b]]
        hand = nxt
    assert hand.size == 0, "keys left in the scratch"
    assert np.array_equal(w, end), "cursors end at the regions' ends"
    return rounds


def make(kind: str, n: int, rng) -> np.ndarray:
    u = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    if kind == "uniform":
        return u
    if kind == "zipf":
        return (rng.zipf(1.3, n) % (2 ** 32)).astype(np.uint32)
    if kind == "sorted":
        return np.sort(u)
    if kind == "reversed":
        return np.sort(u)[::-1].copy()
    if kind == "one_bucket":
        return np.full(n, 0x7F000000, np.uint32)
    if kind == "two_buckets":
        return rng.choice(np.array([0x01000000, 0xFE000000], np.uint32), n)
    raise ValueError(kind)


@pytest.mark.parametrize("kind", ["uniform", "zipf", "sorted", "reversed", "one_bucket", "two_buckets"])
@pytest.mark.parametrize("n,half", [(0, 5), (1, 1), (100_000, 7_000), (100_000, 50_000), (123_457, 4_096),
                                    (50_000, 999), (20_000, 100)])
def test_rounds_partition_and_bound(kind, n, half):
    rng = np.random.default_rng(n + half)
    a = make(kind, n, rng)
    orig = a.copy()
    rounds = partition_rounds(a, 24, half)
    assert rounds <= -(-n // half) + 1
    assert np.array_equal(np.sort(a), np.sort(orig))  # a permutation of the input
    d = (a >> 24) & 255
    assert np.all(d[1:] >= d[:-1])  # buckets in order
