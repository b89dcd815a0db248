"""CPU model of the prepared first pass (csrc/pa_histogram.cu,
tile_counts_kernel and launch_tile_counts): the chunking of the first
pass's tiles over CTAs, the per-tile byte-0 counts recovered from two
never-cleared counter sets used on alternate steps, the per-tile prefix
within a chunk and the chunk prefix written by the last CTA.  Checked on
the invariant the pass relies on: tile_prefix[t] + chunk_excl[t // tpc] is
the exclusive prefix of the byte-0 counts over tiles, and the chunks'
totals are the byte-0 histogram.  No GPU; the kernels themselves are
checked against the oracle in tests/test_gpu_prepared_pass.py."""
import numpy as np
import pytest

MAX_CHUNKS = 160  # kTileCountMaxChunks


def chunking(n: int, tile_keys: int, sms: int) -> tuple[int, int, int]:
    """(tiles, tiles per chunk, chunks) as launch_tile_counts computes them."""
    tiles = -(-n // tile_keys)
    g0 = max(1, min(min(sms, MAX_CHUNKS), tiles))
    tpc = -(-tiles // g0)
    return tiles, tpc, -(-tiles // tpc)


def prepared_rows(keys: np.ndarray, tile_keys: int, sms: int):
    n = keys.size
    tiles, tpc, chunks = chunking(n, tile_keys, sms)
    d0 = (keys & 255).astype(np.int64)
    tile_prefix = np.zeros((tiles, 256), np.int64)
    chunk_tot = np.zeros((chunks, 256), np.int64)
    for c in range(chunks):
        t0, t1 = c * tpc, min((c + 1) * tpc, tiles)
        sets = [np.zeros(256, np.int64), np.zeros(256, np.int64)]  # cumulative, never cleared
        seen = [np.zeros(256, np.int64), np.zeros(256, np.int64)]
        run = np.zeros(256, np.int64)
        for t in range(t0, t1):
            p = (t - t0) & 1
            sets[p] += np.bincount(d0[t * tile_keys:min(n, (t + 1) * tile_keys)], minlength=256)
            total = sets[p].copy()
            cnt = total - seen[p]
            seen[p] = total
            tile_prefix[t] = run
            run = run + cnt
        chunk_tot[c] = run
    chunk_excl = np.cumsum(chunk_tot, axis=0) - chunk_tot
    return tiles, tpc, chunks, tile_prefix, chunk_excl, chunk_tot


@pytest.mark.parametrize("tile_keys", [4096, 6144, 8192])
@pytest.mark.parametrize("mult,extra", [(0, 8193), (2, 0), (152, 0), (152, 1), (305, -1), (457, 5000),
                                        (0, 1_000_003), (321, 3)])
def test_prefix_rows_give_the_exclusive_tile_prefix(tile_keys, mult, extra):
    n = mult * tile_keys + extra
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] &= np.uint32(0xFFFFFF03)  # a skewed byte 0 in the first third
    tiles, tpc, chunks, tile_prefix, chunk_excl, chunk_tot = prepared_rows(keys, tile_keys, 152)
    assert chunks <= MAX_CHUNKS and (chunks - 1) * tpc < tiles <= chunks * tpc  # every chunk has a tile
    d0 = (keys & 255).astype(np.int64)
    per_tile = np.stack([np.bincount(d0[t * tile_keys:(t + 1) * tile_keys], minlength=256) for t in range(tiles)])
    want = np.cumsum(per_tile, axis=0) - per_tile
    got = tile_prefix + chunk_excl[np.arange(tiles) // tpc]
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(chunk_tot.sum(axis=0), np.bincount(d0, minlength=256))
    assert int(got.max()) < 2 ** 30  # u32 rows (the prepared pass is used below 2^30 keys)


@pytest.mark.parametrize("sms", [1, 2, 148, 152, 160, 200])
def test_chunking_bounds(sms):
    for tile_keys in (4096, 6144, 8192):
        for n in (tile_keys + 1, 7 * tile_keys, 1_000_003, 100_000_000, (1 << 30) - 1):
            tiles, tpc, chunks = chunking(n, tile_keys, sms)
            assert 1 <= chunks <= min(MAX_CHUNKS, sms, tiles)
            assert (chunks - 1) * tpc < tiles <= chunks * tpc
            assert tiles * 256 * 4 == -(-n // tile_keys) * 1024  # tile_prefix rows: 1 KB per tile
