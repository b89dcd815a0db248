"""Generates tests/golden/reference_golden.npz from the reference's own CPU
code compiled unchanged (oracle/_ref/libpa_ref.so, see oracle/build.py).

The reference ships no golden vectors or known-answer tests; its only pins
are self-checks against std::sort / std::stable_sort / std::nth_element /
std::accumulate (RadixSortLsdBenchmark.cpp:47,95; RadixSelectBenchmark.cpp:51;
SumBenchmark.cpp:91,135,188).  These fixtures record what the reference
itself returns on small seeded inputs built with its own input recipes
(ParallelAlgorithms.cpp:91-115 uniform, :151-163 nearly presorted,
:188-190 constant), so that the oracle restatement and the GPU path can be
checked against it on machines where the reference cannot be built.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_golden.npz"
SIZES = [0, 1, 2, 7, 31, 99, 100, 101, 255, 256, 1000, 4097, 8191]


def mt_u32(seed: int, n: int) -> np.ndarray:
    """(unsigned)std::mt19937_64(seed)(), the reference's key recipe."""
    return _mt19937_64(seed, n).astype(np.uint32)


def _mt19937_64(seed: int, n: int) -> np.ndarray:
    # MT19937-64 (Matsumoto & Nishimura), the engine behind std::mt19937_64.
    NN, MM = 312, 156
    A = 0xB5026F5AA96619E9
    UM, LM = 0xFFFFFFFF80000000, 0x7FFFFFFF
    mask = (1 << 64) - 1
    mt = [0] * NN
    mt[0] = seed & mask
    for i in range(1, NN):
        mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & mask
    out = np.empty(n, np.uint64)
    idx = NN
    for j in range(n):
        if idx >= NN:
            for i in range(NN):
                x = (mt[i] & UM) | (mt[(i + 1) % NN] & LM)
                xa = x >> 1
                if x & 1:
                    xa ^= A
                mt[i] = mt[(i + MM) % NN] ^ xa
            idx = 0
        x = mt[idx]
        idx += 1
        x ^= (x >> 29) & 0x5555555555555555
        x ^= (x << 17) & 0x71D67FFFEDA60000
        x ^= (x << 37) & 0xFFF7EEE000000000
        x ^= x >> 43
        out[j] = x & mask
    return out


def inputs(n: int) -> dict[str, np.ndarray]:
    nearly = np.arange(n, dtype=np.uint32)
    nearly[::100] = 0x1010
    return {
        "uniform": mt_u32(1234, n),
        "nearly": nearly,
        "constant": np.full(n, 0x10101010, np.uint32),
        "c42": np.full(n, 42, np.uint32),
    }


def main() -> None:
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("the compiled reference is required (oracle/build.py could not build it)")
    g: dict[str, np.ndarray] = {}
    for n in SIZES:
        for dist, a in inputs(n).items():
            key = f"{dist}_{n}"
            g[f"in_{key}"] = a
            s = a.copy()
            ref.sort_radix_par(s)
            g[f"sort_{key}"] = s
            if n:
                a2, b2 = a.copy(), np.zeros_like(a)
                ref.sort_two_phase_par(a2, b2)
                g[f"twophase_a_{key}"], g[f"twophase_b_{key}"] = a2, b2
                g[f"histbc_{key}"] = ref.hist_byte_components(a, 0, n - 1)
                for sh in (0, 8, 13, 24, 31):
                    g[f"hist1_s{sh}_{key}"] = ref.hist_one_byte(a, 0, n - 1, sh)
                ks = sorted({0, n // 2, max(0, n - 21), n - 1})
                g[f"selk_{key}"] = np.array(ks, np.uint64)
                g[f"selv_{key}"] = np.array([ref.select(a, k) for k in ks], np.uint64)
                wq = max(1, n // 5)
                q = (n - 1) // wq + 1
                g[f"qc_{key}"] = ref.hist_qc(a, 0, n - 1, wq, q, 1)
                g[f"sob_{key}"] = ref.start_of_bins(a, n, wq, q, 0)
            g[f"sum32_{key}"] = np.array([ref.sum_nonrec(a)], np.uint64)
            g[f"sumtpl_{key}"] = np.array([ref.sum_template_u32(a)], np.int64)
            a64 = a.astype(np.uint64) * np.uint64(0x100000001)
            g[f"sum64_{key}"] = np.array([ref.sum_nonrec(a64)], np.uint64)
            g[f"sum64r_{key}"] = np.array([ref.sum_recursive_u64(a64)], np.uint64)
    # sub-range cases: l > 0 and inclusive r
    a = mt_u32(1234, 5000)
    g["sub_in"] = a
    g["sub_histbc"] = ref.hist_byte_components(a, 17, 4321)
    g["sub_hist1"] = ref.hist_one_byte(a, 5, 4999, 16)
    g["sub_qc"] = ref.hist_qc(a, 123, 4444, 1000, 5, 2)
    g["sub_sum"] = np.array([ref.sum_nonrec(a, 10, 4990)], np.uint64)
    g["sub_sel"] = np.array([ref.select(a, 2600, start=1000, length=3000)], np.uint64)
    u8 = (mt_u32(77, 10007) & 0xFF).astype(np.uint8)
    g["u8_in"] = u8
    g["u8_hist"] = ref.hist_u8(u8, 0, u8.size)
    g["u8_hist_sub"] = ref.hist_u8(u8, 3, 9000)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(g)} arrays)")


if __name__ == "__main__":
    main()
