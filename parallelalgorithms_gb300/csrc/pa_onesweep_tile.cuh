// Device-side building blocks of the onesweep digit pass, shared by the
// plain sort (pa_onesweep.cu) and the batched segmented sort
// (pa_segmented.cu).  See pa_onesweep.cu for the algorithm.
#pragma once

#include <type_traits>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace os {


constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kNibbleBins = 16;
#ifndef PA_LOOKBACK_WIDTH
#define PA_LOOKBACK_WIDTH 4
#endif
constexpr int kLookbackWidth = PA_LOOKBACK_WIDTH;  // predecessor tiles read per round trip

template <typename S>
struct StatusWord;
template <>
struct StatusWord<uint32_t> {
  static constexpr uint32_t kAgg = 1u << 30;
  static constexpr uint32_t kIncl = 2u << 30;
  static constexpr uint32_t kMask = (1u << 30) - 1;
  static constexpr int kShift = 30;
};
template <>
struct StatusWord<unsigned long long> {
  static constexpr unsigned long long kAgg = 1ull << 62;
  static constexpr unsigned long long kIncl = 2ull << 62;
  static constexpr unsigned long long kMask = (1ull << 62) - 1;
  static constexpr int kShift = 62;
};

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS>
struct Geometry {
  static constexpr int kWarps = BLOCK / 32;
  static constexpr int kTile = BLOCK * ITEMS;
  static constexpr size_t kKeysOff = 0;
  static constexpr size_t kValsOff = kKeysOff + (size_t)kTile * sizeof(K);
  static constexpr size_t kCntOff = kValsOff + (HAS_VALS ? (size_t)kTile * 4 : 0);
  // counter (nibble s, thread t) lives at word s * kCntRow + t + t / 32
  static constexpr int kCntRow = BLOCK + 32;
  static constexpr size_t kBinBaseOff = kCntOff + (size_t)kNibbleBins * kCntRow * 4;
  static constexpr size_t kBinStartOff = kBinBaseOff + (size_t)kRadix * 8;
  static constexpr size_t kBinEndOff = kBinStartOff + (size_t)kRadix * 4;
  static constexpr size_t kWarpTotOff = kBinEndOff + (size_t)kRadix * 4;
  static constexpr size_t kBarOff = kWarpTotOff + (size_t)kWarps * 4 + 8 - ((size_t)kWarps * 4) % 8;
  static constexpr size_t kTileIdOff = kBarOff + 8;
  static constexpr size_t kAbortOff = kTileIdOff + 4;
  static constexpr size_t kBytes = kAbortOff + 4;
  static_assert(kTile % 4 == 0, "tile starts must stay 16-byte aligned");
  static_assert((ITEMS * sizeof(K)) % 16 == 0, "a thread's run of keys is read as 16-byte vectors");
  static_assert(BLOCK >= kRadix, "one thread per bin in the look-back");
};

// Block-wide exclusive scan of one value per thread.  Contains one
// __syncthreads(); s_warp holds BLOCK / 32 words.
template <int BLOCK>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp) {
  constexpr int W = BLOCK / 32;
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  // every warp scans the W warp totals, lane l holding total l
  const uint32_t wt = lane < (uint32_t)W ? s_warp[lane] : 0u;
  uint32_t wincl = wt;
#pragma unroll
  for (int o = 1; o < W; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULL, wincl, o);
    if (lane >= (uint32_t)o) wincl += t;
  }
  return __shfl_sync(FULL, wincl - wt, warp) + incl - v;
}

// Byte `shift / 8` of a key (digits are byte aligned): one byte-permute.
template <typename K>
__device__ __forceinline__ uint32_t digit8(K key, uint32_t sel, bool upper) {
  uint32_t w;
  if constexpr (sizeof(K) == 4) {
    (void)upper;
    w = (uint32_t)key;
  } else {
    w = upper ? (uint32_t)(key >> 32) : (uint32_t)key;
  }
  return __byte_perm(w, 0u, sel);
}

// Counters: (nibble s, thread t) lives at word s * (BLOCK + 32) + t + t / 32.
// Rows are a multiple of 32 words and each warp's 32 columns are shifted by
// one bank per warp, so that both access patterns are free of bank
// conflicts: counting (a warp touches 32 different threads' columns, any
// nibbles) and the scan (a warp walks one row, each lane 16 consecutive
// words).

// One stable counting pass over the tile on the 4-bit nibble at `sh`: keys
// (and payloads) held by each thread in `k` / `v` are written to their
// nibble-sorted positions in s_keys / s_vals.  Ends with a barrier, after
// which the tile in shared memory is in the new order.
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS>
__device__ __forceinline__ void nibble_pass(const K (&k)[ITEMS], const uint32_t (&v)[HAS_VALS ? ITEMS : 1],
                                            uint32_t sh, K* s_keys, uint32_t* s_vals, uint32_t* s_cnt,
                                            uint32_t* s_warp) {
  const uint32_t tid = threadIdx.x;
  uint32_t* col = s_cnt + tid + (tid >> 5);  // this thread's column: word col[s * (BLOCK + 32)]
  // Only this thread touches its column until the scan.
#pragma unroll
  for (int s = 0; s < kNibbleBins; ++s) col[s * (BLOCK + 32)] = 0;
  // Rank of each key among this thread's earlier keys of the same nibble
  // (at most ITEMS - 1 <= 15), packed four bits per key.
  uint32_t r[(ITEMS + 7) / 8];
#pragma unroll
  for (int q = 0; q < (ITEMS + 7) / 8; ++q) r[q] = 0;
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    uint32_t* c = col + ((uint32_t)(k[j] >> sh) & 15u) * (uint32_t)(BLOCK + 32);
    const uint32_t x = *c;
    r[j / 8] += x << (4 * (j % 8));
    *c = x + 1;
  }
  __syncthreads();
  // Exclusive scan of the 16 x BLOCK counters in (nibble, thread) order:
  // thread t owns the 16 consecutive counters [16t, 16t + 16) of that order,
  // which sit in one row at consecutive words (a 16-aligned run of columns
  // never crosses a 32-column group).
  const uint32_t lin = 16u * tid;
  const uint32_t row = lin / BLOCK, col0 = lin % BLOCK;
  uint32_t* cb = s_cnt + row * (uint32_t)(BLOCK + 32) + col0 + (col0 >> 5);
  uint32_t c[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) c[i] = cb[i];
  uint32_t run = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t t = c[i];
    c[i] = run;
    run += t;
  }
  const uint32_t base = block_exclusive_scan<BLOCK>(run, s_warp);
#pragma unroll
  for (int i = 0; i < 16; ++i) cb[i] = c[i] + base;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t pos = col[((uint32_t)(k[j] >> sh) & 15u) * (uint32_t)(BLOCK + 32)] +
                         ((r[j / 8] >> (4 * (j % 8))) & 15u);
    s_keys[pos] = k[j];
    if (HAS_VALS) s_vals[pos] = v[j];
  }
  __syncthreads();
}

// Loads this thread's ITEMS consecutive keys (and payloads) from shared
// memory with 16-byte vector reads.
template <typename K, bool HAS_VALS, int ITEMS>
__device__ __forceinline__ void load_run(K (&k)[ITEMS], uint32_t (&v)[HAS_VALS ? ITEMS : 1], const K* s_keys,
                                         const uint32_t* s_vals) {
  const uint4* src = reinterpret_cast<const uint4*>(s_keys + threadIdx.x * ITEMS);
  constexpr int PER = 16 / (int)sizeof(K);
#pragma unroll
  for (int q = 0; q < ITEMS / PER; ++q) {
    const uint4 x = src[q];
    const K* e = reinterpret_cast<const K*>(&x);
#pragma unroll
    for (int i = 0; i < PER; ++i) k[q * PER + i] = e[i];
  }
  if (HAS_VALS) {
    const uint4* vs = reinterpret_cast<const uint4*>(s_vals + threadIdx.x * ITEMS);
#pragma unroll
    for (int q = 0; q < ITEMS / 4; ++q) {
      const uint4 x = vs[q];
      v[4 * q + 0] = x.x;
      v[4 * q + 1] = x.y;
      v[4 * q + 2] = x.z;
      v[4 * q + 3] = x.w;
    }
  }
}

// What one tile of one onesweep pass needs.  `in`/`out` (and `vin`/`vout`)
// are the array being sorted (a whole sort, or one segment of a batch),
// `n` its length, `bin_start` its 256 global bin starts for this digit and
// `status` its [tiles][256] look-back words for this pass.
template <typename K, typename S>
struct TileJob {
  const K* in;
  K* out;
  const uint32_t* vin;
  uint32_t* vout;
  size_t n;
  size_t out_n;  // output positions are below this (n, or the output array's length)
  uint32_t tile;
  uint32_t shift;
  bool tin;
  bool tout;
  const unsigned long long* bin_start;
  S* status;
  uint32_t* err;
  uint32_t spin_limit;  // look-back polls before giving up (kSpinLimit unless a test lowers it)
  // Prepared offsets (the first pass of a 32-bit keys-only sort, multisplit
  // ranking only): bin b of this tile starts at bin_start[b] + tile_prefix[tile][b]
  // + chunk_excl[tile / tiles_per_chunk][b]; the tile neither publishes nor
  // looks back.
  const uint32_t* tile_prefix = nullptr;
  const uint32_t* chunk_excl = nullptr;
  uint32_t tiles_per_chunk = 0;
};

// One tile of an onesweep digit pass (steps 2-6 above).  Called by all
// BLOCK threads after a barrier that ends every earlier use of `smem`;
// `s_bar` is an initialised mbarrier outside the tile's layout and `parity`
// the phase the next bulk copy completes (flipped here when one is used).
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, typename S>
__device__ __forceinline__ void onesweep_tile(const TileJob<K, S>& job, unsigned char* smem, uint64_t* s_bar,
                                              uint32_t& parity) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  static_assert(ITEMS <= 16, "per-thread ranks are packed in 4 bits");
  using SW = StatusWord<S>;
  constexpr int TILE = G::kTile;
  K* s_keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem + G::kCntOff);
  unsigned long long* s_bin_base = reinterpret_cast<unsigned long long*>(smem + G::kBinBaseOff);
  uint32_t* s_bin_start = reinterpret_cast<uint32_t*>(smem + G::kBinStartOff);
  uint32_t* s_bin_end = reinterpret_cast<uint32_t*>(smem + G::kBinEndOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + G::kWarpTotOff);
  uint32_t* s_abort = reinterpret_cast<uint32_t*>(smem + G::kAbortOff);

  // No __restrict__/read-only path: in a batched launch the input of a pass
  // was written by other CTAs of the same launch.
  const K* in = job.in;
  K* out = job.out;
  const uint32_t* vin = job.vin;
  uint32_t* vout = job.vout;
  const bool tin = job.tin;
  const bool tout = job.tout;
  const uint32_t shift = job.shift;
  const uint32_t tid = threadIdx.x;
  const uint32_t tile = job.tile;
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, job.n - tile_base);
  if (tid == 0) *s_abort = 0;

  // ---- 2. tile -> shared memory ---------------------------------------------
  const bool tma_ok = ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) &&
                      (!HAS_VALS || (reinterpret_cast<uintptr_t>(vin) & 15u) == 0);
  uint32_t loaded = 0;  // keys [0, loaded) arrive by bulk copy
  if (tma_ok) {
    const uint32_t kbulk = (tile_n * (uint32_t)sizeof(K)) & ~15u;
    const uint32_t vbulk = HAS_VALS ? ((tile_n * 4u) & ~15u) : 0u;
    if (tid == 0) {
      mbar_arrive_expect_tx(s_bar, kbulk + vbulk);
      fence_proxy_async();
      if (kbulk) bulk_load_g2s(s_keys, in + tile_base, kbulk, s_bar);
      if (HAS_VALS && vbulk) bulk_load_g2s(s_vals, vin + tile_base, vbulk, s_bar);
    }
    loaded = kbulk / (uint32_t)sizeof(K);
    if (HAS_VALS)
      for (uint32_t i = vbulk / 4u + tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
  } else if (HAS_VALS) {
    for (uint32_t i = tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
  }
  for (uint32_t i = loaded + tid; i < tile_n; i += BLOCK) s_keys[i] = in[tile_base + i];
  // padding: all-ones keys sort after every real key of any digit
  for (uint32_t i = tile_n + tid; i < (uint32_t)TILE; i += BLOCK) s_keys[i] = ~(K)0;
  for (uint32_t i = tid; i < (uint32_t)kRadix; i += BLOCK) {
    s_bin_start[i] = 0;
    s_bin_end[i] = 0;
  }
  bool tma_pending = false;  // this thread's wait for the tile's bulk copy gave up
  if (tma_ok) {
    tma_pending = !mbar_wait_bounded(s_bar, parity, job.err);
    if (tma_pending) *s_abort = 1;
    parity ^= 1u;
  }
  __syncthreads();

  // ---- 3. sort the tile by the digit: low nibble, then high nibble ------------
  K k[ITEMS];
  uint32_t v[HAS_VALS ? ITEMS : 1];
  load_run<K, HAS_VALS, ITEMS>(k, v, s_keys, s_vals);
  if (tin) {
    const uint32_t first = tid * ITEMS;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
      if (first + j < tile_n) k[j] = to_ordered(k[j], true);
  }
  nibble_pass<K, HAS_VALS, BLOCK, ITEMS>(k, v, shift, s_keys, s_vals, s_cnt, s_warp);
  load_run<K, HAS_VALS, ITEMS>(k, v, s_keys, s_vals);
  nibble_pass<K, HAS_VALS, BLOCK, ITEMS>(k, v, shift + 4, s_keys, s_vals, s_cnt, s_warp);

  // ---- 4. bin counts from run boundaries; publish --------------------------
  const uint32_t dsel = 0x4440u | ((shift >> 3) & 3u);
  const bool dupper = shift >= 32;
  const bool full = tile_n == (uint32_t)TILE;
  {
    const uint32_t first = tid * ITEMS;
    K run[ITEMS];
    uint32_t unused[1];
    load_run<K, false, ITEMS>(run, unused, s_keys, nullptr);
    uint32_t prev = first > 0 ? digit8(s_keys[first - 1], dsel, dupper) : 0xFFFFFFFFu;
    if (full) {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t d = digit8(run[j], dsel, dupper);
        if (d != prev) {
          s_bin_start[d] = first + j;
          if (first + j > 0) s_bin_end[prev] = first + j;
        }
        prev = d;
      }
      if (first + ITEMS == (uint32_t)TILE) s_bin_end[prev] = TILE;
    } else {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t i = first + j;
        if (i < tile_n) {
          const uint32_t d = digit8(run[j], dsel, dupper);
          if (d != prev) {
            s_bin_start[d] = i;
            if (i > 0) s_bin_end[prev] = i;
          }
          if (i + 1 == tile_n) s_bin_end[d] = tile_n;
          prev = d;
        }
      }
    }
  }
  __syncthreads();
  uint32_t count = 0;
  if (tid < (uint32_t)kRadix) {
    count = s_bin_end[tid] - s_bin_start[tid];
    S* st = job.status + (size_t)tile * kRadix + tid;
    st_relaxed_gpu(st, (S)((tile == 0 ? SW::kIncl : SW::kAgg) | (S)count));
  }

  // ---- 5. decoupled look-back ---------------------------------------------
  // Offsets are kept in the status word type: 32-bit when n < 2^30.
  S* s_base = reinterpret_cast<S*>(s_bin_base);
  if (tid < (uint32_t)kRadix) {
    S excl = 0;
    if (tile > 0) {
      const S* base = job.status + tid;
      long long t = (long long)tile - 1;
      uint32_t spins = 0;
      bool done = false;
      while (!done) {
        S sw[kLookbackWidth];
#pragma unroll
        for (int i = 0; i < kLookbackWidth; ++i)
          sw[i] = (t - i >= 0) ? ld_relaxed_gpu(base + (size_t)(t - i) * kRadix) : (S)SW::kIncl;
        int used = 0;
#pragma unroll
        for (int i = 0; i < kLookbackWidth; ++i) {
          if (done || used != i) break;
          const uint32_t flag = (uint32_t)(sw[i] >> SW::kShift);
          if (flag == 0) break;
          excl += sw[i] & SW::kMask;
          ++used;
          if (flag == 2u) done = true;
        }
        t -= used;
        if (!done && used == 0) {
          ++spins;
          if (spins > job.spin_limit || ((spins & 1023u) == 0 && ld_relaxed_gpu(job.err) != 0)) {
            raise_error(job.err, DEVERR_LOOKBACK_TIMEOUT);
            *s_abort = 1;
            break;
          }
        }
      }
      S* st = job.status + (size_t)tile * kRadix + tid;
      st_relaxed_gpu(st, (S)(SW::kIncl | (S)(excl + count)));
    }
    s_base[tid] = (S)job.bin_start[tid] + excl - (S)s_bin_start[tid];
  }
  __syncthreads();

  // ---- 6. write out in bin-contiguous runs -----------------------------------
  // A tile whose look-back or load gave up has no valid offsets: it writes
  // nothing (the call reports the failure), and every store is bounds-checked.
  // A bulk copy that was waited for in vain gets one more bounded wait, so
  // that it cannot land in shared memory after the CTA has moved on.
  if (*s_abort) {
    if (tma_pending) mbar_wait_bounded(s_bar, parity ^ 1u, job.err);
    return;
  }
  const S n_out = (S)job.out_n;
  auto scatter = [&](auto transform) {
    if (full) {
#pragma unroll 4
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t i = (uint32_t)j * BLOCK + tid;
        const K key = s_keys[i];
        const S o = s_base[digit8(key, dsel, dupper)] + i;
        if (o < n_out) {
          out[o] = transform(key);
          if (HAS_VALS) vout[o] = s_vals[i];
        }
      }
    } else {
      for (uint32_t i = tid; i < tile_n; i += BLOCK) {
        const K key = s_keys[i];
        const S o = s_base[digit8(key, dsel, dupper)] + i;
        if (o < n_out) {
          out[o] = transform(key);
          if (HAS_VALS) vout[o] = s_vals[i];
        }
      }
    }
  };
  if (tout)
    scatter([](K x) { return from_ordered(x, true); });
  else
    scatter([](K x) { return x; });
}


// 8-bit warp multisplit: the mask of lanes whose digit equals this lane's,
// from eight ballots (no match instruction: on this GPU it runs on a slow
// pipe).  For bit b: p = bit b of d; ballot(p); keep lanes that agree.
__device__ __forceinline__ uint32_t match_digit8(uint32_t d) {
  uint32_t peers = 0xFFFFFFFFu;
#define PA_MATCH_BIT(B)                                         \
  asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\t"                   \
      "and.b32 t, %1, " #B ";\n\t"                                \
      "setp.ne.u32 p, t, 0;\n\t"                                  \
      "vote.sync.ballot.b32 t, p, 0xffffffff;\n\t"                \
      "@!p not.b32 t, t;\n\t"                                     \
      "and.b32 %0, %0, t;\n\t}"                                   \
      : "+r"(peers)                                              \
      : "r"(d));
  PA_MATCH_BIT(1)
  PA_MATCH_BIT(2)
  PA_MATCH_BIT(4)
  PA_MATCH_BIT(8)
  PA_MATCH_BIT(16)
  PA_MATCH_BIT(32)
  PA_MATCH_BIT(64)
  PA_MATCH_BIT(128)
#undef PA_MATCH_BIT
  return peers;
}

// Shared-memory places one multisplit tile uses: the tile buffer (keys and
// payloads) and the per-tile scratch (per-warp bin counters, bin bases and
// starts, tile bin counts, abort flag).
template <typename K, typename S>
struct TileSmem {
  K* keys;
  uint32_t* vals;
  uint32_t* wh;      // [warps][256] counters (and [warps][256] match words)
  S* base;           // [256] global base of each bin for this tile
  uint32_t* tstart;  // [256] first in-tile position of each bin
  uint32_t* tcount;  // [256] keys of each bin in the tile
  uint32_t* abort;
  uint32_t* pre = nullptr;  // [2][256]: the tile's prepared offset rows (tile_prefix, chunk_excl), if any
};

// Whether a pass can bulk-copy its tiles (16-byte aligned key and payload
// arrays); otherwise every key is read with plain loads.
template <typename K, bool HAS_VALS, typename S>
__device__ __forceinline__ bool tile_tma_ok(const TileJob<K, S>& job) {
  return ((reinterpret_cast<uintptr_t>(job.in) & 15u) == 0) &&
         (!HAS_VALS || (reinterpret_cast<uintptr_t>(job.vin) & 15u) == 0);
}

// Starts the bulk copy of tile `tile` into `keys` / `vals`, completing on
// `bar` (one thread calls it; the 16-byte multiple head of the tile only, the
// body reads the ragged rest), and with prepared offsets their two 1 KB rows
// into `pre`.  Nothing is issued for a pass that cannot bulk-copy.
template <typename K, bool HAS_VALS, int TILE, typename S>
__device__ __forceinline__ void tile_issue_load(const TileJob<K, S>& job, uint32_t tile, K* keys, uint32_t* vals,
                                                uint64_t* bar, uint32_t* pre = nullptr) {
  if (!tile_tma_ok<K, HAS_VALS>(job)) return;
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, job.n - tile_base);
  const uint32_t kbulk = (tile_n * (uint32_t)sizeof(K)) & ~15u;
  const uint32_t vbulk = HAS_VALS ? ((tile_n * 4u) & ~15u) : 0u;
  const bool prepared = pre != nullptr && job.tile_prefix != nullptr;
  const uint32_t pbulk = prepared ? 2u * kRadix * 4u : 0u;
  fence_proxy_async();
  mbar_arrive_expect_tx(bar, kbulk + vbulk + pbulk);
  if (kbulk) bulk_load_g2s(keys, job.in + tile_base, kbulk, bar);
  if (HAS_VALS && vbulk) bulk_load_g2s(vals, job.vin + tile_base, vbulk, bar);
  if (prepared) {
    bulk_load_g2s(pre, job.tile_prefix + (size_t)tile * kRadix, kRadix * 4u, bar);
    bulk_load_g2s(pre + kRadix, job.chunk_excl + (size_t)(tile / job.tiles_per_chunk) * kRadix, kRadix * 4u, bar);
  }
}

// Tuning switches of the multisplit ranking (compile-time):
//   PA_MATCH_ATOMIC_OR = 1: peers are found through shared memory instead of
//     ballots: each lane ORs its lane bit into its warp's word for its digit
//     and reads the word back; the group's leader clears it again.
#ifndef PA_MATCH_ATOMIC_OR
#define PA_MATCH_ATOMIC_OR 0
#endif
//   PA_MATCH_MIX = m > 0: items j with j % m == 0 find their peers through
//     shared memory (as PA_MATCH_ATOMIC_OR), the others with ballots, so the
//     integer pipe (ballots) and the shared-memory pipe (atomic OR, read
//     back, clear) share the matching work.  Default 3: measured fastest on
//     GB300 (100M u32 sort 1.78 ms against 1.86 ms all-ballot; 2 and 4-6 in
//     between, and all-atomic-OR is slower on skewed keys).  0 = ballots only.
#ifndef PA_MATCH_MIX
#define PA_MATCH_MIX 3
#endif
constexpr int kMatchWords = (PA_MATCH_ATOMIC_OR || PA_MATCH_MIX) ? 2 : 1;  // [warps][256] word arrays in TileSmem::wh

// Applies the float order transform to the tile in shared memory (first
// pass of a float sort), so that the ranking loop reads ordered keys.
template <typename K, int BLOCK>
__device__ __forceinline__ void order_tile_in_place(K* s_keys, uint32_t tile_n) {
  for (uint32_t i = threadIdx.x; i < tile_n; i += BLOCK) s_keys[i] = to_ordered(s_keys[i], true);
}

// One onesweep tile ranked by warp multisplit: warp w owns the contiguous
// run [w * 32 * ITEMS, (w + 1) * 32 * ITEMS) of the tile, lane l its items
// j * 32 + l; for each item the lanes holding the same digit (its peers) are
// found with the eight ballots of match_digit8, or for every PA_MATCH_MIX-th
// item by an atomic OR of the lane bit into the warp's shared word for the
// digit; every lane reads the warp's counter for that digit and takes
// counter + peers below it, then the group's lowest lane bumps the counter,
// so ranks follow tile order.
// Per-bin warp counters are scanned across warps into tile offsets; keys are
// staged in shared memory at their in-tile sorted position and written out
// in bin-contiguous runs after the look-back.
//
// Called by all BLOCK threads after a barrier that ends every earlier use of
// `sm`; the tile's bulk copy (if the pass bulk-copies) was started on `bar`
// with tile_issue_load, and `parity` is the phase it completes (flipped here).
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, typename S>
__device__ __forceinline__ void onesweep_tile_ms_body(const TileJob<K, S>& job, const TileSmem<K, S>& sm,
                                                      uint64_t* s_bar, uint32_t& parity) {
  using SW = StatusWord<S>;
  constexpr int TILE = BLOCK * ITEMS;
  constexpr int WARPS = BLOCK / 32;
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  K* s_keys = sm.keys;
  uint32_t* s_vals = sm.vals;
  uint32_t* s_wh = sm.wh;
  S* s_base = sm.base;
  uint32_t* s_tstart = sm.tstart;
  uint32_t* s_tcount = sm.tcount;
  uint32_t* s_abort = sm.abort;

  const K* in = job.in;
  K* out = job.out;
  const uint32_t* vin = job.vin;
  uint32_t* vout = job.vout;
  const uint32_t shift = job.shift;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const uint32_t tile = job.tile;
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, job.n - tile_base);
  const bool full = tile_n == (uint32_t)TILE;
  if (tid == 0) *s_abort = 0;
  for (uint32_t i = tid; i < (uint32_t)(kMatchWords * WARPS * kRadix); i += BLOCK) s_wh[i] = 0;

  // the ragged end (or, without bulk copies, everything) with plain loads
  const bool tma_ok = tile_tma_ok<K, HAS_VALS>(job);
  // Prepared offsets: their rows came with the bulk copy, or are read here
  // when the pass cannot bulk-copy (the barrier below orders either before use).
  const bool prepared = job.tile_prefix != nullptr;  // (set only where sm.pre is)
  if (prepared && !tma_ok)
    for (uint32_t i = tid; i < (uint32_t)kRadix; i += BLOCK) {
      sm.pre[i] = job.tile_prefix[(size_t)tile * kRadix + i];
      sm.pre[kRadix + i] = job.chunk_excl[(size_t)(tile / job.tiles_per_chunk) * kRadix + i];
    }
  uint32_t loaded = 0;
  if (tma_ok) {
    loaded = ((tile_n * (uint32_t)sizeof(K)) & ~15u) / (uint32_t)sizeof(K);
    if (HAS_VALS)
      for (uint32_t i = ((tile_n * 4u) & ~15u) / 4u + tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
  } else if (HAS_VALS) {
    for (uint32_t i = tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
  }
  for (uint32_t i = loaded + tid; i < tile_n; i += BLOCK) s_keys[i] = in[tile_base + i];
  // A short last tile is padded with all-ones keys: they rank after every
  // real key (in bin 255, after its real keys), so every tile is ranked as a
  // full one; they only raise the last tile's own bin-255 count, which no
  // later tile reads, and they are never written out.
  for (uint32_t i = tile_n + tid; i < (uint32_t)TILE; i += BLOCK) s_keys[i] = ~(K)0;
  bool tma_pending = false;  // this thread's wait for the tile's bulk copy gave up
  if (tma_ok) {
    tma_pending = !mbar_wait_bounded(s_bar, parity, job.err);
    if (tma_pending) *s_abort = 1;
    parity ^= 1u;
  }
  __syncthreads();
  if (job.tin) {
    order_tile_in_place<K, BLOCK>(s_keys, tile_n);
    __syncthreads();
  }

  // rank within the warp
  const uint32_t dsel = 0x4440u | ((shift >> 3) & 3u);
  const bool dupper = shift >= 32;
  const uint32_t lt = lanemask_lt();
  const uint32_t wbase = warp * ITEMS * 32;
  uint32_t* wh = s_wh + warp * kRadix;
  K k[ITEMS];
  uint32_t v[HAS_VALS ? ITEMS : 1];
  uint32_t rk[(ITEMS + 1) / 2];  // in-warp ranks (< 32 * ITEMS), two 16-bit halves per word
#pragma unroll
  for (int q = 0; q < (ITEMS + 1) / 2; ++q) rk[q] = 0;
  // all of the warp's keys into registers first, so that no item's counter
  // chain starts with a shared-memory load
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    k[j] = s_keys[idx];
    if (HAS_VALS) v[j] = s_vals[idx];
  }
  auto rank_item = [&](auto jc) {
    constexpr int j = decltype(jc)::value;
    const uint32_t d = digit8(k[j], dsel, dupper);
#if PA_MATCH_ATOMIC_OR || PA_MATCH_MIX
    constexpr bool kSmemMatch = PA_MATCH_ATOMIC_OR || (PA_MATCH_MIX > 0 && j % (PA_MATCH_MIX > 0 ? PA_MATCH_MIX : 1) == 0);
#else
    constexpr bool kSmemMatch = false;
#endif
    uint32_t peers;
    uint32_t* mw = s_wh + WARPS * kRadix + warp * kRadix + d;
    if constexpr (kSmemMatch) {
      atomicOr(mw, 1u << lane);
      __syncwarp();
      peers = *mw;
    } else {
      peers = match_digit8(d);
    }
    // Every lane reads the warp's counter for its digit; after the warp has
    // read, the group's lowest lane bumps it (and clears the match word).
    const uint32_t pl = peers & lt;
    const uint32_t base = wh[d];
    __syncwarp();
    if (pl == 0) {
      wh[d] = base + __popc(peers);
      if constexpr (kSmemMatch) *mw = 0u;
    }
    rk[j / 2] |= (base + __popc(pl)) << (16 * (j % 2));
    __syncwarp();
  };
  static_for<ITEMS>(rank_item);
  __syncthreads();

  // per bin: exclusive scan over warps, tile count, publish
  if (tid < (uint32_t)kRadix) {
    uint32_t sum = 0;
#pragma unroll 4
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s_wh[w * kRadix + tid];
      s_wh[w * kRadix + tid] = sum;
      sum += c;
    }
    s_tcount[tid] = sum;
    if (!prepared) {
      S* st = job.status + (size_t)tile * kRadix + tid;
      st_relaxed_gpu(st, (S)((tile == 0 ? SW::kIncl : SW::kAgg) | (S)sum));
    }
  }
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the 256 tile counts, 8 bins per lane
    uint32_t c[kRadix / 32];
    uint32_t local = 0;
#pragma unroll
    for (int i = 0; i < kRadix / 32; ++i) {
      c[i] = s_tcount[lane * (kRadix / 32) + i];
      local += c[i];
    }
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(FULL, incl, o);
      if (lane >= (uint32_t)o) incl += t;
    }
    uint32_t run = incl - local;
#pragma unroll
    for (int i = 0; i < kRadix / 32; ++i) {
      s_tstart[lane * (kRadix / 32) + i] = run;
      run += c[i];
    }
  }
  __syncthreads();
  if (tid < (uint32_t)kRadix) {  // fold the tile offset of each bin into the warp offsets
    const uint32_t ts = s_tstart[tid];
#pragma unroll 4
    for (int w = 0; w < WARPS; ++w) s_wh[w * kRadix + tid] += ts;
  }
  __syncthreads();

  // stage keys at their in-tile sorted position; then the look-back
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t pos = wh[digit8(k[j], dsel, dupper)] + ((rk[j / 2] >> (16 * (j % 2))) & 0xFFFFu);
    s_keys[pos] = k[j];
    if (HAS_VALS) s_vals[pos] = v[j];
  }
  if (tid < (uint32_t)kRadix) {
    const uint32_t count = s_tcount[tid];
    S excl = 0;
    if (prepared) {
      excl = (S)sm.pre[tid] + (S)sm.pre[kRadix + tid];
    } else if (tile > 0) {
      const S* base = job.status + tid;
      long long t = (long long)tile - 1;
      uint32_t spins = 0;
      bool done = false;
      while (!done) {
        S sw[kLookbackWidth];
#pragma unroll
        for (int i = 0; i < kLookbackWidth; ++i)
          sw[i] = (t - i >= 0) ? ld_relaxed_gpu(base + (size_t)(t - i) * kRadix) : (S)SW::kIncl;
        int used = 0;
#pragma unroll
        for (int i = 0; i < kLookbackWidth; ++i) {
          if (done || used != i) break;
          const uint32_t flag = (uint32_t)(sw[i] >> SW::kShift);
          if (flag == 0) break;
          excl += sw[i] & SW::kMask;
          ++used;
          if (flag == 2u) done = true;
        }
        t -= used;
        if (!done && used == 0) {
          ++spins;
          // give up once the limit is reached, or early once another tile
          // has already reported a failure (its successors would wait in vain)
          if (spins > job.spin_limit || ((spins & 1023u) == 0 && ld_relaxed_gpu(job.err) != 0)) {
            raise_error(job.err, DEVERR_LOOKBACK_TIMEOUT);
            *s_abort = 1;
            break;
          }
        }
      }
      S* st = job.status + (size_t)tile * kRadix + tid;
      st_relaxed_gpu(st, (S)(SW::kIncl | (S)(excl + count)));
    }
    s_base[tid] = (S)job.bin_start[tid] + excl - (S)s_tstart[tid];
  }
  __syncthreads();

  // write out in bin-contiguous runs (nothing after a failed wait; a bulk
  // copy waited for in vain gets one more bounded wait first)
  if (*s_abort) {
    if (tma_pending) mbar_wait_bounded(s_bar, parity ^ 1u, job.err);
    return;
  }
  const S n_out = (S)job.out_n;
  auto scatter = [&](auto transform) {
    if (full) {
#pragma unroll 4
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t i = (uint32_t)j * BLOCK + tid;
        const K key = s_keys[i];
        const S o = s_base[digit8(key, dsel, dupper)] + i;
        if (o < n_out) {
          out[o] = transform(key);
          if (HAS_VALS) vout[o] = s_vals[i];
        }
      }
    } else {
      for (uint32_t i = tid; i < tile_n; i += BLOCK) {
        const K key = s_keys[i];
        const S o = s_base[digit8(key, dsel, dupper)] + i;
        if (o < n_out) {
          out[o] = transform(key);
          if (HAS_VALS) vout[o] = s_vals[i];
        }
      }
    }
  };
  if (job.tout)
    scatter([](K x) { return from_ordered(x, true); });
  else
    scatter([](K x) { return x; });
}

// ---------------------------------------------------------------------------
// Wide-digit tile: the multisplit tile for RB-bit digits with RB > 8 (11:
// 2048 bins, three passes for 32-bit keys).  Same steps as the 8-bit body
// above, with what changes when a tile has 2048 bins:
//   - the peers of a key come from RB ballots (no shared-memory match words:
//     [warps][2048] of them would not fit next to the counters);
//   - the warps' counters are 16-bit ([warps][2048] x 2 bytes; a warp's count
//     and the in-tile starts folded into it stay below 2^16);
//   - the per-bin scans, the in-tile bin starts and the look-back loop over
//     the bins, each thread owning 2048 / BLOCK of them (its look-back walks
//     them in lockstep, their loads in flight together);
//   - the digit is (key >> shift) & (2^RB - 1).
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int RB>
struct WideGeometry {
  static constexpr int kWarps = BLOCK / 32;
  static constexpr int kTile = BLOCK * ITEMS;
  static constexpr int kBins = 1 << RB;
  static constexpr size_t kKeysOff = 0;
  static constexpr size_t kValsOff = kKeysOff + (size_t)kTile * sizeof(K);
  static constexpr size_t kWhOff = kValsOff + (HAS_VALS ? (size_t)kTile * 4 : 0);          // [warps][bins] u16
  static constexpr size_t kBaseOff = kWhOff + (((size_t)kWarps * kBins * 2 + 15) & ~(size_t)15);  // [bins] 8 B
  static constexpr size_t kTstartOff = kBaseOff + (size_t)kBins * 8;                          // [bins] u32
  static constexpr size_t kTcountOff = kTstartOff + (size_t)kBins * 4;                        // [bins] u32
  static constexpr size_t kWarpTotOff = kTcountOff + (size_t)kBins * 4;                       // [warps] u32
  static constexpr size_t kBarOff = kWarpTotOff + (((size_t)kWarps * 4 + 7) & ~(size_t)7);
  static constexpr size_t kTileIdOff = kBarOff + 8;
  static constexpr size_t kAbortOff = kTileIdOff + 4;
  static constexpr size_t kBytes = kAbortOff + 4;
  static_assert(kBins % BLOCK == 0, "every thread owns the same number of bins");
  static_assert(kTile + 32 * ITEMS < 65536, "16-bit counters hold in-tile positions");
  static_assert(kTile % 4 == 0 && kValsOff % 16 == 0, "tile buffers stay 16-byte aligned");
};

// Lanes whose RB-bit digit equals this lane's, from RB ballots.
template <int RB>
__device__ __forceinline__ uint32_t match_bits(uint32_t d) {
  uint32_t peers = 0xFFFFFFFFu;
  static_for<RB>([&](auto bc) {
    constexpr uint32_t B = 1u << decltype(bc)::value;
    asm("{\n\t.reg .pred p;\n\t.reg .b32 t;\n\t"
        "and.b32 t, %1, %2;\n\t"
        "setp.ne.u32 p, t, 0;\n\t"
        "vote.sync.ballot.b32 t, p, 0xffffffff;\n\t"
        "@!p not.b32 t, t;\n\t"
        "and.b32 %0, %0, t;\n\t}"
        : "+r"(peers)
        : "r"(d), "n"(B));
  });
  return peers;
}

template <int RB, typename K>
__device__ __forceinline__ uint32_t digit_wide(K key, uint32_t shift) {
  return (uint32_t)(key >> shift) & ((1u << RB) - 1u);
}

// One wide-digit tile in the WideGeometry layout at `smem`: starts its bulk
// copy (thread 0) and sorts, publishes and writes it out.  Called by all
// BLOCK threads after a barrier that ends every earlier use of `smem`.
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int RB, typename S>
__device__ __forceinline__ void onesweep_tile_wide(const TileJob<K, S>& job, unsigned char* smem, uint64_t* s_bar,
                                                   uint32_t& parity) {
  using G = WideGeometry<K, HAS_VALS, BLOCK, ITEMS, RB>;
  using SW = StatusWord<S>;
  constexpr int TILE = G::kTile;
  constexpr int WARPS = G::kWarps;
  constexpr int R = G::kBins;
  constexpr int BPT = R / BLOCK;  // bins per thread
  K* s_keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  uint16_t* s_wh = reinterpret_cast<uint16_t*>(smem + G::kWhOff);
  S* s_base = reinterpret_cast<S*>(smem + G::kBaseOff);
  uint32_t* s_tstart = reinterpret_cast<uint32_t*>(smem + G::kTstartOff);
  uint32_t* s_tcount = reinterpret_cast<uint32_t*>(smem + G::kTcountOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + G::kWarpTotOff);
  uint32_t* s_abort = reinterpret_cast<uint32_t*>(smem + G::kAbortOff);

  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const uint32_t tile = job.tile;
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, job.n - tile_base);
  const uint32_t shift = job.shift;
  if (tid == 0) {
    *s_abort = 0;
    tile_issue_load<K, HAS_VALS, TILE>(job, tile, s_keys, s_vals, s_bar);
  }
  uint32_t* wh_words = reinterpret_cast<uint32_t*>(s_wh);
  for (uint32_t i = tid; i < (uint32_t)(WARPS * R / 2); i += BLOCK) wh_words[i] = 0;
  const bool tma_ok = tile_tma_ok<K, HAS_VALS>(job);
  uint32_t loaded = 0;
  if (tma_ok) {
    loaded = ((tile_n * (uint32_t)sizeof(K)) & ~15u) / (uint32_t)sizeof(K);
    if (HAS_VALS)
      for (uint32_t i = ((tile_n * 4u) & ~15u) / 4u + tid; i < tile_n; i += BLOCK) s_vals[i] = job.vin[tile_base + i];
  } else if (HAS_VALS) {
    for (uint32_t i = tid; i < tile_n; i += BLOCK) s_vals[i] = job.vin[tile_base + i];
  }
  for (uint32_t i = loaded + tid; i < tile_n; i += BLOCK) s_keys[i] = job.in[tile_base + i];
  // a short last tile is padded with all-ones keys (see the 8-bit body)
  for (uint32_t i = tile_n + tid; i < (uint32_t)TILE; i += BLOCK) s_keys[i] = ~(K)0;
  bool tma_pending = false;
  if (tma_ok) {
    tma_pending = !mbar_wait_bounded(s_bar, parity, job.err);
    if (tma_pending) *s_abort = 1;
    parity ^= 1u;
  }
  __syncthreads();
  if (job.tin) {
    order_tile_in_place<K, BLOCK>(s_keys, tile_n);
    __syncthreads();
  }

  // rank within the warp
  const uint32_t lt = lanemask_lt();
  const uint32_t wbase = warp * ITEMS * 32;
  uint16_t* wh = s_wh + warp * R;
  K k[ITEMS];
  uint32_t v[HAS_VALS ? ITEMS : 1];
  uint32_t rk[(ITEMS + 1) / 2];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    k[j] = s_keys[idx];
    if (HAS_VALS) v[j] = s_vals[idx];
  }
#pragma unroll
  for (int q = 0; q < (ITEMS + 1) / 2; ++q) rk[q] = 0;
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t d = digit_wide<RB>(k[j], shift);
    const uint32_t peers = match_bits<RB>(d);
    const uint32_t pl = peers & lt;
    const uint32_t base = wh[d];
    __syncwarp();
    if (pl == 0) wh[d] = (uint16_t)(base + __popc(peers));
    rk[j / 2] |= (base + __popc(pl)) << (16 * (j % 2));
    __syncwarp();
  }
  __syncthreads();

  // per bin: exclusive scan over the warps, tile count, publish
#pragma unroll
  for (int m = 0; m < BPT; ++m) {
    const uint32_t b = tid + (uint32_t)m * BLOCK;
    uint32_t sum = 0;
#pragma unroll 4
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s_wh[w * R + b];
      s_wh[w * R + b] = (uint16_t)sum;
      sum += c;
    }
    s_tcount[b] = sum;
    st_relaxed_gpu(job.status + (size_t)tile * R + b, (S)((tile == 0 ? SW::kIncl : SW::kAgg) | (S)sum));
  }
  __syncthreads();
  {  // in-tile bin starts: thread t scans bins [t * BPT, (t + 1) * BPT)
    uint32_t c[BPT];
    uint32_t local = 0;
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      c[i] = s_tcount[tid * BPT + i];
      local += c[i];
    }
    uint32_t run = block_exclusive_scan<BLOCK>(local, s_warp);
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      s_tstart[tid * BPT + i] = run;
      run += c[i];
    }
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < BPT; ++m) {  // fold the in-tile start of each bin into the warp offsets
    const uint32_t b = tid + (uint32_t)m * BLOCK;
    const uint32_t ts = s_tstart[b];
#pragma unroll 4
    for (int w = 0; w < WARPS; ++w) s_wh[w * R + b] = (uint16_t)(s_wh[w * R + b] + ts);
  }
  __syncthreads();

  // stage keys at their in-tile sorted position; then the look-back
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t pos = wh[digit_wide<RB>(k[j], shift)] + ((rk[j / 2] >> (16 * (j % 2))) & 0xFFFFu);
    s_keys[pos] = k[j];
    if (HAS_VALS) s_vals[pos] = v[j];
  }
  {
    S excl[BPT];
#pragma unroll
    for (int m = 0; m < BPT; ++m) excl[m] = 0;
    if (tile > 0) {
      long long t[BPT];
      bool done[BPT];
#pragma unroll
      for (int m = 0; m < BPT; ++m) {
        t[m] = (long long)tile - 1;
        done[m] = false;
      }
      uint32_t spins = 0;
      bool all_done = false;
      while (!all_done) {
        S sw[BPT][kLookbackWidth];
#pragma unroll
        for (int m = 0; m < BPT; ++m) {
          const S* base = job.status + tid + (size_t)m * BLOCK;
#pragma unroll
          for (int i = 0; i < kLookbackWidth; ++i)
            sw[m][i] = (!done[m] && t[m] - i >= 0) ? ld_relaxed_gpu(base + (size_t)(t[m] - i) * R) : (S)SW::kIncl;
        }
        bool progress = false;
        all_done = true;
#pragma unroll
        for (int m = 0; m < BPT; ++m) {
          if (!done[m]) {
            int used = 0;
#pragma unroll
            for (int i = 0; i < kLookbackWidth; ++i) {
              if (done[m] || used != i) break;
              const uint32_t flag = (uint32_t)(sw[m][i] >> SW::kShift);
              if (flag == 0) break;
              excl[m] += sw[m][i] & SW::kMask;
              ++used;
              if (flag == 2u) done[m] = true;
            }
            t[m] -= used;
            progress |= used > 0;
          }
          all_done &= done[m];
        }
        if (!all_done && !progress) {
          ++spins;
          if (spins > job.spin_limit || ((spins & 1023u) == 0 && ld_relaxed_gpu(job.err) != 0)) {
            raise_error(job.err, DEVERR_LOOKBACK_TIMEOUT);
            *s_abort = 1;
            break;
          }
        }
      }
    }
#pragma unroll
    for (int m = 0; m < BPT; ++m) {
      const uint32_t b = tid + (uint32_t)m * BLOCK;
      if (tile > 0)  // published even after a timeout, so that no successor waits on this tile
        st_relaxed_gpu(job.status + (size_t)tile * R + b, (S)(SW::kIncl | (excl[m] + (S)s_tcount[b])));
      s_base[b] = (S)job.bin_start[b] + excl[m] - (S)s_tstart[b];
    }
  }
  __syncthreads();

  // write out in bin-contiguous runs (nothing after a failed wait)
  if (*s_abort) {
    if (tma_pending) mbar_wait_bounded(s_bar, parity ^ 1u, job.err);
    return;
  }
  const S n_out = (S)job.out_n;
  const bool full = tile_n == (uint32_t)TILE;
  auto scatter = [&](auto toutc) {
    constexpr bool TOUT = decltype(toutc)::value;
    if (full) {
#pragma unroll 4
      for (int j = 0; j < ITEMS; ++j) {
        const uint32_t i = (uint32_t)j * BLOCK + tid;
        const K key = s_keys[i];
        const S o = s_base[digit_wide<RB>(key, shift)] + i;
        job.out[o] = TOUT ? from_ordered(key, true) : key;
        if (HAS_VALS) job.vout[o] = s_vals[i];
      }
    } else {
      for (uint32_t i = tid; i < tile_n; i += BLOCK) {
        const K key = s_keys[i];
        const S o = s_base[digit_wide<RB>(key, shift)] + i;
        if (o < n_out) {
          job.out[o] = TOUT ? from_ordered(key, true) : key;
          if (HAS_VALS) job.vout[o] = s_vals[i];
        }
      }
    }
  };
  if (job.tout)
    scatter(std::true_type{});
  else
    scatter(std::false_type{});
}

// One multisplit tile in the Geometry layout (one tile buffer at offset 0):
// starts its bulk copy and runs the body.  Used where one CTA handles one
// tile at a time (the batched kernel).
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, typename S>
__device__ __forceinline__ void onesweep_tile_multisplit(const TileJob<K, S>& job, unsigned char* smem,
                                                         uint64_t* s_bar, uint32_t& parity) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  static_assert((size_t)kMatchWords * G::kWarps * kRadix <= (size_t)kNibbleBins * G::kCntRow,
                "warp counters (and match words) fit the counter area");
  TileSmem<K, S> sm;
  sm.keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  sm.vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  sm.wh = reinterpret_cast<uint32_t*>(smem + G::kCntOff);
  sm.base = reinterpret_cast<S*>(smem + G::kBinBaseOff);
  sm.tstart = reinterpret_cast<uint32_t*>(smem + G::kBinStartOff);
  sm.tcount = reinterpret_cast<uint32_t*>(smem + G::kBinEndOff);
  sm.abort = reinterpret_cast<uint32_t*>(smem + G::kAbortOff);
  // the prepared offset rows sit in the counter area's last 2 KB, which the
  // warp counters and match words leave free
  static_assert((size_t)kMatchWords * G::kWarps * kRadix + 2 * kRadix <= (size_t)kNibbleBins * G::kCntRow,
                "the prepared offset rows fit after the warp counters");
  sm.pre = sm.wh + (size_t)kMatchWords * G::kWarps * kRadix;
  if (threadIdx.x == 0) tile_issue_load<K, HAS_VALS, G::kTile>(job, job.tile, sm.keys, sm.vals, s_bar, sm.pre);
  onesweep_tile_ms_body<K, HAS_VALS, BLOCK, ITEMS, S>(job, sm, s_bar, parity);
}

}  // namespace os
}  // namespace pa
