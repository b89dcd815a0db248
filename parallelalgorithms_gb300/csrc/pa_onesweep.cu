// Onesweep digit pass: one launch moves every key (and payload) to its
// position for one 8-bit digit, stably.
//
// GPU form of the reference's per-digit work in SortRadixInnerPar
// (RadixSortLsdParallel.h:253-322): its per-quantum histogram
// (ComputeStartOfBinsPar, :108-165) becomes a per-tile histogram whose
// cross-tile prefix is found by decoupled look-back instead of a serial
// Q x 256 prefix, and its de-randomised per-bin write buffers
// (PermuteDerandomizedNew, :169-212) become a tile sorted by digit in shared
// memory and written out in bin-contiguous runs.
//
// Per CTA (one tile of TILE = BLOCK * ITEMS keys):
//   1. take the next tile ticket (tickets are handed out in launch order, so
//      every tile a CTA waits on in step 5 is owned by a CTA already running);
//   2. bulk-copy the tile global -> shared with the TMA engine, completing on
//      an mbarrier (plain loads for the <16-byte ragged end, or when a buffer
//      is not 16-byte aligned); a partial tile is padded with all-ones keys,
//      which sort after every real key;
//   3. sort the tile by the 8-bit digit in shared memory as two stable 4-bit
//      counting passes (low nibble, then high nibble).  Each thread owns ITEMS
//      consecutive keys, so (thread, item) order is input order; per-thread
//      counters live in shared memory at [nibble][thread], one bank per
//      thread, so counting is conflict-free and needs no warp-wide matching;
//      a block-wide exclusive scan of the counters gives each key its
//      position;
//   4. bin counts of the tile from the run boundaries of the sorted tile;
//      publish them (AGGREGATE, or INCLUSIVE for tile 0);
//   5. per bin, walk back over earlier tiles' words, four tiles per round
//      trip, until an INCLUSIVE one; publish INCLUSIVE;
//   6. write the sorted tile out: consecutive threads write consecutive keys
//      of a bin to consecutive addresses.
#include <cstdio>
#include <cstdlib>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kNibbleBins = 16;
constexpr int kLookbackWidth = 4;  // predecessor tiles read per round trip

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
  static_assert(ITEMS <= 16, "per-thread ranks are packed in 4 bits");
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

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_kernel(const OnesweepArgs args) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  using SW = StatusWord<S>;
  constexpr int TILE = G::kTile;

  const PassCtrl pc = args.ctrl->pass[args.pass];
  if (pc.skip) return;

  extern __shared__ __align__(128) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem + G::kCntOff);
  unsigned long long* s_bin_base = reinterpret_cast<unsigned long long*>(smem + G::kBinBaseOff);
  uint32_t* s_bin_start = reinterpret_cast<uint32_t*>(smem + G::kBinStartOff);
  uint32_t* s_bin_end = reinterpret_cast<uint32_t*>(smem + G::kBinEndOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + G::kWarpTotOff);
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + G::kBarOff);
  uint32_t* s_tile_id = reinterpret_cast<uint32_t*>(smem + G::kTileIdOff);
  uint32_t* s_abort = reinterpret_cast<uint32_t*>(smem + G::kAbortOff);

  const K* __restrict__ in = static_cast<const K*>(pc.src_is_tmp ? args.keys_b : args.keys_a);
  K* __restrict__ out = static_cast<K*>(pc.src_is_tmp ? args.keys_a : args.keys_b);
  const uint32_t* __restrict__ vin = pc.src_is_tmp ? args.vals_b : args.vals_a;
  uint32_t* __restrict__ vout = pc.src_is_tmp ? args.vals_a : args.vals_b;
  const bool tin = args.is_float && pc.transform_in;
  const bool tout = args.is_float && pc.transform_out;
  const uint32_t shift = args.shift;
  const uint32_t tid = threadIdx.x;

  // ---- 1. ticket -------------------------------------------------------------
  if (tid == 0) {
    *s_tile_id = atomicAdd(args.tile_counter, 1u);
    *s_abort = 0;
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const uint32_t tile = *s_tile_id;
  const size_t num_tiles = (args.n + TILE - 1) / TILE;
  if ((size_t)tile >= num_tiles) {  // a ticket counter that was not reset
    if (tid == 0) raise_error(args.err, DEVERR_BAD_STATE);
    return;
  }
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, args.n - tile_base);

  // ---- 2. tile -> shared memory ---------------------------------------------
  const bool tma_ok = ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) &&
                      (!HAS_VALS || (reinterpret_cast<uintptr_t>(vin) & 15u) == 0);
  uint32_t loaded = 0;  // keys [0, loaded) arrive by bulk copy
  if (tma_ok) {
    const uint32_t kbulk = (tile_n * (uint32_t)sizeof(K)) & ~15u;
    const uint32_t vbulk = HAS_VALS ? ((tile_n * 4u) & ~15u) : 0u;
    if (tid == 0) {
      mbar_arrive_expect_tx(s_bar, kbulk + vbulk);
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
  if (tma_ok && !mbar_wait_bounded(s_bar, 0, args.err)) *s_abort = 1;
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
    S* st = static_cast<S*>(args.status) + (size_t)tile * kRadix + tid;
    st_relaxed_gpu(st, (S)((tile == 0 ? SW::kIncl : SW::kAgg) | (S)count));
  }

  // ---- 5. decoupled look-back ---------------------------------------------
  // Offsets are kept in the status word type: 32-bit when n < 2^30.
  S* s_base = reinterpret_cast<S*>(s_bin_base);
  if (tid < (uint32_t)kRadix) {
    S excl = 0;
    if (tile > 0) {
      const S* base = static_cast<const S*>(args.status) + tid;
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
        if (!done && used == 0 && ++spins > kSpinLimit) {
          raise_error(args.err, DEVERR_LOOKBACK_TIMEOUT);
          *s_abort = 1;
          break;
        }
      }
      S* st = static_cast<S*>(args.status) + (size_t)tile * kRadix + tid;
      st_relaxed_gpu(st, (S)(SW::kIncl | (S)(excl + count)));
    }
    s_base[tid] = (S)args.bin_start[tid] + excl - (S)s_bin_start[tid];
  }
  __syncthreads();

  // ---- 6. write out in bin-contiguous runs -----------------------------------
  // A tile whose look-back or load gave up has no valid offsets: it writes
  // nothing (the call reports the failure), and every store is bounds-checked.
  if (*s_abort) return;
  const S n_out = (S)args.n;
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

template <typename K>
__global__ void final_copy_kernel(K* keys_a, const K* keys_b, uint32_t* vals_a, const uint32_t* vals_b, size_t n,
                                  const SortCtrl* ctrl) {
  if (!ctrl->final_in_tmp) return;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    keys_a[i] = keys_b[i];
    if (vals_a) vals_a[i] = vals_b[i];
  }
}

// Tile geometries.  Each is (threads, keys per thread, CTAs per SM the
// register budget is cut for).  The active one per (key type, payload) is
// the first entry unless PA_ONESWEEP_GEOMETRY selects another (tuning).
struct GeomChoice {
  int block, items, minb;
};
constexpr GeomChoice kGeomU32[] = {{512, 16, 2}, {256, 16, 4}, {384, 16, 3}, {1024, 8, 1}, {512, 8, 3}};
constexpr GeomChoice kGeomU32Kv[] = {{512, 12, 2}, {256, 12, 4}, {512, 8, 3}};
constexpr GeomChoice kGeomU64[] = {{256, 12, 4}, {512, 12, 2}, {512, 8, 3}};
constexpr GeomChoice kGeomU64Kv[] = {{256, 12, 3}, {256, 8, 4}, {512, 8, 2}};

int geometry_index(int count) {
  static int idx = -2;
  if (idx == -2) {
    const char* e = std::getenv("PA_ONESWEEP_GEOMETRY");
    idx = e ? std::atoi(e) : 0;
  }
  return (idx >= 0 && idx < count) ? idx : 0;
}

template <typename K, bool HAS_VALS>
GeomChoice active_geometry() {
  if (sizeof(K) == 4 && !HAS_VALS) return kGeomU32[geometry_index(5)];
  if (sizeof(K) == 4) return kGeomU32Kv[geometry_index(3)];
  if (!HAS_VALS) return kGeomU64[geometry_index(3)];
  return kGeomU64Kv[geometry_index(3)];
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S>
cudaError_t launch_g(const OnesweepArgs& a, cudaStream_t stream) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  auto kern = onesweep_kernel<K, HAS_VALS, BLOCK, ITEMS, MINB, S>;
  static bool configured = false;  // one attribute call per instantiation
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kBytes);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const size_t tiles = ceil_div(a.n, (size_t)G::kTile);
  kern<<<(unsigned)tiles, BLOCK, G::kBytes, stream>>>(a);
  return cudaGetLastError();
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB>
cudaError_t launch_s(const OnesweepArgs& a, cudaStream_t stream) {
  if (a.n < (1ull << 30)) return launch_g<K, HAS_VALS, BLOCK, ITEMS, MINB, uint32_t>(a, stream);
  return launch_g<K, HAS_VALS, BLOCK, ITEMS, MINB, unsigned long long>(a, stream);
}

#define PA_GEOM_CASE(B, I, M) \
  if (g.block == B && g.items == I && g.minb == M) return launch_s<K, HAS_VALS, B, I, M>(a, stream);

template <typename K, bool HAS_VALS>
cudaError_t launch_kv(const OnesweepArgs& a, cudaStream_t stream) {
  const GeomChoice g = active_geometry<K, HAS_VALS>();
  if constexpr (sizeof(K) == 4 && !HAS_VALS) {
    PA_GEOM_CASE(512, 16, 2)
    PA_GEOM_CASE(256, 16, 4)
    PA_GEOM_CASE(384, 16, 3)
    PA_GEOM_CASE(1024, 8, 1)
    PA_GEOM_CASE(512, 8, 3)
  } else if constexpr (sizeof(K) == 4) {
    PA_GEOM_CASE(512, 12, 2)
    PA_GEOM_CASE(256, 12, 4)
    PA_GEOM_CASE(512, 8, 3)
  } else if constexpr (!HAS_VALS) {
    PA_GEOM_CASE(256, 12, 4)
    PA_GEOM_CASE(512, 12, 2)
    PA_GEOM_CASE(512, 8, 3)
  } else {
    PA_GEOM_CASE(256, 12, 3)
    PA_GEOM_CASE(256, 8, 4)
    PA_GEOM_CASE(512, 8, 2)
  }
  return cudaErrorInvalidConfiguration;
}

}  // namespace

size_t onesweep_tile_keys(int key_bytes, bool has_vals) {
  GeomChoice g;
  if (key_bytes == 4)
    g = has_vals ? active_geometry<uint32_t, true>() : active_geometry<uint32_t, false>();
  else
    g = has_vals ? active_geometry<unsigned long long, true>() : active_geometry<unsigned long long, false>();
  return (size_t)g.block * g.items;
}

size_t onesweep_status_bytes(size_t n) { return n < (1ull << 30) ? 4 : 8; }

cudaError_t launch_onesweep_pass(const OnesweepArgs& a, int key_bytes, bool has_vals, cudaStream_t stream) {
  if (a.n == 0) return cudaSuccess;
  if (key_bytes == 4) return has_vals ? launch_kv<uint32_t, true>(a, stream) : launch_kv<uint32_t, false>(a, stream);
  return has_vals ? launch_kv<unsigned long long, true>(a, stream) : launch_kv<unsigned long long, false>(a, stream);
}

cudaError_t launch_final_copy(void* keys_a, const void* keys_b, uint32_t* vals_a, const uint32_t* vals_b,
                              size_t n, int key_bytes, const SortCtrl* ctrl, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const int block = 256;
  const unsigned grid = (unsigned)min(ceil_div(n, (size_t)block), (size_t)device_info().sm_count * 8);
  if (key_bytes == 4)
    final_copy_kernel<uint32_t><<<grid, block, 0, stream>>>(static_cast<uint32_t*>(keys_a),
                                                            static_cast<const uint32_t*>(keys_b), vals_a, vals_b, n,
                                                            ctrl);
  else
    final_copy_kernel<unsigned long long><<<grid, block, 0, stream>>>(
        static_cast<unsigned long long*>(keys_a), static_cast<const unsigned long long*>(keys_b), vals_a, vals_b, n,
        ctrl);
  return cudaGetLastError();
}

}  // namespace pa
