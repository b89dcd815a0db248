// Onesweep digit pass: one launch moves every key (and payload) to its
// position for one 8-bit digit, stably.
//
// GPU form of the reference's per-digit work in SortRadixInnerPar
// (RadixSortLsdParallel.h:253-322): its per-quantum histogram
// (ComputeStartOfBinsPar, :108-165) becomes a per-tile histogram whose
// cross-tile prefix is found by decoupled look-back instead of a serial
// Q x 256 prefix, and its de-randomised per-bin write buffers
// (PermuteDerandomizedNew, :169-212) become a tile staged by bin in shared
// memory and written out in bin-contiguous runs.
//
// Per CTA (one tile of TILE = BLOCK * ITEMS keys):
//   1. take the next tile ticket (tiles are handed out in launch order, so
//      every tile a CTA waits on in step 4 is owned by a CTA already running);
//   2. bulk-copy the tile global -> shared with the TMA engine, completing on
//      an mbarrier (plain loads for the <16-byte ragged end, or when a
//      buffer is not 16-byte aligned);
//   3. rank: each warp owns a contiguous 32 * ITEMS run of the tile; for each
//      item, __match_any_sync groups lanes holding the same digit, the group
//      leader bumps the warp's shared counter for that digit, and lanes take
//      rank = counter + peers below them.  Items are visited in tile order, so
//      ranks preserve input order (stability);
//   4. per bin: prefix of the warp counters, publish the tile's count
//      (AGGREGATE), walk back over earlier tiles' words until an INCLUSIVE
//      one, publish INCLUSIVE;
//   5. write keys into shared memory at their in-tile sorted position;
//   6. write the sorted tile out: consecutive threads write consecutive keys
//      of a bin to consecutive addresses.
#include <cstdio>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;

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
  static constexpr size_t kWarpHistOff = kValsOff + (HAS_VALS ? (size_t)kTile * 4 : 0);
  static constexpr size_t kBinBaseOff = kWarpHistOff + (size_t)kWarps * kRadix * 4;
  static constexpr size_t kTileCountOff = kBinBaseOff + (size_t)kRadix * 8;
  static constexpr size_t kTileStartOff = kTileCountOff + (size_t)kRadix * 4;
  static constexpr size_t kExclOff = kTileStartOff + (size_t)kRadix * 4;
  static constexpr size_t kBarOff = kExclOff + (size_t)kRadix * 8;
  static constexpr size_t kTileIdOff = kBarOff + 8;
  static constexpr size_t kAbortOff = kTileIdOff + 4;
  static constexpr size_t kBytes = kAbortOff + 4;
  static_assert(kTile % 4 == 0, "tile must keep 16-byte alignment of tile starts");
  static_assert(BLOCK >= kRadix, "one thread per bin in the look-back");
};

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, typename S>
__global__ void __launch_bounds__(BLOCK) onesweep_kernel(const OnesweepArgs args) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  using SW = StatusWord<S>;
  constexpr int TILE = G::kTile;
  constexpr uint32_t FULL = 0xFFFFFFFFu;

  const PassCtrl pc = args.ctrl->pass[args.pass];
  if (pc.skip) return;

  extern __shared__ __align__(128) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  uint32_t* s_wh = reinterpret_cast<uint32_t*>(smem + G::kWarpHistOff);
  unsigned long long* s_bin_base = reinterpret_cast<unsigned long long*>(smem + G::kBinBaseOff);
  uint32_t* s_tile_count = reinterpret_cast<uint32_t*>(smem + G::kTileCountOff);
  uint32_t* s_tile_start = reinterpret_cast<uint32_t*>(smem + G::kTileStartOff);
  unsigned long long* s_excl = reinterpret_cast<unsigned long long*>(smem + G::kExclOff);
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
  const uint32_t warp = tid >> 5;
  const uint32_t lane = tid & 31u;

  if (tid == 0) {
    *s_tile_id = atomicAdd(args.tile_counter, 1u);
    *s_abort = 0;
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  for (uint32_t i = tid; i < (uint32_t)(G::kWarps * kRadix); i += BLOCK) s_wh[i] = 0;
  __syncthreads();

  const uint32_t tile = *s_tile_id;
  const size_t num_tiles = (args.n + TILE - 1) / TILE;
  if ((size_t)tile >= num_tiles) {  // a ticket counter that was not reset
    if (tid == 0) raise_error(args.err, DEVERR_BAD_STATE);
    return;
  }
  const size_t tile_base = (size_t)tile * TILE;
  const uint32_t tile_n = (uint32_t)min((size_t)TILE, args.n - tile_base);

  // ---- 2. load the tile into shared memory ---------------------------------
  const bool tma_ok = ((reinterpret_cast<uintptr_t>(in) & 15u) == 0) &&
                      (!HAS_VALS || (reinterpret_cast<uintptr_t>(vin) & 15u) == 0);
  if (tma_ok) {
    const uint32_t kbulk = (tile_n * (uint32_t)sizeof(K)) & ~15u;
    const uint32_t vbulk = HAS_VALS ? ((tile_n * 4u) & ~15u) : 0u;
    if (tid == 0) {
      mbar_arrive_expect_tx(s_bar, kbulk + vbulk);
      if (kbulk) bulk_load_g2s(s_keys, in + tile_base, kbulk, s_bar);
      if (HAS_VALS && vbulk) bulk_load_g2s(s_vals, vin + tile_base, vbulk, s_bar);
    }
    for (uint32_t i = kbulk / (uint32_t)sizeof(K) + tid; i < tile_n; i += BLOCK) s_keys[i] = in[tile_base + i];
    if (HAS_VALS)
      for (uint32_t i = vbulk / 4u + tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
    mbar_wait_bounded(s_bar, 0, args.err);
  } else {
    for (uint32_t i = tid; i < tile_n; i += BLOCK) s_keys[i] = in[tile_base + i];
    if (HAS_VALS)
      for (uint32_t i = tid; i < tile_n; i += BLOCK) s_vals[i] = vin[tile_base + i];
  }
  __syncthreads();

  // ---- 3. rank within the warp -------------------------------------------
  const bool full = tile_n == (uint32_t)TILE;
  const uint32_t wbase = warp * ITEMS * 32;
  K k[ITEMS];
  uint32_t v[HAS_VALS ? ITEMS : 1];
  uint32_t rank[ITEMS];
  uint32_t* wh = s_wh + warp * kRadix;
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    const bool valid = full || idx < tile_n;
    k[j] = valid ? to_ordered(s_keys[idx], tin) : (K)0;
    if (HAS_VALS) v[j] = valid ? s_vals[idx] : 0u;
  }
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    const bool valid = full || idx < tile_n;
    const uint32_t d = valid ? digit_of(k[j], shift, kRadix - 1) : (uint32_t)kRadix;
    const uint32_t peers = __match_any_sync(FULL, d);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader && valid) {
      base = wh[d];
      wh[d] = base + __popc(peers);
    }
    base = __shfl_sync(FULL, base, leader);
    rank[j] = base + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();

  // ---- 4. tile counts, publish, look-back --------------------------------
  if (tid < kRadix) {
    uint32_t sum = 0;
#pragma unroll 4
    for (int w = 0; w < G::kWarps; ++w) {
      const uint32_t c = s_wh[w * kRadix + tid];
      s_wh[w * kRadix + tid] = sum;
      sum += c;
    }
    s_tile_count[tid] = sum;
    S* st = static_cast<S*>(args.status) + (size_t)tile * kRadix + tid;
    st_relaxed_gpu(st, (S)((tile == 0 ? SW::kIncl : SW::kAgg) | (S)sum));
  }
  __syncthreads();
  if (warp == 0) {
    // exclusive scan of the 256 tile counts: 8 consecutive bins per lane
    uint32_t c[kRadix / 32];
    uint32_t local = 0;
#pragma unroll
    for (int i = 0; i < kRadix / 32; ++i) {
      c[i] = s_tile_count[lane * (kRadix / 32) + i];
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
      s_tile_start[lane * (kRadix / 32) + i] = run;
      run += c[i];
    }
  }
  if (tid < kRadix) {
    unsigned long long excl = 0;
    if (tile > 0) {
      const S* base = static_cast<const S*>(args.status) + tid;
      long long t = (long long)tile - 1;
      uint32_t spins = 0;
      while (true) {
        const S s = ld_relaxed_gpu(base + (size_t)t * kRadix);
        const uint32_t flag = (uint32_t)(s >> SW::kShift);
        if (flag == 0) {
          if (++spins > kSpinLimit) {
            raise_error(args.err, DEVERR_LOOKBACK_TIMEOUT);
            *s_abort = 1;
            break;
          }
          continue;
        }
        excl += (unsigned long long)(s & SW::kMask);
        if (flag == 2u || t == 0) break;
        --t;
      }
      S* st = static_cast<S*>(args.status) + (size_t)tile * kRadix + tid;
      st_relaxed_gpu(st, (S)(SW::kIncl | (S)(excl + s_tile_count[tid])));
    }
    s_excl[tid] = excl;
  }
  __syncthreads();

  // ---- 5. stage by bin in shared memory ----------------------------------
  if (tid < kRadix) s_bin_base[tid] = args.bin_start[tid] + s_excl[tid] - (unsigned long long)s_tile_start[tid];
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t idx = wbase + (uint32_t)j * 32u + lane;
    if (full || idx < tile_n) {
      const uint32_t d = digit_of(k[j], shift, kRadix - 1);
      const uint32_t pos = s_tile_start[d] + wh[d] + rank[j];
      s_keys[pos] = k[j];
      if (HAS_VALS) s_vals[pos] = v[j];
    }
  }
  __syncthreads();

  // ---- 6. write out in bin-contiguous runs --------------------------------
  // A tile whose look-back gave up has no valid offsets: it writes nothing
  // (the call reports the failure), and every store is bounds-checked.
  if (*s_abort) return;
  const unsigned long long n_out = args.n;
#pragma unroll
  for (int j = 0; j < ITEMS; ++j) {
    const uint32_t i = (uint32_t)j * BLOCK + tid;
    if (full || i < tile_n) {
      const K key = s_keys[i];
      const uint32_t d = digit_of(key, shift, kRadix - 1);
      const unsigned long long o = s_bin_base[d] + i;
      if (o < n_out) {
        out[o] = from_ordered(key, tout);
        if (HAS_VALS) vout[o] = s_vals[i];
      }
    }
  }
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

// Tile geometry per key type.  32-bit keys: 512 threads x 16 keys; wider
// records use fewer items per thread so that keys, payloads and ranks stay
// in registers.
constexpr int kBlock = 512;
constexpr int kItemsU32 = 16;
constexpr int kItemsU32Kv = 12;
constexpr int kItemsU64 = 12;
constexpr int kItemsU64Kv = 8;

template <typename K, bool HAS_VALS, int ITEMS, typename S>
cudaError_t launch_t(const OnesweepArgs& a, cudaStream_t stream) {
  using G = Geometry<K, HAS_VALS, kBlock, ITEMS>;
  auto kern = onesweep_kernel<K, HAS_VALS, kBlock, ITEMS, S>;
  static bool configured = false;  // one attribute call per instantiation
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::kBytes);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const size_t tiles = ceil_div(a.n, (size_t)G::kTile);
  kern<<<(unsigned)tiles, kBlock, G::kBytes, stream>>>(a);
  return cudaGetLastError();
}

template <typename K, bool HAS_VALS, int ITEMS>
cudaError_t launch_k(const OnesweepArgs& a, cudaStream_t stream) {
  if (a.n < (1ull << 30)) return launch_t<K, HAS_VALS, ITEMS, uint32_t>(a, stream);
  return launch_t<K, HAS_VALS, ITEMS, unsigned long long>(a, stream);
}

}  // namespace

size_t onesweep_tile_keys(int key_bytes, bool has_vals) {
  if (key_bytes == 4) return (size_t)kBlock * (has_vals ? kItemsU32Kv : kItemsU32);
  return (size_t)kBlock * (has_vals ? kItemsU64Kv : kItemsU64);
}

size_t onesweep_status_bytes(size_t n) { return n < (1ull << 30) ? 4 : 8; }

cudaError_t launch_onesweep_pass(const OnesweepArgs& a, int key_bytes, bool has_vals, cudaStream_t stream) {
  if (a.n == 0) return cudaSuccess;
  if (key_bytes == 4) {
    return has_vals ? launch_k<uint32_t, true, kItemsU32Kv>(a, stream)
                    : launch_k<uint32_t, false, kItemsU32>(a, stream);
  }
  return has_vals ? launch_k<unsigned long long, true, kItemsU64Kv>(a, stream)
                  : launch_k<unsigned long long, false, kItemsU64>(a, stream);
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
