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
//      is not 16-byte aligned);
//   3. rank every key within the tile by its 8-bit digit (stable).  Default:
//      warp multisplit (pa_onesweep_tile.cuh, onesweep_tile_ms_body) -- per
//      item, the lanes holding the same digit are found by ballots or by a
//      shared-memory atomic OR, one of them bumps the warp's counter for the
//      digit; the warps' counters are scanned into the tile's bin offsets.
//      Alternative (PA_ONESWEEP_RANK=counting): two stable 4-bit counting
//      passes over the tile with per-thread counters (onesweep_tile);
//   4. publish the tile's bin counts (AGGREGATE, or INCLUSIVE for tile 0);
//   5. per bin, walk back over earlier tiles' words, four tiles per round
//      trip, until an INCLUSIVE one; publish INCLUSIVE.  (The first pass of
//      a 32-bit keys-only sort skips steps 4-5: its tiles' offsets were
//      prepared by the histogram, launch_tile_counts, and arrive with the
//      tile's bulk copy);
//   6. stage the keys at their in-tile sorted position in shared memory and
//      write them out: consecutive threads write consecutive keys of a bin to
//      consecutive addresses.
// Small inputs (at most small_sort_max_keys) are sorted whole by one CTA in
// shared memory instead (small_sort_kernel).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pa_common.cuh"
#include "pa_kernels.cuh"
#include "pa_onesweep_tile.cuh"

namespace pa {
namespace {

using namespace os;

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S, bool MULTISPLIT>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_kernel(const OnesweepArgs args) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  constexpr int TILE = G::kTile;
  const PassCtrl pc = args.ctrl->pass[args.pass];
  if (pc.skip) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + G::kBarOff);
  uint32_t* s_tile_id = reinterpret_cast<uint32_t*>(smem + G::kTileIdOff);
  // 1. tile ticket: tiles are taken in launch order
  if (threadIdx.x == 0) {
    *s_tile_id = atomicAdd(args.tile_counter, 1u);
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const uint32_t tile = *s_tile_id;
  // keys to move: args.n, or fewer counted on the device (tiles past them exit)
  const size_t n = args.n_dev ? min((size_t)*args.n_dev, args.n) : args.n;
  if ((size_t)tile >= (n + TILE - 1) / TILE) {
    if (!args.n_dev && threadIdx.x == 0) raise_error(args.err, DEVERR_BAD_STATE);  // a ticket counter not reset
    return;
  }
  TileJob<K, S> job;
  job.in = static_cast<const K*>(pc.src_is_tmp ? args.keys_b : args.keys_a);
  job.out = static_cast<K*>(pc.src_is_tmp ? args.keys_a : args.keys_b);
  job.vin = pc.src_is_tmp ? args.vals_b : args.vals_a;
  job.vout = pc.src_is_tmp ? args.vals_a : args.vals_b;
  job.n = n;
  job.out_n = args.out_n ? args.out_n : n;
  job.tile = tile;
  job.shift = args.shift;
  job.tin = args.is_float && pc.transform_in;
  job.tout = args.is_float && pc.transform_out;
  job.bin_start = args.bin_start;
  job.status = static_cast<S*>(args.status);
  job.err = args.err;
  job.spin_limit = args.spin_limit ? args.spin_limit : kSpinLimit;
  job.tile_prefix = args.tile_prefix;  // prepared offsets (used by the multisplit ranking)
  job.chunk_excl = args.chunk_excl;
  job.tiles_per_chunk = args.tiles_per_chunk;
  uint32_t parity = 0;
  if constexpr (MULTISPLIT)
    onesweep_tile_multisplit<K, HAS_VALS, BLOCK, ITEMS, S>(job, smem, s_bar, parity);
  else
    onesweep_tile<K, HAS_VALS, BLOCK, ITEMS, S>(job, smem, s_bar, parity);
}

// Wide-digit pass (11-bit digits, 2048 bins): onesweep_tile_wide.
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S, int RB>
__global__ void __launch_bounds__(BLOCK, MINB) onesweep_wide_kernel(const OnesweepArgs args) {
  using G = WideGeometry<K, HAS_VALS, BLOCK, ITEMS, RB>;
  constexpr int TILE = G::kTile;
  const PassCtrl pc = args.ctrl->pass[args.pass];
  if (pc.skip) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + G::kBarOff);
  uint32_t* s_tile_id = reinterpret_cast<uint32_t*>(smem + G::kTileIdOff);
  if (threadIdx.x == 0) {  // tile ticket: tiles are taken in launch order
    *s_tile_id = atomicAdd(args.tile_counter, 1u);
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const uint32_t tile = *s_tile_id;
  if ((size_t)tile >= (args.n + TILE - 1) / TILE) {  // a ticket counter that was not reset
    if (threadIdx.x == 0) raise_error(args.err, DEVERR_BAD_STATE);
    return;
  }
  TileJob<K, S> job;
  job.in = static_cast<const K*>(pc.src_is_tmp ? args.keys_b : args.keys_a);
  job.out = static_cast<K*>(pc.src_is_tmp ? args.keys_a : args.keys_b);
  job.vin = pc.src_is_tmp ? args.vals_b : args.vals_a;
  job.vout = pc.src_is_tmp ? args.vals_a : args.vals_b;
  job.n = args.n;
  job.out_n = args.n;
  job.tile = tile;
  job.shift = args.shift;
  job.tin = args.is_float && pc.transform_in;
  job.tout = args.is_float && pc.transform_out;
  job.bin_start = args.bin_start;
  job.status = static_cast<S*>(args.status);
  job.err = args.err;
  job.spin_limit = args.spin_limit ? args.spin_limit : kSpinLimit;
  uint32_t parity = 0;
  onesweep_tile_wide<K, HAS_VALS, BLOCK, ITEMS, RB, S>(job, smem, s_bar, parity);
}

// A whole sort of at most BLOCK * ITEMS keys by one CTA, in shared memory:
// the keys (and payloads) are read once, sorted by stable 4-bit counting
// passes over every nibble (each thread owns ITEMS consecutive keys, so
// (thread, item) order is input order), and written once.  One launch
// instead of the histogram / scan / digit-pass chain, for small inputs
// whose cost is launch latency.  Padding keys (all ones) sort after every
// real key.
template <typename K, bool HAS_VALS, int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK, 1) small_sort_kernel(K* __restrict__ keys, uint32_t* __restrict__ vals,
                                                             uint32_t n, int is_float) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  constexpr int TILE = G::kTile;
  extern __shared__ __align__(128) unsigned char smem[];
  K* s_keys = reinterpret_cast<K*>(smem + G::kKeysOff);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(smem + G::kValsOff);
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem + G::kCntOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + G::kWarpTotOff);
  const bool flt = is_float != 0;
  for (uint32_t i = threadIdx.x; i < (uint32_t)TILE; i += BLOCK) {
    s_keys[i] = i < n ? to_ordered(keys[i], flt) : ~(K)0;
    if (HAS_VALS) s_vals[i] = i < n ? vals[i] : 0u;
  }
  __syncthreads();
  K k[ITEMS];
  uint32_t v[HAS_VALS ? ITEMS : 1];
  for (uint32_t sh = 0; sh < 8u * (uint32_t)sizeof(K); sh += 4) {
    load_run<K, HAS_VALS, ITEMS>(k, v, s_keys, s_vals);
    nibble_pass<K, HAS_VALS, BLOCK, ITEMS>(k, v, sh, s_keys, s_vals, s_cnt, s_warp);  // ends with a barrier
  }
  for (uint32_t i = threadIdx.x; i < n; i += BLOCK) {
    keys[i] = from_ordered(s_keys[i], flt);
    if (HAS_VALS) vals[i] = s_vals[i];
  }
}

template <typename K, bool HAS_VALS, int ITEMS>
cudaError_t launch_small_t(void* keys, uint32_t* vals, size_t n, bool is_float, cudaStream_t stream) {
  constexpr int kSmallBlock = 512;
  using G = Geometry<K, HAS_VALS, kSmallBlock, ITEMS>;
  auto kern = small_sort_kernel<K, HAS_VALS, kSmallBlock, ITEMS>;
  cudaError_t e = ensure_dynamic_smem(kern, G::kBytes);
  if (e != cudaSuccess) return e;
  kern<<<1, kSmallBlock, G::kBytes, stream>>>(static_cast<K*>(keys), vals, (uint32_t)n, is_float ? 1 : 0);
  return cudaGetLastError();
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

// One grid row per run: run r copies src[runs[3r], +runs[3r+1]) to
// dst[runs[3r+2], ...) with 16-byte vector stores (the loads are plain and
// coalesced: a warp reads consecutive elements); the few elements before the
// destination's first 16-byte boundary and after its last one are copied
// singly.
template <typename K>
__global__ void gather_runs_kernel(const K* __restrict__ src, K* __restrict__ dst,
                                   const unsigned long long* __restrict__ runs) {
  constexpr uint32_t V = 16 / sizeof(K);
  const size_t r = blockIdx.y;
  const K* s = src + runs[3 * r];
  const size_t len = (size_t)runs[3 * r + 1];
  K* d = dst + runs[3 * r + 2];
  size_t head = ((16u - (reinterpret_cast<uintptr_t>(d) & 15u)) & 15u) / sizeof(K);
  if (head > len) head = len;
  const size_t nvec = (len - head) / V;
  const size_t tail = head + nvec * V;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (tid < head) d[tid] = s[tid];
  if (tid < len - tail) d[tail + tid] = s[tail + tid];
  uint4* dv = reinterpret_cast<uint4*>(d + head);
  for (size_t j = tid; j < nvec; j += stride) {
    const K* e = s + head + j * V;
    K v[V];
#pragma unroll
    for (uint32_t k = 0; k < V; ++k) v[k] = e[k];
    dv[j] = *reinterpret_cast<const uint4*>(v);
  }
}

// Tile geometries.  Each is (threads, keys per thread, CTAs per SM the
// register budget is cut for).  The active one per (key type, payload) is
// the first entry unless PA_ONESWEEP_GEOMETRY selects another (tuning).
struct GeomChoice {
  int block, items, minb;
};
constexpr GeomChoice kGeomU32[] = {{384, 16, 3}, {512, 16, 2}, {256, 16, 4}, {1024, 8, 1}, {512, 8, 3}};
constexpr GeomChoice kGeomU32Kv[] = {{512, 12, 2}, {256, 12, 4}, {512, 8, 3}};
constexpr GeomChoice kGeomU64[] = {{512, 12, 2}, {256, 12, 4}, {512, 8, 3}};
constexpr GeomChoice kGeomU64Kv[] = {{256, 12, 3}, {256, 8, 4}, {512, 8, 2}};

int geometry_index(int count) {
  static const int idx = [] {  // read once (thread-safe initialisation)
    const char* e = std::getenv("PA_ONESWEEP_GEOMETRY");
    return e ? std::atoi(e) : 0;
  }();
  return (idx >= 0 && idx < count) ? idx : 0;
}

template <typename K, bool HAS_VALS>
GeomChoice active_geometry() {
  if (sizeof(K) == 4 && !HAS_VALS) return kGeomU32[geometry_index(5)];
  if (sizeof(K) == 4) return kGeomU32Kv[geometry_index(3)];
  if (!HAS_VALS) return kGeomU64[geometry_index(3)];
  return kGeomU64Kv[geometry_index(3)];
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S, bool MS>
cudaError_t launch_g2(const OnesweepArgs& a, cudaStream_t stream) {
  using G = Geometry<K, HAS_VALS, BLOCK, ITEMS>;
  auto kern = onesweep_kernel<K, HAS_VALS, BLOCK, ITEMS, MINB, S, MS>;
  cudaError_t e = ensure_dynamic_smem(kern, G::kBytes);
  if (e != cudaSuccess) return e;
  size_t tiles = ceil_div(a.n, (size_t)G::kTile);
  if (a.max_ctas && a.max_ctas < tiles) tiles = a.max_ctas;
  kern<<<(unsigned)tiles, BLOCK, G::kBytes, stream>>>(a);
  return cudaGetLastError();
}

// Ranking method of a pass: the warp multisplit (default) or the in-tile
// counting sort (PA_ONESWEEP_RANK=counting).  A persistent form of the
// multisplit pass that copied each CTA's next tile in while it worked on the
// current one was measured slower on GB300 (tickets taken early make
// successors wait in the look-back) and is not built.
bool use_multisplit() {
  static const bool v = [] {
    const char* e = std::getenv("PA_ONESWEEP_RANK");
    return !(e && std::strcmp(e, "counting") == 0);
  }();
  return v;
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB, typename S>
cudaError_t launch_g(const OnesweepArgs& a, cudaStream_t stream) {
  if (use_multisplit()) return launch_g2<K, HAS_VALS, BLOCK, ITEMS, MINB, S, true>(a, stream);
  if constexpr (ITEMS <= 16) return launch_g2<K, HAS_VALS, BLOCK, ITEMS, MINB, S, false>(a, stream);
  return cudaErrorInvalidConfiguration;  // the counting ranking packs ranks in 4 bits (at most 16 items)
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB>
cudaError_t launch_s(const OnesweepArgs& a, cudaStream_t stream) {
  if (a.n < (1ull << 30) && a.out_n < (1ull << 30))
    return launch_g<K, HAS_VALS, BLOCK, ITEMS, MINB, uint32_t>(a, stream);
  return launch_g<K, HAS_VALS, BLOCK, ITEMS, MINB, unsigned long long>(a, stream);
}

#define PA_GEOM_CASE(B, I, M) \
  if (g.block == B && g.items == I && g.minb == M) return launch_s<K, HAS_VALS, B, I, M>(a, stream);

// Wide-digit geometries (threads, keys per thread, CTAs per SM), the first
// one active unless PA_WIDE_GEOMETRY selects another (tuning).  The 16-bit
// warp counters of 2048 bins take 4 KB per warp.
constexpr GeomChoice kWide[] = {{512, 8, 2}, {256, 16, 2}, {512, 16, 1}};

int wide_geometry_index() {
  static const int idx = [] {
    const char* e = std::getenv("PA_WIDE_GEOMETRY");
    const int i = e ? std::atoi(e) : 0;
    return (i >= 0 && i < 3) ? i : 0;
  }();
  return idx;
}

template <typename K, bool HAS_VALS, int BLOCK, int ITEMS, int MINB>
cudaError_t launch_wide_t(const OnesweepArgs& a, cudaStream_t stream) {
  using G = WideGeometry<K, HAS_VALS, BLOCK, ITEMS, 11>;
  auto go = [&](auto* kern) {
    cudaError_t e = ensure_dynamic_smem(kern, G::kBytes);
    if (e != cudaSuccess) return e;
    size_t tiles = ceil_div(a.n, (size_t)G::kTile);
    if (a.max_ctas && a.max_ctas < tiles) tiles = a.max_ctas;
    kern<<<(unsigned)tiles, BLOCK, G::kBytes, stream>>>(a);
    return cudaGetLastError();
  };
  if (a.n < (1ull << 30)) return go(onesweep_wide_kernel<K, HAS_VALS, BLOCK, ITEMS, MINB, uint32_t, 11>);
  return go(onesweep_wide_kernel<K, HAS_VALS, BLOCK, ITEMS, MINB, unsigned long long, 11>);
}

template <typename K, bool HAS_VALS>
cudaError_t launch_wide(const OnesweepArgs& a, cudaStream_t stream) {
  const GeomChoice g = kWide[wide_geometry_index()];
  if (g.block == 512 && g.items == 8) return launch_wide_t<K, HAS_VALS, 512, 8, 2>(a, stream);
  if (g.block == 256 && g.items == 16) return launch_wide_t<K, HAS_VALS, 256, 16, 2>(a, stream);
  return launch_wide_t<K, HAS_VALS, 512, 16, 1>(a, stream);
}

template <typename K, bool HAS_VALS>
cudaError_t launch_kv(const OnesweepArgs& a, cudaStream_t stream) {
  if (a.radix_bits == 11) return launch_wide<K, HAS_VALS>(a, stream);
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

size_t onesweep_tile_keys(int key_bytes, bool has_vals, int radix_bits) {
  if (radix_bits == 11) {
    const GeomChoice g = kWide[wide_geometry_index()];
    return (size_t)g.block * g.items;
  }
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

size_t small_sort_max_keys(int key_bytes, bool has_vals) {
  (void)has_vals;
  return key_bytes == 4 ? 512 * 16 : 512 * 8;
}

cudaError_t launch_small_sort(void* keys, uint32_t* vals, size_t n, int key_bytes, bool is_float, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (n > small_sort_max_keys(key_bytes, vals != nullptr)) return cudaErrorInvalidValue;
  if (key_bytes == 4)
    return vals ? launch_small_t<uint32_t, true, 16>(keys, vals, n, is_float, stream)
                : launch_small_t<uint32_t, false, 16>(keys, vals, n, is_float, stream);
  if (key_bytes == 8)
    return vals ? launch_small_t<unsigned long long, true, 8>(keys, vals, n, false, stream)
                : launch_small_t<unsigned long long, false, 8>(keys, vals, n, false, stream);
  return cudaErrorInvalidValue;
}

cudaError_t launch_gather_runs(const void* src, void* dst, const unsigned long long* runs, size_t nruns,
                               size_t max_run, int key_bytes, cudaStream_t stream) {
  if (nruns == 0 || max_run == 0) return cudaSuccess;
  if (nruns > 65535) return cudaErrorInvalidValue;
  const int block = 256;
  const size_t vec = 16 / (size_t)key_bytes;
  const unsigned gx = (unsigned)max((size_t)1, min(ceil_div(max_run, (size_t)block * vec * 8),
                                                   (size_t)device_info().sm_count * 2));
  const dim3 grid(gx, (unsigned)nruns);
  if (key_bytes == 4)
    gather_runs_kernel<uint32_t><<<grid, block, 0, stream>>>(static_cast<const uint32_t*>(src),
                                                             static_cast<uint32_t*>(dst), runs);
  else if (key_bytes == 8)
    gather_runs_kernel<unsigned long long><<<grid, block, 0, stream>>>(
        static_cast<const unsigned long long*>(src), static_cast<unsigned long long*>(dst), runs);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
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
