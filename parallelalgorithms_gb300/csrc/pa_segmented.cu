// Batched segmented sort: thousands of uint32 arrays of uneven size, each
// sorted independently (stable, ascending), in ONE persistent kernel launch
// fed by a device work queue, launched through a captured CUDA graph.
//
// No reference counterpart: the reference sorts one array per call
// (SortRadixPar, RadixSortLsdParallel.h:367); its nearest idea is bundling
// small work items (BundleSmallWorkItems.cpp:36).  Per segment the result is
// exactly SortRadixPar's.
//
// Work items, in queue order (a CTA takes the next item with one atomicAdd):
//   HIST  one chunk of a large segment: its four byte-digit counts, added
//         into the segment's histogram;
//   SCAN  one large segment: bin starts of its four digits;
//   PASS  (11-bit plans) one tile of one large segment for digit pass p: the
//         onesweep tile of the plain sort (pa_onesweep_tile.cuh), look-back
//         within the segment.  8-bit plans run each pass as its own launch
//         after the persistent kernel instead (seg_pass_kernel: the plain
//         sort's pass geometry over all large segments' tiles at once, no
//         work-queue round trips per tile);
//   SMALL one small segment (<= the small/large cutoff) sorted entirely in
//         shared memory by eight stable 4-bit counting passes, read once and
//         written once.
// Small items are spread between the large-segment stages so that CTAs
// waiting on a stage have work.  An item waits only on earlier items of the
// same segment (per-segment completion counters: HIST chunks before SCAN,
// SCAN before pass 0, all tiles of pass p before pass p + 1); items are taken
// in queue order by running CTAs, so the earliest unfinished item can always
// proceed.  Every wait is bounded and reports through the plan's error word.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "pa_common.cuh"
#include "pa_gpu.h"
#include "pa_kernels.cuh"
#include "pa_onesweep_tile.cuh"
#include "pa_segmented.cuh"

namespace pa {
namespace seg {

using namespace os;

// Bounded wait until *ctr >= need (acquire).  Thread 0 only.
__device__ __forceinline__ void wait_count(const uint32_t* ctr, uint32_t need, uint32_t* err) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (ld_acquire_gpu(ctr) >= need) return;
    __nanosleep(64);
  }
  raise_error(err, DEVERR_LOOKBACK_TIMEOUT);
}

// Lane copies of each HIST counter: the 8-bit table (4 x 256) keeps 8, the
// 11-bit one (3 x 2048) 2, so that both fit shared memory.
template <int RB>
__host__ __device__ constexpr int hist_lanes() { return RB == 11 ? 2 : kHistLanes; }

template <int RB>
__device__ __forceinline__ void hist_item(const PlanDev& P, const Item& it, unsigned char* smem) {
  constexpr uint32_t D = RB == 11 ? 3u : 4u, R = 1u << RB;
  constexpr uint32_t L = hist_lanes<RB>();
  const LargeSeg L_ = P.large[it.seg];
  uint32_t* h = reinterpret_cast<uint32_t*>(smem);
  constexpr uint32_t kWords = D * R * L;
  for (uint32_t i = threadIdx.x; i < kWords; i += kBlock) h[i] = 0;
  __syncthreads();
  const uint32_t lo = it.idx * kHistChunk;
  const uint32_t len = min(kHistChunk, L_.len - lo);
  const uint32_t* src = P.keys + L_.base + lo;
  uint32_t* my = h + (threadIdx.x % L);
  for (uint32_t i = threadIdx.x; i < len; i += kBlock) {
    const uint32_t k = src[i];
#pragma unroll
    for (uint32_t d = 0; d < D; ++d) atomicAdd(my + (d * R + ((k >> (RB * d)) & (R - 1))) * L, 1u);
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < D * R; e += kBlock) {
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t j = 0; j < L; ++j) sum += h[e * L + ((j + e) % L)];
    if (sum) atomicAdd(&P.hist[(size_t)it.seg * D * R + e], sum);
  }
}

template <int RB>
__device__ __forceinline__ void scan_item(const PlanDev& P, const Item& it, unsigned char* smem) {
  constexpr uint32_t D = RB == 11 ? 3u : 4u, R = 1u << RB;
  constexpr uint32_t PER = R >= kBlock ? R / kBlock : 1;  // bins per thread
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem);
  const uint32_t tid = threadIdx.x;
  for (uint32_t d = 0; d < D; ++d) {
    const uint32_t* hd = P.hist + (size_t)it.seg * D * R + d * R;
    uint32_t c[PER];
    uint32_t local = 0;
#pragma unroll
    for (uint32_t i = 0; i < PER; ++i) {
      const uint32_t b = tid * PER + i;
      c[i] = b < R ? hd[b] : 0u;
      local += c[i];
    }
    uint32_t run = block_exclusive_scan<kBlock>(local, s_warp);
#pragma unroll
    for (uint32_t i = 0; i < PER; ++i) {
      const uint32_t b = tid * PER + i;
      if (b < R) P.bin_start[(size_t)it.seg * D * R + d * R + b] = run;
      run += c[i];
    }
    __syncthreads();  // s_warp is reused by the next digit's scan
  }
}

template <int PASS_ITEMS, int RB>
__device__ __forceinline__ void pass_item(const PlanDev& P, const Item& it, unsigned char* smem, uint64_t* bar,
                                          uint32_t& parity) {
  constexpr uint32_t D = RB == 11 ? 3u : 4u, R = 1u << RB;
  const LargeSeg L = P.large[it.seg];
  const bool even = (it.pass & 1u) == 0;
  TileJob<uint32_t, uint32_t> job;
  job.in = (even ? P.keys : P.tmp) + L.base;
  job.out = (even ? P.tmp : P.keys) + L.base;
  job.vin = nullptr;
  job.vout = nullptr;
  job.n = L.len;
  job.out_n = L.len;
  job.tile = it.idx;
  job.shift = RB * it.pass;
  job.tin = false;
  job.tout = false;
  job.bin_start = P.bin_start + (size_t)it.seg * D * R + it.pass * R;
  job.status = P.status + ((size_t)it.pass * P.total_tiles + L.tile_base) * R;
  job.err = P.err;
  job.spin_limit = kSpinLimit;
  if constexpr (RB == 11)
    onesweep_tile_wide<uint32_t, false, kBlock, PASS_ITEMS, 11, uint32_t>(job, smem, bar, parity);
  else
    onesweep_tile_multisplit<uint32_t, false, kBlock, PASS_ITEMS, uint32_t>(job, smem, bar, parity);
}

template <int SMALL_ITEMS>
__device__ __forceinline__ void small_item(const PlanDev& P, const Item& it, unsigned char* smem) {
  using GS = Geometry<uint32_t, false, kBlock, SMALL_ITEMS>;
  constexpr uint32_t TILE = GS::kTile;
  uint32_t* s_keys = reinterpret_cast<uint32_t*>(smem + GS::kKeysOff);
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem + GS::kCntOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + GS::kWarpTotOff);
  const unsigned long long base = P.seg_off[it.seg];
  const uint32_t len = (uint32_t)(P.seg_off[it.seg + 1] - base);
  const uint32_t* keys = P.keys + base;
  uint32_t* out = result_buffer(P) + base;
  for (uint32_t i = threadIdx.x; i < TILE; i += kBlock) s_keys[i] = i < len ? keys[i] : 0xFFFFFFFFu;
  __syncthreads();
  uint32_t k[SMALL_ITEMS];
  uint32_t v[1];
#pragma unroll 1
  for (uint32_t sh = 0; sh < 32; sh += 4) {
    load_run<uint32_t, false, SMALL_ITEMS>(k, v, s_keys, nullptr);
    nibble_pass<uint32_t, false, kBlock, SMALL_ITEMS>(k, v, sh, s_keys, nullptr, s_cnt, s_warp);
  }
  for (uint32_t i = threadIdx.x; i < len; i += kBlock) out[i] = s_keys[i];
}

template <int PASS_ITEMS, int SMALL_ITEMS, int RB>
__global__ void __launch_bounds__(kBlock, 2) segsort_kernel(const PlanDev P) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ Item s_item;
  __shared__ uint32_t s_index;
  // The bulk-copy barrier lives outside the dynamic area, which every item
  // kind lays out differently.
  __shared__ __align__(8) uint64_t s_bar_storage;
  uint64_t* s_bar = &s_bar_storage;
  if (threadIdx.x == 0) {
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  uint32_t parity = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t i = atomicAdd(P.head, 1u);
      s_index = i;
      if (i < P.num_items) s_item = P.items[i];
    }
    __syncthreads();
    if (s_index >= P.num_items) break;
    const Item it = s_item;
    if (it.kind == ITEM_SCAN || it.kind == ITEM_PASS) {
      if (threadIdx.x == 0) {
        const LargeSeg L = P.large[it.seg];
        const uint32_t* d = P.done + (size_t)it.seg * kStages;
        if (it.kind == ITEM_SCAN)
          wait_count(d + ST_HIST, L.hist_chunks, P.err);
        else if (it.pass == 0)
          wait_count(d + ST_SCAN, 1, P.err);
        else
          wait_count(d + ST_PASS0 + it.pass - 1, L.tiles, P.err);
        fence_proxy_async();
      }
      __syncthreads();
    }
    if (it.kind == ITEM_SMALL)
      small_item<SMALL_ITEMS>(P, it, smem);
    else if (it.kind == ITEM_HIST)
      hist_item<RB>(P, it, smem);
    else if (it.kind == ITEM_SCAN)
      scan_item<RB>(P, it, smem);
    else
      pass_item<PASS_ITEMS, RB>(P, it, smem, s_bar, parity);
    __syncthreads();
    if (it.kind != ITEM_SMALL && threadIdx.x == 0) {
      __threadfence();
      const uint32_t st = it.kind == ITEM_HIST ? ST_HIST : it.kind == ITEM_SCAN ? ST_SCAN : ST_PASS0 + it.pass;
      atomicAdd(P.done + (size_t)it.seg * kStages + st, 1u);
    }
  }
}

// One digit pass over every large segment of an 8-bit plan: tiles taken in
// launch order (ticket), each mapped to its segment through the plan's tile
// table; the onesweep tile of the plain sort with the segment as the array,
// so the look-back stays inside the segment (its first tile publishes an
// INCLUSIVE word).  Runs after the persistent kernel has finished every
// HIST and SCAN item, so no item waits.
using PassGeometry = Geometry<uint32_t, false, kPassBlock, kPassItems>;

__global__ void __launch_bounds__(kPassBlock, 3) seg_pass_kernel(const PlanDev P, uint32_t pass) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* s_bar = reinterpret_cast<uint64_t*>(smem + PassGeometry::kBarOff);
  uint32_t* s_tile = reinterpret_cast<uint32_t*>(smem + PassGeometry::kTileIdOff);
  if (threadIdx.x == 0) {
    *s_tile = atomicAdd(P.pass_ticket, 1u);
    mbar_init(s_bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  const uint32_t g = *s_tile;
  if (g >= P.pass_tiles) {  // a ticket counter that was not cleared
    if (threadIdx.x == 0) raise_error(P.err, DEVERR_BAD_STATE);
    return;
  }
  const uint32_t seg = P.tile_seg[g];
  const LargeSeg L = P.large[seg];
  const bool even = (pass & 1u) == 0;
  TileJob<uint32_t, uint32_t> job;
  job.in = (even ? P.keys : P.tmp) + L.base;
  job.out = (even ? P.tmp : P.keys) + L.base;
  job.vin = nullptr;
  job.vout = nullptr;
  job.n = L.len;
  job.out_n = L.len;
  job.tile = g - L.ptile_base;
  job.shift = 8u * pass;
  job.tin = false;
  job.tout = false;
  job.bin_start = P.bin_start + (size_t)seg * 4 * 256 + pass * 256;
  job.status = P.pass_status + (size_t)L.ptile_base * 256;
  job.err = P.err;
  job.spin_limit = kSpinLimit;
  uint32_t parity = 0;
  onesweep_tile_multisplit<uint32_t, false, kPassBlock, kPassItems, uint32_t>(job, smem, s_bar, parity);
}

// ---- host side ---------------------------------------------------------------
template <int PI, int SI, int RB>
constexpr size_t smem_bytes_for() {
  using GS = Geometry<uint32_t, false, kBlock, SI>;
  size_t b = RB == 11 ? WideGeometry<uint32_t, false, kBlock, PI, 11>::kBytes : Geometry<uint32_t, false, kBlock, PI>::kBytes;
  if (GS::kBytes > b) b = GS::kBytes;
  const size_t hist = (size_t)(RB == 11 ? 3 : 4) * (1u << RB) * hist_lanes<RB>() * 4;
  if (hist > b) b = hist;
  return b;
}


template <int PI, int SI, int RB>
KernelChoice choice() {
  return {segsort_kernel<PI, SI, RB>, smem_bytes_for<PI, SI, RB>(), (uint32_t)kBlock * PI, (uint32_t)kBlock * SI};
}

template <int RB>
bool pick_kernel_rb(int pi, int si, KernelChoice* out) {
  if (pi == 8 && si == 4) *out = choice<8, 4, RB>();
  if (pi == 8 && si == 8) *out = choice<8, 8, RB>();
  if (pi == 8 && si == 16) *out = choice<8, 16, RB>();
  if (pi == 16 && si == 4) *out = choice<16, 4, RB>();
  if (pi == 16 && si == 8) *out = choice<16, 8, RB>();
  if (pi == 16 && si == 16) *out = choice<16, 16, RB>();
  return true;
}

bool pick_kernel(int tile_keys, int small_cutoff, int radix_bits, KernelChoice* out) {
  const int pi = tile_keys == 4096 ? 8 : tile_keys == 8192 ? 16 : 0;
  const int si = small_cutoff == 2048 ? 4 : small_cutoff == 4096 ? 8 : small_cutoff == 8192 ? 16 : 0;
  if (!pi || !si) return false;
  return radix_bits == 11 ? pick_kernel_rb<11>(pi, si, out) : pick_kernel_rb<8>(pi, si, out);
}

// ---- host-side planning --------------------------------------------------------
int build_host_plan(const uint64_t* off_host, size_t num_segments, const pa_segsort_config* cfg, HostPlan* hp,
                    int passes) {
  if (passes < 1 || passes > kPasses) return record_error(PA_ERR_ARG, "a batched plan runs 1 to 4 digit passes");
  pa_segsort_config c{};
  if (cfg) c = *cfg;
  for (int r : c.reserved)
    if (r) return record_error(PA_ERR_ARG, "pa_segsort_config.reserved must be zero");
  if (c.small_cutoff == 0) c.small_cutoff = 4096;
  if (c.tile_keys == 0) c.tile_keys = 8192;
  if (c.digit_bits == 0) c.digit_bits = 8;
  if (c.digit_bits != 8 && c.digit_bits != 11)
    return record_error(PA_ERR_ARG, "digit_bits must be 8 or 11 for the batched sort");
  if (c.digit_bits == 11) passes = 3;
  KernelChoice kc{};
  if (!pick_kernel(c.tile_keys, c.small_cutoff, c.digit_bits, &kc))
    return record_error(PA_ERR_ARG, "tile_keys must be 4096 or 8192 and small_cutoff 2048, 4096 or 8192");
  const uint64_t* off = off_host;
  for (size_t i = 0; i < num_segments; ++i) {
    if (off[i + 1] < off[i]) return record_error(PA_ERR_ARG, "seg_offsets must be non-decreasing");
    if (off[i + 1] - off[i] > kMaxSegmentKeys)
      return record_error(PA_ERR_ARG, "a segment exceeds 2^30 - 1 keys (the batched sort's limit)");
  }
  hp->cfg = c;
  hp->kc = kc;
  hp->passes = (uint32_t)passes;
  hp->radix_bits = (uint32_t)c.digit_bits;
  hp->split = c.digit_bits == 8;
  hp->tile_seg.clear();
  hp->pass_tiles = 0;
  hp->off.assign(off, off + num_segments + 1);
  hp->items.clear();
  hp->large.clear();
  std::vector<uint32_t> small_ids;
  uint32_t total_tiles = 0;
  for (size_t i = 0; i < num_segments; ++i) {
    const uint64_t len = off[i + 1] - off[i];
    if (len == 0 || (len == 1 && (passes % 2) == 0)) continue;  // (an odd pass count moves even single keys to tmp)
    if (len <= (uint64_t)kc.small_tile && len <= (uint64_t)c.small_cutoff) {
      small_ids.push_back((uint32_t)i);
    } else {
      LargeSeg L{};
      L.base = off[i];
      L.len = (uint32_t)len;
      L.tiles = (uint32_t)((len + kc.pass_tile - 1) / kc.pass_tile);
      L.hist_chunks = (uint32_t)((len + kHistChunk - 1) / kHistChunk);
      L.tile_base = total_tiles;
      total_tiles += L.tiles;
      if (hp->split) {
        const uint32_t pt = (uint32_t)((len + kPassTile - 1) / kPassTile);
        L.ptile_base = hp->pass_tiles;
        hp->pass_tiles += pt;
        hp->tile_seg.insert(hp->tile_seg.end(), pt, (uint32_t)hp->large.size());
      }
      hp->large.push_back(L);
    }
  }
  // largest small segments first (they take longest)
  std::stable_sort(small_ids.begin(), small_ids.end(),
                   [&](uint32_t a, uint32_t b) { return off[a + 1] - off[a] > off[b + 1] - off[b]; });
  auto& items = hp->items;
  size_t next_small = 0;
  // small items go after HIST, after SCAN and (PASS items) after each pass but the last
  const size_t gaps = hp->split ? 2 : 1 + 1 + (size_t)passes;
  auto add_small = [&](size_t share_of) {
    const size_t upto = std::min(small_ids.size(), (small_ids.size() * share_of + gaps - 1) / gaps);
    for (; next_small < upto; ++next_small) items.push_back({ITEM_SMALL, 0, small_ids[next_small], 0});
  };
  const uint32_t nlarge = (uint32_t)hp->large.size();
  for (uint32_t l = 0; l < nlarge; ++l)
    for (uint32_t ch = 0; ch < hp->large[l].hist_chunks; ++ch) items.push_back({ITEM_HIST, 0, l, ch});
  add_small(1);
  for (uint32_t l = 0; l < nlarge; ++l) items.push_back({ITEM_SCAN, 0, l, 0});
  add_small(2);
  if (!hp->split) {
    for (uint32_t p = 0; p < (uint32_t)passes; ++p) {
      for (uint32_t l = 0; l < nlarge; ++l)
        for (uint32_t t = 0; t < hp->large[l].tiles; ++t) items.push_back({ITEM_PASS, p, l, t});
      add_small(3 + p);
    }
  }
  add_small(gaps);
  hp->total_tiles = total_tiles;
  hp->num_small = (uint32_t)small_ids.size();
  hp->num_large = nlarge;
  // device layout
  const size_t nl = std::max<size_t>(nlarge, 1);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    o = (o + 255) & ~(size_t)255;
    const size_t at = o;
    o += bytes;
    return at;
  };
  hp->o_items = take(std::max<size_t>(items.size(), 1) * sizeof(Item));
  hp->o_off = take(hp->off.size() * 8);
  hp->o_large = take(nl * sizeof(LargeSeg));
  hp->o_tile_seg = take(std::max<size_t>(hp->tile_seg.size(), 1) * 4);  // (the uploaded image ends here)
  const size_t per_seg = (size_t)seg_digits(hp->radix_bits) * seg_bins(hp->radix_bits);
  hp->o_bins = take(nl * per_seg * 8);
  hp->o_err = take(256);
  hp->o_head = take(256);  // everything from here on is cleared per run
  hp->o_done = take(nl * kStages * 4);
  hp->o_hist = take(nl * per_seg * 4);
  hp->o_status = take(hp->split ? 0 : (size_t)passes * std::max<uint32_t>(total_tiles, 1) * seg_bins(hp->radix_bits) * 4);
  hp->o_pticket = take(256);
  hp->o_pstatus = take((size_t)std::max<uint32_t>(hp->pass_tiles, 1) * 256 * 4);
  hp->bytes = o;
  return PA_OK;
}

PlanDev device_view(const HostPlan& hp, char* dev, uint32_t* keys, uint32_t* tmp) {
  PlanDev d{};
  d.keys = keys;
  d.tmp = tmp;
  d.passes = hp.passes;
  d.items = reinterpret_cast<const Item*>(dev + hp.o_items);
  d.num_items = (uint32_t)hp.items.size();
  d.total_tiles = hp.total_tiles;
  d.seg_off = reinterpret_cast<const unsigned long long*>(dev + hp.o_off);
  d.large = reinterpret_cast<const LargeSeg*>(dev + hp.o_large);
  d.head = reinterpret_cast<uint32_t*>(dev + hp.o_head);
  d.done = reinterpret_cast<uint32_t*>(dev + hp.o_done);
  d.hist = reinterpret_cast<uint32_t*>(dev + hp.o_hist);
  d.status = reinterpret_cast<uint32_t*>(dev + hp.o_status);
  d.bin_start = reinterpret_cast<unsigned long long*>(dev + hp.o_bins);
  d.err = reinterpret_cast<uint32_t*>(dev + hp.o_err);
  d.radix_bits = hp.radix_bits;
  d.tile_seg = reinterpret_cast<const uint32_t*>(dev + hp.o_tile_seg);
  d.pass_tiles = hp.pass_tiles;
  d.pass_ticket = reinterpret_cast<uint32_t*>(dev + hp.o_pticket);
  d.pass_status = reinterpret_cast<uint32_t*>(dev + hp.o_pstatus);
  return d;
}

size_t plan_image_bytes(const HostPlan& hp) { return hp.o_tile_seg + std::max<size_t>(hp.tile_seg.size(), 1) * 4; }

cudaError_t upload_plan(const HostPlan& hp, char* dev, cudaStream_t s, void* pinned_staging) {
  cudaError_t e = cudaSuccess;
  if (pinned_staging) {
    char* img = static_cast<char*>(pinned_staging);
    const size_t bytes = plan_image_bytes(hp);
    std::memset(img, 0, bytes);
    if (!hp.items.empty()) std::memcpy(img + hp.o_items, hp.items.data(), hp.items.size() * sizeof(Item));
    std::memcpy(img + hp.o_off, hp.off.data(), hp.off.size() * 8);
    if (!hp.large.empty()) std::memcpy(img + hp.o_large, hp.large.data(), hp.large.size() * sizeof(LargeSeg));
    if (!hp.tile_seg.empty()) std::memcpy(img + hp.o_tile_seg, hp.tile_seg.data(), hp.tile_seg.size() * 4);
    e = cudaMemcpyAsync(dev, img, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dev + hp.o_err, 0, 256, s);
    return e;
  }
  if (!hp.items.empty())
    e = cudaMemcpyAsync(dev + hp.o_items, hp.items.data(), hp.items.size() * sizeof(Item), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dev + hp.o_off, hp.off.data(), hp.off.size() * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !hp.large.empty())
    e = cudaMemcpyAsync(dev + hp.o_large, hp.large.data(), hp.large.size() * sizeof(LargeSeg),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !hp.tile_seg.empty())
    e = cudaMemcpyAsync(dev + hp.o_tile_seg, hp.tile_seg.data(), hp.tile_seg.size() * 4, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dev + hp.o_err, 0, 256, s);
  return e;
}

unsigned plan_grid(const HostPlan& hp) {
  if (ensure_dynamic_smem(hp.kc.fn, hp.kc.smem) != cudaSuccess) cudaGetLastError();  // the launch reports it
  if (hp.split && ensure_dynamic_smem(seg_pass_kernel, PassGeometry::kBytes) != cudaSuccess) cudaGetLastError();
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hp.kc.fn, kBlock, hp.kc.smem) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  unsigned grid = (unsigned)std::max(1, per_sm) * (unsigned)device_info().sm_count;
  const uint32_t items = (uint32_t)hp.items.size();
  if (items < grid) grid = std::max<uint32_t>(items, 1);
  return grid;
}

cudaError_t launch_plan(const HostPlan& hp, const PlanDev& pd, char* dev, unsigned grid, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(dev + hp.o_head, 0, hp.o_pticket - hp.o_head, s);
  if (e != cudaSuccess) return e;
  if (!hp.items.empty()) {
    hp.kc.fn<<<grid, kBlock, hp.kc.smem, s>>>(pd);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (!hp.split || hp.pass_tiles == 0) return cudaSuccess;
  for (uint32_t p = 0; p < hp.passes && e == cudaSuccess; ++p) {
    e = cudaMemsetAsync(dev + hp.o_pticket, 0, hp.bytes - hp.o_pticket, s);
    if (e == cudaSuccess) {
      seg_pass_kernel<<<hp.pass_tiles, kPassBlock, PassGeometry::kBytes, s>>>(pd, p);
      e = cudaGetLastError();
    }
  }
  return e;
}

}  // namespace seg
}  // namespace pa

using namespace pa;
using namespace pa::seg;

struct pa_segsort_plan {
  int device = -1;
  size_t num_segments = 0;
  unsigned long long total_keys = 0;
  HostPlan hp;
  unsigned grid = 0;
  char* dev = nullptr;
  PlanDev pd{};
  uint32_t* err_host = nullptr;
  cudaStream_t cap_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t* g_keys = nullptr;
  uint32_t* g_tmp = nullptr;
};

namespace {

int cfail(cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  cudaGetLastError();
  return record_error(e == cudaErrorMemoryAllocation ? PA_ERR_OOM : PA_ERR_CUDA, buf);
}

#define PA_SEG_CUDA(call)                                 \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cfail(e_, #call);       \
  } while (0)

bool dev_ptr(const void* p) {
  cudaPointerAttributes at;
  if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int d = 0;
  cudaGetDevice(&d);
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == d;
}

void destroy_graph(pa_segsort_plan* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  p->g_keys = p->g_tmp = nullptr;
}

int enqueue(pa_segsort_plan* p, cudaStream_t s) {
  PA_SEG_CUDA(launch_plan(p->hp, p->pd, p->dev, p->grid, s));
  // an odd number of passes (11-bit digits: three) leaves every segment in tmp
  if (p->hp.passes & 1u)
    PA_SEG_CUDA(cudaMemcpyAsync(p->pd.keys, p->pd.tmp, (size_t)p->total_keys * 4, cudaMemcpyDeviceToDevice, s));
  return PA_OK;
}

}  // namespace

extern "C" {

int pa_segsort_plan_create(const uint64_t* seg_offsets, size_t num_segments, const pa_segsort_config* cfg,
                           pa_segsort_plan** out) {
  if (!out) return record_error(PA_ERR_ARG, "out is NULL");
  *out = nullptr;
  if (!seg_offsets) return record_error(PA_ERR_ARG, "seg_offsets is NULL");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return record_error(PA_ERR_NO_DEVICE, "no CUDA device");
  }
  // The offsets must be readable on the host to plan the work.
  std::vector<uint64_t> off(num_segments + 1);
  if (dev_ptr(seg_offsets)) {
    PA_SEG_CUDA(cudaMemcpy(off.data(), seg_offsets, off.size() * 8, cudaMemcpyDeviceToHost));
  } else {
    std::memcpy(off.data(), seg_offsets, off.size() * 8);
  }
  auto* p = new pa_segsort_plan();
  if (int rc = build_host_plan(off.data(), num_segments, cfg, &p->hp)) {
    delete p;
    return rc;
  }
  cudaGetDevice(&p->device);
  p->num_segments = num_segments;
  p->total_keys = num_segments ? off[num_segments] : 0;
  cudaError_t e = cudaMalloc(&p->dev, p->hp.bytes);
  if (e != cudaSuccess) {
    delete p;
    return cfail(e, "cudaMalloc(plan)");
  }
  e = cudaMallocHost(&p->err_host, sizeof(uint32_t));
  if (e == cudaSuccess) e = upload_plan(p->hp, p->dev, (cudaStream_t)0);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    pa_segsort_plan_destroy(p);
    return cfail(e, "plan set-up");
  }
  p->grid = plan_grid(p->hp);
  p->pd = device_view(p->hp, p->dev, nullptr, nullptr);
  *out = p;
  return PA_OK;
}

int pa_segsort_plan_info(const pa_segsort_plan* p, uint32_t* num_small, uint32_t* num_large, uint32_t* num_items) {
  if (!p) return record_error(PA_ERR_ARG, "plan is NULL");
  if (num_small) *num_small = p->hp.num_small;
  if (num_large) *num_large = p->hp.num_large;
  if (num_items) *num_items = (uint32_t)p->hp.items.size();
  return PA_OK;
}

int pa_segsort_plan_run(pa_segsort_plan* p, uint32_t* keys, uint32_t* tmp, const pa_opts* opts) {
  if (!p) return record_error(PA_ERR_ARG, "plan is NULL");
  if (p->total_keys == 0) return PA_OK;
  if (!dev_ptr(keys) || !dev_ptr(tmp))
    return record_error(PA_ERR_ARG, "keys and tmp must be device memory holding the plan's total key count");
  cudaStream_t s = opts ? static_cast<cudaStream_t>(opts->stream) : (cudaStream_t)0;
  p->pd.keys = keys;
  p->pd.tmp = tmp;
  if (p->hp.cfg.use_graph) {
    if (!p->exec || p->g_keys != keys || p->g_tmp != tmp) {
      destroy_graph(p);
      PA_SEG_CUDA(cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal));
      const int rc = enqueue(p, p->cap_stream);
      cudaGraph_t g = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(p->cap_stream, &g);
      if (rc != PA_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ec != cudaSuccess) return cfail(ec, "cudaStreamEndCapture");
      p->graph = g;
      PA_SEG_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
      p->g_keys = keys;
      p->g_tmp = tmp;
    }
    PA_SEG_CUDA(cudaGraphLaunch(p->exec, s));
  } else {
    if (int rc = enqueue(p, s)) return rc;
  }
  if (opts && opts->async_device) return PA_OK;
  return pa_segsort_plan_sync(p, opts ? opts->stream : nullptr);
}

int pa_segsort_plan_sync(pa_segsort_plan* p, void* stream) {
  if (!p) return record_error(PA_ERR_ARG, "plan is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  PA_SEG_CUDA(cudaMemcpyAsync(p->err_host, p->pd.err, 4, cudaMemcpyDeviceToHost, s));
  PA_SEG_CUDA(cudaStreamSynchronize(s));
  if (*p->err_host) {
    PA_SEG_CUDA(cudaMemsetAsync(p->pd.err, 0, 4, s));
    PA_SEG_CUDA(cudaStreamSynchronize(s));
    return record_error(PA_ERR_TIMEOUT, "a bounded device-side wait of the batched sort gave up");
  }
  return PA_OK;
}

int pa_segsort_plan_destroy(pa_segsort_plan* p) {
  if (!p) return PA_OK;
  destroy_graph(p);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->dev) cudaFree(p->dev);
  if (p->err_host) cudaFreeHost(p->err_host);
  delete p;
  return PA_OK;
}

int pa_segmented_sort_u32(uint32_t* keys, const uint64_t* seg_offsets, size_t num_segments,
                          const pa_segsort_config* cfg, const pa_opts* opts) {
  if (num_segments == 0) return PA_OK;
  if (!keys || !seg_offsets) return record_error(PA_ERR_ARG, "NULL buffer");
  pa_segsort_plan* p = nullptr;
  pa_segsort_config c{};
  if (cfg) c = *cfg;
  c.use_graph = 0;  // one-shot: nothing to replay
  if (int rc = pa_segsort_plan_create(seg_offsets, num_segments, &c, &p)) return rc;
  const size_t n = (size_t)p->total_keys;
  cudaStream_t s = opts ? static_cast<cudaStream_t>(opts->stream) : (cudaStream_t)0;
  uint32_t* d_keys = keys;
  uint32_t* d_tmp = nullptr;
  const bool host = !dev_ptr(keys);
  cudaError_t e = cudaSuccess;
  if (n && host) e = cudaMalloc(&d_keys, n * 4);
  if (e == cudaSuccess && n) e = cudaMalloc(&d_tmp, n * 4);
  if (e == cudaSuccess && n && host) e = cudaMemcpyAsync(d_keys, keys, n * 4, cudaMemcpyHostToDevice, s);
  int rc = PA_OK;
  if (e != cudaSuccess) {
    rc = cfail(e, "batched sort buffers");
  } else if (n) {
    pa_opts o{};
    if (opts) o = *opts;
    o.async_device = 0;
    rc = pa_segsort_plan_run(p, d_keys, d_tmp, &o);
    if (rc == PA_OK && host) {
      e = cudaMemcpyAsync(keys, d_keys, n * 4, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) rc = cfail(e, "copy back");
    }
  }
  if (d_tmp) cudaFree(d_tmp);
  if (host && d_keys && d_keys != keys) cudaFree(d_keys);
  pa_segsort_plan_destroy(p);
  return rc;
}

}  // extern "C"
