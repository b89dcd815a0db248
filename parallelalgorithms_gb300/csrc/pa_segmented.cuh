// Host-side interface of the batched segmented sort (pa_segmented.cu), used
// by its C ABI and by the serving loop (pa_serve.cu) to launch coalesced
// batches on their own streams with caller-provided device memory.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "pa_gpu.h"

namespace pa {
namespace seg {

constexpr int kBlock = 512;
constexpr int kPasses = 4;                  // uint32 keys, 8-bit digits (11-bit digits: 3 passes)
constexpr uint32_t kHistChunk = 64 * 1024;  // keys per HIST item
constexpr int kHistLanes = 8;               // lane-banked copies of each counter
constexpr uint32_t kMaxSegmentKeys = (1u << 30) - 1;  // 32-bit look-back words

enum : uint32_t { ITEM_SMALL = 0, ITEM_HIST = 1, ITEM_SCAN = 2, ITEM_PASS = 3 };
enum : uint32_t { ST_HIST = 0, ST_SCAN = 1, ST_PASS0 = 2, kStages = 2 + kPasses };

struct Item {
  uint32_t kind;
  uint32_t pass;
  uint32_t seg;  // segment index (SMALL) or large-segment index
  uint32_t idx;  // tile (PASS) or chunk (HIST)
};

struct LargeSeg {
  unsigned long long base;
  uint32_t len;
  uint32_t tiles;
  uint32_t hist_chunks;
  uint32_t tile_base;   // first tile of this segment in each pass's status array (PASS items)
  uint32_t ptile_base;  // first tile of this segment in a pass launch (8-bit plans)
  uint32_t pad;
};

// 8-bit plans run their digit passes as separate launches after the
// persistent kernel: one onesweep launch per pass over every large
// segment's tiles (the plain sort's pass geometry), look-back within each
// segment.
constexpr int kPassBlock = 384;
constexpr int kPassItems = 16;
constexpr uint32_t kPassTile = (uint32_t)kPassBlock * kPassItems;

struct PlanDev {
  uint32_t* keys;
  uint32_t* tmp;
  uint32_t passes;                 // low digits sorted by the large segments' passes (4: all);
                                   // results end in keys for an even count, in tmp for an odd one
  const Item* items;
  uint32_t num_items;
  uint32_t total_tiles;
  const unsigned long long* seg_off;
  const LargeSeg* large;
  uint32_t* head;                  // zeroed per run
  uint32_t* done;                  // [large][kStages], zeroed per run
  uint32_t* hist;                  // [large][digits][bins], zeroed per run
  uint32_t* status;                // [passes][total_tiles][bins], zeroed per run
  unsigned long long* bin_start;   // [large][digits][bins]
  uint32_t* err;
  uint32_t radix_bits;             // 8 (256 bins, 4 digits) or 11 (2048 bins, 3 digits)
  // pass launches (8-bit plans)
  const uint32_t* tile_seg;        // [pass_tiles] large segment of each tile
  uint32_t pass_tiles;
  uint32_t* pass_ticket;           // zeroed before each pass
  uint32_t* pass_status;           // [pass_tiles][256], zeroed before each pass
};

// Digits of a 32-bit key and bins per digit for a digit width.
__host__ __device__ inline uint32_t seg_digits(uint32_t radix_bits) { return radix_bits == 11 ? 3u : 4u; }
__host__ __device__ inline uint32_t seg_bins(uint32_t radix_bits) { return 1u << radix_bits; }

using KernelFn = void (*)(const PlanDev);

// The persistent kernel instantiation for a (tile, small cutoff) choice.
struct KernelChoice {
  KernelFn fn;
  size_t smem;
  uint32_t pass_tile;
  uint32_t small_tile;
};

// A batch planned on the host: the work queue, the large segments, the
// offsets, and the layout of the device block the launch needs.
struct HostPlan {
  pa_segsort_config cfg{};
  KernelChoice kc{};
  std::vector<Item> items;
  std::vector<LargeSeg> large;
  std::vector<uint64_t> off;
  uint32_t total_tiles = 0, num_small = 0, num_large = 0;
  uint32_t passes = kPasses;  // digit passes of the large segments (3: every segment's top byte is
                              // constant; 3 with 11-bit digits)
  uint32_t radix_bits = 8;
  bool split = false;              // digit passes as separate launches (8-bit plans)
  uint32_t pass_tiles = 0;
  std::vector<uint32_t> tile_seg;
  size_t o_items = 0, o_off = 0, o_large = 0, o_tile_seg = 0, o_bins = 0, o_err = 0, o_head = 0, o_done = 0,
         o_hist = 0, o_status = 0, o_pticket = 0, o_pstatus = 0, bytes = 0;
};

// Validates the offsets and plans the queue and the device block layout.
// `passes` < 4 sorts large segments by their low `passes` bytes only (for
// segments whose higher bytes are constant); results then end in tmp when
// `passes` is odd (result_buffer).  With cfg->digit_bits = 11 the plan runs
// three 11-bit passes (and `passes` is ignored).
int build_host_plan(const uint64_t* off_host, size_t num_segments, const pa_segsort_config* cfg, HostPlan* hp,
                    int passes = kPasses);
// Pointers of a device block laid out by `hp` (keys / tmp: the batch's keys).
PlanDev device_view(const HostPlan& hp, char* dev, uint32_t* keys, uint32_t* tmp);
// Where a run of `pd` leaves the sorted keys: keys after an even number of
// passes, tmp after an odd one.
__host__ __device__ inline uint32_t* result_buffer(const PlanDev& pd) { return (pd.passes & 1u) ? pd.tmp : pd.keys; }
// Copies the queue, offsets and segment table into the block; clears its error word.
// With `pinned_staging` (page-locked, at least plan_image_bytes(hp) bytes, left
// untouched by the caller until the copy has run) the three tables go up in
// one asynchronous copy; without it they are copied from the plan's own
// pageable vectors, which makes the runtime wait for the stream first.
cudaError_t upload_plan(const HostPlan& hp, char* dev, cudaStream_t s, void* pinned_staging = nullptr);
// Bytes of the block's leading image (queue, offsets, segment table).
size_t plan_image_bytes(const HostPlan& hp);
// Persistent grid for the plan's kernel on the current device.
unsigned plan_grid(const HostPlan& hp);
// Clears the per-run state and launches the persistent kernel (and, for an
// 8-bit plan, the pass launches after it).
cudaError_t launch_plan(const HostPlan& hp, const PlanDev& pd, char* dev, unsigned grid, cudaStream_t s);

}  // namespace seg
}  // namespace pa
