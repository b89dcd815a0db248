// In-place partition of 32-bit keys by one 8-bit digit, through a scratch
// buffer of fixed size: the level step of the in-place MSD radix sort
// (pa_sort_u32_inplace), GPU form of parallel_hybrid_inplace_msd_radix_sort
// (RadixSortMsdParallel.h:291-317).
//
// The reference partitions the array by its top digit in place (a parallel
// histogram, then one serial swap cycle per bin, RadixSortMsdParallel.h:31-63),
// recurses into every bin in parallel tasks (:65-99) and finishes bins under
// 100 keys by insertion sort; besides the keys it holds O(1) memory per level.
// A serial swap cycle has no GPU form, so here a level moves keys in rounds
// through two scratch halves C[0], C[1] of H keys each, never through a second
// array of n keys.  Per bucket b of the range (region [start_b, end_b) from
// the digit histogram):
//   w_b  write cursor: [start_b, w_b) already holds bucket b's keys;
//   r_b  end of the unread part: [w_b, r_b) still holds original keys,
//        [r_b, end_b) was read into the scratch and is free.
// One round, with the keys in hand in C[p] and their digit counts cnt[p]:
//   1. top-up: the first H - |C[p]| unread keys, taken from the tops of the
//      unread parts bucket by bucket, are appended to C[p] (r_b lowered);
//   2. with need_t keys of digit t in hand, the unread keys in
//      [w_t, min(w_t + need_t, r_t)) are copied to C[p ^ 1] (they are in
//      the way) and w_t advances by need_t;
//   3. the keys in hand are scattered into [old w_t, old w_t + need_t) by an
//      onesweep digit pass (pa_onesweep.cu) whose bin starts are those
//      cursors and whose key count is read on the device.
// Every key is read once from its unread place and written once to its final
// one (16 bytes of traffic per key, scratch included); a round places every
// key in hand, so ceil(len / H) + 1 rounds always suffice (rounds after the
// last key is placed find nothing to do).  The scratch half written by a
// round's copies is read back by its pass while still in L2.
#include <algorithm>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kBins = 256;
constexpr int kPlanThreads = kBins;  // plan kernels: one thread per bucket
constexpr int kMoveBlock = 256;  // threads of the copy kernel (and of the plan kernels' scans)
constexpr int kMoveWarps = kMoveBlock / 32;
static_assert(kMoveBlock == kPlanThreads, "the block scan serves both");

// Exclusive prefix of v over the 256 threads of the CTA; *total = the sum.
// s_warp: 8 words of shared memory.  Contains barriers: every thread calls it.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* s_warp, T* total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  T incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  T run = 0, all = 0;
#pragma unroll
  for (int w = 0; w < kMoveWarps; ++w) {
    if ((uint32_t)w < warp) run += s_warp[w];
    all += s_warp[w];
  }
  *total = all;
  __syncthreads();
  return run + incl - v;
}

__device__ __forceinline__ uint32_t digit_at(uint32_t k, uint32_t shift) { return (k >> shift) & (kBins - 1); }

// Regions from the range's digit counts; nothing in hand.
__global__ void __launch_bounds__(kPlanThreads) inplace_init_kernel(const unsigned long long* hist,
                                                                    InplaceState* st) {
  __shared__ unsigned long long s_warp[kMoveWarps];
  const uint32_t t = threadIdx.x;
  unsigned long long total;
  const unsigned long long c = hist[t];
  const unsigned long long start = block_excl_scan(c, s_warp, &total);
  st->w[t] = start;
  st->r[t] = start + c;
  st->cursor[t] = 0;
  st->cnt[0][t] = 0;
  st->cnt[1][t] = 0;
  if (t == 0) {
    st->hand[0] = st->hand[1] = 0;
    st->total = 0;
    st->run_base = st->run_keys = 0;
    st->ticket = 0;
  }
  if (t < sizeof(SortCtrl) / 4) reinterpret_cast<uint32_t*>(&st->ctrl)[t] = 0;  // pass 0: keys_a -> keys_b
}

// Step 1's plan: run t = the top g_t keys of bucket t's unread part, where
// the g_t take the first H - hand[p] unread keys in bucket order.
__global__ void __launch_bounds__(kPlanThreads) inplace_plan_topup_kernel(InplaceState* st, int p,
                                                                          unsigned long long half) {
  __shared__ unsigned long long s_warp[kMoveWarps];
  const uint32_t t = threadIdx.x;
  const unsigned long long hand = st->hand[p];
  const unsigned long long want = half > hand ? half - hand : 0;
  const unsigned long long u = st->r[t] - st->w[t];
  unsigned long long all;
  const unsigned long long before = block_excl_scan(u, s_warp, &all);
  const unsigned long long g = before >= want ? 0 : min(u, want - before);
  const unsigned long long top = st->r[t] - g;
  st->r[t] = top;
  st->run_src[t] = top;
  st->run_len[t] = g;
  unsigned long long taken;
  const unsigned long long at = block_excl_scan(g, s_warp, &taken);
  st->run_dst[t] = hand + at;
  if (t == 0) {
    st->run_base = hand;
    st->run_keys = taken;
    st->total = hand + taken;
  }
}

// Step 2's plan: the scatter cursors, the runs in the way, the new cursors.
__global__ void __launch_bounds__(kPlanThreads) inplace_plan_swap_kernel(InplaceState* st, int p) {
  __shared__ unsigned long long s_warp[kMoveWarps];
  const uint32_t t = threadIdx.x;
  const unsigned long long need = st->cnt[p][t];
  st->cnt[p][t] = 0;
  const unsigned long long w = st->w[t], r = st->r[t];
  const unsigned long long stop = min(w + need, r);
  const unsigned long long x = stop > w ? stop - w : 0;
  st->cursor[t] = w;
  st->run_src[t] = w;
  st->run_len[t] = x;
  unsigned long long all;
  st->run_dst[t] = block_excl_scan(x, s_warp, &all);
  st->w[t] = w + need;
  st->r[t] = max(r, w + need);
  if (t == 0) {
    st->ticket = 0;   // the round's pass takes tiles from 0
    st->hand[p] = 0;  // every key in hand is placed by this round's scatter
    st->hand[p ^ 1] = all;
    st->run_base = 0;
    st->run_keys = all;
  }
}

// Copies the plan's runs keys[run_src[b], +run_len[b]) to
// dst[run_dst[b], ...) and adds their digit counts into cnt; zeroes
// zero[0, zero_words) on the way (the next pass's look-back words).  Chunks
// of kGatherChunk destination keys per CTA step: a chunk inside one run (the
// common case: runs average the scratch half / 256 keys) is one straight
// copy, others find each key's run by binary search among the chunk's runs.
constexpr int kGatherItems = 8;
constexpr int kGatherChunk = kMoveBlock * kGatherItems;
__global__ void __launch_bounds__(kMoveBlock) inplace_gather_kernel(const uint32_t* keys, uint32_t* dst,
                                                                    const InplaceState* st,
                                                                    unsigned long long* cnt, uint32_t shift,
                                                                    uint32_t* zero, size_t zero_words) {
  __shared__ unsigned long long s_dst[kBins];
  __shared__ unsigned long long s_src[kBins];
  __shared__ uint32_t s_h[kBins];
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  for (size_t z = (size_t)blockIdx.x * kMoveBlock + tid; z < zero_words; z += (size_t)gridDim.x * kMoveBlock)
    zero[z] = 0;
  s_dst[tid] = st->run_dst[tid];
  s_src[tid] = st->run_src[tid];
  s_h[tid] = 0;
  const unsigned long long base = st->run_base, end = base + st->run_keys;
  __syncthreads();
  // the run holding i: the last b in [lo, 255] with s_dst[b] <= i (empty runs
  // share their start with the next run, so the last such b is never empty)
  auto run_of = [&](unsigned long long i, uint32_t lo) {
    uint32_t b = lo;
    for (uint32_t step = 128; step > 0; step >>= 1)
      if (b + step < kBins && s_dst[b + step] <= i) b += step;
    return b;
  };
  for (unsigned long long c0 = base + (unsigned long long)blockIdx.x * kGatherChunk; c0 < end;
       c0 += (unsigned long long)gridDim.x * kGatherChunk) {
    const uint32_t cn = (uint32_t)min((unsigned long long)kGatherChunk, end - c0);
    const uint32_t b_lo = run_of(c0, 0);
    const uint32_t b_hi = run_of(c0 + cn - 1, b_lo);
    // every load of the chunk first (all in flight together), then the stores
    uint32_t kk[kGatherItems];
#pragma unroll
    for (int j = 0; j < kGatherItems; ++j) {
      const uint32_t o = (uint32_t)j * kMoveBlock + tid;
      kk[j] = 0;
      if (o < cn) {
        const unsigned long long i = c0 + o;
        const uint32_t b = b_lo == b_hi ? b_lo : run_of(i, b_lo);
        kk[j] = keys[s_src[b] + (i - s_dst[b])];
      }
    }
#pragma unroll
    for (int j = 0; j < kGatherItems; ++j) {
      const uint32_t o = (uint32_t)j * kMoveBlock + tid;
      if (o < cn) dst[c0 + o] = kk[j];
    }
#pragma unroll
    for (int j = 0; j < kGatherItems; ++j) {
      const bool valid = (uint32_t)j * kMoveBlock + tid < cn;
      const uint32_t k = kk[j];
      // digit counts; a warp whose keys share one digit (skewed inputs) adds
      // them with one atomic instead of 32 on the same word
      // (every lane runs the shuffle: a full-mask collective skipped by some
      // lanes never completes)
      const uint32_t d = digit_at(k, shift);
      const uint32_t act = __ballot_sync(0xFFFFFFFFu, valid);
      const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, __ffs(act | 1u) - 1);
      const bool same = __all_sync(0xFFFFFFFFu, !valid || d == d0);
      if (same) {
        if (act && lane == (uint32_t)(__ffs(act) - 1)) atomicAdd(&s_h[d], (uint32_t)__popc(act));
      } else if (valid) {
        atomicAdd(&s_h[d], 1u);
      }
    }
  }
  __syncthreads();
  if (s_h[tid]) atomicAdd(&cnt[tid], (unsigned long long)s_h[tid]);
}

}  // namespace

size_t inplace_status_bytes(size_t n, size_t half) {
  return ceil_div(half, onesweep_tile_keys(4, false)) * 256 * onesweep_status_bytes(std::max(n, half));
}

cudaError_t launch_inplace_partition(uint32_t* keys, size_t n, uint32_t shift, const unsigned long long* hist,
                                     uint32_t* c0, uint32_t* c1, size_t half, InplaceState* st, void* status,
                                     uint32_t* err, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (half == 0 || shift > 24) return cudaErrorInvalidValue;
  const unsigned sms = (unsigned)device_info().sm_count;
  const unsigned gather_grid = (unsigned)min(ceil_div(half, (size_t)kGatherChunk), (size_t)sms * 8);
  const size_t status_words = inplace_status_bytes(n, half) / 4;
  inplace_init_kernel<<<1, kPlanThreads, 0, stream>>>(hist, st);
  cudaError_t e = cudaGetLastError();
  // step 3 is an onesweep digit pass over the keys in hand (their count read
  // on the device) into the array at the round's cursors
  OnesweepArgs pass{};
  pass.vals_a = pass.vals_b = nullptr;
  pass.n = half;
  pass.n_dev = &st->total;
  pass.out_n = n;
  pass.shift = shift;
  pass.pass = 0;
  pass.is_float = 0;
  pass.bin_start = st->cursor;
  pass.status = status;
  pass.tile_counter = &st->ticket;
  pass.ctrl = &st->ctrl;
  pass.err = err;
  pass.keys_b = keys;
  const size_t rounds = ceil_div(n, half) + 1;
  for (size_t round = 0; round < rounds && e == cudaSuccess; ++round) {
    const int p = (int)(round & 1);
    uint32_t* in_hand = p ? c1 : c0;
    uint32_t* next_hand = p ? c0 : c1;
    inplace_plan_topup_kernel<<<1, kPlanThreads, 0, stream>>>(st, p, (unsigned long long)half);
    inplace_gather_kernel<<<gather_grid, kMoveBlock, 0, stream>>>(keys, in_hand, st, st->cnt[p], shift, nullptr, 0);
    inplace_plan_swap_kernel<<<1, kPlanThreads, 0, stream>>>(st, p);
    inplace_gather_kernel<<<gather_grid, kMoveBlock, 0, stream>>>(keys, next_hand, st, st->cnt[p ^ 1], shift,
                                                                  static_cast<uint32_t*>(status), status_words);
    e = cudaGetLastError();
    if (e != cudaSuccess) break;
    pass.keys_a = in_hand;
    e = launch_onesweep_pass(pass, 4, false, stream);
  }
  return e;
}

}  // namespace pa
