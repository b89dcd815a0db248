// Digit histograms.
//
// digit_counts_kernel is the GPU form of HistogramByteComponentsParallel
// (HistogramParallel.h:249-329): one read of the keys produces the counts of
// every digit at once (the "1" of the reference's (1 + D)-pass two-phase
// design, RadixSortLsdParallel.h:43-83).  The same kernel with one digit at an
// arbitrary shift is HistogramOneByteComponentParallel (:535-576), and with
// 1-byte keys the unsigned-char overloads (:16-247).
//
// Each CTA keeps its counters in shared memory "lane-banked": counter
// (digit d, bin b) is replicated once per lane, at word (d * 2^radix_bits + b)
// * LANES + lane % LANES, so the 32 atomics of a warp-wide update always land
// in distinct banks whatever the key distribution (constant input included).
// A CTA streams a grid-strided share of the keys with 16-byte loads, then
// folds the lane copies and adds its counts into the 64-bit global result.
//
// Also here: the per-quantum counts and start of bins (ComputeStartOfBinsPar),
// the scan + pass control of the sort, and the byte counting sort's fill.
#include <algorithm>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kHistBlock = 1024;

// Keys per 16-byte vector.
template <typename K>
constexpr int kVec = 16 / (int)sizeof(K);

// Lane copies per counter: the most (32 = one bank per lane, then 16, 8, ...)
// for which the table fits 160 KB of shared memory.
template <int ND, int RB>
constexpr int kLanes = (ND * (1 << RB) * 32 * 4 <= 160 * 1024)   ? 32
                       : (ND * (1 << RB) * 16 * 4 <= 160 * 1024) ? 16
                       : (ND * (1 << RB) * 8 * 4 <= 160 * 1024)  ? 8
                       : (ND * (1 << RB) * 4 * 4 <= 160 * 1024)  ? 4
                       : (ND * (1 << RB) * 2 * 4 <= 160 * 1024)  ? 2
                                                                  : 1;

template <int ND, int RB>
constexpr size_t hist_smem_bytes() {
  return (size_t)ND * (1 << RB) * kLanes<ND, RB> * 4;
}

// BYTES: the digits are the key's bytes shift0 / 8, shift0 / 8 + 1, ... (the
// sorts' histograms): each is extracted by one byte permute instead of a
// shift and a mask.  FLT: 32-bit float keys, counted in their ordered form.
template <typename K, int ND, int RB, bool BYTES, bool FLT>
__global__ void __launch_bounds__(kHistBlock, 1) digit_counts_kernel(const K* __restrict__ keys, size_t n,
                                                                       uint32_t shift0, uint32_t step,
                                                                       unsigned long long* __restrict__ out) {
  constexpr int R = 1 << RB;
  constexpr int V = kVec<K>;
  constexpr int L = kLanes<ND, RB>;
  constexpr uint32_t kWords = (uint32_t)ND * R * L;
  extern __shared__ uint32_t s_h[];
  for (uint32_t i = threadIdx.x; i < kWords; i += kHistBlock) s_h[i] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x % L;
  uint32_t* my = s_h + lane;
  const uint32_t byte0 = shift0 / 8;

  auto count = [&](K key) {
    if constexpr (sizeof(K) == 4 && FLT) key = to_ordered(key, true);
#pragma unroll
    for (int d = 0; d < ND; ++d) {
      uint32_t b;
      if constexpr (BYTES && RB == 8) {
        const uint32_t byte = byte0 + (uint32_t)d;
        if constexpr (sizeof(K) == 8)
          b = __byte_perm(byte < 4 ? (uint32_t)key : (uint32_t)(key >> 32), 0u, 0x4440u | (byte & 3u));
        else if constexpr (sizeof(K) == 4)
          b = __byte_perm((uint32_t)key, 0u, 0x4440u | (byte & 3u));
        else
          b = (uint32_t)key;
      } else {
        b = (uint32_t)(key >> (shift0 + (uint32_t)d * step)) & (R - 1);
      }
      atomicAdd(my + ((uint32_t)d * R + b) * L, 1u);
    }
  };

  // Split [0, n) into an unaligned head, whole 16-byte vectors, and a tail.
  const uintptr_t addr = reinterpret_cast<uintptr_t>(keys);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > n) head = n;
  const size_t nvec = (n - head) / V;
  const size_t tail_start = head + nvec * V;
  const uint4* vec = reinterpret_cast<const uint4*>(keys + head);
  const size_t stride = (size_t)gridDim.x * kHistBlock;
  size_t i = (size_t)blockIdx.x * kHistBlock + threadIdx.x;
  for (; i + stride < nvec; i += 2 * stride) {  // two 16-byte loads in flight
    const uint4 q0 = ld_stream_v4(vec + i);
    const uint4 q1 = ld_stream_v4(vec + i + stride);
    const K* k0 = reinterpret_cast<const K*>(&q0);
    const K* k1 = reinterpret_cast<const K*>(&q1);
#pragma unroll
    for (int e = 0; e < V; ++e) count(k0[e]);
#pragma unroll
    for (int e = 0; e < V; ++e) count(k1[e]);
  }
  for (; i < nvec; i += stride) {
    const uint4 q0 = ld_stream_v4(vec + i);
    const K* k0 = reinterpret_cast<const K*>(&q0);
#pragma unroll
    for (int e = 0; e < V; ++e) count(k0[e]);
  }
  if (blockIdx.x == 0) {  // head and tail: fewer than 2 * V keys
    const size_t rest = head + (n - tail_start);
    for (size_t r = threadIdx.x; r < rest; r += kHistBlock) count(keys[r < head ? r : tail_start + (r - head)]);
  }
  __syncthreads();
  // Fold the lane copies: thread e sums counter e's L copies, starting at a
  // lane-dependent copy so that a warp's reads hit distinct banks.
  for (uint32_t e = threadIdx.x; e < (uint32_t)(ND * R); e += kHistBlock) {
    uint32_t sum = 0;
#pragma unroll 8
    for (int j = 0; j < L; ++j) sum += s_h[e * L + ((j + e) % L)];
    if (sum) atomicAdd(&out[e], (unsigned long long)sum);
  }
}

template <typename K, int ND, int RB, bool BYTES, bool FLT>
cudaError_t launch_counts_k(const void* keys, size_t n, uint32_t shift0, uint32_t step, unsigned long long* out,
                            cudaStream_t stream) {
  constexpr int V = kVec<K>;
  auto kern = digit_counts_kernel<K, ND, RB, BYTES, FLT>;
  constexpr size_t smem = hist_smem_bytes<ND, RB>();
  cudaError_t e = ensure_dynamic_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const size_t work = ceil_div(ceil_div(n, (size_t)V), (size_t)kHistBlock * 4);
  size_t blocks = work < (size_t)device_info().sm_count ? work : (size_t)device_info().sm_count;
  if (blocks < 1) blocks = 1;
  kern<<<(unsigned)blocks, kHistBlock, smem, stream>>>(static_cast<const K*>(keys), n, shift0, step, out);
  return cudaGetLastError();
}

template <typename K, int ND, int RB>
cudaError_t launch_counts_t(const void* keys, size_t n, uint32_t shift0, uint32_t step, bool is_float,
                            unsigned long long* out, cudaStream_t stream) {
  const bool bytes = RB == 8 && shift0 % 8 == 0 && (ND == 1 || step == 8) && (sizeof(K) > 1 || shift0 == 0);
  if (sizeof(K) == 4 && is_float)
    return bytes ? launch_counts_k<K, ND, RB, true, true>(keys, n, shift0, step, out, stream)
                 : launch_counts_k<K, ND, RB, false, true>(keys, n, shift0, step, out, stream);
  return bytes ? launch_counts_k<K, ND, RB, true, false>(keys, n, shift0, step, out, stream)
               : launch_counts_k<K, ND, RB, false, false>(keys, n, shift0, step, out, stream);
}

// The 32-bit sort's histogram with the first pass's tile offsets
// (launch_tile_counts).  CTA c owns the first pass's tiles [c * tpc,
// (c + 1) * tpc) and reads them in order, one tile per step, each of the
// NT = tile_keys / 8 threads two 16-byte vectors of the tile (the pairs of
// the next two tiles are in flight while the current one is counted: one
// CTA per SM needs about two tiles' bytes in flight to keep up with HBM).
// Bytes 1-3 go to lane-banked counters as in digit_counts_kernel; byte 0
// goes to one of two lane-banked sets, by the parity of the step.  The sets
// are never cleared: after the step's barrier, thread b < 256 sums its bin's
// copies in the step's set, and the difference from that set's previous sum
// is the tile's count of byte-0 value b; the chunk's running total before
// the tile is the tile's tile_prefix row.  While thread b sums one set the
// others count the next tile into the other one, and the next barrier ends
// the sum before the set is counted into again.  (Named barriers that let
// the counting threads run up to two tiles ahead of the summing ones
// measured slower: 0.129 against 0.114 ms per 100M keys.)  The last CTA to
// finish (ticket) turns the chunks' totals into chunk_excl.
constexpr uint32_t kTcLanes = 32;
constexpr size_t kTcSmemBytes = (size_t)(3 + 2) * 256 * kTcLanes * 4;  // 160 KB
static_assert((size_t)kTileCountMaxChunks * 256 * 4 <= kTcSmemBytes, "the chunks' totals fit the counters' space");

template <bool FLT, int NT>
__global__ void __launch_bounds__(NT, 1) tile_counts_kernel(const uint32_t* __restrict__ keys, size_t n,
                                                              uint32_t tile_keys, uint32_t tiles, uint32_t tpc,
                                                              unsigned long long* __restrict__ out,
                                                              uint32_t* __restrict__ tile_prefix,
                                                              uint32_t* chunk_tot, uint32_t* __restrict__ chunk_excl,
                                                              uint32_t* ticket) {
  constexpr uint32_t L = kTcLanes;
  extern __shared__ __align__(16) uint32_t s_tc[];
  uint32_t* s_hi = s_tc;                  // bytes 1..3: [3][256][L]
  uint32_t* s_set0 = s_tc + 3 * 256 * L;  // byte 0, even steps: [256][L]
  uint32_t* s_set1 = s_set0 + 256 * L;    // byte 0, odd steps
  __shared__ uint32_t s_last;
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  constexpr uint32_t nt = NT;  // tile_keys / 8
  for (uint32_t i = tid; i < 5u * 256u * L; i += nt) s_tc[i] = 0;
  __syncthreads();
  const uint32_t c = blockIdx.x;
  const uint32_t t0 = c * tpc, t1 = min(t0 + tpc, tiles);
  const uint32_t vpt = tile_keys / 4u;  // 16-byte vectors per tile (2 * nt)
  const uint4* vec = reinterpret_cast<const uint4*>(keys);
  auto is_full = [&](uint32_t t) { return (size_t)(t + 1) * tile_keys <= n; };
  auto count = [&](uint32_t key, uint32_t* set) {
    if constexpr (FLT) key = to_ordered(key, true);
    atomicAdd(set + __byte_perm(key, 0u, 0x4440u) * L + lane, 1u);
    atomicAdd(s_hi + (0u * 256u + __byte_perm(key, 0u, 0x4441u)) * L + lane, 1u);
    atomicAdd(s_hi + (1u * 256u + __byte_perm(key, 0u, 0x4442u)) * L + lane, 1u);
    atomicAdd(s_hi + (2u * 256u + __byte_perm(key, 0u, 0x4443u)) * L + lane, 1u);
  };
  // q: tile t's pair, r: tile t + 1's (loaded when the tile is a full one of the chunk)
  uint4 q0 = make_uint4(0u, 0u, 0u, 0u), q1 = q0, r0 = q0, r1 = q0;
  auto fetch = [&](uint32_t t, uint4& v0, uint4& v1) {
    if (t < t1 && is_full(t)) {
      v0 = ld_stream_v4(vec + (size_t)t * vpt + tid);
      v1 = ld_stream_v4(vec + (size_t)t * vpt + nt + tid);
    }
  };
  fetch(t0, q0, q1);
  fetch(t0 + 1, r0, r1);
  // thread b < 256: keys of byte-0 value b in the chunk's tiles so far, and
  // the two sets' last sums for bin b
  uint32_t run = 0, seen0 = 0, seen1 = 0;
  for (uint32_t t = t0; t < t1; ++t) {
    const bool odd = ((t - t0) & 1u) != 0;
    uint32_t* set = odd ? s_set1 : s_set0;
    if (is_full(t)) {
      const uint4 a = q0, b = q1;
      q0 = r0;
      q1 = r1;
      fetch(t + 2, r0, r1);
      count(a.x, set);
      count(a.y, set);
      count(a.z, set);
      count(a.w, set);
      count(b.x, set);
      count(b.y, set);
      count(b.z, set);
      count(b.w, set);
    } else {  // the array's last tile, shorter than a tile: plain loads
      for (size_t i = (size_t)t * tile_keys + tid; i < n; i += nt) count(keys[i], set);
    }
    __syncthreads();
    if (tid < 256u) {
      // the bin's L copies as 16-byte reads, rotated by bin so that each
      // quarter warp's reads cover the 32 banks once
      const uint4* row = reinterpret_cast<const uint4*>(set + tid * L);
      uint32_t sum = 0;
#pragma unroll
      for (uint32_t j = 0; j < L / 4u; ++j) {
        const uint4 x = row[(j + tid) & (L / 4u - 1u)];
        sum += x.x + x.y + x.z + x.w;
      }
      const uint32_t cnt = sum - (odd ? seen1 : seen0);
      if (odd)
        seen1 = sum;
      else
        seen0 = sum;
      tile_prefix[(size_t)t * 256u + tid] = run;
      run += cnt;
    }
  }
  if (tid < 256u) {
    chunk_tot[(size_t)c * 256u + tid] = run;
    if (run) atomicAdd(&out[tid], (unsigned long long)run);
  }
  // bytes 1..3: fold the lane copies (every thread has passed the last step's
  // barrier, so all counting is done)
  for (uint32_t e = tid; e < 3u * 256u; e += nt) {
    uint32_t sum = 0;
#pragma unroll 8
    for (uint32_t j = 0; j < L; ++j) sum += s_hi[e * L + ((j + e) & (L - 1u))];
    if (sum) atomicAdd(&out[256u + e], (unsigned long long)sum);
  }
  // the last CTA to finish turns the chunks' totals into chunk_excl
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1u) ? 1u : 0u;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const uint32_t chunks = gridDim.x;
  const uint4* tot4 = reinterpret_cast<const uint4*>(chunk_tot);
  uint4* s_tot4 = reinterpret_cast<uint4*>(s_tc);  // the counters are folded: their space is free
  // every load issued before any is used (one round trip, not one per row)
  constexpr uint32_t kPer = ((uint32_t)kTileCountMaxChunks * 64u + nt - 1u) / nt;
  uint4 v[kPer];
#pragma unroll
  for (uint32_t j = 0; j < kPer; ++j) {
    const uint32_t i = tid + j * nt;
    if (i < chunks * 64u) v[j] = __ldcg(tot4 + i);
  }
#pragma unroll
  for (uint32_t j = 0; j < kPer; ++j) {
    const uint32_t i = tid + j * nt;
    if (i < chunks * 64u) s_tot4[i] = v[j];
  }
  __syncthreads();
  if (tid < 256u) {
    uint32_t acc = 0;
    for (uint32_t cc = 0; cc < chunks; ++cc) {
      const uint32_t v = s_tc[cc * 256u + tid];
      chunk_excl[(size_t)cc * 256u + tid] = acc;
      acc += v;
    }
  }
}

// Several arrays' one-digit histograms in one launch: CTAs walk the
// flattened list of (job, chunk) items; each chunk is counted in lane-banked
// shared counters (one copy per lane of an 8-lane group) and added into its
// job's global counts.
constexpr int kMultiBlock = 512;
constexpr int kMultiLanes = 8;

template <typename K>
__global__ void __launch_bounds__(kMultiBlock) digit_counts_multi_kernel(const HistJob* __restrict__ jobs, int njobs,
                                                                         uint32_t total_chunks) {
  __shared__ uint32_t s_h[256 * kMultiLanes];
  __shared__ int s_job;
  const uint32_t lane = threadIdx.x % kMultiLanes;
  for (uint32_t item = blockIdx.x; item < total_chunks; item += gridDim.x) {
    if (threadIdx.x == 0) {  // the job whose chunks hold `item`: last first_chunk <= item
      int lo = 0, hi = njobs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].first_chunk <= item) lo = mid;
        else hi = mid - 1;
      }
      s_job = lo;
    }
    for (uint32_t i = threadIdx.x; i < 256 * kMultiLanes; i += kMultiBlock) s_h[i] = 0;
    __syncthreads();
    const HistJob J = jobs[s_job];
    const unsigned long long lo = (unsigned long long)(item - J.first_chunk) * kHistJobChunk;
    const unsigned long long hi = min(J.n, lo + kHistJobChunk);
    const K* keys = static_cast<const K*>(J.keys);
    for (unsigned long long i = lo + threadIdx.x; i < hi; i += kMultiBlock)
      atomicAdd(&s_h[((uint32_t)(keys[i] >> J.shift) & 255u) * kMultiLanes + lane], 1u);
    __syncthreads();
    if (threadIdx.x < 256) {
      uint32_t sum = 0;
#pragma unroll
      for (int j = 0; j < kMultiLanes; ++j) sum += s_h[threadIdx.x * kMultiLanes + j];
      if (sum) atomicAdd(&J.out[threadIdx.x], (unsigned long long)sum);
    }
    __syncthreads();
  }
}

// Counts per work quantum over keys[l, r): a CTA covers one chunk that never
// straddles a quantum boundary; quanta are numbered by absolute index
// (i / work_quanta) as in HistogramByteComponentsAcrossWorkQuantasQC
// (HistogramParallel.h:351-393).  `keys` points at index l.
constexpr int kQcBlock = 256;
constexpr size_t kQcChunk = 64 * 1024;

__global__ void __launch_bounds__(kQcBlock) quanta_counts_kernel(const uint32_t* __restrict__ keys, size_t l,
                                                                 size_t r, size_t work_quanta, size_t q0,
                                                                 size_t chunks_per_quantum, uint32_t shift,
                                                                 unsigned long long* __restrict__ out) {
  __shared__ uint32_t s_hist[256];
  for (int i = threadIdx.x; i < 256; i += kQcBlock) s_hist[i] = 0;
  __syncthreads();
  const size_t q = q0 + blockIdx.x / chunks_per_quantum;
  const size_t c = blockIdx.x % chunks_per_quantum;
  const size_t qs = q * work_quanta;
  size_t s = qs + c * kQcChunk;
  size_t e = s + kQcChunk;
  if (e > qs + work_quanta) e = qs + work_quanta;
  if (s < l) s = l;
  if (e > r) e = r;
  for (size_t i = s + threadIdx.x; i < e; i += kQcBlock) atomicAdd(&s_hist[(keys[i - l] >> shift) & 255u], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += kQcBlock)
    if (s_hist[i]) atomicAdd(&out[q * 256 + i], (unsigned long long)s_hist[i]);
}

// start_of_bins from per-quantum counts.  Block b (one per bin) walks the
// quanta; bin totals are then turned into bin offsets by one small block.
__global__ void quanta_column_prefix_kernel(const unsigned long long* counts, size_t quanta,
                                            unsigned long long* sob, unsigned long long* bin_total) {
  const int b = blockIdx.x;
  if (threadIdx.x != 0) return;
  unsigned long long run = 0;
  for (size_t q = 0; q < quanta; ++q) {
    sob[q * 256 + b] = run;
    run += counts[q * 256 + b];
  }
  bin_total[b] = run;
}

__global__ void quanta_add_bin_offsets_kernel(unsigned long long* sob, size_t quanta,
                                              const unsigned long long* bin_total) {
  __shared__ unsigned long long s_off[256];
  if (threadIdx.x == 0) {
    unsigned long long run = 0;
    for (int b = 0; b < 256; ++b) {
      s_off[b] = run;
      run += bin_total[b];
    }
  }
  __syncthreads();
  const size_t total = quanta * 256;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
    sob[i] += s_off[i & 255];
}

// Exclusive scan of each pass's counts and the pass control block.
constexpr int kScanBlock = 256;

template <int R>
__global__ void __launch_bounds__(kScanBlock) scan_digits_kernel(const unsigned long long* __restrict__ counts,
                                                                 int passes, size_t n, int is_float, int allow_skip,
                                                                 unsigned long long* __restrict__ bin_start,
                                                                 SortCtrl* ctrl) {
  constexpr int PER = R / kScanBlock;
  __shared__ unsigned long long s_warp[kScanBlock / 32];
  __shared__ uint32_t s_trivial[kMaxPasses];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int p = 0; p < passes; ++p) {
    unsigned long long c[PER];
    unsigned long long local = 0;
    bool trivial = false;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      c[i] = counts[(size_t)p * R + threadIdx.x * PER + i];
      local += c[i];
      trivial |= (c[i] == (unsigned long long)n);
    }
    unsigned long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
      if (lane >= (uint32_t)o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    const int any_trivial = __syncthreads_or(trivial ? 1 : 0);
    unsigned long long woff = 0;
    for (uint32_t w = 0; w < warp; ++w) woff += s_warp[w];
    unsigned long long run = woff + incl - local;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      bin_start[(size_t)p * R + threadIdx.x * PER + i] = run;
      run += c[i];
    }
    if (threadIdx.x == 0) s_trivial[p] = (allow_skip && any_trivial) ? 1u : 0u;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int last_exec = -1, first_exec = -1;
    uint32_t in_tmp = 0, executed = 0;
    for (int p = 0; p < kMaxPasses; ++p) {
      PassCtrl& pc = ctrl->pass[p];
      pc.skip = (p >= passes) ? 1u : s_trivial[p];
      pc.src_is_tmp = in_tmp;
      pc.transform_in = 0;
      pc.transform_out = 0;
      if (!pc.skip) {
        if (first_exec < 0) first_exec = p;
        last_exec = p;
        in_tmp ^= 1u;
        ++executed;
      }
    }
    if (first_exec >= 0 && is_float) {
      ctrl->pass[first_exec].transform_in = 1;
      ctrl->pass[last_exec].transform_out = 1;
    }
    ctrl->final_in_tmp = in_tmp;
    ctrl->executed = executed;
  }
}

}  // namespace

bool tile_counts_supported(size_t tile_keys) { return tile_keys == 4096 || tile_keys == 6144 || tile_keys == 8192; }

cudaError_t launch_tile_counts(const uint32_t* keys, size_t n, size_t tile_keys, bool is_float,
                               unsigned long long* out, uint32_t* tile_prefix, uint32_t* chunk_tot,
                               uint32_t* chunk_excl, uint32_t* ticket, uint32_t* tpc, cudaStream_t stream) {
  if (n == 0 || n >= ((size_t)1 << 30) || !tile_counts_supported(tile_keys) ||
      (reinterpret_cast<uintptr_t>(keys) & 15u) != 0)
    return cudaErrorInvalidValue;
  const size_t tiles = ceil_div(n, tile_keys);
  size_t g0 = std::min((size_t)device_info().sm_count, (size_t)kTileCountMaxChunks);
  g0 = std::max((size_t)1, std::min(g0, tiles));
  const size_t per = ceil_div(tiles, g0);
  const size_t grid = ceil_div(tiles, per);  // every chunk holds at least one tile
  auto go = [&](auto* kern) {
    cudaError_t e = ensure_dynamic_smem(kern, kTcSmemBytes);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)grid, (unsigned)(tile_keys / 8), kTcSmemBytes, stream>>>(
        keys, n, (uint32_t)tile_keys, (uint32_t)tiles, (uint32_t)per, out, tile_prefix, chunk_tot, chunk_excl,
        ticket);
    *tpc = (uint32_t)per;
    return cudaGetLastError();
  };
  if (tile_keys == 4096) return is_float ? go(tile_counts_kernel<true, 512>) : go(tile_counts_kernel<false, 512>);
  if (tile_keys == 6144) return is_float ? go(tile_counts_kernel<true, 768>) : go(tile_counts_kernel<false, 768>);
  return is_float ? go(tile_counts_kernel<true, 1024>) : go(tile_counts_kernel<false, 1024>);
}

cudaError_t launch_digit_counts(const void* keys, size_t n, int key_bytes, int num_digits, int radix_bits,
                                uint32_t shift0, uint32_t shift_step, bool is_float, unsigned long long* out,
                                cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (radix_bits == 8) {
    if (key_bytes == 4) {
      if (num_digits == 4) return launch_counts_t<uint32_t, 4, 8>(keys, n, shift0, shift_step, is_float, out, stream);
      if (num_digits == 2) return launch_counts_t<uint32_t, 2, 8>(keys, n, shift0, shift_step, is_float, out, stream);
      if (num_digits == 1) return launch_counts_t<uint32_t, 1, 8>(keys, n, shift0, shift_step, is_float, out, stream);
    } else if (key_bytes == 8) {
      if (num_digits == 8)
        return launch_counts_t<unsigned long long, 8, 8>(keys, n, shift0, shift_step, false, out, stream);
      if (num_digits == 1)
        return launch_counts_t<unsigned long long, 1, 8>(keys, n, shift0, shift_step, false, out, stream);
    } else if (key_bytes == 1 && num_digits == 1) {
      return launch_counts_t<uint8_t, 1, 8>(keys, n, shift0, shift_step, false, out, stream);
    }
  } else if (radix_bits == 11) {
    if (key_bytes == 4 && num_digits == 3)
      return launch_counts_t<uint32_t, 3, 11>(keys, n, shift0, shift_step, is_float, out, stream);
    if (key_bytes == 8 && num_digits == 6)
      return launch_counts_t<unsigned long long, 6, 11>(keys, n, shift0, shift_step, false, out, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_digit_counts_multi(const HistJob* jobs, int njobs, uint32_t total_chunks, int key_bytes,
                                      cudaStream_t stream) {
  if (njobs <= 0 || total_chunks == 0) return cudaSuccess;
  const unsigned grid = (unsigned)min((size_t)total_chunks, (size_t)device_info().sm_count * 4);
  if (key_bytes == 4)
    digit_counts_multi_kernel<uint32_t><<<grid, kMultiBlock, 0, stream>>>(jobs, njobs, total_chunks);
  else if (key_bytes == 8)
    digit_counts_multi_kernel<unsigned long long><<<grid, kMultiBlock, 0, stream>>>(jobs, njobs, total_chunks);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_quanta_counts(const uint32_t* keys, size_t l, size_t r, size_t work_quanta,
                                 uint32_t which_byte, unsigned long long* out, cudaStream_t stream) {
  if (r <= l || work_quanta == 0) return cudaSuccess;
  const size_t q0 = l / work_quanta, q1 = (r - 1) / work_quanta;
  const size_t cpq = ceil_div(work_quanta, kQcChunk);
  const size_t blocks = cpq * (q1 - q0 + 1);
  if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  quanta_counts_kernel<<<(unsigned)blocks, kQcBlock, 0, stream>>>(keys, l, r, work_quanta, q0, cpq, 8u * which_byte,
                                                                   out);
  return cudaGetLastError();
}

cudaError_t launch_quanta_start_of_bins(const unsigned long long* counts, size_t quanta,
                                        unsigned long long* start_of_bins, cudaStream_t stream) {
  if (quanta == 0) return cudaSuccess;
  // bin totals live just past the quanta x 256 output (the caller sizes it).
  unsigned long long* bin_total = start_of_bins + quanta * 256;
  quanta_column_prefix_kernel<<<256, 32, 0, stream>>>(counts, quanta, start_of_bins, bin_total);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)min(ceil_div(quanta * 256, (size_t)256), (size_t)1024);
  quanta_add_bin_offsets_kernel<<<grid, 256, 0, stream>>>(start_of_bins, quanta, bin_total);
  return cudaGetLastError();
}

// Byte counting sort's fill (CountingSortParallel.h:48-68): every CTA
// rebuilds the 256 value starts (exclusive prefix of the counts) in shared
// memory; each thread writes 16-byte runs of a[i] = the value whose range
// holds i, walking a per-thread value cursor forward (its positions only
// grow), with single bytes before the first and after the last 16-byte
// boundary of the array.
__global__ void __launch_bounds__(256) counting_fill_kernel(uint8_t* __restrict__ a, size_t n,
                                                            const unsigned long long* __restrict__ counts) {
  __shared__ unsigned long long s_start[257];
  __shared__ unsigned long long s_warp[8];
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const unsigned long long c = counts[t];
  unsigned long long incl = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  unsigned long long before = 0;
  for (uint32_t w = 0; w < warp; ++w) before += s_warp[w];
  s_start[t] = before + incl - c;
  if (t == 255) s_start[256] = before + incl;
  __syncthreads();
  // value holding position p: the largest v with s_start[v] <= p (empty values skipped)
  auto value_at = [&](unsigned long long p) {
    uint32_t lo = 0, hi = 255;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (s_start[mid] <= p) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  const size_t head = min(n, (size_t)((16u - (reinterpret_cast<uintptr_t>(a) & 15u)) & 15u));
  const size_t nvec = (n - head) / 16;
  const size_t tail = head + nvec * 16;
  const size_t gt = (size_t)blockIdx.x * blockDim.x + t;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  if (gt < head) a[gt] = (uint8_t)value_at(gt);
  if (gt < n - tail) a[tail + gt] = (uint8_t)value_at(tail + gt);
  uint4* av = reinterpret_cast<uint4*>(a + head);
  uint32_t v = 0;
  bool have = false;
  for (size_t j = gt; j < nvec; j += stride) {
    const unsigned long long p0 = head + j * 16;
    if (!have) {
      v = value_at(p0);
      have = true;
    }
    while (s_start[v + 1] <= p0) ++v;  // the cursor only moves forward
    uint32_t w[4];
    if (s_start[v + 1] >= p0 + 16) {  // the whole run holds one value
      const uint32_t rep = v * 0x01010101u;
      w[0] = w[1] = w[2] = w[3] = rep;
    } else {
      uint32_t u = v;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t word = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const unsigned long long p = p0 + 4 * q + b;
          while (s_start[u + 1] <= p) ++u;
          word |= u << (8 * b);
        }
        w[q] = word;
      }
    }
    av[j] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

cudaError_t launch_counting_fill(uint8_t* a, size_t n, const unsigned long long* counts, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const size_t vec = n / 16 + 1;
  const unsigned grid = (unsigned)min(ceil_div(vec, (size_t)256 * 8), (size_t)device_info().sm_count * 8);
  counting_fill_kernel<<<grid < 1 ? 1 : grid, 256, 0, stream>>>(a, n, counts);
  return cudaGetLastError();
}

cudaError_t launch_scan_digits(const unsigned long long* counts, int passes, int radix_bits, size_t n,
                               bool is_float, bool allow_skip, unsigned long long* bin_start, SortCtrl* ctrl,
                               cudaStream_t stream) {
  if (passes < 1 || passes > kMaxPasses) return cudaErrorInvalidValue;
  if (radix_bits == 8)
    scan_digits_kernel<256><<<1, kScanBlock, 0, stream>>>(counts, passes, n, is_float ? 1 : 0, allow_skip ? 1 : 0,
                                                           bin_start, ctrl);
  else if (radix_bits == 11)
    scan_digits_kernel<2048><<<1, kScanBlock, 0, stream>>>(counts, passes, n, is_float ? 1 : 0, allow_skip ? 1 : 0,
                                                            bin_start, ctrl);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace pa
