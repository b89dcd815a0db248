// Digit histograms.
//
// digit_counts_kernel is the GPU form of HistogramByteComponentsParallel
// (HistogramParallel.h:249-329): one read of the keys produces the counts of
// every digit at once (the "1" of the reference's (1 + D)-pass two-phase
// design, RadixSortLsdParallel.h:43-83).  The same kernel with one digit at an
// arbitrary shift is HistogramOneByteComponentParallel (:535-576), and with
// 1-byte keys the unsigned-char overloads (:16-247).
//
// Each CTA keeps num_digits x 2^radix_bits u32 counters in shared memory,
// streams a grid-strided share of the keys with 16-byte loads, and adds its
// counters into the 64-bit global result once at the end.  When all 32
// lanes of a warp hold the same digit (constant or presorted runs) the warp
// makes one shared atomic of 32 instead of 32 colliding ones.
#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kHistBlock = 512;

template <typename K, int ND, int RB>
__device__ __forceinline__ void count_key(uint32_t* s_hist, K key, bool valid, uint32_t shift0, uint32_t step) {
  constexpr uint32_t R = 1u << RB;
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t vmask = __ballot_sync(FULL, valid);
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const uint32_t b = valid ? (uint32_t)(key >> (shift0 + (uint32_t)d * step)) & (R - 1) : 0u;
    const uint32_t b0 = __shfl_sync(FULL, b, __ffs(vmask) - 1);
    if (__all_sync(FULL, !valid || b == b0)) {
      if ((threadIdx.x & 31u) == 0 && vmask) atomicAdd(&s_hist[d * R + b0], (uint32_t)__popc(vmask));
    } else if (valid) {
      atomicAdd(&s_hist[d * R + b], 1u);
    }
  }
}

// Keys per 16-byte vector.
template <typename K>
constexpr int kVec = 16 / (int)sizeof(K);

template <typename K, int ND, int RB>
__global__ void __launch_bounds__(kHistBlock) digit_counts_kernel(const K* __restrict__ keys, size_t n,
                                                                    uint32_t shift0, uint32_t step, int is_float,
                                                                    unsigned long long* __restrict__ out) {
  constexpr int R = 1 << RB;
  constexpr int V = kVec<K>;
  __shared__ uint32_t s_hist[ND * R];
  for (int i = threadIdx.x; i < ND * R; i += kHistBlock) s_hist[i] = 0;
  __syncthreads();

  // Split [0, n) into an unaligned head, whole 16-byte vectors, and a tail.
  const uintptr_t addr = reinterpret_cast<uintptr_t>(keys);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > n) head = n;
  const size_t nvec = (n - head) / V;
  const size_t tail_start = head + nvec * V;
  const uint4* vec = reinterpret_cast<const uint4*>(keys + head);

  const size_t warps_total = (size_t)gridDim.x * (kHistBlock / 32);
  const size_t gwarp = (size_t)blockIdx.x * (kHistBlock / 32) + (threadIdx.x >> 5);
  const uint32_t lane = threadIdx.x & 31u;
  // Warp-uniform trip count: every lane of a warp runs the same iterations,
  // so the warp-wide votes in count_key see all 32 lanes.
  for (size_t w = gwarp; w * 32 < nvec; w += warps_total) {
    const size_t vi = w * 32 + lane;
    const bool valid = vi < nvec;
    uint4 q = make_uint4(0, 0, 0, 0);
    if (valid) q = ld_stream_v4(vec + vi);
    const K* ks = reinterpret_cast<const K*>(&q);
#pragma unroll
    for (int e = 0; e < V; ++e) {
      K key = ks[e];
      if (sizeof(K) == 4) key = to_ordered(key, is_float != 0);
      count_key<K, ND, RB>(s_hist, key, valid, shift0, step);
    }
  }
  // Head and tail (fewer than 2 * V keys in total) go to the first warp.
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    const size_t rest = head + (n - tail_start);
    for (size_t base = 0; base < rest; base += 32) {
      const size_t r = base + lane;
      const bool valid = r < rest;
      K key = 0;
      if (valid) key = keys[r < head ? r : tail_start + (r - head)];
      if (sizeof(K) == 4) key = to_ordered(key, is_float != 0);
      count_key<K, ND, RB>(s_hist, key, valid, shift0, step);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ND * R; i += kHistBlock) {
    const uint32_t c = s_hist[i];
    if (c) atomicAdd(&out[i], (unsigned long long)c);
  }
}

template <typename K, int ND, int RB>
cudaError_t launch_counts_t(const void* keys, size_t n, uint32_t shift0, uint32_t step, bool is_float,
                            unsigned long long* out, cudaStream_t stream) {
  constexpr int V = kVec<K>;
  const size_t work_warps = ceil_div(ceil_div(n, (size_t)V), (size_t)32 * 8);
  const size_t max_blocks = (size_t)device_info().sm_count * 4;
  size_t blocks = ceil_div(work_warps, (size_t)(kHistBlock / 32));
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks < 1) blocks = 1;
  digit_counts_kernel<K, ND, RB><<<(unsigned)blocks, kHistBlock, 0, stream>>>(static_cast<const K*>(keys), n, shift0,
                                                                             step, is_float ? 1 : 0, out);
  return cudaGetLastError();
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

cudaError_t launch_digit_counts(const void* keys, size_t n, int key_bytes, int num_digits, int radix_bits,
                                uint32_t shift0, uint32_t shift_step, bool is_float, unsigned long long* out,
                                cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (radix_bits == 8) {
    if (key_bytes == 4) {
      if (num_digits == 4) return launch_counts_t<uint32_t, 4, 8>(keys, n, shift0, shift_step, is_float, out, stream);
      if (num_digits == 1) return launch_counts_t<uint32_t, 1, 8>(keys, n, shift0, shift_step, is_float, out, stream);
    } else if (key_bytes == 8) {
      if (num_digits == 8)
        return launch_counts_t<unsigned long long, 8, 8>(keys, n, shift0, shift_step, false, out, stream);
      if (num_digits == 1)
        return launch_counts_t<unsigned long long, 1, 8>(keys, n, shift0, shift_step, false, out, stream);
    } else if (key_bytes == 1 && num_digits == 1) {
      return launch_counts_t<uint8_t, 1, 8>(keys, n, shift0, shift_step, false, out, stream);
    }
  }
  return cudaErrorInvalidValue;
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

cudaError_t launch_scan_digits(const unsigned long long* counts, int passes, int radix_bits, size_t n,
                               bool is_float, bool allow_skip, unsigned long long* bin_start, SortCtrl* ctrl,
                               cudaStream_t stream) {
  if (passes < 1 || passes > kMaxPasses || radix_bits != 8) return cudaErrorInvalidValue;
  scan_digits_kernel<256><<<1, kScanBlock, 0, stream>>>(counts, passes, n, is_float ? 1 : 0, allow_skip ? 1 : 0,
                                                         bin_start, ctrl);
  return cudaGetLastError();
}

}  // namespace pa
