// Kernels of the pipelined host-buffer sort of 32-bit keys (pa_capi.cu,
// pipelined_host_sort): the input arrives in chunks, each chunk is sorted on
// its top 16 bits while the next one is still being copied in, and once all
// chunks are in, each 16-bit bucket (keys sharing their top 16 bits) is
// gathered from its run in every chunk and sorted on its low 16 bits by one
// CTA in shared memory, straight into its final place.  The keys then cross
// HBM once after the chunk passes (one read, one write), against the three
// digit passes plus a gather a bucket sort by 8-bit buckets would need.
//
//   bucket_bounds_kernel  per chunk: where each 16-bit bucket starts in the
//                         chunk (binary search inside its top-byte bucket,
//                         whose start the chunk's top-digit scan gives);
//   bucket_totals_kernel  each bucket's total over the chunks, and per top
//                         byte the key count and the largest 16-bit bucket
//                         (for the host's plan);
//   bucket_positions_kernel  each bucket's global start (exclusive scan);
//   bucket_sort_kernel    one CTA per bucket: gather, four stable 4-bit
//                         counting passes on the low 16 bits, write out.
#include "pa_common.cuh"
#include "pa_kernels.cuh"
#include "pa_onesweep_tile.cuh"

namespace pa {
namespace {

using namespace os;

constexpr uint32_t kBuckets = 1u << 16;      // 16-bit buckets
constexpr uint32_t kStartsStride = kBuckets + 1;

// starts[j] = first index of the chunk (sorted on its top 16 bits) whose key
// has top 16 bits >= j, for j in [0, 65536]; top_start: the chunk's 256
// exclusive top-byte starts.
__global__ void bucket_bounds_kernel(const uint32_t* __restrict__ keys, uint32_t n,
                                     const unsigned long long* __restrict__ top_start, uint32_t* __restrict__ starts) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > kBuckets) return;
  if (j == kBuckets) {
    starts[j] = n;
    return;
  }
  const uint32_t t = j >> 8;
  uint32_t lo = (uint32_t)top_start[t];
  uint32_t hi = t == 255 ? n : (uint32_t)top_start[t + 1];
  while (lo < hi) {  // first index in [lo, hi) with (key >> 16) >= j
    const uint32_t mid = lo + (hi - lo) / 2;
    if ((keys[mid] >> 16) < j)
      lo = mid + 1;
    else
      hi = mid;
  }
  starts[j] = lo;
}

// Bucket totals, one CTA per top byte (256 buckets): tot[j] = bucket j's
// keys over the chunks, summary[t] = keys of top byte t, summary[256 + t] =
// its largest bucket.
__global__ void __launch_bounds__(256) bucket_totals_kernel(const uint32_t* __restrict__ starts, int nc,
                                                            uint32_t* __restrict__ tot,
                                                            unsigned long long* __restrict__ summary) {
  __shared__ unsigned long long s_sum[8];
  __shared__ uint32_t s_max[8];
  const uint32_t j = blockIdx.x * 256u + threadIdx.x, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t v = 0;
#pragma unroll
  for (int c = 0; c < kMaxChunkRuns; ++c) {
    if (c < nc) {
      const uint32_t* s = starts + (size_t)c * kStartsStride + j;
      v += s[1] - s[0];
    }
  }
  tot[j] = v;
  unsigned long long sum = v;
  uint32_t mx = v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  }
  if (lane == 0) {
    s_sum[warp] = sum;
    s_max[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    uint32_t m = 0;
    for (int w = 0; w < 8; ++w) {
      t += s_sum[w];
      m = max(m, s_max[w]);
    }
    summary[blockIdx.x] = t;
    summary[256 + blockIdx.x] = m;
  }
}

// Bucket positions, one CTA per top byte: pos[j] = keys in top bytes below
// j's (each CTA adds up summary[0, t) itself) + keys in the buckets of its
// own top byte below j (block scan of tot); pos[65536] = all keys.
__global__ void __launch_bounds__(256) bucket_positions_kernel(const uint32_t* __restrict__ tot,
                                                               const unsigned long long* __restrict__ summary,
                                                               unsigned long long* __restrict__ pos) {
  __shared__ unsigned long long s_w[8];
  const uint32_t t = blockIdx.x, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  // keys of the top bytes below t
  unsigned long long below = threadIdx.x < t ? summary[threadIdx.x] : 0ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xFFFFFFFFu, below, o);
  if (lane == 0) s_w[warp] = below;
  __syncthreads();
  unsigned long long base = 0;
  for (int w = 0; w < 8; ++w) base += s_w[w];
  __syncthreads();
  // exclusive scan of this top byte's 256 bucket totals
  const uint32_t v = tot[t * 256u + threadIdx.x];
  unsigned long long incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  if (lane == 31) s_w[warp] = incl;
  __syncthreads();
  for (uint32_t w = 0; w < warp; ++w) base += s_w[w];
  pos[t * 256u + threadIdx.x] = base + incl - v;
  if (t == 255 && threadIdx.x == 255) pos[kBuckets] = base + incl;
}

// One CTA per 16-bit bucket b = first + blockIdx.x: its run in every chunk
// (chunk c's keys with top 16 bits b, at src[chunks.lo[c] + starts[c][b],
// ... starts[c][b + 1])) is gathered into shared memory, padded with
// all-ones keys to the tile, sorted by four stable 4-bit counting passes on
// the low 16 bits (the top 16 are b for every real key; padding sorts after
// them), and written to dst[pos[b], pos[b + 1]).  A bucket larger than the
// tile raises DEVERR_BAD_STATE (the host sends such groups elsewhere).
template <int BLOCK, int ITEMS>
__global__ void __launch_bounds__(BLOCK) bucket_sort_kernel(const uint32_t* __restrict__ src, const ChunkRuns chunks,
                                                            const uint32_t* __restrict__ starts,
                                                            const unsigned long long* __restrict__ pos, uint32_t first,
                                                            uint32_t* __restrict__ dst, uint32_t* err) {
  using G = Geometry<uint32_t, false, BLOCK, ITEMS>;
  constexpr uint32_t TILE = (uint32_t)G::kTile;
  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t* s_keys = reinterpret_cast<uint32_t*>(smem + G::kKeysOff);
  uint32_t* s_cnt = reinterpret_cast<uint32_t*>(smem + G::kCntOff);
  uint32_t* s_warp = reinterpret_cast<uint32_t*>(smem + G::kWarpTotOff);
  __shared__ unsigned long long s_src[kMaxChunkRuns];
  __shared__ uint32_t s_off[kMaxChunkRuns + 1];
  const uint32_t b = first + blockIdx.x;
  const unsigned long long base = pos[b];
  const uint32_t total = (uint32_t)(pos[b + 1] - base);
  if (total == 0) return;
  if (total > TILE) {
    if (threadIdx.x == 0) raise_error(err, DEVERR_BAD_STATE);
    return;
  }
  if (threadIdx.x == 0) {
    uint32_t off = 0;
#pragma unroll
    for (int c = 0; c < kMaxChunkRuns; ++c) {  // (constant indices keep the table in parameter space)
      if (c < chunks.count) {
        const uint32_t* s = starts + (size_t)c * kStartsStride + b;
        s_src[c] = chunks.lo[c] + s[0];
        s_off[c] = off;
        off += s[1] - s[0];
      }
    }
    s_off[chunks.count] = off;
  }
  __syncthreads();
  // gather: consecutive threads read consecutive keys of a run, all of a
  // thread's loads in flight at once
  uint32_t g[ITEMS];
#pragma unroll
  for (int q = 0; q < ITEMS; ++q) {
    const uint32_t i = threadIdx.x + (uint32_t)q * BLOCK;
    g[q] = 0xFFFFFFFFu;
    if (i < total) {
      int c = 0;
      while (i >= s_off[c + 1]) ++c;
      g[q] = src[s_src[c] + (i - s_off[c])];
    }
  }
#pragma unroll
  for (int q = 0; q < ITEMS; ++q) s_keys[threadIdx.x + (uint32_t)q * BLOCK] = g[q];
  __syncthreads();
  uint32_t k[ITEMS];
  uint32_t unused[1];
  for (uint32_t sh = 0; sh < 16; sh += 4) {
    load_run<uint32_t, false, ITEMS>(k, unused, s_keys, nullptr);
    nibble_pass<uint32_t, false, BLOCK, ITEMS>(k, unused, sh, s_keys, nullptr, s_cnt, s_warp);  // ends with a barrier
  }
  for (uint32_t i = threadIdx.x; i < total; i += BLOCK) dst[base + i] = s_keys[i];
}

template <int BLOCK, int ITEMS>
cudaError_t launch_bucket_sort_t(const uint32_t* src, const ChunkRuns& chunks, const uint32_t* starts,
                                 const unsigned long long* pos, uint32_t first, uint32_t num, uint32_t* dst,
                                 uint32_t* err, cudaStream_t stream) {
  using G = Geometry<uint32_t, false, BLOCK, ITEMS>;
  auto kern = bucket_sort_kernel<BLOCK, ITEMS>;
  cudaError_t e = ensure_dynamic_smem(kern, G::kBytes);
  if (e != cudaSuccess) return e;
  kern<<<num, BLOCK, G::kBytes, stream>>>(src, chunks, starts, pos, first, dst, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_bucket_bounds(const uint32_t* keys, size_t n, const unsigned long long* top_start, uint32_t* starts,
                                 cudaStream_t stream) {
  if (n >= ((size_t)1 << 32)) return cudaErrorInvalidValue;
  constexpr unsigned kBlock = 256;
  bucket_bounds_kernel<<<(kBuckets + 1 + kBlock - 1) / kBlock, kBlock, 0, stream>>>(keys, (uint32_t)n, top_start,
                                                                                     starts);
  return cudaGetLastError();
}

cudaError_t launch_bucket_totals(const uint32_t* starts, int num_chunks, uint32_t* tot, unsigned long long* pos,
                                 unsigned long long* summary, cudaStream_t stream) {
  if (num_chunks < 1 || num_chunks > kMaxChunkRuns) return cudaErrorInvalidValue;
  bucket_totals_kernel<<<256, 256, 0, stream>>>(starts, num_chunks, tot, summary);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  bucket_positions_kernel<<<256, 256, 0, stream>>>(tot, summary, pos);
  return cudaGetLastError();
}

size_t bucket_sort_max_keys() { return 8192; }

cudaError_t launch_bucket_sort(const uint32_t* src, const ChunkRuns& chunks, const uint32_t* starts,
                               const unsigned long long* pos, uint32_t first_bucket, uint32_t num_buckets,
                               size_t max_bucket_keys, uint32_t* dst, uint32_t* err, cudaStream_t stream) {
  if (num_buckets == 0) return cudaSuccess;
  if (chunks.count < 1 || chunks.count > kMaxChunkRuns || (size_t)first_bucket + num_buckets > kBuckets)
    return cudaErrorInvalidValue;
  if (max_bucket_keys <= 2048)
    return launch_bucket_sort_t<256, 8>(src, chunks, starts, pos, first_bucket, num_buckets, dst, err, stream);
  if (max_bucket_keys <= 4096)
    return launch_bucket_sort_t<256, 16>(src, chunks, starts, pos, first_bucket, num_buckets, dst, err, stream);
  if (max_bucket_keys <= 8192)
    return launch_bucket_sort_t<512, 16>(src, chunks, starts, pos, first_bucket, num_buckets, dst, err, stream);
  return cudaErrorInvalidValue;
}

}  // namespace pa
