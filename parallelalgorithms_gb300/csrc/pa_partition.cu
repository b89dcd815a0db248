// Radix partition around a few ascending indices k[0, m): GPU form of
// PartitionRadix (RadixPartition.h:92-185).  The reference narrows digit by
// digit with an in-place swap loop; here the k-th smallest key of each k is
// found by the select (pa_select.cu), and the keys are then split into the
// 2m + 1 buckets those m pivot values define:
//   bucket 2i     keys strictly between pivot i - 1 and pivot i,
//   bucket 2i + 1 keys equal to pivot i,
//   bucket 2m     keys above the last pivot.
// (With equal pivots the buckets between and for the repeats stay empty.)
// In bucket order every a[k_i] lands inside the "equal to pivot i" bucket
// (its first position is the number of keys below pivot i, at most k_i, and
// the bucket holds every key equal to it), nothing before it is larger and
// nothing after it is smaller: the reference's contract.  The order of the
// keys inside a bucket is not specified (the reference's is an artefact of
// its serial swap loop).
//
// Two reads and one write of the keys: every CTA counts its chunk's keys per
// bucket (no global atomics: a few cursors shared by thousands of CTAs made
// a hot spot), one CTA per bucket scans that bucket's counts over the chunks,
// then every CTA ranks its chunk's keys per bucket in shared memory (lanes of
// a warp that share a bucket found with four ballots, one shared atomic per
// group) and writes each key at its bucket's start + its chunk's offset +
// its rank.
#include <type_traits>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kPartBlock = 256;
constexpr int kPartItems = 16;
constexpr int kPartTile = kPartBlock * kPartItems;

// Bucket of key x among the M sorted pivots: the number of pivots below x
// plus the number of pivots at or below it.  This is non-decreasing in x,
// puts the keys equal to a pivot in a bucket of their own between the keys
// below and above it (with equal pivots, several buckets stay empty), and
// takes values 0 .. 2M.
template <int M>
__device__ __forceinline__ uint32_t bucket_of(uint32_t x, const uint32_t (&p)[M]) {
  uint32_t b = 0;
#pragma unroll
  for (int i = 0; i < M; ++i) b += (x > p[i] ? 1u : 0u) + (x >= p[i] ? 1u : 0u);
  return b;
}

// Lanes of the warp whose BITS-bit value equals this lane's.
template <int BITS>
__device__ __forceinline__ uint32_t match_small(uint32_t b) {
  uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
  for (int bit = 0; bit < BITS; ++bit) {
    const uint32_t v = __ballot_sync(0xFFFFFFFFu, (b >> bit) & 1u);
    peers &= ((b >> bit) & 1u) ? v : ~v;
  }
  return peers;
}

// Bits of the largest bucket number, 2M.
template <int M>
struct BucketBits {
  static constexpr int value = 2 * M < 2 ? 1 : 2 * M < 4 ? 2 : 2 * M < 8 ? 3 : 4;
};

// Chunk c's count of bucket b into cnt[b * chunks + c]: per-thread counters
// in registers, summed over the warp by shuffles and over the CTA in shared
// memory.
template <int M>
__global__ void __launch_bounds__(kPartBlock) partition_count_kernel(const uint32_t* __restrict__ in, size_t n,
                                                                     const uint32_t* __restrict__ pivots,
                                                                     unsigned long long* __restrict__ cnt) {
  constexpr int NB = 2 * M + 1;
  constexpr int kWarps = kPartBlock / 32;
  __shared__ uint32_t s_wc[kWarps][NB];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  uint32_t p[M];
#pragma unroll
  for (int i = 0; i < M; ++i) p[i] = pivots[i];
  const size_t chunk = (size_t)blockIdx.x * kPartTile;
  uint32_t x[kPartItems];
#pragma unroll
  for (int j = 0; j < kPartItems; ++j) {
    const size_t i = chunk + (size_t)j * kPartBlock + tid;
    x[j] = i < n ? in[i] : 0u;
  }
  uint32_t c[NB];
#pragma unroll
  for (int b = 0; b < NB; ++b) c[b] = 0;
#pragma unroll
  for (int j = 0; j < kPartItems; ++j) {
    const uint32_t bk = chunk + (size_t)j * kPartBlock + tid < n ? bucket_of<M>(x[j], p) : 0xFFu;
#pragma unroll
    for (int b = 0; b < NB; ++b) c[b] += bk == (uint32_t)b ? 1u : 0u;
  }
#pragma unroll
  for (int b = 0; b < NB; ++b) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c[b] += __shfl_xor_sync(0xFFFFFFFFu, c[b], o);
  }
  if (lane == 0)
#pragma unroll
    for (int b = 0; b < NB; ++b) s_wc[warp][b] = c[b];
  __syncthreads();
  if (tid < (uint32_t)NB) {
    unsigned long long sum = 0;
    for (int w = 0; w < kWarps; ++w) sum += s_wc[w][tid];
    cnt[(size_t)tid * gridDim.x + blockIdx.x] = sum;
  }
}

// Writes every key of chunk blockIdx.x to out at its bucket's start (the
// lower buckets' totals) + the chunk's offset in the bucket (cnt, scanned
// over the chunks) + its warp's offset + its rank among the warp's keys of
// that bucket (lanes sharing a bucket found with ballots; one counter per
// warp and bucket, bumped by the group's lowest lane).
template <int M>
__global__ void __launch_bounds__(kPartBlock) partition_write_kernel(const uint32_t* __restrict__ in,
                                                                     uint32_t* __restrict__ out, size_t n,
                                                                     const uint32_t* __restrict__ pivots,
                                                                     const unsigned long long* __restrict__ cnt,
                                                                     const unsigned long long* __restrict__ total) {
  constexpr int NB = 2 * M + 1;
  constexpr int kWarps = kPartBlock / 32;
  __shared__ uint32_t s_wc[kWarps][16];
  __shared__ unsigned long long s_pos[kWarps][16];
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  uint32_t p[M];
#pragma unroll
  for (int i = 0; i < M; ++i) p[i] = pivots[i];
  if (tid < kWarps * 16) s_wc[tid / 16][tid % 16] = 0;
  __syncthreads();
  const uint32_t lt = lanemask_lt();
  const size_t chunk = (size_t)blockIdx.x * kPartTile;
  uint32_t x[kPartItems];
  uint32_t br[kPartItems];  // bucket << 16 | rank inside the warp's run of that bucket
#pragma unroll
  for (int j = 0; j < kPartItems; ++j) {
    const size_t i = chunk + (size_t)j * kPartBlock + tid;
    x[j] = i < n ? in[i] : 0u;
  }
  uint32_t* wc = s_wc[warp];
#pragma unroll
  for (int j = 0; j < kPartItems; ++j) {
    const bool valid = chunk + (size_t)j * kPartBlock + tid < n;
    const uint32_t b = bucket_of<M>(x[j], p);
    const uint32_t peers = match_small<BucketBits<M>::value>(b) & __ballot_sync(0xFFFFFFFFu, valid);
    const uint32_t pl = peers & lt;
    const uint32_t base = wc[b];
    __syncwarp();
    if (valid && pl == 0) wc[b] = base + __popc(peers);
    br[j] = (b << 16) | (base + __popc(pl));
    __syncwarp();
  }
  __syncthreads();
  if (tid < (uint32_t)NB) {  // each warp's first position in the bucket
    unsigned long long run = cnt[(size_t)tid * gridDim.x + blockIdx.x];
    for (uint32_t b = 0; b < tid; ++b) run += total[b];
    for (int w = 0; w < kWarps; ++w) {
      s_pos[w][tid] = run;
      run += s_wc[w][tid];
    }
  }
  __syncthreads();
  const unsigned long long* pos = s_pos[warp];
#pragma unroll
  for (int j = 0; j < kPartItems; ++j) {
    const size_t i = chunk + (size_t)j * kPartBlock + tid;
    if (i < n) {
      const unsigned long long o = pos[br[j] >> 16] + (br[j] & 0xFFFFu);
      if (o < n) out[o] = x[j];
    }
  }
}

// One CTA per bucket b: cnt[b * chunks + c] -> exclusive prefix over the
// chunks (in place), and the bucket's total into total[b].
constexpr int kPartScanBlock = 1024;
__global__ void __launch_bounds__(kPartScanBlock) partition_scan_kernel(unsigned long long* cnt, size_t chunks,
                                                                        unsigned long long* total) {
  __shared__ unsigned long long s_warp[kPartScanBlock / 32];
  unsigned long long* col = cnt + (size_t)blockIdx.x * chunks;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const size_t per = ceil_div(chunks, (size_t)kPartScanBlock);
  const size_t lo = min(chunks, tid * per), hi = min(chunks, lo + per);
  unsigned long long local = 0;
  for (size_t c = lo; c < hi; ++c) local += col[c];
  unsigned long long incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  unsigned long long run = incl - local;
  for (uint32_t w = 0; w < warp; ++w) run += s_warp[w];
  if (tid == kPartScanBlock - 1) total[blockIdx.x] = run + local;
  for (size_t c = lo; c < hi; ++c) {
    const unsigned long long v = col[c];
    col[c] = run;
    run += v;
  }
}

}  // namespace

size_t partition_scratch_words(size_t n, int m) {
  return (size_t)(2 * m + 1) * (ceil_div(n, (size_t)kPartTile) + 1);
}

cudaError_t launch_partition(const uint32_t* in, uint32_t* out, size_t n, const uint32_t* pivots, int m,
                             unsigned long long* scratch, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (m < 1 || m > kPartitionMaxPivots) return cudaErrorInvalidValue;
  const size_t chunks = ceil_div(n, (size_t)kPartTile);
  if (chunks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  const int nb = 2 * m + 1;
  unsigned long long* cnt = scratch;                   // [nb][chunks]
  unsigned long long* total = scratch + nb * chunks;  // [nb]
  cudaError_t e = cudaSuccess;
  auto count = [&](auto mc) {
    constexpr int M = decltype(mc)::value;
    partition_count_kernel<M><<<(unsigned)chunks, kPartBlock, 0, stream>>>(in, n, pivots, cnt);
  };
  auto write = [&](auto mc) {
    constexpr int M = decltype(mc)::value;
    partition_write_kernel<M><<<(unsigned)chunks, kPartBlock, 0, stream>>>(in, out, n, pivots, cnt, total);
  };
  auto by_m = [&](auto&& f) {
    switch (m) {
      case 1: f(std::integral_constant<int, 1>{}); break;
      case 2: f(std::integral_constant<int, 2>{}); break;
      case 3: f(std::integral_constant<int, 3>{}); break;
      case 4: f(std::integral_constant<int, 4>{}); break;
      case 5: f(std::integral_constant<int, 5>{}); break;
      case 6: f(std::integral_constant<int, 6>{}); break;
      default: f(std::integral_constant<int, 7>{}); break;
    }
  };
  by_m(count);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  partition_scan_kernel<<<nb, kPartScanBlock, 0, stream>>>(cnt, chunks, total);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  by_m(write);
  return cudaGetLastError();
}

}  // namespace pa
