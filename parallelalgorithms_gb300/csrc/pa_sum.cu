// Exact 64-bit sum: GPU form of SumParallelNonRecursive / SumParallel
// (SumParallel.h:162-307).  The reference cuts the array into 16K-element
// tasks and adds the per-task sums serially; here the array streams through
// shared memory by bulk copies (pa_bulkstream.cuh), each consumer thread
// accumulates 16-byte vectors into a 64-bit register, warps and CTAs reduce
// with shuffles,
// each CTA writes one partial, and the last CTA to finish (ticket) adds the
// partials in CTA order.  Integer addition modulo 2^64 is associative, so
// the result equals the reference's bit for bit whatever the split.
#include "pa_bulkstream.cuh"
#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

// The aligned body of the array streams through shared memory by bulk copies
// (four 32 KB stages per CTA, one CTA per SM); the unaligned head and tail
// (fewer than two vectors) are read directly.
constexpr int kStages = 4;
constexpr int kChunk = 32 * 1024;
constexpr int kConsumers = 512;
using Ring = BulkRing<kStages, kChunk, kConsumers>;
constexpr int kMaxSumBlocks = 152 * 8;

template <typename K>
__global__ void __launch_bounds__(Ring::kThreads, 1) sum_kernel(const K* __restrict__ keys, size_t n,
                                                               unsigned long long* __restrict__ partials,
                                                               uint32_t* ticket, unsigned long long* __restrict__ out,
                                                               uint32_t* err) {
  extern __shared__ __align__(128) unsigned char ring[];
  constexpr int V = 16 / (int)sizeof(K);
  const uintptr_t addr = reinterpret_cast<uintptr_t>(keys);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > n) head = n;
  const size_t nvec = (n - head) / V;
  const size_t tail_start = head + nvec * V;

  unsigned long long acc = 0;
  bulk_stream<kStages, kChunk, kConsumers>(keys + head, nvec * 16, ring, err, [&](const uint4* st, uint32_t nv) {
    for (uint32_t v = threadIdx.x; v < nv; v += kConsumers) {
      const uint4 a = st[v];
      if (sizeof(K) == 4)
        acc += (unsigned long long)a.x + a.y + (unsigned long long)a.z + a.w;
      else
        acc += ((unsigned long long)a.y << 32 | a.x) + ((unsigned long long)a.w << 32 | a.z);
    }
  });
  if (blockIdx.x == 0) {
    const size_t rest = head + (n - tail_start);
    for (size_t r = threadIdx.x; r < rest; r += Ring::kThreads)
      acc += (unsigned long long)keys[r < head ? r : tail_start + (r - head)];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  __shared__ unsigned long long s_w[Ring::kThreads / 32];
  __shared__ bool s_last;
  if ((threadIdx.x & 31u) == 0) s_w[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < Ring::kThreads / 32; ++w) t += s_w[w];
    partials[blockIdx.x] = t;
    __threadfence();
    s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x < 32) {
    __threadfence();
    unsigned long long t = 0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += 32) t += ld_relaxed_gpu(&partials[b]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    if (threadIdx.x == 0) {
      *out = t;
      *ticket = 0;  // leave the ticket ready for the next call on this workspace
    }
  }
}

template <typename K>
cudaError_t launch_sum_t(const K* keys, size_t n, unsigned long long* partials, uint32_t* ticket,
                         unsigned long long* out, uint32_t* err, cudaStream_t stream) {
  cudaError_t e = ensure_dynamic_smem(sum_kernel<K>, Ring::kBytes);
  if (e != cudaSuccess) return e;
  const size_t chunks = ceil_div(n * sizeof(K), (size_t)kChunk);
  size_t blocks = min((size_t)device_info().sm_count, (size_t)kMaxSumBlocks);
  if (blocks > chunks) blocks = chunks;
  if (blocks < 1) blocks = 1;
  sum_kernel<K><<<(unsigned)blocks, Ring::kThreads, Ring::kBytes, stream>>>(keys, n, partials, ticket, out, err);
  return cudaGetLastError();
}

}  // namespace

size_t sum_partials_needed() { return kMaxSumBlocks; }

cudaError_t launch_sum(const void* keys, size_t n, int key_bytes, unsigned long long* partials, uint32_t* ticket,
                       unsigned long long* out, uint32_t* err, cudaStream_t stream) {
  if (key_bytes == 4)
    return launch_sum_t(static_cast<const uint32_t*>(keys), n, partials, ticket, out, err, stream);
  if (key_bytes == 8)
    return launch_sum_t(static_cast<const unsigned long long*>(keys), n, partials, ticket, out, err, stream);
  return cudaErrorInvalidValue;
}

}  // namespace pa
