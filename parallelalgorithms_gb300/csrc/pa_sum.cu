// Exact 64-bit sum: GPU form of SumParallelNonRecursive / SumParallel
// (SumParallel.h:162-307).  The reference cuts the array into 16K-element
// tasks and adds the per-task sums serially; here each thread accumulates
// 16-byte vectors into a 64-bit register, warps and CTAs reduce with shuffles,
// each CTA writes one partial, and the last CTA to finish (ticket) adds the
// partials in CTA order.  Integer addition modulo 2^64 is associative, so
// the result equals the reference's bit for bit whatever the split.
#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {
namespace {

constexpr int kSumBlock = 512;
constexpr int kMaxSumBlocks = 152 * 8;

template <typename K>
__global__ void __launch_bounds__(kSumBlock) sum_kernel(const K* __restrict__ keys, size_t n,
                                                        unsigned long long* __restrict__ partials, uint32_t* ticket,
                                                        unsigned long long* __restrict__ out) {
  constexpr int V = 16 / (int)sizeof(K);
  const uintptr_t addr = reinterpret_cast<uintptr_t>(keys);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > n) head = n;
  const size_t nvec = (n - head) / V;
  const size_t tail_start = head + nvec * V;
  const uint4* vec = reinterpret_cast<const uint4*>(keys + head);

  unsigned long long acc = 0;
  const size_t stride = (size_t)gridDim.x * kSumBlock;
  size_t i = (size_t)blockIdx.x * kSumBlock + threadIdx.x;
  // two independent 16-byte loads in flight per iteration
  for (; i + stride < nvec; i += 2 * stride) {
    const uint4 a = ld_stream_v4(vec + i);
    const uint4 b = ld_stream_v4(vec + i + stride);
    if (sizeof(K) == 4) {
      acc += (unsigned long long)a.x + a.y + (unsigned long long)a.z + a.w;
      acc += (unsigned long long)b.x + b.y + (unsigned long long)b.z + b.w;
    } else {
      acc += ((unsigned long long)a.y << 32 | a.x) + ((unsigned long long)a.w << 32 | a.z);
      acc += ((unsigned long long)b.y << 32 | b.x) + ((unsigned long long)b.w << 32 | b.z);
    }
  }
  for (; i < nvec; i += stride) {
    const uint4 a = ld_stream_v4(vec + i);
    if (sizeof(K) == 4)
      acc += (unsigned long long)a.x + a.y + (unsigned long long)a.z + a.w;
    else
      acc += ((unsigned long long)a.y << 32 | a.x) + ((unsigned long long)a.w << 32 | a.z);
  }
  if (blockIdx.x == 0) {
    const size_t rest = head + (n - tail_start);
    for (size_t r = threadIdx.x; r < rest; r += kSumBlock)
      acc += (unsigned long long)keys[r < head ? r : tail_start + (r - head)];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  __shared__ unsigned long long s_w[kSumBlock / 32];
  __shared__ bool s_last;
  if ((threadIdx.x & 31u) == 0) s_w[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kSumBlock / 32; ++w) t += s_w[w];
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

}  // namespace

size_t sum_partials_needed() { return kMaxSumBlocks; }

cudaError_t launch_sum(const void* keys, size_t n, int key_bytes, unsigned long long* partials, uint32_t* ticket,
                       unsigned long long* out, cudaStream_t stream) {
  const size_t per_vec = 16 / (size_t)key_bytes;
  size_t blocks = ceil_div(ceil_div(n, per_vec), (size_t)kSumBlock * 4);
  const size_t cap = (size_t)min(device_info().sm_count * 4, kMaxSumBlocks);
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (key_bytes == 4)
    sum_kernel<uint32_t><<<(unsigned)blocks, kSumBlock, 0, stream>>>(static_cast<const uint32_t*>(keys), n, partials,
                                                                    ticket, out);
  else if (key_bytes == 8)
    sum_kernel<unsigned long long><<<(unsigned)blocks, kSumBlock, 0, stream>>>(
        static_cast<const unsigned long long*>(keys), n, partials, ticket, out);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace pa
