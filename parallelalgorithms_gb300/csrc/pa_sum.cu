// Exact 64-bit sum: GPU form of SumParallelNonRecursive / SumParallel
// (SumParallel.h:162-307).  The reference cuts the array into 16K-element
// tasks and adds the per-task sums serially; here the array streams through
// shared memory by bulk copies (pa_bulkstream.cuh), each consumer thread
// accumulates 16-byte vectors into a 64-bit register, warps and CTAs reduce
// with shuffles,
// each CTA writes one partial, and the last CTA to finish (ticket) adds the
// partials in CTA order.  Integer addition modulo 2^64 is associative, so
// the result equals the reference's bit for bit whatever the split.  Any
// element type of 1, 2, 4 or 8 bytes is summed the same way after widening
// to 64 bits (the reference's template SumParallel<_Type>, :207-237).
#include <type_traits>

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

// Element kinds (pa_gpu.h PA_ELEM_*): each element is widened to 64 bits
// (zero-extended unsigned, sign-extended signed, float and double truncated
// toward zero as the reference's (long long) cast does; out-of-range values,
// undefined behaviour in the reference, saturate here) and summed modulo 2^64.
template <typename T>
__device__ __forceinline__ unsigned long long widen(T x) {
  if constexpr (std::is_floating_point<T>::value || std::is_signed<T>::value)
    return (unsigned long long)(long long)x;
  else
    return (unsigned long long)x;
}

// Sum of the elements of one 16-byte vector.
template <typename T>
__device__ __forceinline__ unsigned long long vec_sum(const uint4& a) {
  if constexpr (std::is_same<T, uint32_t>::value) {
    return (unsigned long long)a.x + a.y + (unsigned long long)a.z + a.w;
  } else if constexpr (std::is_same<T, unsigned long long>::value) {
    return ((unsigned long long)a.y << 32 | a.x) + ((unsigned long long)a.w << 32 | a.z);
  } else if constexpr (std::is_same<T, uint8_t>::value || std::is_same<T, int8_t>::value) {
    // byte sums of each word by sum-of-absolute-differences against zero
    const uint32_t u = __vsadu4(a.x, 0u) + __vsadu4(a.y, 0u) + __vsadu4(a.z, 0u) + __vsadu4(a.w, 0u);
    if constexpr (std::is_same<T, uint8_t>::value) {
      return u;
    } else {  // a signed byte b >= 128 stands for b - 256
      const uint32_t neg = __popc(a.x & 0x80808080u) + __popc(a.y & 0x80808080u) + __popc(a.z & 0x80808080u) +
                           __popc(a.w & 0x80808080u);
      return (unsigned long long)((long long)u - 256ll * (long long)neg);
    }
  } else {
    const T* e = reinterpret_cast<const T*>(&a);
    unsigned long long acc = 0;
#pragma unroll
    for (int i = 0; i < (int)(16 / sizeof(T)); ++i) acc += widen(e[i]);
    return acc;
  }
}

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
    for (uint32_t v = threadIdx.x; v < nv; v += kConsumers) acc += vec_sum<K>(st[v]);
  });
  if (blockIdx.x == 0) {
    const size_t rest = head + (n - tail_start);
    for (size_t r = threadIdx.x; r < rest; r += Ring::kThreads)
      acc += widen(keys[r < head ? r : tail_start + (r - head)]);
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

// Per-chunk sums: chunk c is keys[c * chunk, min(n, (c + 1) * chunk)).  One
// warp per chunk (warps stride over chunks); lanes read the chunk coalesced,
// lane 0 stores its sum and adds it to *total (addition modulo 2^64 is
// associative, so the atomic order does not matter).
template <typename K>
__global__ void __launch_bounds__(256) sum_chunks_kernel(const K* __restrict__ keys, size_t n, size_t chunk,
                                                         size_t nchunks, unsigned long long* __restrict__ sums,
                                                         unsigned long long* total) {
  const size_t warps = (size_t)gridDim.x * (blockDim.x / 32);
  const uint32_t lane = threadIdx.x & 31u;
  for (size_t c = (size_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); c < nchunks; c += warps) {
    const size_t lo = c * chunk, hi = min(n, lo + chunk);
    unsigned long long acc = 0;
    for (size_t i = lo + lane; i < hi; i += 32) acc += widen(keys[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    if (lane == 0) {
      sums[c] = acc;
      atomicAdd(total, acc);
    }
  }
}

template <typename K>
cudaError_t launch_chunks_t(const void* keys, size_t n, size_t chunk, unsigned long long* sums,
                            unsigned long long* total, cudaStream_t stream) {
  const size_t nchunks = ceil_div(n, chunk);
  const size_t grid = min(ceil_div(nchunks, (size_t)8), (size_t)device_info().sm_count * 16);
  sum_chunks_kernel<K><<<(unsigned)(grid < 1 ? 1 : grid), 256, 0, stream>>>(static_cast<const K*>(keys), n, chunk,
                                                                           nchunks, sums, total);
  return cudaGetLastError();
}

}  // namespace

size_t sum_partials_needed() { return kMaxSumBlocks; }

int sum_elem_bytes(int elem_kind) {
  switch (elem_kind) {
    case kElemU8: case kElemI8: return 1;
    case kElemU16: case kElemI16: return 2;
    case kElemU32: case kElemI32: case kElemF32: return 4;
    case kElemU64: case kElemI64: case kElemF64: return 8;
    default: return 0;
  }
}

cudaError_t launch_sum(const void* keys, size_t n, int elem_kind, unsigned long long* partials, uint32_t* ticket,
                       unsigned long long* out, uint32_t* err, cudaStream_t stream) {
  switch (elem_kind) {
    case kElemU8: return launch_sum_t(static_cast<const uint8_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemI8: return launch_sum_t(static_cast<const int8_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemU16: return launch_sum_t(static_cast<const uint16_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemI16: return launch_sum_t(static_cast<const int16_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemU32: return launch_sum_t(static_cast<const uint32_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemI32: return launch_sum_t(static_cast<const int32_t*>(keys), n, partials, ticket, out, err, stream);
    case kElemU64:
      return launch_sum_t(static_cast<const unsigned long long*>(keys), n, partials, ticket, out, err, stream);
    case kElemI64: return launch_sum_t(static_cast<const long long*>(keys), n, partials, ticket, out, err, stream);
    case kElemF32: return launch_sum_t(static_cast<const float*>(keys), n, partials, ticket, out, err, stream);
    case kElemF64: return launch_sum_t(static_cast<const double*>(keys), n, partials, ticket, out, err, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sum_chunks(const void* keys, size_t n, int elem_kind, size_t chunk, unsigned long long* sums,
                              unsigned long long* total, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  if (chunk == 0) return cudaErrorInvalidValue;
  switch (elem_kind) {
    case kElemU8: return launch_chunks_t<uint8_t>(keys, n, chunk, sums, total, stream);
    case kElemI8: return launch_chunks_t<int8_t>(keys, n, chunk, sums, total, stream);
    case kElemU16: return launch_chunks_t<uint16_t>(keys, n, chunk, sums, total, stream);
    case kElemI16: return launch_chunks_t<int16_t>(keys, n, chunk, sums, total, stream);
    case kElemU32: return launch_chunks_t<uint32_t>(keys, n, chunk, sums, total, stream);
    case kElemI32: return launch_chunks_t<int32_t>(keys, n, chunk, sums, total, stream);
    case kElemU64: return launch_chunks_t<unsigned long long>(keys, n, chunk, sums, total, stream);
    case kElemI64: return launch_chunks_t<long long>(keys, n, chunk, sums, total, stream);
    case kElemF32: return launch_chunks_t<float>(keys, n, chunk, sums, total, stream);
    case kElemF64: return launch_chunks_t<double>(keys, n, chunk, sums, total, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pa
