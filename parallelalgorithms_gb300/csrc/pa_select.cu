// Radix select: exact k-th smallest key (0-based).
//
// GPU form of RadixSelectiontNonRecursiveInner (RadixSelect.h:83-129).  The
// reference narrows MSD digit by digit: count the digit over the current
// range (HistogramOneComponentOpt), find the bin holding k, move that bin's
// keys together (MoveOutsideOfKthBinIn, :36-55), recurse into the bin.
// Here nothing is moved: each step re-counts the next digit over the keys
// whose already-decided high digits equal the prefix found so far, and the
// last CTA of the step (ticket) picks the bin holding k and extends the
// prefix.  After the first step, when the keys sharing the prefix fit the
// candidate buffer, the step also compacts them, and later steps read only
// that buffer.  All state lives on the device, so the host enqueues
// key_bits / 8 launches and never waits between them.
#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {

struct SelectState {
  unsigned long long hist[256];
  unsigned long long prefix;       // decided high digits, right-aligned
  unsigned long long k;            // rank sought among keys sharing prefix
  unsigned long long count;        // keys sharing prefix
  unsigned long long cand_n;       // keys in the candidate buffer
  unsigned long long cand_fill;    // compaction cursor of the current step
  uint32_t prefix_bits;
  uint32_t src;                    // 0: the input array, 1: candidate buffer
  uint32_t ticket;
  uint32_t pad;
};

namespace {

constexpr int kSelBlock = 512;

template <typename K>
__device__ __forceinline__ bool matches(K key, unsigned long long prefix, uint32_t prefix_bits) {
  constexpr uint32_t W = 8u * sizeof(K);
  if (prefix_bits == 0) return true;
  return (unsigned long long)(key >> (W - prefix_bits)) == prefix;
}

template <typename K>
__global__ void __launch_bounds__(kSelBlock) select_step_kernel(const K* __restrict__ keys, size_t n,
                                                                K* __restrict__ cand, size_t cand_cap,
                                                                SelectState* st, uint32_t shift, K* out) {
  constexpr uint32_t W = 8u * sizeof(K);
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  __shared__ uint32_t s_hist[256];
  __shared__ bool s_last;
  for (int i = threadIdx.x; i < 256; i += kSelBlock) s_hist[i] = 0;

  const unsigned long long prefix = st->prefix;
  const uint32_t prefix_bits = st->prefix_bits;
  const uint32_t src = st->src;
  const bool compact = src == 0 && prefix_bits > 0 && st->count <= (unsigned long long)cand_cap;
  const K* __restrict__ in = src ? cand : keys;
  const size_t len = src ? (size_t)st->cand_n : n;
  // Compaction happens at most once (only while reading the input array),
  // so it never overlaps its own source.
  K* __restrict__ dst = cand;
  __syncthreads();

  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt = lanemask_lt();
  const size_t warps_total = (size_t)gridDim.x * (kSelBlock / 32);
  const size_t gwarp = (size_t)blockIdx.x * (kSelBlock / 32) + (threadIdx.x >> 5);
  for (size_t w = gwarp; w * 32 < len; w += warps_total) {
    const size_t i = w * 32 + lane;
    K key = 0;
    bool m = false;
    if (i < len) {
      key = in[i];
      m = matches(key, prefix, prefix_bits);
    }
    if (m) atomicAdd(&s_hist[(uint32_t)(key >> shift) & 255u], 1u);
    if (compact) {
      const uint32_t ballot = __ballot_sync(FULL, m);
      if (ballot) {
        const uint32_t leader = __ffs(ballot) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&st->cand_fill, (unsigned long long)__popc(ballot));
        base = __shfl_sync(FULL, base, leader);
        if (m) dst[base + __popc(ballot & lt)] = key;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += kSelBlock)
    if (s_hist[i]) atomicAdd(&st->hist[i], (unsigned long long)s_hist[i]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    unsigned long long k = st->k, cum = 0;
    uint32_t bin = 255;
    for (uint32_t b = 0; b < 256; ++b) {
      const unsigned long long c = ld_relaxed_gpu(&st->hist[b]);
      if (k < cum + c) {
        bin = b;
        break;
      }
      cum += c;
    }
    const unsigned long long c = ld_relaxed_gpu(&st->hist[bin]);
    st->prefix = (prefix << 8) | bin;
    st->prefix_bits = prefix_bits + 8;
    st->k = k - cum;
    st->count = c;
    if (compact) {
      st->src = 1;
      st->cand_n = ld_relaxed_gpu(&st->cand_fill);
    }
    st->cand_fill = 0;
    st->ticket = 0;
    if (prefix_bits + 8 == W) *out = (K)((prefix << 8) | bin);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += kSelBlock) st->hist[i] = 0;
}

template <typename K>
cudaError_t launch_select_t(const K* keys, size_t n, K* cand, size_t cand_cap, SelectState* st, K* out,
                            cudaStream_t stream) {
  constexpr uint32_t W = 8u * sizeof(K);
  const unsigned grid = (unsigned)max(1, device_info().sm_count * 4);
  for (uint32_t s = 0; s < W / 8; ++s) {
    const uint32_t shift = W - 8u * (s + 1);
    select_step_kernel<K><<<grid, kSelBlock, 0, stream>>>(keys, n, cand, cand_cap, st, shift, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

__global__ void select_init_kernel(SelectState* st, unsigned long long k, unsigned long long n) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) st->hist[i] = 0;
  if (threadIdx.x == 0) {
    st->prefix = 0;
    st->k = k;
    st->count = n;
    st->cand_n = 0;
    st->cand_fill = 0;
    st->prefix_bits = 0;
    st->src = 0;
    st->ticket = 0;
  }
}

}  // namespace

size_t select_state_bytes() { return sizeof(SelectState); }

cudaError_t launch_select(const void* keys, size_t n, size_t k, int key_bytes, void* cand, size_t cand_cap,
                          void* work, void* out, uint32_t* err, cudaStream_t stream) {
  (void)err;
  SelectState* st = static_cast<SelectState*>(work);
  select_init_kernel<<<1, 256, 0, stream>>>(st, k, n);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (key_bytes == 4)
    return launch_select_t<uint32_t>(static_cast<const uint32_t*>(keys), n, static_cast<uint32_t*>(cand), cand_cap, st,
                                     static_cast<uint32_t*>(out), stream);
  if (key_bytes == 8)
    return launch_select_t<unsigned long long>(static_cast<const unsigned long long*>(keys), n,
                                               static_cast<unsigned long long*>(cand), cand_cap, st,
                                               static_cast<unsigned long long*>(out), stream);
  return cudaErrorInvalidValue;
}

}  // namespace pa
