// Radix select: exact k-th smallest key (0-based).
//
// GPU form of RadixSelectiontNonRecursiveInner (RadixSelect.h:83-129).  The
// reference narrows MSD digit by digit: count the digit over the current
// range (HistogramOneComponentOpt), find the bin holding k, move that bin's
// keys together (MoveOutsideOfKthBinIn, :36-55), recurse into the bin.
// Here nothing is moved in the input:
//   step 0   every digit's counts over all keys come from one read by the
//            one-read histogram kernel (digit_counts_kernel); a one-CTA pick
//            finds the top digit's bin holding k;
//   step s   while every key still shares the prefix found so far (one bin
//            held them all), digit s's counts over all keys are the ones
//            needed and no key is read; otherwise every key whose decided
//            high digits equal the prefix is counted on digit s (lane-banked
//            shared counters, 16-byte loads) and the last CTA of the step
//            (ticket) picks the bin.
// The first filtering step also copies the keys sharing the prefix into a
// candidate buffer when they fit it, and later steps read only that buffer.
// All state lives on the device, so the host enqueues key_bits / 8 + 2
// launches and never waits between them.
#include "pa_bulkstream.cuh"
#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {

struct SelectState {
  unsigned long long hist_all[8][256];  // counts of every digit over all keys (step 0)
  unsigned long long hist[256];
  unsigned long long prefix;       // decided high digits, right-aligned
  unsigned long long k;            // rank sought among keys sharing prefix
  unsigned long long count;        // keys sharing prefix
  unsigned long long cand_n;       // keys in the candidate buffer
  unsigned long long cand_fill;    // compaction cursor of the current step
  uint32_t prefix_bits;
  uint32_t src;                    // 0: the input array, 1: candidate buffer
  uint32_t ticket;
  uint32_t all_digits;             // hist_all holds every digit (else only the top one)
};

namespace {

// A filtering step streams its source through shared memory by bulk copies
// (three 16 KB stages per CTA, two CTAs per SM, 512 consumer threads each
// taking two vectors of every chunk).
constexpr int kStages = 3;
constexpr int kChunk = 16 * 1024;
constexpr int kConsumers = 512;
constexpr int kPerThread = kChunk / 16 / kConsumers;
static_assert(kPerThread * kConsumers * 16 == kChunk, "a chunk splits evenly over the consumers");
using Ring = BulkRing<kStages, kChunk, kConsumers>;
constexpr int kSelBlock = Ring::kThreads;
constexpr int kSelLanes = 32;  // lane copies of each shared counter
// Candidates a CTA gathers in shared memory before one global reservation
// (12 KB, so that counters and buffer stay under 48 KB of static shared
// memory).
template <typename K>
constexpr int kCandBuf = 12 * 1024 / (int)sizeof(K);

template <typename K>
__device__ __forceinline__ bool matches(K key, unsigned long long prefix, uint32_t prefix_bits) {
  constexpr uint32_t W = 8u * sizeof(K);
  if (prefix_bits == 0) return true;
  return (unsigned long long)(key >> (W - prefix_bits)) == prefix;
}

// Picks the bin of h (256 complete counts of the next digit over the keys
// sharing the prefix) holding rank st->k and narrows the state to it (called
// by every thread of one CTA of at least 256 threads).  `compacted`: this
// step filled the candidate buffer.
template <typename K>
__device__ void pick_bin(SelectState* st, const unsigned long long* h, bool compacted, K* out) {
  constexpr uint32_t W = 8u * sizeof(K);
  __shared__ unsigned long long s_tot[8];
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  const unsigned long long c = t < 256 ? ld_relaxed_gpu(&h[t]) : 0ull;
  unsigned long long incl = c;  // inclusive scan of the 256 counts
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  if (t < 256 && lane == 31) s_tot[warp] = incl;
  __syncthreads();
  if (t < 256) {
    unsigned long long before = 0;
    for (uint32_t w = 0; w < warp; ++w) before += s_tot[w];
    const unsigned long long excl = before + incl - c;
    const unsigned long long k = st->k;
    if (c != 0 && excl <= k && k < excl + c) {  // exactly one bin holds rank k
      const unsigned long long prefix = (st->prefix << 8) | t;
      st->prefix = prefix;
      st->prefix_bits += 8;
      st->k = k - excl;
      st->count = c;
      if (compacted) {
        st->src = 1;
        st->cand_n = ld_relaxed_gpu(&st->cand_fill);  // filled by every CTA's atomics
      }
      st->cand_fill = 0;
      if (st->prefix_bits == W) *out = (K)prefix;
    }
  }
  __syncthreads();
  if (t < 256) st->hist[t] = 0;
  if (t == 0) st->ticket = 0;
}

template <typename K>
__global__ void __launch_bounds__(256) select_pick_kernel(SelectState* st, K* out) {
  constexpr uint32_t W = 8u * sizeof(K);
  pick_bin<K>(st, st->hist_all[W / 8 - 1], false, out);
}

// One filtering step: counts digit `shift` of the keys sharing the prefix,
// optionally copies them to the candidate buffer; the last CTA picks.
template <typename K>
__global__ void __launch_bounds__(kSelBlock, 2) select_step_kernel(const K* keys, size_t n, K* cand, size_t cand_cap,
                                                                   SelectState* st, uint32_t shift, K* out,
                                                                   uint32_t* err) {
  extern __shared__ __align__(128) unsigned char ring[];
  constexpr int V = 16 / (int)sizeof(K);
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  constexpr uint32_t CB = (uint32_t)kCandBuf<K>;
  __shared__ uint32_t s_h[256 * kSelLanes];
  __shared__ K s_cand[CB];
  __shared__ uint32_t s_cn, s_valid;
  __shared__ unsigned long long s_base;
  __shared__ bool s_last;
  for (uint32_t i = threadIdx.x; i < 256u * kSelLanes; i += kSelBlock) s_h[i] = 0;
  if (threadIdx.x == 0) {
    s_cn = 0;
    s_valid = CB;
  }

  // The state read here changes only in the last CTA, after every CTA has
  // taken its ticket.  When every key shares the prefix, digit `shift`'s
  // counts over all keys (step 0) are the ones needed and nothing is read.
  const bool all_share = st->all_digits && st->count == (unsigned long long)n;
  const unsigned long long prefix = st->prefix;
  const uint32_t prefix_bits = st->prefix_bits;
  const uint32_t src = st->src;
  // Compaction happens at most once (only while reading the input array),
  // so it never overlaps its own source.
  const bool compact = !all_share && src == 0 && st->count <= (unsigned long long)cand_cap;
  const K* in = src ? cand : keys;
  const size_t len = all_share ? 0 : src ? (size_t)st->cand_n : n;
  __syncthreads();

  const uint32_t lane = threadIdx.x & 31u;
  uint32_t* my = s_h + lane;
  auto count_key = [&](K key) { atomicAdd(my + (((uint32_t)(key >> shift) & 255u) * kSelLanes), 1u); };
  // Warp-aggregated append of this thread's matched keys (kk where mm):
  // into the CTA's shared buffer while it has room, else straight to the
  // candidate buffer.  Shared reservations only grow, so the first one that
  // does not fit marks the end of the valid shared entries (s_valid).
  auto append = [&](const K* kk, const bool* mm, int nk) {
    uint32_t cnt = 0;
    for (int e = 0; e < nk; ++e) cnt += mm[e] ? 1u : 0u;
    if (__ballot_sync(FULL, cnt != 0) == 0) return;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(FULL, incl, o);
      if (lane >= (uint32_t)o) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    uint32_t pos = 0;
    if (lane == 31) {
      pos = atomicAdd(&s_cn, total);
      if (pos + total > CB) atomicMin(&s_valid, pos);
    }
    pos = __shfl_sync(FULL, pos, 31);
    if (pos + total <= CB) {
      uint32_t at = pos + (incl - cnt);
      for (int e = 0; e < nk; ++e)
        if (mm[e]) s_cand[at++] = kk[e];
      return;
    }
    unsigned long long base = 0;
    if (lane == 31) base = atomicAdd(&st->cand_fill, (unsigned long long)total);
    base = __shfl_sync(FULL, base, 31) + (incl - cnt);
    for (int e = 0; e < nk; ++e)
      if (mm[e]) cand[base++] = kk[e];
  };

  // Split [0, len) into an unaligned head, whole 16-byte vectors and a tail;
  // the vectors stream through the bulk-copy ring.
  const uintptr_t addr = reinterpret_cast<uintptr_t>(in);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > len) head = len;
  const size_t nvec = (len - head) / V;
  const size_t tail_start = head + nvec * V;
  bulk_stream<kStages, kChunk, kConsumers>(in + head, nvec * 16, ring, err, [&](const uint4* stq, uint32_t nv) {
    // a full chunk is one round of kPerThread vectors per thread; a short last
    // chunk masks the missing ones (same trip count on every lane)
    K kk[kPerThread * V];
    bool mm[kPerThread * V];
#pragma unroll
    for (int u = 0; u < kPerThread; ++u) {
      const uint32_t v = (uint32_t)u * kConsumers + threadIdx.x;
      const bool in_range = v < nv;
      const uint4 q = in_range ? stq[v] : make_uint4(0, 0, 0, 0);
      const K* e = reinterpret_cast<const K*>(&q);
#pragma unroll
      for (int j = 0; j < V; ++j) {
        kk[u * V + j] = e[j];
        mm[u * V + j] = in_range && matches(e[j], prefix, prefix_bits);
        if (mm[u * V + j]) count_key(e[j]);
      }
    }
    if (compact) append(kk, mm, kPerThread * V);
  });
  if (blockIdx.x == 0 && threadIdx.x < 32) {  // head and tail: fewer than 2 * V keys, one warp
    const size_t rest = head + (len - tail_start);
    for (size_t r0 = 0; r0 < rest; r0 += 32) {
      const size_t r = r0 + threadIdx.x;
      K key = 0;
      bool m = false;
      if (r < rest) {
        key = in[r < head ? r : tail_start + (r - head)];
        m = matches(key, prefix, prefix_bits);
        if (m) count_key(key);
      }
      if (compact) append(&key, &m, 1);
    }
  }
  __syncthreads();
  if (compact) {  // the CTA's shared candidates go out with one reservation
    const uint32_t nv = min(s_cn, s_valid);
    if (threadIdx.x == 0) s_base = nv ? atomicAdd(&st->cand_fill, (unsigned long long)nv) : 0ull;
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < nv; j += kSelBlock) cand[s_base + j] = s_cand[j];
  }
  // fold the lane copies (staggered so a warp's reads hit distinct banks)
  for (uint32_t b = threadIdx.x; b < 256u; b += kSelBlock) {
    uint32_t sum = 0;
    for (uint32_t j = 0; j < (uint32_t)kSelLanes; ++j) sum += s_h[b * kSelLanes + ((j + b) % kSelLanes)];
    if (sum) atomicAdd(&st->hist[b], (unsigned long long)sum);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  pick_bin<K>(st, all_share ? st->hist_all[shift / 8] : st->hist, compact, out);
}

template <typename K>
cudaError_t launch_select_t(const K* keys, size_t n, K* cand, size_t cand_cap, SelectState* st, K* out,
                            uint32_t* err, cudaStream_t stream) {
  constexpr uint32_t W = 8u * sizeof(K);
  // step 0: the one-read histogram kernel counts every digit of 32-bit keys
  // (the lower digits serve steps whose prefix all keys share, such as a
  // constant input); for 64-bit keys eight digits cost more than the reads
  // they save, so it counts only the top digit
  cudaError_t e = sizeof(K) == 4
                      ? launch_digit_counts(keys, n, 4, 4, 8, 0, 8, false, &st->hist_all[0][0], stream)
                      : launch_digit_counts(keys, n, 8, 1, 8, W - 8, 0, false, &st->hist_all[W / 8 - 1][0], stream);
  if (e != cudaSuccess) return e;
  select_pick_kernel<K><<<1, 256, 0, stream>>>(st, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = ensure_dynamic_smem(select_step_kernel<K>, Ring::kBytes);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)max(1, device_info().sm_count * 2);  // two CTAs per SM
  for (uint32_t s = 1; s < W / 8; ++s) {
    const uint32_t shift = W - 8u * (s + 1);
    select_step_kernel<K><<<grid, kSelBlock, Ring::kBytes, stream>>>(keys, n, cand, cand_cap, st, shift, out, err);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

__global__ void select_init_kernel(SelectState* st, unsigned long long k, unsigned long long n, uint32_t all_digits) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) st->hist[i] = 0;
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&st->hist_all[0][0])[i] = 0;
  if (threadIdx.x == 0) {
    st->prefix = 0;
    st->k = k;
    st->count = n;
    st->cand_n = 0;
    st->cand_fill = 0;
    st->prefix_bits = 0;
    st->src = 0;
    st->ticket = 0;
    st->all_digits = all_digits;
  }
}

}  // namespace

size_t select_state_bytes() { return sizeof(SelectState); }

cudaError_t launch_select(const void* keys, size_t n, size_t k, int key_bytes, void* cand, size_t cand_cap,
                          void* work, void* out, uint32_t* err, cudaStream_t stream) {
  SelectState* st = static_cast<SelectState*>(work);
  select_init_kernel<<<1, 256, 0, stream>>>(st, k, n, key_bytes == 4 ? 1u : 0u);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (key_bytes == 4)
    return launch_select_t<uint32_t>(static_cast<const uint32_t*>(keys), n, static_cast<uint32_t*>(cand), cand_cap, st,
                                     static_cast<uint32_t*>(out), err, stream);
  if (key_bytes == 8)
    return launch_select_t<unsigned long long>(static_cast<const unsigned long long*>(keys), n,
                                               static_cast<unsigned long long*>(cand), cand_cap, st,
                                               static_cast<unsigned long long*>(out), err, stream);
  return cudaErrorInvalidValue;
}

}  // namespace pa
