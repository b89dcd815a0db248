// Radix select: exact k-th smallest key (0-based).
//
// GPU form of RadixSelectiontNonRecursiveInner (RadixSelect.h:83-129).  The
// reference narrows MSD digit by digit: count the digit over the current
// range (HistogramOneComponentOpt), find the bin holding k, move that bin's
// keys together (MoveOutsideOfKthBinIn, :36-55), recurse into the bin.  The
// result is the same order statistic; here the input is read once in the
// usual case and never moved:
//   sample   eight CTAs take kSample keys at even strides and the last of
//            them finds, by the same MSD digit narrowing in shared memory,
//            the sample's keys
//            `lo` and `hi` a few standard deviations below and above rank k
//            (the extreme ranks give the key type's minimum / maximum);
//   range    one streaming read of the input counts the keys below lo and
//            equal to lo and to hi and copies the keys strictly between
//            them (the candidates) to a buffer, branch-free per key; the
//            last CTA (ticket) then either has the answer (lo or hi), or
//            continues with rank k among the candidates and picks their top
//            digit (counted as each warp flushed its candidates), or (rank
//            k outside the bracket, or the
//            candidates overflowed: an unrepresentative sample) restarts the
//            plain digit-by-digit narrowing over the whole input;
//   step s   the digit below the decided prefix is counted over the keys of
//            the current source (input or a candidate buffer) that share
//            the prefix (lane-banked shared counters), and the last CTA
//            picks the bin.  A step whose digit is already decided (or
//            whose answer is already written) returns at once.
// A step may copy the keys sharing the prefix into the other candidate
// buffer (input -> A, A -> B, B -> A) when they fit it, and later steps read
// only that buffer; once a step has copied few keys, its last CTA finishes
// the remaining digits in shared memory.  All state lives on the device, so the host
// enqueues key_bits / 8 + 3 launches and never waits between them.
#include <cmath>

#include "pa_common.cuh"
#include "pa_kernels.cuh"

namespace pa {

constexpr int kSelectSample = 8192;  // keys in the bracketing sample

struct SelectState {
  unsigned long long sample[kSelectSample];  // the sample, gathered by several CTAs
  unsigned long long hist[256];
  unsigned long long prefix;        // decided high digits, right-aligned
  unsigned long long k;             // rank sought among the current source's keys sharing prefix
  unsigned long long count;         // keys sharing prefix
  unsigned long long cand_n[2];     // keys in candidate buffer A / B
  unsigned long long cand_fill;     // compaction cursor of the current step
  unsigned long long lo, hi;        // the sample's bracket around rank k
  unsigned long long below, eq_lo, eq_hi;  // range pass: keys < lo, == lo, == hi (hi != lo)
  uint32_t prefix_bits;
  uint32_t src;                     // 0: the input array, 1: buffer A, 2: buffer B
  uint32_t ticket;
  uint32_t done;                    // the result is written
  uint32_t overflow;                // the range pass's candidates did not fit buffer A
};

namespace {

// A streaming kernel runs one CTA of 1024 threads per SM; each thread keeps
// kUnroll 16-byte loads in flight per grid-strided round.
constexpr int kSelBlock = 1024;
constexpr int kSelWarps = kSelBlock / 32;
constexpr int kUnroll = 4;
constexpr int kSelLanes = 16;  // lane copies of each shared counter
// Candidates are staged per warp in shared memory (a segment holding one
// round of the warp, so that one visit always fits after a flush) and leave
// with one global reservation per segment.
constexpr int kSegBytes = 32 * kUnroll * 16;
template <typename K>
constexpr uint32_t kSegKeys = (uint32_t)(kSegBytes / sizeof(K));
constexpr size_t kStreamSmem = (size_t)kSelWarps * kSegBytes;
// Sample size and bracket width: the sample's rank of the k-th key has
// standard deviation sqrt(S p (1 - p)) (p = k / n); the bracket spans five
// of them on each side, so about 5.5 % of a uniform input lies inside it
// for the median and the sample misses rank k with probability ~1e-6.
constexpr int kSampleLog2 = 13;
constexpr int kSample = 1 << kSampleLog2;
static_assert(kSample == kSelectSample, "the state block holds the sample");
constexpr int kSampleThreads = 1024;
constexpr double kBracketSigmas = 5.0;

template <typename K>
__device__ __forceinline__ bool matches(K key, unsigned long long prefix, uint32_t prefix_bits) {
  constexpr uint32_t W = 8u * sizeof(K);
  if (prefix_bits == 0) return true;
  return (unsigned long long)(key >> (W - prefix_bits)) == prefix;
}

// Picks the bin of h (256 complete counts of the next digit over the keys
// sharing the prefix) holding rank st->k and narrows the state to it (called
// by every thread of one CTA of at least 256 threads).  `compacted_to`: the
// candidate buffer (1: A, 2: B) this step filled, which becomes the source;
// 0: none.
template <typename K>
__device__ void pick_bin(SelectState* st, const unsigned long long* h, uint32_t compacted_to, K* out) {
  constexpr uint32_t W = 8u * sizeof(K);
  __shared__ unsigned long long s_tot[8];
  const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
  // Every thread reads the state it tests before the barrier below, and the
  // one thread whose bin holds rank k writes it only after that barrier: a
  // thread reading st->k after the update would see the narrowed rank and
  // could wrongly match a lower bin as well.
  const unsigned long long k = st->k, prefix0 = st->prefix;
  const uint32_t bits0 = st->prefix_bits;
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
    if (c != 0 && excl <= k && k < excl + c) {  // exactly one bin holds rank k
      const unsigned long long prefix = (prefix0 << 8) | t;
      st->prefix = prefix;
      st->prefix_bits = bits0 + 8;
      st->k = k - excl;
      st->count = c;
      if (compacted_to) {
        st->cand_n[compacted_to - 1] = ld_relaxed_gpu(&st->cand_fill);  // filled by every CTA's atomics
        st->src = compacted_to;
      }
      st->cand_fill = 0;
      if (bits0 + 8 == W) {
        *out = (K)prefix;
        st->done = 1;
      }
    }
  }
  __syncthreads();
  if (t < 256) st->hist[t] = 0;
  if (t == 0) st->ticket = 0;
}

// The bracket: kSample keys at even strides, and their order statistics at
// the ranks kBracketSigmas standard deviations either side of rank k's
// image, both found at once by MSD digit narrowing over the sample in
// shared memory.  kSample / kSampleThreads CTAs gather the sample (strided
// loads over the whole input go faster from several SMs) into the state
// block; the last of them (ticket) reads it back from L2 and narrows.
template <typename K>
__global__ void __launch_bounds__(kSampleThreads) select_sample_kernel(const K* keys, size_t n, SelectState* st) {
  constexpr uint32_t W = 8u * sizeof(K);
  extern __shared__ __align__(16) unsigned char sample_raw[];
  K* s = reinterpret_cast<K*>(sample_raw);
  __shared__ uint32_t s_h[2][256];
  __shared__ unsigned long long s_pref[2], s_rank[2];
  __shared__ bool s_lo_min, s_hi_max, s_last;
  const uint32_t tid = threadIdx.x;
  const uint32_t ns = (uint32_t)(n < (size_t)kSample ? n : (size_t)kSample);
  // key j of the sample sits at (j n + n / 2) / ns: a shift when ns is the
  // full sample (a power of two), j itself when the input is smaller
  {
    const uint32_t j = blockIdx.x * kSampleThreads + tid;
    if (j < ns)
      st->sample[j] = (unsigned long long)keys[ns == (uint32_t)kSample ? ((size_t)j * n + n / 2) >> kSampleLog2
                                                                        : (size_t)j];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
#pragma unroll
  for (int q = 0; q < kSample / kSampleThreads; ++q) {  // (L2 reads: other SMs wrote them)
    const uint32_t j = tid + (uint32_t)q * kSampleThreads;
    if (j < ns) s[j] = (K)__ldcg(&st->sample[j]);
  }
  if (tid == 0) {
    st->ticket = 0;
    const double p = ((double)st->k + 0.5) / (double)n;
    long long r = (long long)(p * (double)ns);
    if (r > (long long)ns - 1) r = (long long)ns - 1;
    const long long m = (long long)(kBracketSigmas * sqrt((double)ns * p * (1.0 - p))) + 2;
    const long long r_lo = r > m ? r - m : 0;
    const long long r_hi = r + m < (long long)ns - 1 ? r + m : (long long)ns - 1;
    s_rank[0] = (unsigned long long)r_lo;
    s_rank[1] = (unsigned long long)r_hi;
    s_lo_min = r_lo == 0;  // no sample key below the bracket: open it down to the minimum
    s_hi_max = r_hi == (long long)ns - 1;
    s_pref[0] = s_pref[1] = 0;
  }
  uint32_t pbits = 0;
  for (int d = (int)W / 8 - 1; d >= 0; --d) {
    const uint32_t shift = 8u * (uint32_t)d;
    for (uint32_t i = tid; i < 512u; i += kSampleThreads) (&s_h[0][0])[i] = 0;
    __syncthreads();
    const unsigned long long p0 = s_pref[0], p1 = s_pref[1];
    for (uint32_t j = tid; j < ns; j += kSampleThreads) {
      const K key = s[j];
      const uint32_t dig = (uint32_t)(key >> shift) & 255u;
      if (matches(key, p0, pbits)) atomicAdd(&s_h[0][dig], 1u);
      if (matches(key, p1, pbits)) atomicAdd(&s_h[1][dig], 1u);
    }
    __syncthreads();
    if (tid < 64) {  // warp t narrows target t; lane l owns bins [8l, 8l + 8)
      const uint32_t t = tid >> 5, lane = tid & 31u;
      uint32_t c[8], sum = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        c[i] = s_h[t][8 * lane + i];
        sum += c[i];
      }
      uint32_t incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
      }
      const unsigned long long rk = s_rank[t];
      const unsigned long long pref = s_pref[t];
      __syncwarp();  // every lane has read the target before one lane narrows it
      uint32_t acc = incl - sum;
      if ((unsigned long long)acc <= rk && rk < (unsigned long long)incl) {
        for (int i = 0; i < 8; ++i) {
          if (rk < (unsigned long long)(acc + c[i])) {
            s_pref[t] = (pref << 8) | (8u * lane + (uint32_t)i);
            s_rank[t] = rk - acc;
            break;
          }
          acc += c[i];
        }
      }
    }
    pbits += 8;
    __syncthreads();
  }
  if (tid == 0) {
    st->lo = s_lo_min ? 0ull : s_pref[0];
    st->hi = s_hi_max ? (unsigned long long)(K)~(K)0 : s_pref[1];
  }
}

// A consumer warp's candidate segment in shared memory: `fill` keys (the
// same value in every lane).  seg_flush writes them to dst with one global
// reservation (one past the capacity only raises st->overflow), and with
// `top` set also counts each written key's top digit into the lane-banked
// shared counters at `top` (a warp-uniform loop: counting here costs far
// less than a per-key branch while streaming);
// seg_append adds this thread's matched keys (kk[e] where bit e of mm is
// set), flushing first when they would not fit.  Both are warp-collective.
template <typename K>
__device__ __forceinline__ void seg_flush(K* seg, uint32_t& fill, K* dst, size_t cap, SelectState* st,
                                          uint32_t* top = nullptr) {
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  constexpr uint32_t W = 8u * sizeof(K);
  if (fill == 0) return;
  const uint32_t lane = threadIdx.x & 31u;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(&st->cand_fill, (unsigned long long)fill);
  base = __shfl_sync(FULL, base, 0);
  __syncwarp();  // every lane's segment writes are visible
  if (base + fill <= cap) {
    for (uint32_t i = lane; i < fill; i += 32) {
      const K key = seg[i];
      dst[base + i] = key;
      if (top) atomicAdd(top + (((uint32_t)(key >> (W - 8)) & 255u) * kSelLanes), 1u);
    }
  } else if (lane == 0) {
    st->overflow = 1;
  }
  __syncwarp();  // the segment is read out before it is refilled
  fill = 0;
}

template <typename K>
__device__ __forceinline__ void seg_append(const K* kk, uint32_t mm, int nk, K* seg, uint32_t& fill, K* dst,
                                           size_t cap, SelectState* st, uint32_t* top = nullptr) {
  constexpr uint32_t FULL = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t cnt = __popc(mm);
  if (__ballot_sync(FULL, cnt != 0) == 0) return;
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(FULL, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  const uint32_t total = __shfl_sync(FULL, incl, 31);
  if (fill + total > kSegKeys<K>) seg_flush<K>(seg, fill, dst, cap, st, top);
  uint32_t at = fill + incl - cnt;
  for (int e = 0; e < nk; ++e)
    if ((mm >> e) & 1u) seg[at++] = kk[e];
  fill += total;
}

// Streams src[0, len) with 16-byte loads straight into registers, kUnroll
// of them in flight per thread (vectors i, i + stride, ... of a grid-strided
// round); visit(keys, valid, nk) is called by every thread once per round,
// the same number of times on every lane, with bit e of `valid` set when key
// e is present (a compile-time all-ones mask in the full rounds, so that the
// masking costs nothing there), and once more per 32 keys by the first
// CTA's first warp for the unaligned head and tail (one key per lane).
// Called by all threads; ends with a barrier.
template <typename K, typename F>
__device__ __forceinline__ void stream_keys(const K* in, size_t len, F&& visit) {
  constexpr int V = 16 / (int)sizeof(K);
  const uintptr_t addr = reinterpret_cast<uintptr_t>(in);
  size_t head = ((16u - (addr & 15u)) & 15u) / sizeof(K);
  if (head > len) head = len;
  const size_t nvec = (len - head) / V;
  const size_t tail_start = head + nvec * V;
  const uint4* vec = reinterpret_cast<const uint4*>(in + head);
  const size_t stride = (size_t)gridDim.x * kSelBlock;
  const size_t per_round = (size_t)kUnroll * stride;
  const size_t full = nvec / per_round;  // rounds with every vector present
  size_t i = (size_t)blockIdx.x * kSelBlock + threadIdx.x;
  auto round = [&](bool masked) {
    uint4 q[kUnroll];
    uint32_t valid = 0xFFFFFFFFu;
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const size_t j = i + (size_t)u * stride;
      if (masked && j >= nvec) {
        q[u] = make_uint4(0, 0, 0, 0);
        valid &= ~(((1u << V) - 1u) << (u * V));
      } else {
        q[u] = ld_stream_v4(vec + j);
      }
    }
    K kk[kUnroll * V];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const K* e = reinterpret_cast<const K*>(&q[u]);
#pragma unroll
      for (int j = 0; j < V; ++j) kk[u * V + j] = e[j];
    }
    if (masked)
      visit(kk, valid, kUnroll * V);
    else
      visit(kk, 0xFFFFFFFFu, kUnroll * V);
  };
  for (size_t r = 0; r < full; ++r, i += per_round) round(false);
  if (full * per_round < nvec) round(true);  // the last, partial round (the same on every thread)
  if (blockIdx.x == 0 && threadIdx.x < 32) {  // head and tail: fewer than 2 * V keys, one warp
    const size_t rest = head + (len - tail_start);
    for (size_t r0 = 0; r0 < rest; r0 += 32) {
      const size_t r = r0 + threadIdx.x;
      K key = 0;
      const bool ok = r < rest;
      if (ok) key = in[r < head ? r : tail_start + (r - head)];
      visit(&key, ok ? 1u : 0u, 1);
    }
  }
  __syncthreads();
}

// Folds the lane copies of the shared counters into st->hist (staggered so
// a warp's reads hit distinct banks); CTAs that counted nothing skip it.
// Called by all threads.
__device__ __forceinline__ void fold_counts(const uint32_t* s_h, SelectState* st, bool counted) {
  if (!__syncthreads_or(counted ? 1 : 0)) return;
  for (uint32_t b = threadIdx.x; b < 256u; b += kSelBlock) {
    uint32_t sum = 0;
    for (uint32_t j = 0; j < (uint32_t)kSelLanes; ++j) sum += s_h[b * kSelLanes + ((j + b) % kSelLanes)];
    if (sum) atomicAdd(&st->hist[b], (unsigned long long)sum);
  }
}

// One read of the input against the bracket [lo, hi]; the last CTA decides
// how the select continues.
template <typename K>
__global__ void __launch_bounds__(kSelBlock, 1) select_range_kernel(const K* keys, size_t n, K* cand_a, size_t cap_a,
                                                                    SelectState* st, K* out) {
  extern __shared__ __align__(128) unsigned char seg_smem[];
  __shared__ uint32_t s_h[256 * kSelLanes];  // the candidates' top digit, lane-banked
  __shared__ uint32_t s_cnt[3];
  __shared__ bool s_last;
  __shared__ int s_mode;
  for (uint32_t i = threadIdx.x; i < 256u * kSelLanes; i += kSelBlock) s_h[i] = 0;
  if (threadIdx.x == 0) s_cnt[0] = s_cnt[1] = s_cnt[2] = 0;
  const K lo = (K)st->lo, hi = (K)st->hi;
  // strictly inside (lo, hi)  <=>  key - (lo + 1) < hi - lo - 1 (unsigned);
  // nothing is inside when hi == lo
  const K lo1 = (K)(lo + 1), w = hi > lo ? (K)(hi - lo - 1) : (K)0;
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5;
  K* seg = reinterpret_cast<K*>(seg_smem) + (size_t)warp * kSegKeys<K>;
  uint32_t fill = 0;
  uint32_t* my_top = s_h + (threadIdx.x % kSelLanes);
  uint32_t below = 0, eq_lo = 0, eq_hi = 0;
  // branch-free per key: three counts and a match bit (per-key branches
  // or shared atomics here would cost more than the read itself; the
  // candidates' top digit is counted as each warp flushes its segment)
  stream_keys<K>(keys, n, [&](const K* kk, uint32_t valid, int nk) {
    uint32_t mm = 0;
#pragma unroll
    for (int e = 0; e < nk; ++e) {
      const K key = kk[e];
      const bool v = (valid >> e) & 1u;
      below += (v && key < lo) ? 1u : 0u;
      eq_lo += (v && key == lo) ? 1u : 0u;
      eq_hi += (v && key == hi) ? 1u : 0u;  // (discarded below when hi == lo)
      mm |= (v && (K)(key - lo1) < w) ? (1u << e) : 0u;
    }
    seg_append<K>(kk, mm, nk, seg, fill, cand_a, cap_a, st, my_top);
  });
  seg_flush<K>(seg, fill, cand_a, cap_a, st, my_top);
  if (below) atomicAdd(&s_cnt[0], below);
  if (eq_lo) atomicAdd(&s_cnt[1], eq_lo);
  if (eq_hi) atomicAdd(&s_cnt[2], eq_hi);
  fold_counts(s_h, st, true);  // (its barrier also orders the count atomics above)
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_cnt[0]) atomicAdd(&st->below, (unsigned long long)s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&st->eq_lo, (unsigned long long)s_cnt[1]);
    if (s_cnt[2]) atomicAdd(&st->eq_hi, (unsigned long long)s_cnt[2]);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (threadIdx.x == 0) {
    const unsigned long long k = st->k, b = ld_relaxed_gpu(&st->below), el = ld_relaxed_gpu(&st->eq_lo),
                             eh = hi != lo ? ld_relaxed_gpu(&st->eq_hi) : 0ull,
                             inside = ld_relaxed_gpu(&st->cand_fill);
    const bool overflow = *(volatile uint32_t*)&st->overflow != 0;
    int mode = 0;  // 0: restart over the input, 1: answer written, 2: continue in the candidates
    if (k >= b && k < b + el) {
      *out = lo;
      mode = 1;
    } else if (k >= b + el && k < b + el + inside) {
      mode = overflow ? 0 : 2;
    } else if (k >= b + el + inside && k < b + el + inside + eh) {
      *out = hi;
      mode = 1;
    }
    if (mode == 1) st->done = 1;
    if (mode == 2) {  // continue in the candidates: their top digit is picked below
      st->k = k - b - el;
      st->count = inside;
      st->cand_n[0] = inside;
      st->src = 1;
    }
    if (mode == 0) {  // an unrepresentative sample: the plain narrowing over the input
      st->count = n;
      st->src = 0;
      st->overflow = 0;
    }
    st->cand_fill = 0;
    s_mode = mode;
  }
  __syncthreads();
  if (s_mode == 2) {
    pick_bin<K>(st, st->hist, 0u, out);  // (resets the ticket and the counts)
  } else {
    if (threadIdx.x < 256) st->hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) st->ticket = 0;
  }
}

// When the keys this step compacted are few (at most kFinishKeys), the
// step's last CTA finishes the select itself: it loads the ones sharing the
// new prefix from the buffer just written (other CTAs wrote it: L2 reads)
// into shared memory and narrows their remaining digits there, so the later
// step launches return at once.  Called by every thread of the last CTA
// after pick_bin.
template <typename K>
constexpr uint32_t kFinishKeys = (uint32_t)(kStreamSmem / sizeof(K));
template <typename K>
__device__ void finish_in_cta(SelectState* st, const K* buf, K* s_keys, K* out) {
  constexpr uint32_t W = 8u * sizeof(K);
  __shared__ uint32_t s_fc[256];
  __shared__ uint32_t s_n;
  __shared__ unsigned long long s_pref, s_rank;
  __shared__ bool s_go;
  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
    const uint32_t src = st->src;
    s_go = !st->done && src != 0 && st->cand_n[src - 1] <= (unsigned long long)kFinishKeys<K>;
    s_n = 0;
    s_pref = st->prefix;
    s_rank = st->k;
  }
  __syncthreads();
  if (!s_go) return;
  uint32_t pbits = st->prefix_bits;
  const unsigned long long prefix = s_pref;
  const uint32_t len = (uint32_t)st->cand_n[st->src - 1];
  for (uint32_t i = tid; i < len; i += kSelBlock) {
    const K key = __ldcg(&buf[i]);
    if (matches(key, prefix, pbits)) s_keys[atomicAdd(&s_n, 1u)] = key;
  }
  __syncthreads();
  const uint32_t m = s_n;
  for (; pbits < W; pbits += 8) {
    const uint32_t shift = W - 8u - pbits;
    for (uint32_t i = tid; i < 256u; i += kSelBlock) s_fc[i] = 0;
    __syncthreads();
    const unsigned long long p = s_pref;
    for (uint32_t j = tid; j < m; j += kSelBlock)
      if (matches(s_keys[j], p, pbits)) atomicAdd(&s_fc[(uint32_t)(s_keys[j] >> shift) & 255u], 1u);
    __syncthreads();
    if (tid < 32) {  // lane l owns bins [8l, 8l + 8)
      const uint32_t lane = tid;
      uint32_t c[8], sum = 0;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        c[i] = s_fc[8 * lane + i];
        sum += c[i];
      }
      uint32_t incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
      }
      const unsigned long long rk = s_rank, pref = s_pref;
      __syncwarp();  // every lane has read the target before one lane narrows it
      uint32_t acc = incl - sum;
      if ((unsigned long long)acc <= rk && rk < (unsigned long long)incl) {
        for (int i = 0; i < 8; ++i) {
          if (rk < (unsigned long long)(acc + c[i])) {
            s_pref = (pref << 8) | (8u * lane + (uint32_t)i);
            s_rank = rk - acc;
            break;
          }
          acc += c[i];
        }
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    *out = (K)s_pref;
    st->prefix = s_pref;
    st->prefix_bits = W;
    st->done = 1;
  }
}

// One narrowing step on digit `shift`: counts the digit over the current
// source's keys sharing the prefix, optionally copies them to the next
// candidate buffer; the last CTA picks.  Returns at once unless this digit
// is the next undecided one.
template <typename K>
__global__ void __launch_bounds__(kSelBlock, 1) select_step_kernel(const K* keys, size_t n, K* cand_a, size_t cap_a,
                                                                   K* cand_b, size_t cap_b, SelectState* st,
                                                                   uint32_t shift, K* out) {
  extern __shared__ __align__(128) unsigned char seg_smem[];
  constexpr uint32_t W = 8u * sizeof(K);
  // The state read here changes only in the last CTA, after every CTA has
  // taken its ticket (or in an earlier launch).
  if (st->done || st->prefix_bits != W - 8u - shift) return;
  __shared__ uint32_t s_h[256 * kSelLanes];
  __shared__ bool s_last;
  for (uint32_t i = threadIdx.x; i < 256u * kSelLanes; i += kSelBlock) s_h[i] = 0;
  const unsigned long long prefix = st->prefix;
  const uint32_t prefix_bits = st->prefix_bits;
  const uint32_t src = st->src;
  const K* in = src == 0 ? keys : src == 1 ? cand_a : cand_b;
  const size_t len = src == 0 ? n : (size_t)st->cand_n[src - 1];
  // compaction goes to the other candidate buffer (the input to A, A to B,
  // B to A), so it never overlaps its own source
  const uint32_t to = src == 1 ? 2u : 1u;
  K* dst = to == 1 ? cand_a : cand_b;
  const size_t cap = to == 1 ? cap_a : cap_b;
  const bool compact = st->count <= (unsigned long long)cap;
  __syncthreads();
  const uint32_t warp = threadIdx.x >> 5;
  K* seg = reinterpret_cast<K*>(seg_smem) + (size_t)warp * kSegKeys<K>;
  uint32_t fill = 0;
  uint32_t* my = s_h + (threadIdx.x % kSelLanes);
  bool counted = false;
  stream_keys<K>(in, len, [&](const K* kk, uint32_t valid, int nk) {
    uint32_t mm = 0;
    for (int e = 0; e < nk; ++e) {
      if (((valid >> e) & 1u) && matches(kk[e], prefix, prefix_bits)) {
        atomicAdd(my + (((uint32_t)(kk[e] >> shift) & 255u) * kSelLanes), 1u);
        counted = true;
        mm |= 1u << e;
      }
    }
    if (compact) seg_append<K>(kk, mm, nk, seg, fill, dst, cap, st);
  });
  if (compact) seg_flush<K>(seg, fill, dst, cap, st);
  fold_counts(s_h, st, counted);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  pick_bin<K>(st, st->hist, compact ? to : 0u, out);
  if (compact) finish_in_cta<K>(st, dst, reinterpret_cast<K*>(seg_smem), out);
}

template <typename K>
cudaError_t launch_select_t(const K* keys, size_t n, K* cand, size_t cand_cap, SelectState* st, K* out,
                            uint32_t* err, cudaStream_t stream) {
  constexpr uint32_t W = 8u * sizeof(K);
  (void)err;  // no kernel of the select waits on another CTA's progress
  // buffer A takes the range pass's candidates (or the first compaction of
  // the input), buffer B the compaction after the next digit; A's length is
  // a whole number of 16-byte vectors so that B stays aligned
  size_t cap_b = cand_cap / 8;
  size_t cap_a = (cand_cap - cap_b) & ~(size_t)(16 / sizeof(K) - 1);
  cap_b = cand_cap - cap_a;
  K* cand_a = cand;
  K* cand_b = cand + cap_a;
  const size_t sample_smem = (size_t)kSample * sizeof(K);
  cudaError_t e = ensure_dynamic_smem(select_sample_kernel<K>, sample_smem);
  if (e != cudaSuccess) return e;
  select_sample_kernel<K><<<kSample / kSampleThreads, kSampleThreads, sample_smem, stream>>>(keys, n, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)max(1, device_info().sm_count);  // one CTA per SM
  e = ensure_dynamic_smem(select_range_kernel<K>, kStreamSmem);
  if (e != cudaSuccess) return e;
  select_range_kernel<K><<<grid, kSelBlock, kStreamSmem, stream>>>(keys, n, cand_a, cap_a, st, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = ensure_dynamic_smem(select_step_kernel<K>, kStreamSmem);
  if (e != cudaSuccess) return e;
  for (uint32_t s = 0; s < W / 8; ++s) {
    const uint32_t shift = W - 8u * (s + 1);
    select_step_kernel<K><<<grid, kSelBlock, kStreamSmem, stream>>>(keys, n, cand_a, cap_a, cand_b, cap_b, st,
                                                                        shift, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

__global__ void select_init_kernel(SelectState* st, unsigned long long k) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) st->hist[i] = 0;
  if (threadIdx.x == 0) {
    st->prefix = 0;
    st->k = k;
    st->count = 0;
    st->cand_n[0] = st->cand_n[1] = 0;
    st->cand_fill = 0;
    st->lo = st->hi = 0;
    st->below = st->eq_lo = st->eq_hi = 0;
    st->prefix_bits = 0;
    st->src = 0;
    st->ticket = 0;
    st->done = 0;
    st->overflow = 0;
  }
}

// Index of a key equal to *value in keys[0, n), into *idx (set to all ones
// by the launcher first): k itself when keys[k] already holds it, else the smallest
// such index.  CTAs walk 16 K-key chunks in chunk order; a chunk that starts
// past an index already found is skipped, so the walk stops early.
constexpr int kFindBlock = 256;
constexpr size_t kFindChunk = (size_t)kFindBlock * 64;

__global__ void __launch_bounds__(kFindBlock) find_key_kernel(const uint32_t* __restrict__ keys, size_t n, size_t k,
                                                              const uint32_t* __restrict__ value,
                                                              unsigned long long* idx) {
  const uint32_t v = *value;
  if (keys[k] == v) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicMin(idx, (unsigned long long)k);
    return;
  }
  __shared__ unsigned long long s_best;
  for (size_t c = blockIdx.x; c * kFindChunk < n; c += gridDim.x) {
    const size_t lo = c * kFindChunk;
    if (threadIdx.x == 0) s_best = ld_relaxed_gpu(idx);
    __syncthreads();
    const bool past = lo > s_best;
    __syncthreads();
    if (past) return;  // every later chunk starts later still
    const size_t hi = min(n, lo + kFindChunk);
    for (size_t i = lo + threadIdx.x; i < hi; i += kFindBlock)
      if (keys[i] == v) atomicMin(idx, (unsigned long long)i);
  }
}

// keys[k] <-> keys[*idx] (one thread); nothing when *idx is k or not found.
__global__ void swap_key_kernel(uint32_t* keys, size_t n, size_t k, const unsigned long long* idx) {
  const unsigned long long j = *idx;
  if (j >= n || j == k) return;
  const uint32_t t = keys[k];
  keys[k] = keys[j];
  keys[j] = t;
}

}  // namespace

size_t select_state_bytes() { return sizeof(SelectState); }

cudaError_t launch_find_key(const uint32_t* keys, size_t n, size_t k, const uint32_t* value, unsigned long long* idx,
                            cudaStream_t stream) {
  if (n == 0 || k >= n) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(idx, 0xFF, sizeof(*idx), stream);  // "not found yet"
  if (e != cudaSuccess) return e;
  const size_t chunks = ceil_div(n, kFindChunk);
  const unsigned grid = (unsigned)min(chunks, (size_t)device_info().sm_count * 8);
  find_key_kernel<<<grid, kFindBlock, 0, stream>>>(keys, n, k, value, idx);
  return cudaGetLastError();
}

cudaError_t launch_swap_key(uint32_t* keys, size_t n, size_t k, const unsigned long long* idx, cudaStream_t stream) {
  swap_key_kernel<<<1, 1, 0, stream>>>(keys, n, k, idx);
  return cudaGetLastError();
}

cudaError_t launch_select(const void* keys, size_t n, size_t k, int key_bytes, void* cand, size_t cand_cap,
                          void* work, void* out, uint32_t* err, cudaStream_t stream) {
  SelectState* st = static_cast<SelectState*>(work);
  select_init_kernel<<<1, 256, 0, stream>>>(st, k);
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
