// Device-side building blocks shared by every kernel of the radix hot path:
// key traits (digit extraction, float32 order transform), inline-PTX wrappers
// for mbarrier + bulk (TMA) copies, relaxed/acquire global accesses for the
// decoupled look-back, and the device error word.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

namespace pa {

// ---------------------------------------------------------------------------
// Device error word.  Every spin-wait in these kernels is bounded; when a
// bound is hit the kernel ORs one of these bits into the call's error word,
// publishes whatever it must so that no other CTA waits on it forever, and
// returns.  The host reads the word after the call and reports
// PA_ERR_TIMEOUT.
// ---------------------------------------------------------------------------
enum : uint32_t {
  DEVERR_LOOKBACK_TIMEOUT = 1u << 0,
  DEVERR_TMA_TIMEOUT = 1u << 1,
  DEVERR_BAD_STATE = 1u << 2,
};

// Polls allowed before a look-back or barrier wait gives up.  Each poll is an
// L2 round trip (hundreds of ns) or a suspended try_wait, so the bound is
// well above a second; in a healthy run a wait lasts microseconds.
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit) {
  if (err) atomicOr(err, bit);
}

// ---------------------------------------------------------------------------
// Keys.  Digits are taken from the "ordered" form of a key: the key itself
// for unsigned integers, and for float32 the bit pattern with the sign-flip
// transform applied, so that unsigned order equals IEEE total order
// (-inf < ... < -0.0 < +0.0 < ... < +inf).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t f32_to_ordered(uint32_t b) {
  return b ^ ((b >> 31) ? 0xFFFFFFFFu : 0x80000000u);
}
__device__ __forceinline__ uint32_t ordered_to_f32(uint32_t o) {
  return o ^ ((o >> 31) ? 0x80000000u : 0xFFFFFFFFu);
}

template <typename K>
__device__ __forceinline__ uint32_t digit_of(K key, uint32_t shift, uint32_t mask) {
  return (uint32_t)(key >> shift) & mask;
}

template <typename K>
__device__ __forceinline__ K to_ordered(K k, bool is_float) {
  if constexpr (sizeof(K) == 4) {
    return is_float ? (K)f32_to_ordered((uint32_t)k) : k;
  } else {
    return k;
  }
}
template <typename K>
__device__ __forceinline__ K from_ordered(K k, bool is_float) {
  if constexpr (sizeof(K) == 4) {
    return is_float ? (K)ordered_to_f32((uint32_t)k) : k;
  } else {
    return k;
  }
}

// ---------------------------------------------------------------------------
// Lane helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------------------
// Global accesses for inter-CTA status words (decoupled look-back).  The
// flag and the count share one word, so relaxed atomicity at GPU scope is
// all the protocol needs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk copy (the TMA engine's non-tensor form: a contiguous run of
// bytes, 16-byte aligned on both sides, size a multiple of 16).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
}

// Makes the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and raises the error
// bit) if the phase did not complete within the poll budget.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t* err) {
  for (uint32_t i = 0; i < kSpinLimit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  raise_error(err, DEVERR_TMA_TIMEOUT);
  return false;
}

// Orders this thread's earlier (generic-proxy) view of global memory before
// its later bulk copies (async proxy): needed when the data a bulk copy reads
// was written by other CTAs of the same launch and published to this thread
// through an acquire.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async;" ::: "memory"); }

// Global -> shared bulk copy completing on `bar` (complete_tx counts bytes).
__device__ __forceinline__ void bulk_load_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Streaming 16-byte load that does not allocate in L1.
__device__ __forceinline__ uint4 ld_stream_v4(const void* p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__host__ __device__ constexpr inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }

// Calls f(std::integral_constant<int, i>{}) for i = 0 .. N-1, unrolled at
// compile time (so that per-item choices can be made with if constexpr).
template <typename F, int... I>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

}  // namespace pa
