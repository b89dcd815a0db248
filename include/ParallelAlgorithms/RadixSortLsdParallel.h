// Drop-in replacement for the reference's RadixSortLsdParallel.h: the same
// entry points with the same signatures and in-place semantics, running on
// the GPU through the C ABI in pa_gpu.h (link with libpa_gb300.so).
//
// The reference's threshold parameters (parallelThreshold,
// ParallelWorkQuantum) size CPU work quanta; they are accepted and ignored.
// Unlike the reference, failures are reported: std::bad_alloc when device
// memory runs out, std::runtime_error for a CUDA failure.
#ifndef PA_DROPIN_RADIXSORTLSDPARALLEL_H
#define PA_DROPIN_RADIXSORTLSDPARALLEL_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// RadixSortLsdParallel.h:367 -- result in a; tmp_work_buff is scratch.
inline void SortRadixPar(unsigned* a, unsigned* tmp_work_buff, size_t a_size, size_t parallelThreshold = 512 * 1024) {
  (void)parallelThreshold;
  pa_detail::check(pa_sort_u32(a, tmp_work_buff, a_size, nullptr), "SortRadixPar");
}

// RadixSortLsdParallel.h:340 -- allocates its own scratch.
inline void SortRadixPar(unsigned* a, size_t a_size, size_t parallelThreshold = 64 * 1024) {
  (void)parallelThreshold;
  pa_detail::check(pa_sort_u32(a, nullptr, a_size, nullptr), "SortRadixPar");
}

// RadixSortLsdParallel.h:215 -- result in inputArray.
template <unsigned long PowerOfTwoRadix, unsigned long Log2ofPowerOfTwoRadix>
inline void SortRadixInnerPar(unsigned* inputArray, unsigned* workArray, size_t inputSize,
                              size_t ParallelWorkQuantum = 64 * 1024) {
  static_assert(PowerOfTwoRadix == 256 && Log2ofPowerOfTwoRadix == 8, "the GPU path implements 8-bit digits");
  (void)ParallelWorkQuantum;
  pa_detail::check(pa_sort_u32(inputArray, workArray, inputSize, nullptr), "SortRadixInnerPar");
}

// RadixSortLsdParallel.h:86 -- afterwards a and b both hold the sorted keys.
inline void RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(unsigned* a, unsigned* b, unsigned long a_size) {
  pa_detail::check(pa_sort_two_phase_u32(a, b, a_size, nullptr), "RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase");
}

// RadixSortLsdParallel.h:491.  The reference's body is commented out for
// a_size >= 100 (:503); this gives the intended result, as above.
inline void RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize(unsigned* a, unsigned* b, size_t a_size) {
  pa_detail::check(pa_sort_two_phase_u32(a, b, a_size, nullptr),
                   "RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize");
}

// Additive overloads (no reference counterpart): 64-bit keys, float keys by
// IEEE total order, and keys with a stable uint32 payload.
inline void SortRadixPar(unsigned long long* a, unsigned long long* tmp_work_buff, size_t a_size) {
  pa_detail::check(pa_sort_u64(reinterpret_cast<uint64_t*>(a), reinterpret_cast<uint64_t*>(tmp_work_buff), a_size,
                               nullptr),
                   "SortRadixPar(u64)");
}
inline void SortRadixPar(float* a, float* tmp_work_buff, size_t a_size) {
  pa_detail::check(pa_sort_f32(a, tmp_work_buff, a_size, nullptr), "SortRadixPar(float)");
}
inline void SortRadixParKV(unsigned* keys, unsigned* payload, size_t a_size) {
  pa_detail::check(pa_sort_kv_u32(keys, payload, nullptr, nullptr, a_size, nullptr), "SortRadixParKV");
}
inline void SortRadixParKV(unsigned long long* keys, unsigned* payload, size_t a_size) {
  pa_detail::check(pa_sort_kv_u64(reinterpret_cast<uint64_t*>(keys), payload, nullptr, nullptr, a_size, nullptr),
                   "SortRadixParKV(u64)");
}
inline void SortRadixParKV(float* keys, unsigned* payload, size_t a_size) {
  pa_detail::check(pa_sort_kv_f32(keys, payload, nullptr, nullptr, a_size, nullptr), "SortRadixParKV(float)");
}

}  // namespace ParallelAlgorithms

#endif  // PA_DROPIN_RADIXSORTLSDPARALLEL_H
