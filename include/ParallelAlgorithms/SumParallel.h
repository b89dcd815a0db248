// Drop-in replacement for the reference's SumParallel.h entry points on the
// radix path: exact sums in a 64-bit accumulator, [l, r) with r exclusive.
// The reference underflows on an empty range (SumParallel.h:263-268); here
// an empty range sums to 0.
#ifndef PA_DROPIN_SUMPARALLEL_H
#define PA_DROPIN_SUMPARALLEL_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// SumParallel.h:261
inline unsigned long long SumParallelNonRecursive(unsigned in_array[], size_t l, size_t r,
                                                  size_t parallelThreshold = 16 * 1024) {
  (void)parallelThreshold;
  uint64_t s = 0;
  pa_detail::check(pa_sum_u32(in_array + l, r > l ? r - l : 0, &s, nullptr), "SumParallelNonRecursive");
  return s;
}

// SumParallel.h:285
inline unsigned long long SumParallelNonRecursive(unsigned long long in_array[], size_t l, size_t r,
                                                  size_t parallelThreshold = 16 * 1024) {
  (void)parallelThreshold;
  uint64_t s = 0;
  pa_detail::check(pa_sum_u64(reinterpret_cast<const uint64_t*>(in_array) + l, r > l ? r - l : 0, &s, nullptr),
                   "SumParallelNonRecursive");
  return s;
}

// SumParallel.h:162
inline unsigned long long SumParallel(unsigned long long in_array[], size_t l, size_t r,
                                      size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}

// SumParallel.h:207 -- SumParallel<unsigned>(...) -> long long: the same
// 64-bit sum read as signed.
inline long long SumParallel(unsigned in_array[], size_t l, size_t r, size_t parallelThreshold = 16 * 1024) {
  return (long long)SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}

}  // namespace ParallelAlgorithms

#endif  // PA_DROPIN_SUMPARALLEL_H
