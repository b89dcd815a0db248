// Drop-in replacement for the reference's CountingSortParallel.h byte-array
// counting sort: the bytes a[l, r) (r exclusive) sorted in place by a
// one-read histogram and a parallel fill on the GPU.  The thresholds are
// accepted and have no effect.
#ifndef PA_DROPIN_COUNTINGSORTPARALLEL_H
#define PA_DROPIN_COUNTINGSORTPARALLEL_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// CountingSortParallel.h:29
template <unsigned long NumberOfBins>
inline void counting_sort_parallel_inner(unsigned char* array_to_sort, size_t l, size_t r,
                                         size_t threshold_count = 64 * 1024, size_t threshold_fill = 64 * 1024) {
  static_assert(NumberOfBins == 256, "byte values have 256 bins");
  (void)threshold_count;
  (void)threshold_fill;
  if (r <= l) return;
  pa_detail::check(pa_counting_sort_u8(reinterpret_cast<uint8_t*>(array_to_sort) + l, r - l, nullptr),
                   "counting_sort_parallel_inner");
}

// CountingSortParallel.h:81
inline void counting_sort_parallel(unsigned char* a, size_t a_size) {
  counting_sort_parallel_inner<256>(a, 0, a_size);
}

}  // namespace ParallelAlgorithms

#endif
