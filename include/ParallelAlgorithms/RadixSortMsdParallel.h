// Drop-in replacement for the reference's RadixSortMsdParallel.h entry point:
// in-place sort of unsigned keys that, like the reference, needs no second
// array of a_size keys: pa_sort_u32_inplace partitions in place by digit
// through a bounded device scratch (2^24 keys) and sorts the buckets in
// groups.  The reference's MSD sort is unstable; for keys alone any sort
// gives the same array.
#ifndef PA_DROPIN_RADIXSORTMSDPARALLEL_H
#define PA_DROPIN_RADIXSORTMSDPARALLEL_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// RadixSortMsdParallel.h:291
inline void parallel_hybrid_inplace_msd_radix_sort(unsigned* a, size_t a_size) {
  if (a_size < 2) return;
  pa_detail::check(pa_sort_u32_inplace(a, a_size, 0, nullptr), "parallel_hybrid_inplace_msd_radix_sort");
}

}  // namespace ParallelAlgorithms

#endif
