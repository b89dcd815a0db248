// Drop-in replacement for the reference's ParallelMergeSort.h entry points
// that use LSD radix sort as their leaf: the whole range is sorted by the
// GPU radix sort (stable; the same result as the reference's merge of
// radix-sorted blocks).  Indices follow the reference: r is INCLUSIVE.
// Threshold and memory-fraction arguments are accepted and have no effect.
#ifndef PA_DROPIN_PARALLELMERGESORT_H
#define PA_DROPIN_PARALLELMERGESORT_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// ParallelMergeSort.h:287 -- result in dst[l, r] when srcToDst (src holds
// scratch afterwards), else in src[l, r] (dst is the scratch).
inline void parallel_merge_sort_hybrid_radix(unsigned* src, size_t l, size_t r, unsigned* dst, bool srcToDst = true,
                                             size_t parallelThreshold = 24 * 1024) {
  (void)parallelThreshold;
  if (r < l) return;
  const size_t n = r - l + 1;
  if (srcToDst)
    pa_detail::check(pa_sort_copy_u32(src + l, dst + l, n, nullptr), "parallel_merge_sort_hybrid_radix");
  else
    pa_detail::check(pa_sort_u32(src + l, dst ? dst + l : nullptr, n, nullptr), "parallel_merge_sort_hybrid_radix");
}

// ParallelMergeSort.h:298
inline void parallel_merge_sort_hybrid_radix_single_buffer(unsigned* src, size_t l, size_t r, unsigned* dst,
                                                           bool srcToDst = true, size_t parallelThreshold = 24 * 1024) {
  parallel_merge_sort_hybrid_radix(src, l, r, dst, srcToDst, parallelThreshold);
}

// ParallelMergeSort.h:549: sorts src in place.
inline void parallel_linear_in_place_preventative_adaptive_sort(unsigned* src, size_t src_size, bool stable = true,
                                                                double physical_memory_threshold_post = 0.75,
                                                                size_t parallelThreshold = 24 * 1024) {
  (void)stable;
  (void)physical_memory_threshold_post;
  (void)parallelThreshold;
  pa_detail::check(pa_sort_u32(src, nullptr, src_size, nullptr), "parallel_linear_in_place_preventative_adaptive_sort");
}

}  // namespace ParallelAlgorithms

#endif
