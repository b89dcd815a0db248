// Drop-in replacement for the reference's RadixSelect.h entry points (global
// namespace, like the reference).  Returns the exact k-th smallest element
// and, like the reference, leaves it at a[k]: the GPU path swaps a[k] with the
// first element of the range that holds the answer, so the range stays a
// permutation of its input.  The reference rearranges the range further as
// it narrows (its in-place partitioning); nothing else of the range is moved
// here.
#ifndef PA_DROPIN_RADIXSELECT_H
#define PA_DROPIN_RADIXSELECT_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

// RadixSelect.h:139 -- k is an absolute index in [start, start + length).
inline unsigned SelectRadix(unsigned arrayToBeSelected[], size_t start, size_t length, size_t k) {
  uint32_t v = 0;
  ParallelAlgorithms::pa_detail::check(pa_select_radix_u32(arrayToBeSelected, start, length, k, &v, nullptr),
                                       "SelectRadix");
  return v;
}

// RadixSelect.h:157
inline unsigned SelectRadix(unsigned arrayToBeSelected[], size_t length, size_t k) {
  return SelectRadix(arrayToBeSelected, 0, length, k);
}

#endif  // PA_DROPIN_RADIXSELECT_H
