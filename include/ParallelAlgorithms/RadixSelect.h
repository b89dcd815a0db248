// Drop-in replacement for the reference's RadixSelect.h entry points (global
// namespace, like the reference).  Returns the exact k-th smallest element
// and, like the reference, leaves it at a[k].  The reference also rearranges
// the rest of the range as it narrows; the GPU path leaves it unchanged.
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
