// Drop-in replacement for the reference's RadixPartition.h (global
// functions, as in the reference): in-place partition of unsigned keys
// around one or several ascending indices k.  Afterwards each listed a[k] is
// the k-th smallest of the range, nothing before it is larger and nothing
// after it is smaller; the order inside each part differs from the
// reference's swap loop (for a few k the GPU selects each k-th smallest and
// splits the keys into the buckets between them; for many k it sorts the
// range, which partitions it around every k at once).
#ifndef PA_DROPIN_RADIXPARTITION_H
#define PA_DROPIN_RADIXPARTITION_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

// RadixPartition.h:92
inline unsigned PartitionRadix(unsigned arrayToBePartitioned[], size_t aLength, size_t k) {
  const size_t ks[1] = {k};
  ParallelAlgorithms::pa_detail::check(pa_partition_radix_u32(arrayToBePartitioned, aLength, ks, 1, nullptr), "PartitionRadix");
  return arrayToBePartitioned[k];
}

// RadixPartition.h:124 (k absolute, inside [aStart, aStart + aLength))
inline unsigned PartitionRadix(unsigned arrayToBePartitioned[], size_t aStart, size_t aLength, size_t k) {
  const size_t ks[1] = {k - aStart};
  ParallelAlgorithms::pa_detail::check(pa_partition_radix_u32(arrayToBePartitioned + aStart, aLength, ks, 1, nullptr), "PartitionRadix");
  return arrayToBePartitioned[k];
}

// RadixPartition.h:152 (k[0, kLength) ascending)
inline void PartitionRadix(unsigned arrayToBePartitioned[], size_t aLength, size_t k[], size_t kLength) {
  ParallelAlgorithms::pa_detail::check(pa_partition_radix_u32(arrayToBePartitioned, aLength, k, kLength, nullptr), "PartitionRadix");
}

// RadixPartition.h:165 (k[kStart, kStart + kLength) ascending, absolute)
inline void PartitionRadix(unsigned arrayToBePartitioned[], size_t aStart, size_t aLength, size_t k[], size_t kStart,
                           size_t kLength) {
  if (kLength == 0) return;
  size_t* rel = new size_t[kLength];
  for (size_t i = 0; i < kLength; ++i) rel[i] = k[kStart + i] - aStart;
  const int rc = pa_partition_radix_u32(arrayToBePartitioned + aStart, aLength, rel, kLength, nullptr);
  delete[] rel;
  ParallelAlgorithms::pa_detail::check(rc, "PartitionRadix");
}

#endif
