// Drop-in replacement for the reference's HistogramParallel.h entry points
// on the radix path, with the reference's signatures, index conventions and
// ownership: results are new[]-allocated and released by the caller with
// delete[] (per row, then the outer array, for the 2-D results).
#ifndef PA_DROPIN_HISTOGRAMPARALLEL_H
#define PA_DROPIN_HISTOGRAMPARALLEL_H

#include <cstddef>
#include <cstdint>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

// HistogramParallel.h:249 -- r inclusive.  Returns Log2ofPowerOfTwoRadix = 8
// rows of 256 counts; rows 0-3 are the four byte digits and rows 4-7 are
// zero, as the reference allocates them.
template <unsigned PowerOfTwoRadix, unsigned Log2ofPowerOfTwoRadix>
inline size_t** HistogramByteComponentsParallel(unsigned inArray[], size_t l, size_t r,
                                                size_t parallelThreshold = 64 * 1024) {
  static_assert(PowerOfTwoRadix == 256 && Log2ofPowerOfTwoRadix == 8,
                "the reference's loop is hard-wired to four byte digits");
  (void)parallelThreshold;
  uint64_t counts[4 * 256];
  const size_t n = l <= r ? r - l + 1 : 0;
  pa_detail::check(pa_hist_byte_components_u32(inArray + l, n, counts, nullptr), "HistogramByteComponentsParallel");
  size_t** out = new size_t*[Log2ofPowerOfTwoRadix];
  for (unsigned d = 0; d < Log2ofPowerOfTwoRadix; ++d) {
    out[d] = new size_t[PowerOfTwoRadix];
    for (unsigned b = 0; b < PowerOfTwoRadix; ++b) out[d][b] = d < 4 ? (size_t)counts[d * 256 + b] : 0;
  }
  return out;
}

// HistogramParallel.h:535 -- r inclusive; counts of (a[i] >> shiftRight) & 255.
template <unsigned long PowerOfTwoRadix, unsigned long Log2ofPowerOfTwoRadix>
inline size_t* HistogramOneByteComponentParallel(unsigned inArray[], size_t l, size_t r, unsigned long shiftRight,
                                                 size_t parallelThreshold = 64 * 1024) {
  static_assert(PowerOfTwoRadix == 256 && Log2ofPowerOfTwoRadix == 8, "256 bins of one byte");
  (void)parallelThreshold;
  uint64_t counts[256];
  const size_t n = l <= r ? r - l + 1 : 0;
  pa_detail::check(pa_hist_one_byte_u32(inArray + l, n, (unsigned)shiftRight, counts, nullptr),
                   "HistogramOneByteComponentParallel");
  size_t* out = new size_t[256];
  for (int b = 0; b < 256; ++b) out[b] = (size_t)counts[b];
  return out;
}

// HistogramParallel.h:466 -- same contract.  The reference's leaf loop stops
// one short of its inclusive r (:499); this returns the correct counts.
template <unsigned long PowerOfTwoRadix, unsigned long Log2ofPowerOfTwoRadix>
inline size_t* HistogramOneByteComponentParallel_2(unsigned inArray[], size_t l, size_t r, unsigned long shiftRight,
                                                   size_t parallelThreshold = 64 * 1024) {
  return HistogramOneByteComponentParallel<PowerOfTwoRadix, Log2ofPowerOfTwoRadix>(inArray, l, r, shiftRight,
                                                                                   parallelThreshold);
}

// HistogramParallel.h:17 (and the _2, _3, _4 variants, :117, :184, :58) --
// byte counts of a[l, r), r EXCLUSIVE.
template <unsigned NumberOfBins>
inline size_t* HistogramOneByteComponentParallel(unsigned char inArray[], size_t l, size_t r,
                                                 size_t parallelThreshold = 64 * 1024) {
  static_assert(NumberOfBins == 256, "one bin per byte value");
  (void)parallelThreshold;
  uint64_t counts[256];
  const size_t n = l < r ? r - l : 0;
  pa_detail::check(pa_hist_u8(inArray + l, n, counts, nullptr), "HistogramOneByteComponentParallel(u8)");
  size_t* out = new size_t[256];
  for (int b = 0; b < 256; ++b) out[b] = (size_t)counts[b];
  return out;
}
template <unsigned NumberOfBins>
inline size_t* HistogramOneByteComponentParallel_2(unsigned char inArray[], size_t l, size_t r,
                                                   size_t parallelThreshold = 64 * 1024) {
  return HistogramOneByteComponentParallel<NumberOfBins>(inArray, l, r, parallelThreshold);
}
template <unsigned NumberOfBins>
inline size_t* HistogramOneByteComponentParallel_3(unsigned char inArray[], size_t l, size_t r,
                                                   size_t parallelThreshold = 64 * 1024) {
  return HistogramOneByteComponentParallel<NumberOfBins>(inArray, l, r, parallelThreshold);
}
template <unsigned NumberOfBins>
inline size_t* HistogramOneByteComponentParallel_4(unsigned char inArray[], size_t l, size_t r,
                                                   size_t parallelThreshold = 64 * 1024) {
  return HistogramOneByteComponentParallel<NumberOfBins>(inArray, l, r, parallelThreshold);
}

// HistogramParallel.h:444 -- per-work-quantum counts of byte whichByte over
// a[l..r] (r inclusive); returns numberOfQuantas rows of 256.
template <unsigned PowerOfTwoRadix, unsigned Log2ofPowerOfTwoRadix>
inline size_t** HistogramByteComponentsQCPar(unsigned* inArray, size_t l, size_t r, size_t workQuanta,
                                             size_t numberOfQuantas, unsigned whichByte,
                                             size_t parallelThreshold = 16 * 1024) {
  static_assert(PowerOfTwoRadix == 256 && Log2ofPowerOfTwoRadix == 8, "256 bins of one byte");
  (void)parallelThreshold;
  uint64_t* counts = new uint64_t[numberOfQuantas * 256];
  const int rc = pa_hist_quanta_u32(inArray, l, r, workQuanta, numberOfQuantas, whichByte, counts, nullptr);
  if (rc != PA_OK) {
    delete[] counts;
    pa_detail::check(rc, "HistogramByteComponentsQCPar");
  }
  size_t** out = new size_t*[numberOfQuantas];
  for (size_t q = 0; q < numberOfQuantas; ++q) {
    out[q] = new size_t[256];
    for (int b = 0; b < 256; ++b) out[q][b] = (size_t)counts[q * 256 + b];
  }
  delete[] counts;
  return out;
}

// RadixSortLsdParallel.h:108 -- startOfBin[q][b] for byte `digit`.
template <unsigned PowerOfTwoRadix, unsigned Log2ofPowerOfTwoRadix>
inline size_t** ComputeStartOfBinsPar(unsigned* inArray, size_t size, size_t workQuanta, size_t numberOfQuantas,
                                      unsigned digit, size_t parallelThreshold = 16 * 1024) {
  static_assert(PowerOfTwoRadix == 256 && Log2ofPowerOfTwoRadix == 8, "256 bins of one byte");
  (void)parallelThreshold;
  uint64_t* sob = new uint64_t[numberOfQuantas * 256];
  const int rc = pa_start_of_bins_u32(inArray, size, workQuanta, numberOfQuantas, digit, sob, nullptr);
  if (rc != PA_OK) {
    delete[] sob;
    pa_detail::check(rc, "ComputeStartOfBinsPar");
  }
  size_t** out = new size_t*[numberOfQuantas];
  for (size_t q = 0; q < numberOfQuantas; ++q) {
    out[q] = new size_t[256];
    for (int b = 0; b < 256; ++b) out[q][b] = (size_t)sob[q * 256 + b];
  }
  delete[] sob;
  return out;
}

}  // namespace ParallelAlgorithms

#endif  // PA_DROPIN_HISTOGRAMPARALLEL_H
