// Drop-in replacement for the reference's SumParallel.h: exact sums in a
// 64-bit accumulator over [l, r), r exclusive, on the GPU.  Every public
// function of the reference header is here with its signature; threshold
// and buffer arguments that only steer the reference's CPU tasks are
// accepted and have no effect.  The reference underflows on an empty range
// (SumParallel.h:263-268); here an empty range sums to 0.
#ifndef PA_DROPIN_SUMPARALLEL_H
#define PA_DROPIN_SUMPARALLEL_H

#include <cstddef>
#include <cstdint>
#include <type_traits>

#include "pa_dropin_common.h"

namespace ParallelAlgorithms {

namespace pa_detail {

// PA_ELEM_* kind of an element type (0..9), or -1 for a type with no GPU sum.
template <class T>
constexpr int sum_kind() {
  using U = typename std::remove_cv<T>::type;
  if (std::is_same<U, float>::value) return PA_ELEM_F32;
  if (std::is_same<U, double>::value) return PA_ELEM_F64;
  if (!std::is_integral<U>::value || std::is_same<U, bool>::value) return -1;
  const bool s = std::is_signed<U>::value;
  switch (sizeof(U)) {
    case 1: return s ? PA_ELEM_I8 : PA_ELEM_U8;
    case 2: return s ? PA_ELEM_I16 : PA_ELEM_U16;
    case 4: return s ? PA_ELEM_I32 : PA_ELEM_U32;
    case 8: return s ? PA_ELEM_I64 : PA_ELEM_U64;
    default: return -1;
  }
}

template <class T>
inline uint64_t sum_bits(const T* in_array, size_t l, size_t r, const char* what) {
  static_assert(sum_kind<T>() >= 0, "SumParallel: element type must be an integer or floating type of 1-8 bytes");
  uint64_t s = 0;
  check(pa_sum_typed(in_array + l, r > l ? r - l : 0, sum_kind<T>(), &s, nullptr), what);
  return s;
}

template <class T>
inline uint64_t sum_chunked(const T* in_array, size_t l, size_t r, unsigned long long* sum_array,
                            size_t parallelThreshold, const char* what) {
  uint64_t s = 0;
  check(pa_sum_chunked(in_array + l, r > l ? r - l : 0, sum_kind<T>(), parallelThreshold,
                       reinterpret_cast<uint64_t*>(sum_array), &s, nullptr),
        what);
  return s;
}

}  // namespace pa_detail

// ---- serial leaves (SumParallel.h:40-158): the same sums -------------------
inline unsigned long long Sum(unsigned long long in_array[], size_t l, size_t r) {
  return pa_detail::sum_bits(in_array, l, r, "Sum");
}
inline unsigned long long Sum(unsigned in_array[], size_t l, size_t r) {
  return pa_detail::sum_bits(in_array, l, r, "Sum");
}
inline unsigned long long SumUnrolled(unsigned in_array[], size_t l, size_t r) {
  return pa_detail::sum_bits(in_array, l, r, "SumUnrolled");
}
inline unsigned long long SumBufferedLocally(unsigned in_array[], size_t l, size_t r) {
  return pa_detail::sum_bits(in_array, l, r, "SumBufferedLocally");
}
inline unsigned long long SumBufferedLocally(unsigned long long in_array[], size_t l, size_t r) {
  return pa_detail::sum_bits(in_array, l, r, "SumBufferedLocally");
}
inline unsigned long long SumBufferedExternally(unsigned in_array[], size_t l, size_t r, unsigned buffer[],
                                                size_t buffer_depth) {
  (void)buffer;
  (void)buffer_depth;
  return pa_detail::sum_bits(in_array, l, r, "SumBufferedExternally");
}
inline unsigned long long SumBufferedExternally(unsigned long long in_array[], size_t l, size_t r,
                                                unsigned long long buffer[], size_t buffer_depth) {
  (void)buffer;
  (void)buffer_depth;
  return pa_detail::sum_bits(in_array, l, r, "SumBufferedExternally");
}

// ---- parallel sums ----------------------------------------------------------
// SumParallel.h:162 -- the non-template overload wins for 64-bit unsigned arrays.
inline unsigned long long SumParallel(unsigned long long in_array[], size_t l, size_t r,
                                      size_t parallelThreshold = 16 * 1024) {
  (void)parallelThreshold;
  return pa_detail::sum_bits(in_array, l, r, "SumParallel");
}

// SumParallel.h:207 -- any other numeric element type: each element converted
// to long long (floats truncated toward zero) and summed; the 64-bit sum read
// as signed.
template <class _Type>
inline long long SumParallel(_Type in_array[], size_t l, size_t r, size_t parallelThreshold = 16 * 1024) {
  (void)parallelThreshold;
  return (long long)pa_detail::sum_bits(in_array, l, r, "SumParallel");
}

// SumParallel.h:240
inline unsigned long long SumNonRecursive(unsigned long long in_array[], size_t l, size_t r,
                                          size_t parallelThreshold = 128 * 1024) {
  (void)parallelThreshold;
  return pa_detail::sum_bits(in_array, l, r, "SumNonRecursive");
}

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

// SumParallel.h:309, :337 -- the same sums (the reference's variants differ
// only in how a CPU task reads its chunk).
inline unsigned long long SumParallelNonRecursiveBufferedLocally(unsigned in_array[], size_t l, size_t r,
                                                                 size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}
inline unsigned long long SumParallelNonRecursiveBufferedLocally(unsigned long long in_array[], size_t l, size_t r,
                                                                 size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}

// SumParallel.h:366, :393
inline unsigned long long SumParallelNonRecursiveBuffered(unsigned in_array[], size_t l, size_t r,
                                                          size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}
inline unsigned long long SumParallelNonRecursiveBuffered(unsigned long long in_array[], size_t l, size_t r,
                                                          size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}

// SumParallel.h:419, :442 -- the caller's sum_array (ceil((r - l) /
// parallelThreshold) entries) receives each parallelThreshold-element chunk's
// sum, as the reference's tasks leave them.
inline unsigned long long SumParallelNonRecursive(unsigned in_array[], size_t l, size_t r,
                                                  unsigned long long* sum_array,
                                                  size_t parallelThreshold = 16 * 1024) {
  return pa_detail::sum_chunked(in_array, l, r, sum_array, parallelThreshold, "SumParallelNonRecursive");
}
inline unsigned long long SumParallelNonRecursive(unsigned long long in_array[], size_t l, size_t r,
                                                  unsigned long long* sum_array,
                                                  size_t parallelThreshold = 16 * 1024) {
  return pa_detail::sum_chunked(in_array, l, r, sum_array, parallelThreshold, "SumParallelNonRecursive");
}

// SumParallel.h:466-554 (built by the reference on Windows only): the same sums.
inline unsigned long long SumParallelNonRecursiveNoHyperthreading(unsigned long long in_array[], size_t l, size_t r,
                                                                  size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}
inline unsigned long long SumParallelNonRecursiveNoHyperthreading(unsigned in_array[], size_t l, size_t r,
                                                                  size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}
inline unsigned long long SumParallelNonRecursiveBufferedLocallyNoHyperthreading(
    unsigned in_array[], size_t l, size_t r, size_t parallelThreshold = 16 * 1024) {
  return SumParallelNonRecursive(in_array, l, r, parallelThreshold);
}

}  // namespace ParallelAlgorithms

#endif  // PA_DROPIN_SUMPARALLEL_H
