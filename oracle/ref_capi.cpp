// extern "C" wrapper around the reference's own CPU implementation of the
// radix hot path, compiled unchanged from the reference headers with the
// project-written TBB stand-in (oracle/tbb_shim) and Copy.h stub
// (oracle/ref_stub).  Test infrastructure only: it is the parity checker for
// the oracle restatement and the timed CPU baseline; the GPU product never
// links or calls it.
//
// Each function names the reference entry point it forwards to.
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <random>
#include <thread>
#include <vector>

#include "RadixSortLsdParallel.h"
#include "HistogramParallel.h"
#include "RadixSelect.h"
#include "SumParallel.h"
#include "RadixSortLSD.h"
#include "CountingSortParallel.h"
#include "RadixPartition.h"

// RadixSortLSD.h:37-38 declares these (defined in MemoryUsage.cpp); only the
// memory-adaptive sorts call them, which are not on the path.  Defined here so
// the shared object has no unresolved symbols.
unsigned long long physical_memory_used_in_megabytes() { return 0; }
unsigned long long physical_memory_total_in_megabytes() { return 0; }

extern "C" {

int pa_ref_hardware_concurrency(void) { return tbb::info::default_concurrency(); }

// The reference benchmark's input recipe (ParallelAlgorithms.cpp:91,
// 112-115): std::mt19937_64(seed), key = low 32 bits of each draw.  Lets the
// timed reference run make its own input without loading the GPU library.
void pa_ref_gen_uniform_u32(uint64_t seed, size_t n, uint32_t* out) {
  std::mt19937_64 g(seed);
  for (size_t i = 0; i < n; ++i) out[i] = (uint32_t)g();
}

// RadixSortLsdParallel.h:367 SortRadixPar(a, tmp_work_buff, a_size)
void pa_ref_sort_radix_par_u32(unsigned* a, unsigned* tmp, size_t n) {
  ParallelAlgorithms::SortRadixPar(a, tmp, n);
}

// RadixSortLsdParallel.h:340 SortRadixPar(a, a_size) (allocates its own tmp)
void pa_ref_sort_radix_par_alloc_u32(unsigned* a, size_t n) { ParallelAlgorithms::SortRadixPar(a, n); }

// RadixSortLsdParallel.h:86 (result in b)
void pa_ref_sort_two_phase_par_u32(unsigned* a, unsigned* b, size_t n) {
  ParallelAlgorithms::RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(a, b, (unsigned long)n);
}

// RadixSortLSD.h:518 (serial two-phase, result in a)
void pa_ref_sort_two_phase_serial_u32(unsigned* a, unsigned* b, size_t n) {
  RadixSortLSDPowerOf2Radix_unsigned_TwoPhase(a, b, n);
}

// HistogramParallel.h:249 HistogramByteComponentsParallel<256,8>(a, l, r)
// r inclusive; out receives the 8 rows x 256 counts the reference returns.
void pa_ref_hist_byte_components_par_u32(unsigned* a, size_t l, size_t r, uint64_t* out) {
  size_t** c = ParallelAlgorithms::HistogramByteComponentsParallel<256, 8>(a, l, r);
  for (unsigned d = 0; d < 8; ++d) {
    for (unsigned b = 0; b < 256; ++b) out[d * 256 + b] = c[d][b];
    delete[] c[d];
  }
  delete[] c;
}

// HistogramParallel.h:535 HistogramOneByteComponentParallel<256,8>(a, l, r, shift)
void pa_ref_hist_one_byte_par_u32(unsigned* a, size_t l, size_t r, unsigned long shift, uint64_t* out) {
  size_t* c = ParallelAlgorithms::HistogramOneByteComponentParallel<256, 8>(a, l, r, shift);
  for (unsigned b = 0; b < 256; ++b) out[b] = c[b];
  delete[] c;
}

// HistogramParallel.h:17 HistogramOneByteComponentParallel<256>(uchar a[], l, r)
// r exclusive
void pa_ref_hist_u8_par(unsigned char* a, size_t l, size_t r, uint64_t* out) {
  size_t* c = ParallelAlgorithms::HistogramOneByteComponentParallel<256>(a, l, r);
  for (unsigned b = 0; b < 256; ++b) out[b] = c[b];
  delete[] c;
}

// HistogramParallel.h:444 HistogramByteComponentsQCPar<256,8>; out is Q x 256.
void pa_ref_hist_qc_par_u32(unsigned* a, size_t l, size_t r, size_t work_quanta, size_t quanta,
                            unsigned which_byte, uint64_t* out) {
  size_t** c = ParallelAlgorithms::HistogramByteComponentsQCPar<256, 8>(a, l, r, work_quanta, quanta, which_byte);
  for (size_t q = 0; q < quanta; ++q) {
    for (unsigned b = 0; b < 256; ++b) out[q * 256 + b] = c[q][b];
    delete[] c[q];
  }
  delete[] c;
}

// RadixSortLsdParallel.h:108 ComputeStartOfBinsPar<256,8>; out is Q x 256.
void pa_ref_compute_start_of_bins_par_u32(unsigned* a, size_t n, size_t work_quanta, size_t quanta,
                                          unsigned digit, uint64_t* out) {
  size_t** s = ParallelAlgorithms::ComputeStartOfBinsPar<256, 8>(a, n, work_quanta, quanta, digit);
  for (size_t q = 0; q < quanta; ++q) {
    for (unsigned b = 0; b < 256; ++b) out[q * 256 + b] = s[q][b];
    delete[] s[q];
  }
  delete[] s;
}

// RadixSelect.h:157 SelectRadix(a, length, k).  The reference reads one
// element past the array (RadixSelect.h:112 passes last - start + 1), so the
// caller's buffer must hold n + 1 elements.
unsigned pa_ref_select_radix_u32(unsigned* a_n_plus_1, size_t n, size_t k) {
  return SelectRadix(a_n_plus_1, n, k);
}

// RadixSelect.h:139 SelectRadix(a, start, length, k); buffer must hold
// start + length + 1 elements.
unsigned pa_ref_select_radix_range_u32(unsigned* a, size_t start, size_t length, size_t k) {
  return SelectRadix(a, start, length, k);
}

// SumParallel.h:261 SumParallelNonRecursive(unsigned[], l, r).  The reference
// underflows num_tasks - 1 when r == l (SumParallel.h:263-268), so an empty
// range is answered here without calling it.
unsigned long long pa_ref_sum_par_nonrec_u32(unsigned* a, size_t l, size_t r) {
  if (r <= l) return 0;
  return ParallelAlgorithms::SumParallelNonRecursive(a, l, r);
}

// SumParallel.h:285 SumParallelNonRecursive(unsigned long long[], l, r)
unsigned long long pa_ref_sum_par_nonrec_u64(unsigned long long* a, size_t l, size_t r) {
  if (r <= l) return 0;
  return ParallelAlgorithms::SumParallelNonRecursive(a, l, r);
}

// SumParallel.h:162 SumParallel(unsigned long long[], l, r) (recursive)
unsigned long long pa_ref_sum_par_u64(unsigned long long* a, size_t l, size_t r) {
  return ParallelAlgorithms::SumParallel(a, l, r);
}

// SumParallel.h:207 template SumParallel<unsigned>(a, l, r) -> long long
long long pa_ref_sum_par_template_u32(unsigned* a, size_t l, size_t r) {
  return ParallelAlgorithms::SumParallel(a, l, r);
}

// The same template over other element types: unsigned char (the call of
// SumBenchmark.cpp:101), int and float.
long long pa_ref_sum_par_template_u8(unsigned char* a, size_t l, size_t r) {
  return ParallelAlgorithms::SumParallel(a, l, r);
}
long long pa_ref_sum_par_template_i32(int* a, size_t l, size_t r) { return ParallelAlgorithms::SumParallel(a, l, r); }
long long pa_ref_sum_par_template_f32(float* a, size_t l, size_t r) {
  return ParallelAlgorithms::SumParallel(a, l, r);
}

// SumParallel.h:419 SumParallelNonRecursive(unsigned[], l, r, sum_array,
// parallelThreshold): per-task sums left in sum_array.
unsigned long long pa_ref_sum_par_nonrec_array_u32(unsigned* a, size_t l, size_t r, unsigned long long* sum_array,
                                                   size_t threshold) {
  return ParallelAlgorithms::SumParallelNonRecursive(a, l, r, sum_array, threshold);
}

// CountingSortParallel.h:81 counting_sort_parallel(a, a_size): byte array
// sorted by a parallel histogram and a parallel fill.
void pa_ref_counting_sort_par_u8(unsigned char* a, size_t n) { ParallelAlgorithms::counting_sort_parallel(a, n); }

// RadixPartition.h:152 PartitionRadix(a, aLength, k[], kLength): in-place MSD
// radix partition around every k (k ascending).
void pa_ref_partition_radix_u32(unsigned* a, size_t n, size_t* k, size_t klen) { PartitionRadix(a, n, k, klen); }

// ParallelMergeSort.h:287 parallel_merge_sort_hybrid_radix(src, l, r, dst,
// srcToDst): merge sort with LSD radix sorted leaves, r inclusive.
void pa_ref_merge_sort_hybrid_radix_u32(unsigned* src, size_t l, size_t r, unsigned* dst, int src_to_dst) {
  ParallelAlgorithms::parallel_merge_sort_hybrid_radix(src, l, r, dst, src_to_dst != 0);
}

// ParallelMergeSort.h:549 parallel_linear_in_place_preventative_adaptive_sort.
void pa_ref_preventative_adaptive_sort_u32(unsigned* src, size_t n) {
  ParallelAlgorithms::parallel_linear_in_place_preventative_adaptive_sort(src, n);
}

// RadixSortMsdParallel.h:291 parallel_hybrid_inplace_msd_radix_sort(a, n).
void pa_ref_msd_radix_sort_u32(unsigned* a, size_t n) { ParallelAlgorithms::parallel_hybrid_inplace_msd_radix_sort(a, n); }

// Not in the reference: std::stable_sort baselines for the key types the
// reference has no radix path for (u64, float32 via its bit pattern, and
// key + u32 payload pairs).  Float keys are compared by the sign-flipped bit
// pattern, a total order in which -0.0 sorts before +0.0.
static inline uint32_t f32_order_bits(uint32_t b) { return b ^ ((b >> 31) ? 0xFFFFFFFFu : 0x80000000u); }

void pa_ref_std_stable_sort_u64(unsigned long long* a, size_t n) { std::stable_sort(a, a + n); }

void pa_ref_std_stable_sort_f32_bits(uint32_t* a, size_t n) {
  std::stable_sort(a, a + n, [](uint32_t x, uint32_t y) { return f32_order_bits(x) < f32_order_bits(y); });
}

void pa_ref_std_stable_sort_kv_u64(unsigned long long* k, uint32_t* v, size_t n) {
  std::vector<uint32_t> idx(n);
  for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
  std::stable_sort(idx.begin(), idx.end(), [k](uint32_t x, uint32_t y) { return k[x] < k[y]; });
  std::vector<unsigned long long> k2(n);
  std::vector<uint32_t> v2(n);
  for (size_t i = 0; i < n; ++i) {
    k2[i] = k[idx[i]];
    v2[i] = v[idx[i]];
  }
  std::memcpy(k, k2.data(), n * sizeof(unsigned long long));
  std::memcpy(v, v2.data(), n * sizeof(uint32_t));
}

}  // extern "C"
