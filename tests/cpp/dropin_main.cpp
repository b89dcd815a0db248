// A C++ caller of the reference's radix entry points, switched to the GPU by
// changing only the include path (-I include/ParallelAlgorithms) and linking
// libpa_gb300.so.  Self-checking in the style of the reference's benchmarks
// (RadixSortLsdBenchmark.cpp:78-114, RadixSelectBenchmark.cpp:33-69,
// SumBenchmark.cpp:116-163): each result is compared with the standard
// library and a mismatch exits non-zero.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include "RadixSortLsdParallel.h"
#include "HistogramParallel.h"
#include "RadixSelect.h"
#include "SumParallel.h"
#include "CountingSortParallel.h"
#include "RadixPartition.h"
#include "ParallelMergeSort.h"
#include "RadixSortMsdParallel.h"

static int fail(const char* what) {
  std::printf("FAIL: %s\n", what);
  return 1;
}

int main(int argc, char** argv) {
  const size_t n = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1000003;
  std::mt19937_64 dist(1234);
  std::vector<unsigned> uints(n);
  for (auto& d : uints) d = static_cast<unsigned>(dist());

  // SortRadixPar(a, tmp, n) vs std::stable_sort
  std::vector<unsigned> a(uints), tmp(n), ref(uints);
  std::stable_sort(ref.begin(), ref.end());
  ParallelAlgorithms::SortRadixPar(a.data(), tmp.data(), n);
  if (a != ref) return fail("SortRadixPar(a, tmp, n)");
  std::vector<unsigned> a2(uints);
  ParallelAlgorithms::SortRadixPar(a2.data(), n);
  if (a2 != ref) return fail("SortRadixPar(a, n)");
  std::vector<unsigned> a3(uints), b3(n);
  ParallelAlgorithms::RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(a3.data(), b3.data(), n);
  if (a3 != ref || b3 != ref) return fail("RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase");
  std::vector<unsigned> a4(uints), b4(n);
  ParallelAlgorithms::RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize(a4.data(), b4.data(), n);
  if (b4 != ref) return fail("RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize");
  std::vector<unsigned> a5(uints), w5(n);
  ParallelAlgorithms::SortRadixInnerPar<256, 8>(a5.data(), w5.data(), n);
  if (a5 != ref) return fail("SortRadixInnerPar<256,8>");
  ParallelAlgorithms::SortRadixInnerPar<256, 8>(a5.data(), w5.data(), n, n / 8);  // explicit quantum
  if (a5 != ref) return fail("SortRadixInnerPar<256,8>(quantum)");

  // HistogramByteComponentsParallel<256,8>: 8 rows, rows 4-7 zero
  size_t** h = ParallelAlgorithms::HistogramByteComponentsParallel<256, 8>(uints.data(), 0, n - 1);
  for (unsigned d = 0; d < 8; ++d) {
    std::vector<size_t> c(256, 0);
    if (d < 4)
      for (unsigned v : uints) c[(v >> (8 * d)) & 255]++;
    for (int b = 0; b < 256; ++b)
      if (h[d][b] != c[b]) return fail("HistogramByteComponentsParallel");
    delete[] h[d];
  }
  delete[] h;
  size_t* h1 = ParallelAlgorithms::HistogramOneByteComponentParallel<256, 8>(uints.data(), 0, n - 1, 13);
  {
    std::vector<size_t> c(256, 0);
    for (unsigned v : uints) c[(v >> 13) & 255]++;
    for (int b = 0; b < 256; ++b)
      if (h1[b] != c[b]) return fail("HistogramOneByteComponentParallel");
  }
  delete[] h1;

  // SelectRadix(a, n, k) vs std::nth_element, k = n - 21 as the reference benchmark
  if (n > 21) {
    const size_t k = n - 21;
    std::vector<unsigned> s(uints), nth(uints);
    std::nth_element(nth.begin(), nth.begin() + k, nth.end());
    unsigned v = SelectRadix(s.data(), n, k);
    if (v != nth[k] || s[k] != nth[k]) return fail("SelectRadix");
    std::vector<unsigned> s_sorted(s);
    std::sort(s_sorted.begin(), s_sorted.end());
    if (s_sorted != ref) return fail("SelectRadix left a permutation of the input");
  }

  // SumParallelNonRecursive vs std::accumulate
  const unsigned long long sref = std::accumulate(uints.begin(), uints.end(), 0ULL);
  if (ParallelAlgorithms::SumParallelNonRecursive(uints.data(), 0, n) != sref) return fail("SumParallelNonRecursive");
  if ((unsigned long long)ParallelAlgorithms::SumParallel(uints.data(), 0, n) != sref) return fail("SumParallel");
  if (ParallelAlgorithms::SumParallelNonRecursiveBufferedLocally(uints.data(), 0, n) != sref ||
      ParallelAlgorithms::SumParallelNonRecursiveBuffered(uints.data(), 0, n) != sref)
    return fail("SumParallelNonRecursiveBuffered(Locally)");
  {
    // the caller-buffer form: each parallelThreshold chunk's sum lands in sum_array
    const size_t thr = 16 * 1024, tasks = (n + thr - 1) / thr;
    std::vector<unsigned long long> sum_array(tasks, 0);
    if (ParallelAlgorithms::SumParallelNonRecursive(uints.data(), 0, n, sum_array.data(), thr) != sref)
      return fail("SumParallelNonRecursive(sum_array)");
    for (size_t t = 0; t < tasks; ++t) {
      const size_t hi = std::min(n, (t + 1) * thr);
      if (sum_array[t] != std::accumulate(uints.begin() + t * thr, uints.begin() + hi, 0ULL))
        return fail("SumParallelNonRecursive(sum_array) chunk");
    }
    std::vector<unsigned long long> u64(uints.begin(), uints.end());
    if (ParallelAlgorithms::SumParallel(u64.data(), 0, n) != sref ||
        ParallelAlgorithms::SumParallelNonRecursive(u64.data(), 0, n) != sref)
      return fail("SumParallel(u64)");
  }
  {
    // SumBenchmarkChar's call (SumBenchmark.cpp:72-110): the template
    // SumParallel over unsigned chars, against a plain 64-bit accumulation
    std::vector<unsigned char> u8Array(n);
    for (size_t i = 0; i < n; ++i) u8Array[i] = (unsigned char)uints[i];
    long long sum_ref = 0;
    for (unsigned char c : u8Array) sum_ref += (long long)c;
    long long sum = ParallelAlgorithms::SumParallel(u8Array.data(), 0, uints.size());
    if (sum != sum_ref) return fail("SumParallel(unsigned char)");
    std::vector<int> i32(n);
    std::vector<float> f32(n);
    long long i_ref = 0, f_ref = 0;
    for (size_t i = 0; i < n; ++i) {
      i32[i] = (int)uints[i];
      f32[i] = (float)(int)(uints[i] >> 8) / 7.0f - 100000.0f;
      i_ref += (long long)i32[i];
      f_ref += (long long)f32[i];
    }
    if (ParallelAlgorithms::SumParallel(i32.data(), 0, n) != i_ref) return fail("SumParallel(int)");
    if (ParallelAlgorithms::SumParallel(f32.data(), 0, n) != f_ref) return fail("SumParallel(float)");
  }

  // counting_sort_parallel vs std::sort of the same bytes
  {
    std::vector<unsigned char> bytes(n), want;
    for (size_t i = 0; i < n; ++i) bytes[i] = (unsigned char)(uints[i] >> 13);
    want = bytes;
    std::sort(want.begin(), want.end());
    ParallelAlgorithms::counting_sort_parallel(bytes.data(), n);
    if (bytes != want) return fail("counting_sort_parallel");
  }

  // PartitionRadix around several k: each a[k] is the k-th smallest, parts ordered
  if (n > 8) {
    std::vector<unsigned> p(uints), sorted(uints);
    std::sort(sorted.begin(), sorted.end());
    size_t ks[3] = {0, n / 3, n - 2};
    PartitionRadix(p.data(), n, ks, 3);
    for (size_t k : ks) {
      if (p[k] != sorted[k]) return fail("PartitionRadix value");
      for (size_t i = 0; i < k; ++i)
        if (p[i] > p[k]) return fail("PartitionRadix order");
    }
    std::vector<unsigned> q(uints);
    if (PartitionRadix(q.data(), n, n / 2) != sorted[n / 2]) return fail("PartitionRadix single k");
  }

  // the radix-leaf merge sorts: result in dst (srcToDst) or in src
  if (n > 2) {
    std::vector<unsigned> sorted(uints), src(uints), dst(n, 0u);
    std::sort(sorted.begin(), sorted.end());
    ParallelAlgorithms::parallel_merge_sort_hybrid_radix(src.data(), 0, n - 1, dst.data(), true);
    if (dst != sorted) return fail("parallel_merge_sort_hybrid_radix(srcToDst)");
    std::vector<unsigned> src2(uints), work(n);
    ParallelAlgorithms::parallel_merge_sort_hybrid_radix(src2.data(), 0, n - 1, work.data(), false);
    if (src2 != sorted) return fail("parallel_merge_sort_hybrid_radix(in src)");
    std::vector<unsigned> src3(uints);
    ParallelAlgorithms::parallel_linear_in_place_preventative_adaptive_sort(src3.data(), n);
    if (src3 != sorted) return fail("parallel_linear_in_place_preventative_adaptive_sort");
    std::vector<unsigned> src4(uints);
    ParallelAlgorithms::parallel_hybrid_inplace_msd_radix_sort(src4.data(), n);
    if (src4 != sorted) return fail("parallel_hybrid_inplace_msd_radix_sort");
  }

  std::printf("OK n=%zu\n", n);
  return 0;
}
