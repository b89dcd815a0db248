/*
 * CPU oracle: a plain-C restatement of the reference's radix hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and there only as the
 * checker.  The GPU product never links, loads or calls it.
 *
 * Each function cites the reference file:line it restates.  Parity of this
 * restatement is pinned against the reference's own code compiled unchanged
 * (oracle/_ref, built by oracle/build.py) and against the golden fixtures in
 * tests/golden/, which were produced by that compiled reference.
 *
 * Conventions follow the reference: index ranges are [l, r] inclusive where
 * the reference uses an inclusive r (HistogramParallel.h:249,535) and
 * [l, r) where it uses an exclusive one (SumParallel.h:261).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define PA_ORACLE_OK 0
#define PA_ORACLE_ERR_ARG 1
#define PA_ORACLE_ERR_OOM 2

/* Sign-flip transform that maps IEEE-754 float32 bit patterns to unsigned
 * integers with the same total order (-inf < ... < -0.0 < +0.0 < ... < +inf).
 * Not in the reference (it has no float path); its README lists float keys
 * as future work (README.md:50). */
static inline uint32_t f32_to_ordered(uint32_t b) { return b ^ ((b >> 31) ? 0xFFFFFFFFu : 0x80000000u); }
static inline uint32_t ordered_to_f32(uint32_t o) { return o ^ ((o >> 31) ? 0x80000000u : 0xFFFFFFFFu); }

/* InsertionSort.h:7-22 insertionSortSimilarToSTLnoSelfAssignment; SortRadixPar
 * uses it below 100 elements (RadixSortLsdParallel.h:383-386). */
static void insertion_sort_u32(uint32_t* a, size_t n) {
  for (size_t i = 1; i < n; i++) {
    if (a[i] < a[i - 1]) {
      uint32_t cur = a[i];
      a[i] = a[i - 1];
      size_t j;
      for (j = i - 1; j > 0 && cur < a[j - 1]; j--) a[j] = a[j - 1];
      a[j] = cur;
    }
  }
}

/* Work-quantum size rule of SortRadixPar(a, tmp, n) (RadixSortLsdParallel.h:
 * 374-379) with a fixed core count, since the stable output does not depend
 * on how the array is cut into quanta. */
static size_t quantum_for(size_t n) {
  const size_t cores = 8;
  size_t thr = 512 * 1024;
  if (thr * cores < n) thr = n / cores;
  return thr;
}

/*
 * One LSD digit pass, restating SortRadixInnerPar's loop body
 * (RadixSortLsdParallel.h:253-322):
 *   - per-quantum counts of the digit (HistogramByteComponentsAcrossWorkQuantasQC,
 *     HistogramParallel.h:332-397),
 *   - start of every bin for every quantum (ComputeStartOfBinsPar,
 *     RadixSortLsdParallel.h:128-156): bins in digit order, and within a bin
 *     quanta in array order, which is what makes the pass stable,
 *   - per-quantum scatter (PermuteDerandomizedNew, :169-212; its 64-entry
 *     write buffers only batch the same stores and do not change the output).
 * Keys are read through a 64-bit lane so one body serves 32- and 64-bit keys.
 */
#define DEFINE_LSD_PASS(NAME, KT)                                                                     \
  static int NAME(const KT* in, KT* out, const uint32_t* vin, uint32_t* vout, size_t n, unsigned shift, \
                  unsigned bits) {                                                                     \
    const size_t R = (size_t)1 << bits;                                                                \
    const uint64_t mask = R - 1;                                                                       \
    const size_t quantum = quantum_for(n);                                                             \
    const size_t Q = (n + quantum - 1) / quantum;                                                      \
    uint64_t* count = (uint64_t*)calloc(Q * R, sizeof(uint64_t));                                      \
    uint64_t* start = (uint64_t*)calloc(Q * R, sizeof(uint64_t));                                      \
    if (!count || !start) {                                                                            \
      free(count);                                                                                     \
      free(start);                                                                                     \
      return PA_ORACLE_ERR_OOM;                                                                        \
    }                                                                                                  \
    for (size_t q = 0; q < Q; q++) {                                                                   \
      size_t s = q * quantum, e = s + quantum < n ? s + quantum : n;                                   \
      for (size_t i = s; i < e; i++) count[q * R + (((uint64_t)in[i] >> shift) & mask)]++;            \
    }                                                                                                  \
    uint64_t run = 0;                                                                                  \
    for (size_t b = 0; b < R; b++) {                                                                   \
      for (size_t q = 0; q < Q; q++) {                                                                 \
        start[q * R + b] = run;                                                                        \
        run += count[q * R + b];                                                                       \
      }                                                                                                \
    }                                                                                                  \
    for (size_t q = 0; q < Q; q++) {                                                                   \
      size_t s = q * quantum, e = s + quantum < n ? s + quantum : n;                                   \
      uint64_t* st = start + q * R;                                                                    \
      for (size_t i = s; i < e; i++) {                                                                 \
        uint64_t pos = st[((uint64_t)in[i] >> shift) & mask]++;                                        \
        out[pos] = in[i];                                                                              \
        if (vin) vout[pos] = vin[i];                                                                   \
      }                                                                                                \
    }                                                                                                  \
    free(count);                                                                                       \
    free(start);                                                                                       \
    return PA_ORACLE_OK;                                                                               \
  }

DEFINE_LSD_PASS(lsd_pass_u32, uint32_t)
DEFINE_LSD_PASS(lsd_pass_u64, uint64_t)

/*
 * Stable ascending LSD radix sort of n keys in place in `keys`, with an
 * optional uint32 payload moved with its key.  key_bytes is 4 or 8;
 * digit_bits is 8 (the reference's PowerOfTwoRadix = 256) or 11;
 * is_float = 1 treats 4-byte keys as IEEE-754 float32 bit patterns.
 * tmp / tmp_vals are caller scratch of the same sizes (contents clobbered).
 *
 * For 4-byte unsigned keys, 8-bit digits and no payload this is
 * SortRadixPar(a, tmp, n) (RadixSortLsdParallel.h:367-387) including its
 * insertion-sort branch below 100 keys.  The other key types, digit widths
 * and the payload are not in the reference (its only 64-bit LSD,
 * RadixSortLSD.h:356-400, counts only four digits, Histogram.h:211-223);
 * they widen the same per-quantum structure.
 */
int pa_oracle_lsd_sort(void* keys, void* tmp, uint32_t* vals, uint32_t* tmp_vals, size_t n, int key_bytes,
                       int digit_bits, int is_float) {
  if ((key_bytes != 4 && key_bytes != 8) || (digit_bits != 8 && digit_bits != 11)) return PA_ORACLE_ERR_ARG;
  if (is_float && key_bytes != 4) return PA_ORACLE_ERR_ARG;
  if ((vals == NULL) != (tmp_vals == NULL)) return PA_ORACLE_ERR_ARG;
  if (n == 0) return PA_ORACLE_OK;
  if (key_bytes == 4 && !is_float && !vals && digit_bits == 8 && n < 100) {
    insertion_sort_u32((uint32_t*)keys, n);
    return PA_ORACLE_OK;
  }
  const unsigned width = 8u * (unsigned)key_bytes;
  const unsigned passes = (width + digit_bits - 1) / digit_bits;
  if (is_float) {
    uint32_t* k = (uint32_t*)keys;
    for (size_t i = 0; i < n; i++) k[i] = f32_to_ordered(k[i]);
  }
  void* src = keys;
  void* dst = tmp;
  uint32_t* vsrc = vals;
  uint32_t* vdst = tmp_vals;
  for (unsigned p = 0; p < passes; p++) {
    unsigned shift = p * (unsigned)digit_bits;
    unsigned bits = (unsigned)digit_bits;
    if (shift + bits > width) bits = width - shift;
    int rc = key_bytes == 4 ? lsd_pass_u32((const uint32_t*)src, (uint32_t*)dst, vsrc, vdst, n, shift, bits)
                            : lsd_pass_u64((const uint64_t*)src, (uint64_t*)dst, vsrc, vdst, n, shift, bits);
    if (rc) return rc;
    void* t = src;
    src = dst;
    dst = t;
    uint32_t* vt = vsrc;
    vsrc = vdst;
    vdst = vt;
  }
  if (src != keys) { /* odd number of passes (11-bit digits): copy back */
    memcpy(keys, src, n * (size_t)key_bytes);
    if (vals) memcpy(vals, vsrc, n * sizeof(uint32_t));
  }
  if (is_float) {
    uint32_t* k = (uint32_t*)keys;
    for (size_t i = 0; i < n; i++) k[i] = ordered_to_f32(k[i]);
  }
  return PA_ORACLE_OK;
}

/* HistogramByteComponentsParallel<256,8>(a, l, r) (HistogramParallel.h:249-329):
 * all four byte-digit counts of a[l..r] (r inclusive) in one read.  The
 * reference returns Log2ofPowerOfTwoRadix = 8 rows of which rows 0-3 are
 * filled and rows 4-7 stay zero (:252,:260-293); out is those 8 x 256. */
void pa_oracle_hist_byte_components_u32(const uint32_t* a, size_t l, size_t r, uint64_t* out) {
  memset(out, 0, 8 * 256 * sizeof(uint64_t));
  if (l > r) return;
  for (size_t i = l; i <= r; i++) {
    uint32_t v = a[i];
    out[0 * 256 + (v & 0xff)]++;
    out[1 * 256 + ((v >> 8) & 0xff)]++;
    out[2 * 256 + ((v >> 16) & 0xff)]++;
    out[3 * 256 + ((v >> 24) & 0xff)]++;
  }
}

/* HistogramOneByteComponentParallel<256,8>(a, l, r, shiftRight)
 * (HistogramParallel.h:535-576): counts of (a[i] >> shift) & 255, r inclusive. */
void pa_oracle_hist_one_byte_u32(const uint32_t* a, size_t l, size_t r, unsigned shift, uint64_t* out) {
  memset(out, 0, 256 * sizeof(uint64_t));
  if (l > r) return;
  for (size_t i = l; i <= r; i++) out[(a[i] >> shift) & 0xff]++;
}

/* HistogramOneByteComponentParallel<256>(unsigned char a[], l, r)
 * (HistogramParallel.h:16-54): byte counts of a[l..r), r exclusive. */
void pa_oracle_hist_u8(const uint8_t* a, size_t l, size_t r, uint64_t* out) {
  memset(out, 0, 256 * sizeof(uint64_t));
  for (size_t i = l; i < r; i++) out[a[i]]++;
}

/* Every digit's counts in one read, generalised to the key types and digit
 * widths of pa_oracle_lsd_sort (the fused histogram that precedes the digit
 * passes).  out holds passes x 2^digit_bits counts; float keys are counted
 * after the sign-flip transform. */
int pa_oracle_hist_digits(const void* keys, size_t n, int key_bytes, int digit_bits, int is_float, uint64_t* out) {
  if ((key_bytes != 4 && key_bytes != 8) || (digit_bits != 8 && digit_bits != 11)) return PA_ORACLE_ERR_ARG;
  const unsigned width = 8u * (unsigned)key_bytes;
  const unsigned passes = (width + digit_bits - 1) / digit_bits;
  const size_t R = (size_t)1 << digit_bits;
  memset(out, 0, passes * R * sizeof(uint64_t));
  for (size_t i = 0; i < n; i++) {
    uint64_t k = key_bytes == 4 ? ((const uint32_t*)keys)[i] : ((const uint64_t*)keys)[i];
    if (is_float) k = f32_to_ordered((uint32_t)k);
    for (unsigned p = 0; p < passes; p++) out[p * R + ((k >> (p * digit_bits)) & (R - 1))]++;
  }
  return PA_ORACLE_OK;
}

/* HistogramByteComponentsAcrossWorkQuantasQC / HistogramByteComponentsQCPar
 * (HistogramParallel.h:332-464): counts of byte `which_byte` of a[l..r]
 * (r inclusive) per work quantum; out is quanta x 256. */
void pa_oracle_hist_qc_u32(const uint32_t* a, size_t l, size_t r, size_t work_quanta, size_t quanta,
                           unsigned which_byte, uint64_t* out) {
  memset(out, 0, quanta * 256 * sizeof(uint64_t));
  if (l > r) return;
  for (size_t i = l; i <= r; i++) out[(i / work_quanta) * 256 + ((a[i] >> (8 * which_byte)) & 0xff)]++;
}

/* ComputeStartOfBinsPar<256,8> (RadixSortLsdParallel.h:108-165): for each
 * quantum q and bin b, the output index at which quantum q's first key of
 * bin b lands; out is quanta x 256. */
void pa_oracle_start_of_bins_u32(const uint32_t* a, size_t n, size_t work_quanta, size_t quanta, unsigned digit,
                                 uint64_t* out) {
  uint64_t* count = (uint64_t*)calloc(quanta * 256, sizeof(uint64_t));
  if (!count) return;
  if (n) pa_oracle_hist_qc_u32(a, 0, n - 1, work_quanta, quanta, digit, count);
  uint64_t run = 0;
  for (size_t b = 0; b < 256; b++)
    for (size_t q = 0; q < quanta; q++) {
      out[q * 256 + b] = run;
      run += count[q * 256 + b];
    }
  free(count);
}

/*
 * Radix select restating RadixSelectiontNonRecursiveInner (RadixSelect.h:
 * 83-129) and MoveOutsideOfKthBinIn (:36-55): MSD digit by digit, count the
 * digit over the current range (HistogramOneComponentOpt, Histogram.h:103),
 * find the bin holding k, overwrite out-of-bin slots inside that bin's range
 * with in-bin keys from the left and right of it, narrow to the bin.
 * Destructive like the reference: afterwards only a[k] is defined.
 * The right-hand move uses the range's true length; the reference passes one
 * more (RadixSelect.h:112) and so reads a[last], which can never be moved
 * because the bin's open slots are exhausted first.
 * Returns a[k], the k-th smallest of a[start, start + length) with k an
 * absolute index (SelectRadix, RadixSelect.h:139-168).
 */
#define DEFINE_SELECT(NAME, KT, WIDTH)                                                                \
  static size_t NAME##_move_in(KT* a, size_t ob, size_t ob_len, size_t ib, size_t ib_len, unsigned shift, \
                               uint64_t mask, uint64_t kth) {                                          \
    size_t ib_end = ib + ib_len, ob_end = ob + ob_len;                                                 \
    for (;;) {                                                                                         \
      for (; ob < ob_end; ob++)                                                                        \
        if ((((uint64_t)a[ob] >> shift) & mask) == kth) break;                                         \
      if (ob < ob_end)                                                                                 \
        for (; ib < ib_end; ib++)                                                                      \
          if ((((uint64_t)a[ib] >> shift) & mask) != kth) break;                                       \
      if (ob >= ob_end || ib >= ib_end) break;                                                         \
      a[ib++] = a[ob++];                                                                               \
    }                                                                                                  \
    return ib;                                                                                         \
  }                                                                                                    \
  KT NAME(KT* a, size_t start, size_t length, size_t k) {                                              \
    const unsigned bits = 8;                                                                           \
    const size_t R = 256;                                                                              \
    const uint64_t mask = R - 1;                                                                       \
    uint64_t count[256];                                                                               \
    size_t sob[257];                                                                                   \
    size_t first = start;                                                                              \
    int shift = (WIDTH) - (int)bits;                                                                   \
    while (shift >= 0) {                                                                               \
      size_t last = first + length;                                                                    \
      memset(count, 0, sizeof(count));                                                                 \
      for (size_t i = first; i < last; i++) count[((uint64_t)a[i] >> shift) & mask]++;                \
      sob[0] = first;                                                                                  \
      sob[R] = last;                                                                                   \
      for (size_t i = 1; i < R; i++) sob[i] = sob[i - 1] + count[i - 1];                               \
      size_t kb = 0;                                                                                   \
      for (; kb < R; kb++)                                                                             \
        if (k >= sob[kb] && k < sob[kb + 1]) break;                                                    \
      size_t ib = NAME##_move_in(a, first, sob[kb] - first, sob[kb], sob[kb + 1] - sob[kb], (unsigned)shift, \
                                 mask, kb);                                                            \
      NAME##_move_in(a, sob[kb + 1], last - sob[kb + 1], ib, sob[kb + 1] - ib, (unsigned)shift, mask, kb); \
      if (shift == 0) break;                                                                           \
      shift = shift >= (int)bits ? shift - (int)bits : 0;                                              \
      size_t bin_len = sob[kb + 1] - sob[kb];                                                          \
      if (bin_len > 1) {                                                                               \
        first = sob[kb];                                                                               \
        length = bin_len;                                                                              \
      } else if (bin_len == 1) {                                                                       \
        break;                                                                                         \
      }                                                                                                \
    }                                                                                                  \
    return a[k];                                                                                       \
  }

DEFINE_SELECT(pa_oracle_select_u32, uint32_t, 32)
DEFINE_SELECT(pa_oracle_select_u64, uint64_t, 64)

/* SumParallelNonRecursive(unsigned[], l, r) (SumParallel.h:261-283) and the
 * unsigned long long overload (:285-307): exact sum of a[l..r) (r exclusive)
 * in a 64-bit accumulator, wrapping modulo 2^64.  An empty range sums to 0
 * (the reference underflows num_tasks - 1 there, :263-268). */
uint64_t pa_oracle_sum_u32(const uint32_t* a, size_t l, size_t r) {
  uint64_t s = 0;
  for (size_t i = l; i < r; i++) s += a[i];
  return s;
}

uint64_t pa_oracle_sum_u64(const uint64_t* a, size_t l, size_t r) {
  uint64_t s = 0;
  for (size_t i = l; i < r; i++) s += a[i];
  return s;
}

/* Byte-array counting sort, CountingSortParallel.h:29-79
 * (counting_sort_parallel_inner): the counts of every byte value over
 * a[l, r) (HistogramOneByteComponentParallel_3, :34), their exclusive prefix
 * as each value's start (:56-59), then each value written counts[value]
 * times from its start (the parallel fill, :65-68). */
void pa_oracle_counting_sort_u8(uint8_t* a, size_t l, size_t r) {
  uint64_t counts[256] = {0};
  for (size_t i = l; i < r; ++i) counts[a[i]]++;
  size_t at = l;
  for (unsigned v = 0; v < 256; ++v) {
    memset(a + at, (int)v, (size_t)counts[v]);
    at += (size_t)counts[v];
  }
}

/* In-place MSD radix partition around the sorted indices k[kstart,
 * kstart + klen), RadixPartition.h:30-79 (PartitionRadixMsdUIntInner with
 * 256 bins, 8-bit digits, insertion sort below 48 keys):
 *   1. count the digit at `shift` over a[start, start + n);
 *   2. bins start at the exclusive prefix of the counts; each bin's fill
 *      cursor starts at its start (:42-45);
 *   3. cycle-leader permutation (:47-58): take the element at the current
 *      position; while its bin's cursor is not the current position, swap
 *      it with the element at that cursor and advance the cursor; store it
 *      and advance its bin's cursor; then move to the cursor of the first
 *      bin that is not yet full (the comparison uses the bins' starts with
 *      start[256] = the range start, as the reference does);
 *   4. with digits left (shift > 0), for every bin holding one or more of
 *      the k's (walked in order), recurse into it with those k's when it has
 *      at least 48 keys, else sort it (:59-78). */
static void partition_inner(uint32_t* a, size_t start, size_t n, int shift, const size_t* k, size_t kstart,
                            size_t klen) {
  const size_t last = start + n;
  size_t count[256];
  memset(count, 0, sizeof(count));
  for (size_t i = start; i < last; ++i) count[(a[i] >> shift) & 255u]++;
  size_t bstart[257], cursor[256];
  bstart[0] = cursor[0] = start;
  bstart[256] = start;
  for (int b = 1; b < 256; ++b) bstart[b] = cursor[b] = bstart[b - 1] + count[b - 1];
  size_t next = 1;
  for (size_t cur = start; cur < last;) {
    uint32_t x = a[cur];
    unsigned d;
    while (cursor[d = (x >> shift) & 255u] != cur) {
      const uint32_t t = a[cursor[d]];
      a[cursor[d]++] = x;
      x = t;
    }
    a[cur] = x;
    cursor[d]++;
    while (cursor[next - 1] == bstart[next]) next++;
    cur = cursor[next - 1];
  }
  if (shift <= 0) return;
  const int nshift = shift >= 8 ? shift - 8 : 0;
  size_t ki = kstart;
  for (int b = 0; b < 256 && ki < kstart + klen; ++b) {
    if (bstart[b] < cursor[b] && k[ki] >= bstart[b] && k[ki] < cursor[b]) {
      const size_t first = ki++;
      size_t cnt = 1;
      while (ki < kstart + klen && k[ki] >= bstart[b] && k[ki] < cursor[b]) {
        ++cnt;
        ++ki;
      }
      const size_t m = cursor[b] - bstart[b];
      if (m >= 48) {
        partition_inner(a, bstart[b], m, nshift, k, first, cnt);
      } else {
        for (size_t i = bstart[b] + 1; i < cursor[b]; ++i) {  /* insertion sort */
          const uint32_t v = a[i];
          size_t j = i;
          while (j > bstart[b] && a[j - 1] > v) {
            a[j] = a[j - 1];
            --j;
          }
          a[j] = v;
        }
      }
    }
  }
}

/* PartitionRadix(a, aLength, k[], kLength), RadixPartition.h:152-162. */
void pa_oracle_partition_radix_u32(uint32_t* a, size_t n, const size_t* k, size_t klen) {
  if (n == 0 || klen == 0) return;
  partition_inner(a, 0, n, 24, k, 0, klen);
}

/* The reference benchmark's keys (ParallelAlgorithms.cpp:91, 112-115):
 * low 32 bits of each draw of a 64-bit Mersenne Twister seeded with `seed`
 * (std::mt19937_64).  The generator is the published MT19937-64 of
 * Matsumoto and Nishimura (2000): 312 words of state, twist at 156, tempering
 * shifts 29 / 17 / 37 / 43, initialisation multiplier 6364136223846793005.
 * Lets the CPU baseline make its input without the GPU library. */
void pa_oracle_gen_uniform_u32(uint64_t seed, size_t n, uint32_t* out) {
  enum { NN = 312, MM = 156 };
  const uint64_t matrix_a = 0xB5026F5AA96619E9ull, upper = 0xFFFFFFFF80000000ull, lower = 0x7FFFFFFFull;
  uint64_t mt[NN];
  mt[0] = seed;
  for (int i = 1; i < NN; i++) mt[i] = 6364136223846793005ull * (mt[i - 1] ^ (mt[i - 1] >> 62)) + (uint64_t)i;
  int idx = NN;
  for (size_t k = 0; k < n; k++) {
    if (idx >= NN) {
      for (int i = 0; i < NN; i++) {
        const uint64_t x = (mt[i] & upper) | (mt[(i + 1) % NN] & lower);
        mt[i] = mt[(i + MM) % NN] ^ (x >> 1) ^ ((x & 1u) ? matrix_a : 0u);
      }
      idx = 0;
    }
    uint64_t y = mt[idx++];
    y ^= (y >> 29) & 0x5555555555555555ull;
    y ^= (y << 17) & 0x71D67FFFEDA60000ull;
    y ^= (y << 37) & 0xFFF7EEE000000000ull;
    y ^= y >> 43;
    out[k] = (uint32_t)y;
  }
}
