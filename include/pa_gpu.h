/*
 * pa_gpu.h - C ABI of the GB300 radix hot path (sort, digit histograms,
 * radix select, 64-bit sum) that replaces the CPU implementation in the
 * reference library ParallelAlgorithms.
 *
 * Every entry point:
 *   - is callable from C, C++ (see include/ParallelAlgorithms/ for inline
 *     wrappers with the reference's own C++ signatures), or any FFI;
 *   - takes plain pointers and sizes.  Each buffer may be HOST memory
 *     (pageable or pinned; the call copies it to the GPU and back) or DEVICE
 *     memory of the current CUDA device (used in place).  The kind is found
 *     with cudaPointerGetAttributes;
 *   - returns a pa_status code and never throws or aborts;
 *   - is synchronous (returns after the results are in place) unless
 *     opts->async_device is set and every buffer is device memory.
 * There is no CPU fallback: with no usable GPU every call returns
 * PA_ERR_NO_DEVICE.
 *
 * Citations name the reference entry point each function replaces
 * (file:line within the reference project).
 */
#ifndef PA_GPU_H
#define PA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pa_status {
  PA_OK = 0,
  PA_ERR_ARG = 1,       /* invalid argument (null buffer, k out of range, bad shift, ...) */
  PA_ERR_OOM = 2,       /* device or pinned memory could not be allocated */
  PA_ERR_CUDA = 3,      /* a CUDA runtime call failed; see pa_last_error_message() */
  PA_ERR_TIMEOUT = 4,   /* a bounded device-side wait gave up; results are undefined */
  PA_ERR_NO_DEVICE = 5  /* no CUDA device is usable */
} pa_status;

typedef struct pa_opts {
  void* stream;      /* cudaStream_t to run on; NULL means the legacy default stream */
  int async_device;  /* 1: if every buffer is device memory, return once the work is
                        enqueued; bounded-wait failures are then reported by
                        pa_stream_check(stream) */
  int digit_bits;    /* radix digit width of the LSD sorts: 0 or 8 (the
                        reference's PowerOfTwoRadix = 256; one pass per key
                        byte) or 11 (2048 bins: 3 passes for 32-bit keys, 6 for
                        64-bit ones; same result) */
  int reserved[4];   /* must be zero */
} pa_opts;

/* Human-readable name of a status code. */
const char* pa_status_string(int status);
/* Detail of the most recent failure on the calling thread ("" if none). */
const char* pa_last_error_message(void);
/* 1 if a CUDA device is usable from this process, else 0. */
int pa_device_available(void);
/* Synchronises `stream` and reports (then clears) any bounded-wait failure
 * raised by earlier async_device calls on it. */
int pa_stream_check(void* stream);
/* Releases the cached device and pinned workspaces of every stream. */
int pa_release_workspaces(void);

/* ---- LSD radix sort ------------------------------------------------------
 * Stable ascending sort of keys[0, n) in place.  tmp is caller scratch of n
 * keys whose contents are clobbered; tmp == NULL lets the library use its
 * own scratch.  The digit histograms of every pass are computed in one read
 * of the keys before the digit passes.
 *
 * pa_sort_u32 replaces ParallelAlgorithms::SortRadixPar(unsigned* a,
 *   unsigned* tmp_work_buff, size_t a_size, size_t parallelThreshold)
 *   (RadixSortLsdParallel.h:367) and, with tmp == NULL,
 *   SortRadixPar(unsigned* a, size_t a_size, size_t parallelThreshold)
 *   (RadixSortLsdParallel.h:340), and SortRadixInnerPar<256,8>
 *   (RadixSortLsdParallel.h:215).
 * pa_sort_u64 / pa_sort_f32 / pa_sort_kv_* have no reference counterpart
 *   (the reference sorts only unsigned 32-bit keys, RadixSortLsdParallel.h:216);
 *   they are additive overloads.  Float keys sort by IEEE total order
 *   (-0.0 before +0.0); payloads move with their keys, and equal keys keep
 *   their input order.
 */
int pa_sort_u32(uint32_t* keys, uint32_t* tmp, size_t n, const pa_opts* opts);
int pa_sort_u64(uint64_t* keys, uint64_t* tmp, size_t n, const pa_opts* opts);
int pa_sort_f32(float* keys, float* tmp, size_t n, const pa_opts* opts);
int pa_sort_kv_u32(uint32_t* keys, uint32_t* vals, uint32_t* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts);
int pa_sort_kv_u64(uint64_t* keys, uint32_t* vals, uint64_t* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts);
int pa_sort_kv_f32(float* keys, uint32_t* vals, float* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts);

/* Sorts a[0, n) and leaves the sorted keys in BOTH a and b, which is the end
 * state of RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase(a, b, a_size)
 * (RadixSortLsdParallel.h:86-106) and of the intended (the reference's body
 * is commented out, :503) RadixSortLSDPowerOf2RadixParallel_unsigned_TwoPhase_DeRandomize
 * (RadixSortLsdParallel.h:491). */
int pa_sort_two_phase_u32(uint32_t* a, uint32_t* b, size_t n, const pa_opts* opts);

/* Profiling form of the sorts above (key_kind: PA_KEY_U32 / PA_KEY_U64 /
 * PA_KEY_F32; vals / tmp_vals may be NULL): same result, always synchronous,
 * and phase_ms[i] receives the device time in milliseconds of each kernel,
 * from CUDA events recorded between the launches: [0] the one-read digit
 * histogram, [1] the bin-offset scan, [2 + p] digit pass p (one per
 * digit), [2 + passes] the final copy.  phase_cap bounds the entries written.
 * GPU form of the per-phase timers the reference keeps commented out in its
 * sort (RadixSortLsdParallel.h:255-258, 287, 307-308). */
enum { PA_KEY_U32 = 0, PA_KEY_U64 = 1, PA_KEY_F32 = 2 };
int pa_sort_timed(int key_kind, void* keys, void* tmp, uint32_t* vals, uint32_t* tmp_vals, size_t n,
                  float* phase_ms, int phase_cap, const pa_opts* opts);

/* Allocation-free sort of 32-bit keys.  No counterpart in the reference.
 * For callers that must not allocate GPU memory -- code inside a framework
 * whose caching allocator owns all device memory, or latency-critical loops
 * where cudaMalloc's device-wide synchronisation would stall other streams.
 * Same result as pa_sort_u32, but keys and tmp (n keys each) must both be
 * device memory of the current device, and n is at most 4,194,304: the call
 * works in a fixed ~4 MiB scratch array compiled into the library (held by
 * every GPU that loads it) instead of a workspace it allocates.  The first
 * call on a device looks up that array's device address; make it before any
 * stream capture.  All calls share the array: calls whose work overlaps on
 * the GPU (other streams or threads) race, so issue them one at a time.
 * Synchronous; returns PA_ERR_ARG for host buffers or n above the limit. */
int pa_sort_u32_noalloc(uint32_t* keys, uint32_t* tmp, size_t n, const pa_opts* opts);

/* In-place sort of 32-bit keys with bounded device scratch: replaces
 * parallel_hybrid_inplace_msd_radix_sort(a, a_size) (RadixSortMsdParallel.h:291),
 * whose point is to sort without a second array of n keys.  Besides the keys
 * (for host keys: their device copy) the call holds scratch_keys keys of
 * device scratch (0 = 2^24 = 64 MiB, at least 2^16) and about 1.4 bytes per
 * scratch key + 8 MiB of tables (31 MiB at the default), whatever n is.  Up to scratch_keys keys it is
 * the LSD sort with the scratch as its second buffer; above, ranges are
 * partitioned in place by a digit (top digit first) through the scratch and
 * buckets of at most scratch_keys keys are sorted in groups by the batched
 * segmented sort.  Same sorted array as pa_sort_u32.  For keys above 2^24
 * the call waits for the device once per partitioned range (it reads the
 * range's digit counts back to plan the buckets).  If it fails part way,
 * device keys may be left partly moved (keys in flight through the scratch
 * are not put back); host keys are left as they were. */
int pa_sort_u32_inplace(uint32_t* keys, size_t n, size_t scratch_keys, const pa_opts* opts);

/* ---- digit histograms ----------------------------------------------------
 * pa_hist_byte_components_u32: out[d * 256 + b] = number of keys in a[0, n)
 *   whose byte d (d = 0..3, least significant first) equals b, from one read.
 *   Replaces HistogramByteComponentsParallel<256,8>(a, l, r)
 *   (HistogramParallel.h:249) with a = inArray + l, n = r - l + 1.
 * pa_hist_one_byte_u32: out[b] = number of keys with ((key >> shift) & 255) == b;
 *   shift must be < 32.  Replaces HistogramOneByteComponentParallel<256,8>(a,
 *   l, r, shiftRight) (HistogramParallel.h:535).
 * pa_hist_u8: out[b] = number of bytes equal to b.  Replaces
 *   HistogramOneByteComponentParallel<256>(unsigned char a[], l, r)
 *   (HistogramParallel.h:17) and its _2/_3/_4 variants (:58,:117,:184).
 * pa_hist_quanta_u32: out[q * 256 + b] for q in [0, quanta): number of i in
 *   [l, r] (r inclusive) with i / work_quanta == q and byte which_byte of a[i]
 *   equal to b.  a is the array base (index 0).  Replaces
 *   HistogramByteComponentsQCPar<256,8> (HistogramParallel.h:444).
 * pa_start_of_bins_u32: out[q * 256 + b] = the output index of quantum q's
 *   first key of bin b for byte `digit` over a[0, n).  Replaces
 *   ComputeStartOfBinsPar<256,8> (RadixSortLsdParallel.h:108).
 * out may be host or device memory; it is overwritten.
 */
int pa_hist_byte_components_u32(const uint32_t* a, size_t n, uint64_t* out, const pa_opts* opts);
int pa_hist_one_byte_u32(const uint32_t* a, size_t n, unsigned shift, uint64_t* out, const pa_opts* opts);
int pa_hist_u8(const uint8_t* a, size_t n, uint64_t* out, const pa_opts* opts);
int pa_hist_quanta_u32(const uint32_t* a, size_t l, size_t r, size_t work_quanta, size_t quanta,
                       unsigned which_byte, uint64_t* out, const pa_opts* opts);
int pa_start_of_bins_u32(const uint32_t* a, size_t n, size_t work_quanta, size_t quanta, unsigned digit,
                         uint64_t* out, const pa_opts* opts);

/* ---- radix select ---------------------------------------------------------
 * pa_select_u32 / pa_select_u64: *out = the k-th smallest (0-based) key of
 *   a[0, n); a is not modified.  Requires k < n.
 * pa_select_radix_u32: the reference's contract, SelectRadix(a, start,
 *   length, k) (RadixSelect.h:139; SelectRadix(a, length, k) is start = 0,
 *   RadixSelect.h:157): the (k - start)-th smallest of a[start, start + length)
 *   with k an absolute index in that range, returned in *out AND left at
 *   a[k]: a[k] is swapped with the first element of the range that holds the
 *   answer, so the range stays a permutation of its input.  The reference
 *   rearranges the range further (its in-place partitioning); here no other
 *   element moves.
 */
int pa_select_u32(const uint32_t* a, size_t n, size_t k, uint32_t* out, const pa_opts* opts);
int pa_select_u64(const uint64_t* a, size_t n, size_t k, uint64_t* out, const pa_opts* opts);
int pa_select_radix_u32(uint32_t* a, size_t start, size_t length, size_t k, uint32_t* out, const pa_opts* opts);

/* ---- sum ------------------------------------------------------------------
 * *out = sum of a[0, n) modulo 2^64 (exact; 32-bit inputs cannot wrap below
 * 2^32 elements).  Replaces SumParallelNonRecursive(unsigned[], l, r)
 * (SumParallel.h:261), SumParallelNonRecursive(unsigned long long[], l, r)
 * (:285), SumParallel(unsigned long long[], l, r) (:162) and, reinterpreted as
 * signed, SumParallel<unsigned>(...) -> long long (:207), with a = in_array + l
 * and n = r - l.  An empty range sums to 0.  out may be host or device memory.
 */
int pa_sum_u32(const uint32_t* a, size_t n, uint64_t* out, const pa_opts* opts);
int pa_sum_u64(const uint64_t* a, size_t n, uint64_t* out, const pa_opts* opts);

/* Element kinds of the typed sums. */
enum {
  PA_ELEM_U8 = 0, PA_ELEM_I8 = 1, PA_ELEM_U16 = 2, PA_ELEM_I16 = 3, PA_ELEM_U32 = 4, PA_ELEM_I32 = 5,
  PA_ELEM_U64 = 6, PA_ELEM_I64 = 7, PA_ELEM_F32 = 8, PA_ELEM_F64 = 9
};
/* *out = sum of a[0, n) with every element converted to a 64-bit integer
 * first (unsigned kinds zero-extended, signed kinds sign-extended, float and
 * double truncated toward zero), modulo 2^64: the two's-complement bits of
 * the reference's template SumParallel<_Type>(in_array, l, r) -> long long
 * (SumParallel.h:207-237), with a = in_array + l, n = r - l.  Float values
 * outside the 64-bit range (undefined behaviour in the reference) saturate. */
int pa_sum_typed(const void* a, size_t n, int elem_kind, uint64_t* out, const pa_opts* opts);
/* Per-chunk sums: chunk_sums[i] = sum of a[i * chunk, min(n, (i + 1) * chunk))
 * for the ceil(n / chunk) chunks, *out = their total, each modulo 2^64
 * (elements widened as in pa_sum_typed).  Replaces the caller-buffer
 * overloads SumParallelNonRecursive(in_array, l, r, sum_array,
 * parallelThreshold) (SumParallel.h:419, :442), which leave each task's sum
 * in sum_array, with chunk = parallelThreshold. */
int pa_sum_chunked(const void* a, size_t n, int elem_kind, size_t chunk, uint64_t* chunk_sums, uint64_t* out,
                   const pa_opts* opts);

/* ---- batched segmented sort -----------------------------------------------
 * No reference counterpart (the reference sorts one array per call).  Sorts
 * every segment [seg_offsets[i], seg_offsets[i + 1]) of one uint32 key array
 * independently (stable, ascending; each segment's result equals
 * pa_sort_u32 on it): a persistent kernel fed by a device work queue sorts
 * the segments of up to `small_cutoff` keys inside one CTA's shared memory
 * and counts the longer ones' digits, then (8-bit digits) one onesweep launch
 * per digit pass covers every longer segment (11-bit digits: the passes run
 * as items of the persistent kernel).  A plan is built once
 * for a segmentation and replayed (through a captured CUDA graph when
 * use_graph is set); pa_segmented_sort_u32 is the one-shot form.  Segments
 * must be shorter than 2^30 keys.
 */
typedef struct pa_segsort_config {
  int small_cutoff;  /* 0 (= 4096), 2048, 4096 or 8192 keys */
  int tile_keys;     /* onesweep tile of 11-bit plans: 0 (= 8192), 4096 or 8192 (8-bit
                        plans' pass launches use the plain sort's 6144-key tile) */
  int digit_bits;    /* 0 or 8 (four passes), or 11 (three passes of 2048 bins;
                        the result is copied back from tmp) */
  int use_graph;     /* 1: plan runs replay a captured CUDA graph */
  int reserved[4];   /* must be zero */
} pa_segsort_config;
typedef struct pa_segsort_plan pa_segsort_plan;

/* seg_offsets: num_segments + 1 non-decreasing offsets (host or device). */
int pa_segsort_plan_create(const uint64_t* seg_offsets, size_t num_segments, const pa_segsort_config* cfg,
                           pa_segsort_plan** plan);
/* keys, tmp: device buffers of the plan's total key count; sorted in keys.
 * With opts->async_device the call returns after the launch; then
 * pa_segsort_plan_sync(plan, stream) waits and reports bounded-wait failures. */
int pa_segsort_plan_run(pa_segsort_plan* plan, uint32_t* keys, uint32_t* tmp, const pa_opts* opts);
int pa_segsort_plan_sync(pa_segsort_plan* plan, void* stream);
int pa_segsort_plan_info(const pa_segsort_plan* plan, uint32_t* num_small, uint32_t* num_large, uint32_t* num_items);
int pa_segsort_plan_destroy(pa_segsort_plan* plan);
/* One-shot: keys may be host or device memory. */
int pa_segmented_sort_u32(uint32_t* keys, const uint64_t* seg_offsets, size_t num_segments,
                          const pa_segsort_config* cfg, const pa_opts* opts);

/* ---- serving loop ----------------------------------------------------------
 * No reference counterpart.  A server takes sort / select / histogram
 * requests from any thread as they arrive, admits them while their device
 * memory fits a configured HBM budget (and the memory the GPU reports free),
 * keeps their data device-resident while they run, overlaps requests on
 * several streams, and coalesces waiting 32-bit sorts into one batched
 * launch.  Results equal the plain entry points' (pa_sort_*, pa_select_*,
 * pa_hist_one_byte_*) on the same request.  Host buffers should be pinned
 * for copies to overlap; device buffers are used in place (sort) or read.
 */
enum { PA_REQ_SORT = 0, PA_REQ_SELECT = 1, PA_REQ_HISTOGRAM = 2 };

typedef struct pa_request {
  int op;            /* PA_REQ_SORT, PA_REQ_SELECT or PA_REQ_HISTOGRAM */
  int key_kind;      /* PA_KEY_U32 or PA_KEY_U64 */
  void* keys;        /* n keys (host or device); a sort leaves them sorted here */
  size_t n;
  uint64_t k;        /* select: 0-based rank */
  unsigned shift;    /* histogram: counts of (key >> shift) & 255 */
  uint64_t* result;  /* select: 1 word (the key, zero-extended); histogram: 256 counts (host) */
  int status;        /* written by the server: -1 while pending, then a pa_status */
  int unit_size;     /* written by the server: requests that shared its launch (1 = alone) */
  double t_submit, t_admit, t_done;  /* written by the server: seconds, monotonic clock */
  int internal_device;               /* written by the server */
} pa_request;

typedef struct pa_serve_config {
  size_t hbm_budget_bytes;  /* device memory the server may hold: 0 = 64 GiB */
  int max_inflight;         /* units on the device at once: 0 = 4 */
  int max_batch_requests;   /* 32-bit sorts coalesced into one launch: 0 = 256 */
  int no_coalesce;          /* 1: every request runs alone */
  int num_streams;          /* 0 = 4 */
  int reserve_mib;          /* device memory (MiB, at most the budget) mapped into the
                               server's pool at creation, so that admissions do not wait
                               for the pool to map memory; 0 = map on demand */
  int join_max_keys_log2;   /* only requests of at most 2^this keys share units with
                               others; larger ones run alone: 0 = 20 */
  int unit_max_keys_log2;   /* keys of one shared unit at most 2^this: 0 = 22 */
  int reserved[1];          /* must be zero */
} pa_serve_config;
typedef struct pa_server pa_server;

int pa_server_create(const pa_serve_config* cfg, pa_server** server);
/* Non-blocking; the request must stay alive until it completes. */
int pa_server_submit(pa_server* server, pa_request* req);
/* Blocks until the request completes; returns its status. */
int pa_server_wait(pa_server* server, pa_request* req);
/* Blocks until every submitted request has completed. */
int pa_server_drain(pa_server* server);
/* out[0..8] = submitted, completed, rejected (over budget), units launched,
 * batched units, requests served in batches, peak device bytes held, and the
 * scheduler thread's microseconds spent enqueueing units and completing them
 * (count bounds how many are written). */
int pa_server_stats(pa_server* server, uint64_t* out, int count);
int pa_server_destroy(pa_server* server);

/* Byte-array counting sort, in place: replaces counting_sort_parallel(a,
 * a_size) (CountingSortParallel.h:81-91) and counting_sort_parallel_inner<256>
 * (:29-79): a one-read byte histogram, then a parallel fill of each value's
 * range. */
int pa_counting_sort_u8(uint8_t* a, size_t n, const pa_opts* opts);

/* dst = src sorted (stable, ascending); src is clobbered (used as the
 * scratch).  Replaces the radix-leaf merge sorts that LSD radix sort serves:
 * parallel_merge_sort_hybrid_radix(src, l, r, dst, srcToDst = true)
 * (ParallelMergeSort.h:287) and its _single_buffer form (:298); with
 * srcToDst = false, and parallel_linear_in_place_preventative_adaptive_sort
 * (:549), they sort in place, which is pa_sort_u32. */
int pa_sort_copy_u32(uint32_t* src, uint32_t* dst, size_t n, const pa_opts* opts);

/* Radix partition around the ascending indices k[0, k_len), in place:
 * replaces PartitionRadix(a, aLength, k[], kLength) (RadixPartition.h:152) and
 * its single-k and sub-range forms (:92, :124, :165).  Afterwards, for every
 * k[i], a[k[i]] is the k[i]-th smallest key, no key before it is larger and
 * no key after it is smaller -- the reference's contract.  The order of the
 * other keys inside each part differs from the reference's (an artefact of
 * its serial in-place swap loop): with at most 6 k the keys are split into
 * the buckets the k-th smallest values define (one select per k, then one
 * bucket pass; order inside a bucket unspecified), with more k the whole
 * array comes out sorted (one sort partitions around every k at once). */
int pa_partition_radix_u32(uint32_t* a, size_t n, const size_t* k, size_t k_len, const pa_opts* opts);

/* Failure-detection self-test (no reference counterpart; the reference has
 * no waits that can run out).  Runs one onesweep digit pass of a small sort
 * in which a tile's decoupled look-back polls a predecessor's status word
 * that is never published, with the poll budget lowered to spin_limit, and
 * returns what a sort whose wait ran out returns: PA_ERR_TIMEOUT (the
 * expected result), with the device left usable.  The wait is bounded like
 * every wait in this library; nothing faults or hangs. */
int pa_selftest_wait_expiry(unsigned spin_limit);

/* 256-bin histogram of (key >> shift) & 255 over 64-bit keys (no reference
 * counterpart; the 32-bit form is pa_hist_one_byte_u32). shift < 64. */
int pa_hist_one_byte_u64(const uint64_t* a, size_t n, unsigned shift, uint64_t* out, const pa_opts* opts);

#ifdef __cplusplus
}
#endif

#endif /* PA_GPU_H */
