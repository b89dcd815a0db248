// Host-side launchers of the radix hot-path kernels.  Each launcher enqueues
// work on `stream` and returns a cudaError_t from the launch; none of them
// synchronises.  The C ABI (pa_capi.cu) owns workspace, pointer
// classification and error reporting.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <cuda_runtime.h>

namespace pa {

constexpr int kMaxPasses = 8;  // 64-bit keys, 8-bit digits (11-bit digits: 6 passes)

// Digit widths of the LSD sorts: 8 bits (the reference's PowerOfTwoRadix =
// 256) or 11 bits (2048 bins; three passes for 32-bit keys).
inline int sort_passes(int key_bytes, int radix_bits) { return (8 * key_bytes + radix_bits - 1) / radix_bits; }

// Per-pass control computed on the device from the digit histograms, so the
// host never waits for them: a pass whose digit puts every key in one bin is
// the identity permutation and is skipped; the ping-pong direction and the
// float transform (applied on the first executed pass's loads, undone on the
// last executed pass's stores) follow from the passes that remain.
struct PassCtrl {
  uint32_t skip;
  uint32_t src_is_tmp;
  uint32_t transform_in;
  uint32_t transform_out;
};
struct SortCtrl {
  PassCtrl pass[kMaxPasses];
  uint32_t final_in_tmp;
  uint32_t executed;
};

// Records `message` as the calling thread's pa_last_error_message() and
// returns `status` (for entry points outside pa_capi.cu).
int record_error(int status, const char* message);

// Device properties the launchers size grids with (filled once per device).
struct DeviceInfo {
  int device = -1;
  int sm_count = 0;
  size_t max_smem_optin = 0;
};
const DeviceInfo& device_info();

// Lets `func` use `bytes` of dynamic shared memory on the current device:
// cudaFuncSetAttribute once per (device, function), thread-safe.
cudaError_t ensure_dynamic_smem(const void* func, size_t bytes);
template <typename F>
cudaError_t ensure_dynamic_smem(F* func, size_t bytes) {
  return ensure_dynamic_smem(reinterpret_cast<const void*>(func), bytes);
}

// ---- histograms (pa_histogram.cu) -----------------------------------------
// Counts of `num_digits` digits of width `radix_bits` (digit d taken at bit
// shift0 + d * shift_step of the ordered key) over keys[0, n), ADDED into
// out[num_digits][1 << radix_bits] (unsigned 64-bit).  key_bytes is 1, 4 or 8.
cudaError_t launch_digit_counts(const void* keys, size_t n, int key_bytes, int num_digits, int radix_bits,
                                uint32_t shift0, uint32_t shift_step, bool is_float, unsigned long long* out,
                                cudaStream_t stream);

// The histogram of a 32-bit sort with 8-bit digits that also prepares its
// first digit pass: one read of keys[0, n) (16-byte aligned, n < 2^30)
// ADDS the counts of the four bytes into out[4][256] as launch_digit_counts
// does, and, for the first pass's tiles of tile_keys keys (4096, 6144 or
// 8192), writes
//   tile_prefix[t][b]  keys of byte-0 value b in the earlier tiles of t's chunk,
//   chunk_excl[c][b]   keys of byte-0 value b in the chunks before c,
// where chunk c is the tiles [c * tpc, (c + 1) * tpc) (*tpc set here), so
// that the pass finds each tile's offsets without a look-back.  chunk_tot
// ([kTileCountMaxChunks][256]) is scratch; *ticket starts at zero.
constexpr int kTileCountMaxChunks = 160;
bool tile_counts_supported(size_t tile_keys);
cudaError_t launch_tile_counts(const uint32_t* keys, size_t n, size_t tile_keys, bool is_float,
                               unsigned long long* out, uint32_t* tile_prefix, uint32_t* chunk_tot,
                               uint32_t* chunk_excl, uint32_t* ticket, uint32_t* tpc, cudaStream_t stream);

// Several arrays' 256-bin histograms of (key >> shift) & 255 in one launch
// (the serving loop's coalesced histogram requests).  jobs[0, njobs) in
// device memory; job j's keys are split into kHistJobChunk-key chunks
// numbered from first_chunk on (first_chunk ascending, total_chunks in all);
// counts are ADDED into each job's out[256].  key_bytes 4 or 8.
constexpr uint32_t kHistJobChunk = 64 * 1024;
struct HistJob {
  const void* keys;
  unsigned long long n;
  unsigned long long* out;
  uint32_t shift;
  uint32_t first_chunk;
};
cudaError_t launch_digit_counts_multi(const HistJob* jobs, int njobs, uint32_t total_chunks, int key_bytes,
                                      cudaStream_t stream);

// Byte counting sort's second step: a[0, n) = each byte value v repeated
// counts[v] times, in value order (counts: 256 words summing to n).
cudaError_t launch_counting_fill(uint8_t* a, size_t n, const unsigned long long* counts, cudaStream_t stream);

// Counts of byte `which_byte` of the keys with absolute index in [l, r)
// (keys points at index l), per work quantum (quantum = index / work_quanta),
// ADDED into out[quantum][256].
cudaError_t launch_quanta_counts(const uint32_t* keys, size_t l, size_t r, size_t work_quanta,
                                 uint32_t which_byte, unsigned long long* out, cudaStream_t stream);

// start_of_bins[q][b] = sum of all bins < b over all quanta + sum of bin b over
// quanta < q, from counts[q][256] (RadixSortLsdParallel.h:128-156 on device).
// start_of_bins must hold quanta * 256 + 256 words (the tail holds bin totals).
cudaError_t launch_quanta_start_of_bins(const unsigned long long* counts, size_t quanta,
                                        unsigned long long* start_of_bins, cudaStream_t stream);

// Exclusive scan of each pass's digit counts into bin_start, and the pass
// control block (skips, ping-pong direction, float transform placement).
cudaError_t launch_scan_digits(const unsigned long long* counts, int passes, int radix_bits, size_t n,
                               bool is_float, bool allow_skip, unsigned long long* bin_start, SortCtrl* ctrl,
                               cudaStream_t stream);

// ---- onesweep digit pass (pa_onesweep.cu) --------------------------------
struct OnesweepArgs {
  void* keys_a;  // the caller's key buffer
  void* keys_b;  // the scratch key buffer
  uint32_t* vals_a;
  uint32_t* vals_b;
  size_t n;
  uint32_t shift;
  int pass;
  int is_float;
  const unsigned long long* bin_start;  // this pass's 256 exclusive bin starts
  void* status;                         // this pass's tiles * 256 look-back words
  uint32_t* tile_counter;               // this pass's tile ticket
  const SortCtrl* ctrl;
  uint32_t* err;
  uint32_t spin_limit = 0;  // look-back polls before a tile gives up; 0 = kSpinLimit
  size_t max_ctas = 0;      // CTAs launched; 0 = one per tile (only the wait-expiry self-test sets it)
  int radix_bits = 8;       // digit width: 8 (256 bins) or 11 (2048 bins)
  // 8-bit passes only: the keys to move counted on the device (at most n;
  // the grid is sized for n, tiles past the count exit), and a bound on the
  // output positions when the output is not an n-key array (0: n)
  const unsigned long long* n_dev = nullptr;
  size_t out_n = 0;
  // First pass of a 32-bit keys-only sort: the tiles' offsets prepared by
  // launch_tile_counts (each tile reads its two rows instead of looking back).
  const uint32_t* tile_prefix = nullptr;
  const uint32_t* chunk_excl = nullptr;
  uint32_t tiles_per_chunk = 0;
};

// Tile geometry chosen for (key_bytes, has_vals, radix_bits); the workspace
// is sized with it.
size_t onesweep_tile_keys(int key_bytes, bool has_vals, int radix_bits = 8);
// Bytes of one look-back status word for n keys (4 when n < 2^30, else 8).
size_t onesweep_status_bytes(size_t n);
cudaError_t launch_onesweep_pass(const OnesweepArgs& a, int key_bytes, bool has_vals, cudaStream_t stream);

// Whole sort of n <= small_sort_max_keys(key_bytes, has_vals) keys (and
// payloads) by one CTA in shared memory, in place.
size_t small_sort_max_keys(int key_bytes, bool has_vals);
cudaError_t launch_small_sort(void* keys, uint32_t* vals, size_t n, int key_bytes, bool is_float, cudaStream_t stream);

// Copies `nruns` (at most 65535) runs of elements: run r moves
// src[runs[3r], +runs[3r + 1]) to dst[runs[3r + 2], ...) (element offsets
// and counts; runs in device memory; max_run: the longest run, for the grid).
// key_bytes 4 or 8.
cudaError_t launch_gather_runs(const void* src, void* dst, const unsigned long long* runs, size_t nruns,
                               size_t max_run, int key_bytes, cudaStream_t stream);

// ---- pipelined host-buffer sort of 32-bit keys (pa_pipeline.cu) -----------
// Chunks sorted on their top 16 bits, then 16-bit buckets gathered from
// every chunk and sorted on their low 16 bits into their final places.
constexpr int kMaxChunkRuns = 8;
struct ChunkRuns {
  unsigned long long lo[kMaxChunkRuns];  // first key of each chunk in the source buffer
  int count;
};
// starts[0, 65536]: where each 16-bit bucket starts in keys[0, n) (sorted on
// the top 16 bits; n < 2^32); top_start: the 256 exclusive top-byte starts.
cudaError_t launch_bucket_bounds(const uint32_t* keys, size_t n, const unsigned long long* top_start, uint32_t* starts,
                                 cudaStream_t stream);
// From the chunks' starts ([num_chunks][65537]): tot[0, 65536) each
// bucket's keys, pos[0, 65536] the buckets' global starts; summary[0, 256)
// keys per top byte, summary[256, 512) the largest 16-bit bucket of each.
cudaError_t launch_bucket_totals(const uint32_t* starts, int num_chunks, uint32_t* tot, unsigned long long* pos,
                                 unsigned long long* summary, cudaStream_t stream);
// Buckets [first_bucket, + num_buckets), none larger than max_bucket_keys
// (at most bucket_sort_max_keys()): gathered from src, sorted, written to
// dst[pos[b], pos[b + 1]).
size_t bucket_sort_max_keys();
cudaError_t launch_bucket_sort(const uint32_t* src, const ChunkRuns& chunks, const uint32_t* starts,
                               const unsigned long long* pos, uint32_t first_bucket, uint32_t num_buckets,
                               size_t max_bucket_keys, uint32_t* dst, uint32_t* err, cudaStream_t stream);

// Copies the result back into the caller's buffers when the executed passes
// left it in the scratch buffers (device-side decision from SortCtrl).
cudaError_t launch_final_copy(void* keys_a, const void* keys_b, uint32_t* vals_a, const uint32_t* vals_b,
                              size_t n, int key_bytes, const SortCtrl* ctrl, cudaStream_t stream);

// ---- whole sorts on device buffers (pa_capi.cu) ---------------------------
// Per-call scratch of a device-resident sort: digit counts, tile tickets and
// look-back words (zeroed by enqueue_sort), bin starts, pass control.
struct SortScratch {
  int radix_bits;
  int passes;
  unsigned long long* counts;
  uint32_t* tile_ctr;
  char* status;
  unsigned long long* bin_start;
  SortCtrl* ctrl;
  char* zero_begin;
  size_t zero_bytes;
  size_t tiles;
  size_t status_bytes;
  // launch_tile_counts' tables (32-bit keys only, 8-bit digits, n < 2^30;
  // otherwise null): the first pass then needs no look-back
  uint32_t* tile_prefix;
  uint32_t* chunk_tot;
  uint32_t* chunk_excl;
  uint32_t* tc_ticket;  // zeroed with the counts
};
size_t sort_scratch_bytes(size_t n, int key_bytes, bool has_vals, int radix_bits = 8);
// Carves the scratch from `base` (nullptr measures); returns its size.
size_t sort_scratch_layout(char* base, size_t n, int key_bytes, bool has_vals, SortScratch* s, int radix_bits = 8);
// Enqueues the whole sort (memset, histogram, scan, passes, final copy) of
// device buffers on `stream`; `mark`, when set, runs between launches.
cudaError_t enqueue_sort(const SortScratch& s, void* d_keys, void* d_tmp, uint32_t* d_vals, uint32_t* d_tvals,
                         size_t n, int key_bytes, bool is_float, uint32_t* err, cudaStream_t stream,
                         const std::function<cudaError_t()>& mark = {});

// ---- sum (pa_sum.cu) -------------------------------------------------------
// Element kinds of the sums (the values of pa_gpu.h's PA_ELEM_*).
enum : int {
  kElemU8 = 0, kElemI8 = 1, kElemU16 = 2, kElemI16 = 3, kElemU32 = 4, kElemI32 = 5,
  kElemU64 = 6, kElemI64 = 7, kElemF32 = 8, kElemF64 = 9
};
// Bytes of one element of `elem_kind` (0 for an unknown kind).
int sum_elem_bytes(int elem_kind);
// out = sum of keys[0, n), each element widened to 64 bits, modulo 2^64.
// partials holds sum_partials_needed() words and ticket one zeroed word; a
// bulk-copy wait that gives up raises a bit in *err.
size_t sum_partials_needed();
cudaError_t launch_sum(const void* keys, size_t n, int elem_kind, unsigned long long* partials, uint32_t* ticket,
                       unsigned long long* out, uint32_t* err, cudaStream_t stream);
// sums[c] = sum of chunk c = keys[c * chunk, min(n, (c + 1) * chunk)) and
// *total (zeroed by the caller) += every chunk's sum, modulo 2^64.
cudaError_t launch_sum_chunks(const void* keys, size_t n, int elem_kind, size_t chunk, unsigned long long* sums,
                              unsigned long long* total, cudaStream_t stream);

// ---- partition around a few k (pa_partition.cu) ---------------------------
// Most pivots one partition handles: 2 * 7 + 1 = 15 buckets fit 4 bits.
constexpr int kPartitionMaxPivots = 7;
// out[0, n) = in[0, n) arranged in the 2m + 1 buckets defined by the m sorted
// pivots (device): below pivot 0, equal to it, between pivots 0 and 1, ...,
// above the last one; the order inside a bucket is not specified.  scratch
// holds partition_scratch_words(n, m) words.  in and out must not overlap.
size_t partition_scratch_words(size_t n, int m);
cudaError_t launch_partition(const uint32_t* in, uint32_t* out, size_t n, const uint32_t* pivots, int m,
                             unsigned long long* scratch, cudaStream_t stream);

// ---- in-place partition by one digit (pa_inplace.cu) -----------------------
// Per-bucket cursors and the current round's plan of an in-place partition.
struct InplaceState {
  unsigned long long w[256];       // write cursor
  unsigned long long r[256];       // end of the unread part
  unsigned long long cursor[256];  // the round's scatter cursors
  unsigned long long cnt[2][256];  // digit counts of the keys in hand in each half
  unsigned long long run_src[256], run_len[256], run_dst[256];  // the runs of the next copy
  unsigned long long hand[2];      // keys in hand in each half
  unsigned long long total;        // keys scattered by the round
  unsigned long long run_base, run_keys;  // the copy's destination range
  SortCtrl ctrl;                   // the scatter pass's control (one pass, keys_a -> keys_b)
  uint32_t ticket;                 // the scatter pass's tile ticket
};
// keys[0, n) arranged in place in the buckets of the digit (key >> shift) &
// 255 (bucket order; order inside a bucket unspecified), given hist, the
// range's 256 digit counts (device).  c0, c1: scratch halves of `half` keys
// each; st: device state; status: inplace_status_bytes(n, half) bytes of
// look-back words.  Enqueues ceil(n / half) + 1 rounds of five launches;
// nothing is read back.
size_t inplace_status_bytes(size_t n, size_t half);
cudaError_t launch_inplace_partition(uint32_t* keys, size_t n, uint32_t shift, const unsigned long long* hist,
                                     uint32_t* c0, uint32_t* c1, size_t half, InplaceState* st, void* status,
                                     uint32_t* err, cudaStream_t stream);

// ---- select (pa_select.cu) -------------------------------------------------
struct SelectState;
size_t select_state_bytes();
// k-th smallest (0-based) of keys[0, n) into *out (device).  cand holds
// cand_cap keys; work is select_state_bytes() of scratch (initialised by the
// launcher).
cudaError_t launch_select(const void* keys, size_t n, size_t k, int key_bytes, void* cand, size_t cand_cap,
                          void* work, void* out, uint32_t* err, cudaStream_t stream);
// *idx = k when keys[k] == *value, else the smallest index of a key equal to
// *value in keys[0, n) (all ones if none).
cudaError_t launch_find_key(const uint32_t* keys, size_t n, size_t k, const uint32_t* value, unsigned long long* idx,
                            cudaStream_t stream);
// Swaps keys[k] and keys[*idx] unless *idx is k or not below n.
cudaError_t launch_swap_key(uint32_t* keys, size_t n, size_t k, const unsigned long long* idx, cudaStream_t stream);

}  // namespace pa
