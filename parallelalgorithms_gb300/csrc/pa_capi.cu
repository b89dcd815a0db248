// The C ABI declared in include/pa_gpu.h.
//
// Responsibilities: argument checks, host/device classification of every
// buffer, the per-stream device workspace (grow-only, reused across calls),
// host<->device copies for host buffers, launching the kernel sequence of
// each operation, and turning CUDA errors and device-side bounded-wait
// failures into pa_status codes.  Calls are serialised by one mutex; work on
// different streams uses different workspaces.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "pa_gpu.h"
#include "pa_common.cuh"
#include "pa_kernels.cuh"
#include "pa_segmented.cuh"

namespace pa {

// Lays out sub-buffers in one allocation, 256-byte aligned.  Run once with
// base == nullptr to measure, then with the real base.
struct Carve {
  char* base;
  size_t off = 0;
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* p = reinterpret_cast<T*>(base + off);
    off += count * sizeof(T);
    return p;
  }
};

namespace {

thread_local std::string g_last_error;

int set_error(int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return set_error(PA_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  }
  return set_error(PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define PA_CUDA(call)                                      \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);    \
  } while (0)

constexpr int kMaxEvents = 16;

// PartitionRadix with at most this many k runs one select per k and one
// bucket pass; with more it sorts (a select costs about a sixth of a sort).
constexpr size_t kPartitionSelectMax = 6;
static_assert(kPartitionSelectMax <= (size_t)kPartitionMaxPivots, "the bucket pass holds every pivot");

constexpr int kPipeChunks = 8;   // host-buffer sort: copy-in chunks
static_assert(kPipeChunks <= kMaxChunkRuns, "the bucket sort's chunk table holds every chunk");
constexpr int kPipeGroups = 10;  // host-buffer sort: bucket groups sorted and copied out in turn

struct Workspace {
  char* dev = nullptr;
  size_t dev_cap = 0;
  uint32_t* err = nullptr;       // device error word, zero between calls
  uint32_t* err_host = nullptr;  // pinned mirror for reading it back
  cudaEvent_t ev[kMaxEvents] = {};  // phase timing (created on first use)
  // pipelined host-buffer sort (created on first use)
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t pipe_ev[kPipeChunks + kPipeGroups + 2] = {};
  void* pipe_host = nullptr;                // pinned staging of the pipelined sort (grow-only)
  size_t pipe_host_cap = 0;
};

std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, Workspace> g_ws;

int device_ready() {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(PA_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
  }
  return PA_OK;
}

int get_workspace(cudaStream_t stream, Workspace** out) {
  int dev = 0;
  PA_CUDA(cudaGetDevice(&dev));
  Workspace& ws = g_ws[{dev, stream}];
  if (!ws.err) {
    PA_CUDA(cudaMalloc(&ws.err, 256));
    PA_CUDA(cudaMemset(ws.err, 0, 256));
    PA_CUDA(cudaMallocHost(&ws.err_host, sizeof(uint32_t)));
  }
  *out = &ws;
  return PA_OK;
}

int ensure_dev(Workspace* ws, cudaStream_t stream, size_t bytes) {
  if (bytes <= ws->dev_cap) return PA_OK;
  PA_CUDA(cudaStreamSynchronize(stream));
  if (ws->dev) PA_CUDA(cudaFree(ws->dev));
  ws->dev = nullptr;
  ws->dev_cap = 0;
  const size_t cap = bytes + bytes / 8 + (1u << 20);
  cudaError_t e = cudaMalloc(&ws->dev, cap);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(PA_ERR_OOM, "device workspace of %zu bytes: %s", cap, cudaGetErrorString(e));
  }
  ws->dev_cap = cap;
  return PA_OK;
}

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    int dev = 0;
    cudaGetDevice(&dev);
    return at.device == dev;
  }
  return false;
}

cudaStream_t stream_of(const pa_opts* o) { return o ? static_cast<cudaStream_t>(o->stream) : (cudaStream_t)0; }

int check_opts(const pa_opts* o) {
  if (!o) return PA_OK;
  if (o->digit_bits != 0 && o->digit_bits != 8 && o->digit_bits != 11)
    return set_error(PA_ERR_ARG, "digit_bits must be 0, 8 or 11 (got %d)", o->digit_bits);
  for (int r : o->reserved)
    if (r != 0) return set_error(PA_ERR_ARG, "pa_opts.reserved must be zero");
  return PA_OK;
}

// Synchronises and reports a device-side bounded-wait failure, if any.
int finish(Workspace* ws, cudaStream_t stream, bool async_ok) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  if (async_ok) return PA_OK;
  PA_CUDA(cudaMemcpyAsync(ws->err_host, ws->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  PA_CUDA(cudaStreamSynchronize(stream));
  const uint32_t err = *ws->err_host;
  if (err) {
    PA_CUDA(cudaMemsetAsync(ws->err, 0, sizeof(uint32_t), stream));
    PA_CUDA(cudaStreamSynchronize(stream));
    return set_error(PA_ERR_TIMEOUT, "device-side bounded wait gave up (code 0x%x); results are undefined", err);
  }
  return PA_OK;
}

// ---------------------------------------------------------------------------
// Sort
// ---------------------------------------------------------------------------
// Host-buffer sorts of many keys hide most of the sort behind the host-link
// copies (same result, bit for bit):
//   1. the keys are copied in by chunks on a copy stream; as each chunk
//      arrives, the call's stream sorts it on its top 16 bits (32-bit keys:
//      two onesweep passes, then the start of every 16-bit bucket in it) or
//      splits it into its 256 top-byte buckets (64-bit keys: one pass);
//   2. consecutive top-byte buckets are cut into groups (kPipeRamp), each
//      finished on its own and copied out on the copy stream while the next
//      group is finished: 32-bit groups bucket by 16-bit bucket in shared
//      memory, or (a bucket too large for it, and 64-bit groups) gathered
//      from every chunk in chunk order and sorted by the batched or the
//      plain sort.
// Returns PA_OK after enqueueing everything; the caller's stream waits for
// the last copy.
constexpr size_t kPipeMinKeys = (size_t)1 << 24;

// Group ends at these cumulative shares of the keys, in 64ths: small groups
// first, so that the first copy-out starts soon after the last chunk, then
// groups of 10/64 that a group is finished in less time than the link takes
// to drain the one before (modelled on measured rates: sorting 12.5M keys
// in shared memory 0.18 ms, copying them out 0.26 ms).
constexpr int kPipeRamp[kPipeGroups] = {1, 3, 6, 10, 16, 24, 34, 44, 54, 64};

// PA_HOST_PIPELINE=0 turns the pipelined host-buffer sort off: host buffers
// of any size then take the two-buffer path (copy in, sort, copy out), as a
// comparison point.
bool pipeline_enabled() {
  static const bool v = [] {
    const char* e = std::getenv("PA_HOST_PIPELINE");
    return !(e && std::strcmp(e, "0") == 0);
  }();
  return v;
}

// Host-side fault injection for tests: PA_FAULT_PIPELINE_OOM=1 makes the
// pipelined sort report a device allocation failure before it allocates.
bool fault_pipeline_oom() {
  static const bool v = [] {
    const char* e = std::getenv("PA_FAULT_PIPELINE_OOM");
    return e && std::strcmp(e, "1") == 0;
  }();
  return v;
}

// The workspace's page-locked staging block, grown to at least `bytes`
// (growing frees the old block, which waits for the device: only between
// calls, before any copy from it is queued).  nullptr if it cannot grow.
void* pipe_pinned(Workspace* ws, size_t bytes) {
  if (bytes <= ws->pipe_host_cap) return ws->pipe_host;
  if (ws->pipe_host) cudaFreeHost(ws->pipe_host);
  ws->pipe_host = nullptr;
  ws->pipe_host_cap = 0;
  const size_t cap = std::max(bytes + bytes / 4, (size_t)1 << 20);
  if (cudaMallocHost(&ws->pipe_host, cap) != cudaSuccess) {
    cudaGetLastError();
    ws->pipe_host = nullptr;
    return nullptr;
  }
  ws->pipe_host_cap = cap;
  return ws->pipe_host;
}

int pipelined_host_sort(Workspace* ws, cudaStream_t stream, void* keys, size_t n, int kb) {
  if (fault_pipeline_oom()) return set_error(PA_ERR_OOM, "injected allocation failure (PA_FAULT_PIPELINE_OOM)");
  if (!ws->copy_stream) PA_CUDA(cudaStreamCreateWithFlags(&ws->copy_stream, cudaStreamNonBlocking));
  for (auto& e : ws->pipe_ev)
    if (!e) PA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // 32-bit keys: each chunk is sorted on its top 16 bits as it arrives, and
  // each group of top-byte buckets is finished by sorting its 16-bit buckets
  // (gathered from every chunk) on their low 16 bits in shared memory.
  // 64-bit keys: each chunk is split on its top byte, and each group is
  // gathered bucket by bucket and sorted by the plain sort.
  const bool b16 = kb == 4;
  const int cpass = b16 ? 2 : 1;  // digit passes per chunk
  const uint32_t shift0 = b16 ? 16u : 8u * (uint32_t)kb - 8u;
  const size_t chunk = ((n + kPipeChunks - 1) / kPipeChunks + 3) & ~(size_t)3;
  if (b16 && chunk >= ((size_t)1 << 32))  // (bucket bounds are 32-bit chunk offsets)
    return set_error(PA_ERR_OOM, "chunks of 2^32 keys or more take the two-buffer path");
  const size_t ctiles = ceil_div(chunk, onesweep_tile_keys(kb, false));
  const size_t sb = onesweep_status_bytes(chunk);
  const size_t pstat = ctiles * 256 * sb;  // one chunk pass's look-back words
  // groups that fall back to the batched kernel (a 16-bit bucket past the
  // shared-memory sort) need its plan block: n / 2 bytes of look-back words
  // plus tables at most
  const size_t plan_cap = b16 ? n / 2 + ((size_t)8 << 20) : 0;
  constexpr size_t kStarts = 65537;  // 16-bit bucket starts per chunk
  char *d_keys = nullptr, *d_tmp = nullptr, *d_gs = nullptr, *status = nullptr, *gscratch = nullptr, *plan_dev = nullptr;
  unsigned long long *counts = nullptr, *bin_start = nullptr, *runs = nullptr, *pos16 = nullptr, *summary = nullptr;
  uint32_t *tile_ctr = nullptr, *starts = nullptr, *btot = nullptr;
  SortCtrl* ctrl = nullptr;
  constexpr size_t kMaxRuns = (size_t)256 * kPipeChunks;  // every (bucket, chunk) piece
  auto layout = [&](Carve& c) {
    d_keys = c.take<char>(n * kb);  // input chunks (32-bit: then sorted on the top 16 bits)
    d_tmp = c.take<char>(n * kb);   // 64-bit: chunks split on the top byte; 32-bit: the result
    d_gs = c.take<char>(n * kb);    // the group sorts' scratch
    counts = c.take<unsigned long long>((size_t)kPipeChunks * cpass * 256);
    tile_ctr = c.take<uint32_t>((size_t)kPipeChunks * cpass);
    status = c.take<char>((size_t)kPipeChunks * cpass * pstat);
    bin_start = c.take<unsigned long long>((size_t)kPipeChunks * cpass * 256);
    ctrl = c.take<SortCtrl>(kPipeChunks);
    runs = c.take<unsigned long long>(kMaxRuns * 3);
    gscratch = c.take<char>(sort_scratch_bytes(n, kb, false));
    plan_dev = c.take<char>(plan_cap);
    starts = c.take<uint32_t>(b16 ? (size_t)kPipeChunks * kStarts : 0);
    pos16 = c.take<unsigned long long>(b16 ? kStarts : 0);
    btot = c.take<uint32_t>(b16 ? kStarts : 0);
    summary = c.take<unsigned long long>(b16 ? 512 : 0);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  const size_t zero_bytes = (size_t)(status + (size_t)kPipeChunks * cpass * pstat - reinterpret_cast<char*>(counts));
  cudaEvent_t* ev = ws->pipe_ev;
  cudaStream_t cs = ws->copy_stream;
  char* h = static_cast<char*>(keys);

  // 1. chunked copy-in; each arrived chunk is counted and sorted on its top
  //    16 bits (32-bit keys) or split on its top byte (64-bit keys)
  PA_CUDA(cudaMemsetAsync(counts, 0, zero_bytes, stream));
  PA_CUDA(cudaEventRecord(ev[0], stream));  // earlier work on this workspace is ordered before the copies
  PA_CUDA(cudaStreamWaitEvent(cs, ev[0], 0));
  size_t clo[kPipeChunks + 1];
  int nc = 0;
  for (int c = 0; c < kPipeChunks; ++c) {
    const size_t lo = std::min(n, (size_t)c * chunk), hi = std::min(n, lo + chunk);
    if (lo == hi) break;
    clo[nc++] = lo;
    PA_CUDA(cudaMemcpyAsync(d_keys + lo * kb, h + lo * kb, (hi - lo) * kb, cudaMemcpyHostToDevice, cs));
    PA_CUDA(cudaEventRecord(ev[1 + c], cs));
    PA_CUDA(cudaStreamWaitEvent(stream, ev[1 + c], 0));
    unsigned long long* cnt = counts + (size_t)c * cpass * 256;
    unsigned long long* bs = bin_start + (size_t)c * cpass * 256;
    PA_CUDA(launch_digit_counts(d_keys + lo * kb, hi - lo, kb, cpass, 8, shift0, 8, false, cnt, stream));
    PA_CUDA(launch_scan_digits(cnt, cpass, 8, hi - lo, false, false, bs, &ctrl[c], stream));
    for (int p = 0; p < cpass; ++p) {  // (no pass is skipped: two passes end back in d_keys)
      OnesweepArgs a{};
      a.keys_a = d_keys + lo * kb;
      a.keys_b = d_tmp + lo * kb;
      a.n = hi - lo;
      a.shift = shift0 + 8u * (uint32_t)p;
      a.pass = p;
      a.bin_start = bs + (size_t)p * 256;
      a.status = status + ((size_t)c * cpass + p) * pstat;
      a.tile_counter = tile_ctr + (size_t)c * cpass + p;
      a.ctrl = &ctrl[c];
      a.err = ws->err;
      PA_CUDA(launch_onesweep_pass(a, kb, false, stream));
    }
    if (b16)
      PA_CUDA(launch_bucket_bounds(reinterpret_cast<const uint32_t*>(d_keys) + lo, hi - lo, bs + 256,
                                   starts + (size_t)c * kStarts, stream));
  }
  clo[nc] = n;
  char* split = b16 ? d_keys : d_tmp;  // where each chunk's top-byte buckets lie, in order
  if (b16) PA_CUDA(launch_bucket_totals(starts, nc, btot, pos16, summary, stream));
  std::vector<unsigned long long> hc((size_t)nc * 256);  // [chunks][256] top-byte counts
  std::vector<unsigned long long> bmax(256, 0);           // largest 16-bit bucket per top byte
  {
    const size_t cbytes = (size_t)nc * cpass * 256 * 8;
    unsigned long long* stage =
        static_cast<unsigned long long*>(pipe_pinned(ws, cbytes + (b16 ? 512 * 8 : 0)));
    if (!stage) return set_error(PA_ERR_OOM, "page-locked staging for the pipelined sort");
    PA_CUDA(cudaMemcpyAsync(stage, counts, cbytes, cudaMemcpyDeviceToHost, stream));
    if (b16) PA_CUDA(cudaMemcpyAsync(stage + cbytes / 8, summary, 512 * 8, cudaMemcpyDeviceToHost, stream));
    PA_CUDA(cudaStreamSynchronize(stream));
    for (int c = 0; c < nc; ++c)
      std::memcpy(&hc[(size_t)c * 256], stage + ((size_t)c * cpass + cpass - 1) * 256, 256 * 8);
    if (b16) std::memcpy(bmax.data(), stage + cbytes / 8 + 256, 256 * 8);
  }

  // 2. groups of whole top-byte buckets
  unsigned long long total[257] = {};
  for (int b = 0; b < 256; ++b)
    for (int c = 0; c < nc; ++c) total[b + 1] += hc[(size_t)c * 256 + b];
  for (int b = 0; b < 256; ++b) total[b + 1] += total[b];  // total[b] = keys in buckets < b
  if (total[256] != n) return set_error(PA_ERR_CUDA, "top-digit counts add up to %llu, not %zu", total[256], n);
  int gb[kPipeGroups + 1];  // group g = buckets [gb[g], gb[g + 1])
  int ng = 0;
  gb[0] = 0;
  for (int b = 1; b < 256 && ng < kPipeGroups - 1; ++b)
    if (total[b] >= (unsigned long long)n * kPipeRamp[ng] / 64 && total[b] > total[gb[ng]] && total[b] < n)
      gb[++ng] = b;
  gb[++ng] = 256;
  // 32-bit groups whose 16-bit buckets all fit the shared-memory sort take
  // it; the others (and every 64-bit group) are gathered bucket by bucket
  std::vector<size_t> gmax(ng, 0);
  std::vector<bool> fast(ng, false);
  for (int g = 0; g < ng; ++g) {
    for (int b = gb[g]; b < gb[g + 1]; ++b) gmax[g] = std::max<size_t>(gmax[g], (size_t)bmax[b]);
    fast[g] = b16 && gmax[g] <= bucket_sort_max_keys();
  }
  // bucket b of chunk c starts at clo[c] + (its counts of buckets < b) in `split`
  std::vector<unsigned long long> local((size_t)nc * 257);
  for (int c = 0; c < nc; ++c) {
    local[(size_t)c * 257] = 0;
    for (int b = 0; b < 256; ++b) local[(size_t)c * 257 + b + 1] = local[(size_t)c * 257 + b] + hc[(size_t)c * 256 + b];
  }
  std::vector<unsigned long long> run_tab;  // (src, len, dst) triples of the gathered groups
  std::vector<size_t> run_first(ng + 1), run_max(ng, 0);
  for (int g = 0; g < ng; ++g) {
    run_first[g] = run_tab.size() / 3;
    if (fast[g]) continue;
    const unsigned long long g0 = total[gb[g]];
    for (int b = gb[g]; b < gb[g + 1]; ++b)
      for (int c = 0; c < nc; ++c) {
        const unsigned long long len = hc[(size_t)c * 256 + b];
        if (!len) continue;
        unsigned long long dst = total[b] - g0;  // within the group, bucket b, then chunk order
        for (int c2 = 0; c2 < c; ++c2) dst += hc[(size_t)c2 * 256 + b];
        run_tab.insert(run_tab.end(), {clo[c] + local[(size_t)c * 257 + b], len, dst});
        run_max[g] = std::max<size_t>(run_max[g], (size_t)len);
      }
  }
  run_first[ng] = run_tab.size() / 3;
  // gathered 32-bit groups: batched plans with the buckets as segments and
  // three passes (a bucket's top byte is constant); a plan past the batched
  // sort's limits leaves its group to the plain sort
  std::vector<seg::HostPlan> plans(b16 ? ng : 0);
  std::vector<bool> planned(ng, false);
  std::vector<size_t> image_off(ng + 1, 0);
  for (int g = 0; g < ng; ++g) {
    size_t bytes = 0;
    if (b16 && !fast[g]) {
      std::vector<uint64_t> off(gb[g + 1] - gb[g] + 1);
      for (int b = gb[g]; b <= gb[g + 1]; ++b) off[b - gb[g]] = total[b] - total[gb[g]];
      pa_segsort_config cfg{};
      cfg.small_cutoff = 4096;
      cfg.tile_keys = 8192;
      planned[g] = seg::build_host_plan(off.data(), off.size() - 1, &cfg, &plans[g], 3) == PA_OK &&
                   plans[g].bytes <= plan_cap;
      if (planned[g]) bytes = seg::plan_image_bytes(plans[g]);
    }
    image_off[g + 1] = image_off[g] + (bytes + 255) / 256 * 256;
  }
  const size_t runs_bytes = run_tab.size() * 8;
  const size_t images_at = (runs_bytes + 255) / 256 * 256;  // the plan images follow the run table
  char* stage = static_cast<char*>(pipe_pinned(ws, images_at + image_off[ng] + 256));
  if (!stage) return set_error(PA_ERR_OOM, "page-locked staging for the pipelined sort");
  if (runs_bytes) {
    std::memcpy(stage, run_tab.data(), runs_bytes);
    PA_CUDA(cudaMemcpyAsync(runs, stage, runs_bytes, cudaMemcpyHostToDevice, stream));
  }
  char* images = stage + images_at;
  ChunkRuns chunks{};
  chunks.count = nc;
  for (int c = 0; c < nc; ++c) chunks.lo[c] = clo[c];

  // 3. per group: sort, copy out while the next group runs
  for (int g = 0; g < ng; ++g) {
    const size_t lo = (size_t)total[gb[g]], len = (size_t)(total[gb[g + 1]] - total[gb[g]]);
    if (len == 0) continue;
    char* result = nullptr;
    if (fast[g]) {
      PA_CUDA(launch_bucket_sort(reinterpret_cast<const uint32_t*>(d_keys), chunks, starts, pos16,
                                 (uint32_t)gb[g] * 256u, (uint32_t)(gb[g + 1] - gb[g]) * 256u, gmax[g],
                                 reinterpret_cast<uint32_t*>(d_tmp), ws->err, stream));
      result = d_tmp + lo * kb;
    } else {
      char* gdst = b16 ? d_tmp : d_keys;  // the buffer the chunks' buckets are not in
      PA_CUDA(launch_gather_runs(split, gdst + lo * kb, runs + run_first[g] * 3, run_first[g + 1] - run_first[g],
                                 run_max[g], kb, stream));
      result = gdst + lo * kb;
      if (planned[g]) {
        seg::HostPlan& hp = plans[g];
        PA_CUDA(seg::upload_plan(hp, plan_dev, stream, images + image_off[g]));
        seg::PlanDev pd = seg::device_view(hp, plan_dev, reinterpret_cast<uint32_t*>(gdst + lo * kb),
                                           reinterpret_cast<uint32_t*>(d_gs + lo * kb));
        pd.err = ws->err;
        PA_CUDA(seg::launch_plan(hp, pd, plan_dev, seg::plan_grid(hp), stream));
        result = reinterpret_cast<char*>(seg::result_buffer(pd));
      } else {
        SortScratch sc{};
        sort_scratch_layout(gscratch, len, kb, false, &sc);
        PA_CUDA(enqueue_sort(sc, gdst + lo * kb, d_gs + lo * kb, nullptr, nullptr, len, kb, false, ws->err, stream));
      }
    }
    PA_CUDA(cudaEventRecord(ev[1 + kPipeChunks + g], stream));
    PA_CUDA(cudaStreamWaitEvent(cs, ev[1 + kPipeChunks + g], 0));
    PA_CUDA(cudaMemcpyAsync(h + lo * kb, result, len * kb, cudaMemcpyDeviceToHost, cs));
  }
  PA_CUDA(cudaEventRecord(ev[kPipeChunks + kPipeGroups + 1], cs));
  PA_CUDA(cudaStreamWaitEvent(stream, ev[kPipeChunks + kPipeGroups + 1], 0));
  return PA_OK;
}

// phase_ms (optional, phase_cap entries): device time of each kernel of the
// sort from CUDA events recorded between launches on the call's stream:
// [0] digit histogram, [1] scan, [2 + p] digit pass p, [2 + passes] final
// copy.  Timing forces a synchronous call.
int sort_impl(void* keys, void* tmp, uint32_t* vals, uint32_t* tmp_vals, size_t n, int kb, bool is_float,
              const pa_opts* opts, float* phase_ms = nullptr, int phase_cap = 0) {
  if (int rc = check_opts(opts)) return rc;
  if (n == 0) return PA_OK;
  if (!keys) return set_error(PA_ERR_ARG, "keys is NULL");
  if (tmp_vals && !vals) return set_error(PA_ERR_ARG, "tmp_vals given without vals");
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;

  const bool has_vals = vals != nullptr;
  const bool keys_dev = is_device_ptr(keys);
  const bool tmp_dev = is_device_ptr(tmp);
  const int rb = (opts && opts->digit_bits == 11) ? 11 : 8;
  if (!keys_dev && !has_vals && !is_float && !(phase_ms && phase_cap > 0) && n >= kPipeMinKeys && rb == 8 &&
      pipeline_enabled()) {
    const int rc = pipelined_host_sort(ws, stream, keys, n, kb);
    if (rc == PA_OK) return finish(ws, stream, false);
    // nothing may still copy into the caller's buffer after the call returns
    if (ws->copy_stream) cudaStreamSynchronize(ws->copy_stream);
    cudaStreamSynchronize(stream);
    cudaGetLastError();
    // the pipeline needs a third key-sized device buffer; without the memory
    // for it, the plain host path below (two buffers) still sorts
    if (rc != PA_ERR_OOM) return rc;
  }
  const bool vals_dev = has_vals && is_device_ptr(vals);
  const bool tvals_dev = has_vals && is_device_ptr(tmp_vals);
  void *d_keys = nullptr, *d_tmp = nullptr;
  uint32_t *d_vals = nullptr, *d_tvals = nullptr;
  SortScratch sc{};
  auto layout = [&](Carve& c) {
    d_keys = keys_dev ? keys : c.take<char>(n * kb);
    d_tmp = tmp_dev ? tmp : c.take<char>(n * kb);
    if (has_vals) {
      d_vals = vals_dev ? vals : c.take<uint32_t>(n);
      d_tvals = tvals_dev ? tmp_vals : c.take<uint32_t>(n);
    }
    char* sbase = c.take<char>(sort_scratch_bytes(n, kb, has_vals, rb));
    sort_scratch_layout(sbase, n, kb, has_vals, &sc, rb);
  };
  Carve measure{nullptr};
  layout(measure);
  if (int rc = ensure_dev(ws, stream, measure.off)) return rc;
  Carve real{ws->dev};
  layout(real);

  const size_t key_bytes_total = n * (size_t)kb;
  if (!keys_dev) PA_CUDA(cudaMemcpyAsync(d_keys, keys, key_bytes_total, cudaMemcpyHostToDevice, stream));
  if (has_vals && !vals_dev)
    PA_CUDA(cudaMemcpyAsync(d_vals, vals, n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
  const bool timed = phase_ms && phase_cap > 0;
  int nev = 0;
  auto mark = [&]() -> cudaError_t {
    if (!timed || nev >= kMaxEvents) return cudaSuccess;
    if (!ws->ev[nev]) {
      cudaError_t e = cudaEventCreate(&ws->ev[nev]);
      if (e != cudaSuccess) return e;
    }
    return cudaEventRecord(ws->ev[nev++], stream);
  };
  PA_CUDA(enqueue_sort(sc, d_keys, d_tmp, d_vals, d_tvals, n, kb, is_float, ws->err, stream, mark));
  if (!keys_dev) PA_CUDA(cudaMemcpyAsync(keys, d_keys, key_bytes_total, cudaMemcpyDeviceToHost, stream));
  if (has_vals && !vals_dev)
    PA_CUDA(cudaMemcpyAsync(vals, d_vals, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  const bool all_dev = keys_dev && (!has_vals || vals_dev);
  int rc = finish(ws, stream, !timed && opts && opts->async_device && all_dev);
  if (rc == PA_OK && timed) {
    for (int i = 0; i + 1 < nev && i < phase_cap; ++i) {
      float ms = 0.f;
      PA_CUDA(cudaEventElapsedTime(&ms, ws->ev[i], ws->ev[i + 1]));
      phase_ms[i] = ms;
    }
  }
  return rc;
}

// ---------------------------------------------------------------------------
// In-place sort with bounded scratch
// ---------------------------------------------------------------------------
// An MSD sort of 32-bit keys that holds, besides the keys, a scratch of S
// keys (and small tables) whatever n is.  Up to S keys: the LSD sort with
// the scratch as its second buffer.  Above: a range is partitioned in place
// on its top digit (launch_inplace_partition, rounds through the scratch
// halves); buckets of at most S keys are sorted in groups of consecutive
// buckets (at most S keys a group) on their lower digits by the batched
// segmented sort, with the scratch as its second buffer; larger buckets are
// partitioned again on the next digit.  A range whose keys all share the
// digit is not moved.
constexpr size_t kInplaceDefaultScratch = (size_t)1 << 24;  // keys
constexpr size_t kInplaceMinScratch = (size_t)1 << 16;

int inplace_levels(Workspace* ws, cudaStream_t stream, uint32_t* a, size_t n, size_t S, uint32_t* buf,
                   InplaceState* st, void* status, unsigned long long* hist, char* plan_dev, size_t plan_cap,
                   char* sort_base) {
  struct Range {
    size_t lo, len;
    uint32_t shift;
  };
  std::vector<Range> todo{{0, n, 24}};
  std::vector<unsigned long long> h(256);
  const size_t half = S / 2;
  while (!todo.empty()) {
    const Range rg = todo.back();
    todo.pop_back();
    PA_CUDA(cudaMemsetAsync(hist, 0, 256 * sizeof(unsigned long long), stream));
    PA_CUDA(launch_digit_counts(a + rg.lo, rg.len, 4, 1, 8, rg.shift, 0, false, hist, stream));
    PA_CUDA(cudaMemcpyAsync(h.data(), hist, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    PA_CUDA(cudaStreamSynchronize(stream));
    int nonempty = 0;
    for (unsigned long long c : h) nonempty += c ? 1 : 0;
    if (nonempty <= 1) {  // every key has this digit: nothing moves
      if (rg.shift > 0) todo.push_back({rg.lo, rg.len, rg.shift - 8});
      continue;
    }
    PA_CUDA(launch_inplace_partition(a + rg.lo, rg.len, rg.shift, hist, buf, buf + half, half, st, status, ws->err,
                                     stream));
    if (rg.shift == 0) continue;  // the buckets of the lowest digit hold equal keys
    // groups of consecutive buckets of at most S keys, larger buckets to the next level
    const int passes = (int)(rg.shift / 8);  // digits below this one
    struct Group {
      size_t lo;
      std::vector<uint64_t> off;
    };
    std::vector<Group> groups;
    size_t at = rg.lo;
    bool open = false;
    for (int b = 0; b < 256; ++b) {
      const size_t c = (size_t)h[b];
      if (c == 0) continue;
      if (c > S) {
        todo.push_back({at, c, rg.shift - 8});
        open = false;
      } else {
        if (!open || groups.back().off.back() + c > S) {
          groups.push_back({at, {0}});
          open = true;
        }
        groups.back().off.push_back(groups.back().off.back() + c);
      }
      at += c;
    }
    std::vector<seg::HostPlan> plans(groups.size());
    std::vector<bool> planned(groups.size(), false);
    std::vector<size_t> image_off(groups.size() + 1, 0);
    for (size_t g = 0; g < groups.size(); ++g) {
      size_t bytes = 0;
      if (groups[g].off.back() > 1) {
        pa_segsort_config cfg{};
        cfg.small_cutoff = 4096;
        cfg.tile_keys = 8192;
        planned[g] = seg::build_host_plan(groups[g].off.data(), groups[g].off.size() - 1, &cfg, &plans[g],
                                          passes) == PA_OK &&
                     plans[g].bytes <= plan_cap;
        if (planned[g]) bytes = seg::plan_image_bytes(plans[g]);
      }
      image_off[g + 1] = image_off[g] + (bytes + 255) / 256 * 256;
    }
    char* images = static_cast<char*>(pipe_pinned(ws, image_off.back() + 256));
    if (!images) return set_error(PA_ERR_OOM, "page-locked staging for the in-place sort's plans");
    for (size_t g = 0; g < groups.size(); ++g) {
      uint32_t* ga = a + groups[g].lo;
      const size_t glen = (size_t)groups[g].off.back();
      if (glen < 2) continue;
      if (planned[g]) {
        seg::HostPlan& hp = plans[g];
        PA_CUDA(seg::upload_plan(hp, plan_dev, stream, images + image_off[g]));
        seg::PlanDev pd = seg::device_view(hp, plan_dev, ga, buf);
        pd.err = ws->err;
        PA_CUDA(seg::launch_plan(hp, pd, plan_dev, seg::plan_grid(hp), stream));
        if (seg::result_buffer(pd) != ga)
          PA_CUDA(cudaMemcpyAsync(ga, seg::result_buffer(pd), glen * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                  stream));
      } else {  // the group as one array: its buckets are already in order
        SortScratch sc{};
        sort_scratch_layout(sort_base, glen, 4, false, &sc);
        PA_CUDA(enqueue_sort(sc, ga, buf, nullptr, nullptr, glen, 4, false, ws->err, stream));
      }
    }
  }
  return PA_OK;
}

int inplace_impl(uint32_t* keys, size_t n, size_t scratch_keys, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (opts && opts->digit_bits == 11) return set_error(PA_ERR_ARG, "the in-place sort takes 8-bit digits only");
  if (n == 0) return PA_OK;
  if (!keys) return set_error(PA_ERR_ARG, "keys is NULL");
  if (n == 1) return PA_OK;
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  size_t S = scratch_keys ? std::max(scratch_keys, kInplaceMinScratch) : kInplaceDefaultScratch;
  S &= ~(size_t)1;
  const bool keys_dev = is_device_ptr(keys);
  const size_t sort_keys = std::min(n, S);
  const size_t plan_cap = S / 2 + ((size_t)8 << 20);
  uint32_t *d_keys = nullptr, *buf = nullptr;
  InplaceState* st = nullptr;
  unsigned long long* hist = nullptr;
  char *plan_dev = nullptr, *sort_base = nullptr, *status = nullptr;
  auto layout = [&](Carve& c) {
    d_keys = keys_dev ? keys : c.take<uint32_t>(n);
    buf = c.take<uint32_t>(sort_keys);
    sort_base = c.take<char>(sort_scratch_bytes(sort_keys, 4, false));
    if (n > S) {
      st = c.take<InplaceState>(1);
      hist = c.take<unsigned long long>(256);
      plan_dev = c.take<char>(plan_cap);
      status = c.take<char>(inplace_status_bytes(n, S / 2));
    }
  };
  Carve measure{nullptr};
  layout(measure);
  if (int rc = ensure_dev(ws, stream, measure.off)) return rc;
  Carve real{ws->dev};
  layout(real);
  if (!keys_dev) PA_CUDA(cudaMemcpyAsync(d_keys, keys, n * sizeof(uint32_t), cudaMemcpyHostToDevice, stream));
  if (n <= S) {
    SortScratch sc{};
    sort_scratch_layout(sort_base, n, 4, false, &sc);
    PA_CUDA(enqueue_sort(sc, d_keys, buf, nullptr, nullptr, n, 4, false, ws->err, stream));
  } else if (int rc = inplace_levels(ws, stream, d_keys, n, S, buf, st, status, hist, plan_dev, plan_cap,
                                     sort_base)) {
    cudaStreamSynchronize(stream);
    cudaGetLastError();
    return rc;
  }
  if (!keys_dev) PA_CUDA(cudaMemcpyAsync(keys, d_keys, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && keys_dev);
}

// ---------------------------------------------------------------------------
// Histograms
// ---------------------------------------------------------------------------
// One histogram call: `rows` x 256 counts of the digits selected by
// (key_bytes, num_digits, shift0, step) over a[0, n) into out.
int hist_impl(const void* a, size_t n, int kb, int num_digits, uint32_t shift0, uint32_t step, uint64_t* out,
              const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (!out) return set_error(PA_ERR_ARG, "out is NULL");
  if (n && !a) return set_error(PA_ERR_ARG, "input is NULL");
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool in_dev = is_device_ptr(a);
  const bool out_dev = is_device_ptr(out);
  const size_t out_words = (size_t)num_digits * 256;
  const void* d_in = nullptr;
  unsigned long long* d_out = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? a : c.take<char>(n * kb);
    d_out = out_dev ? reinterpret_cast<unsigned long long*>(out) : c.take<unsigned long long>(out_words);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!in_dev && n) PA_CUDA(cudaMemcpyAsync(const_cast<void*>(d_in), a, n * kb, cudaMemcpyHostToDevice, stream));
  PA_CUDA(cudaMemsetAsync(d_out, 0, out_words * sizeof(uint64_t), stream));
  PA_CUDA(launch_digit_counts(d_in, n, kb, num_digits, 8, shift0, step, false, d_out, stream));
  if (!out_dev) PA_CUDA(cudaMemcpyAsync(out, d_out, out_words * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && in_dev && out_dev);
}

// ---------------------------------------------------------------------------
// Select
// ---------------------------------------------------------------------------
int select_impl(const void* a, size_t n, size_t k, int kb, void* out, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (!a || !out) return set_error(PA_ERR_ARG, "NULL buffer");
  if (k >= n) return set_error(PA_ERR_ARG, "k = %zu is not below n = %zu", k, n);
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool in_dev = is_device_ptr(a);
  const bool out_dev = is_device_ptr(out);
  // Candidates kept after the first digit: a quarter of the input covers
  // uniform and presorted inputs after one step; heavier bins are filtered
  // from the input instead.
  const size_t cand_cap = n / 4 + 1024;
  const void* d_in = nullptr;
  void *cand = nullptr, *work = nullptr, *d_out = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? a : c.take<char>(n * kb);
    cand = c.take<char>(cand_cap * kb);
    work = c.take<char>(select_state_bytes());
    d_out = out_dev ? out : c.take<char>(8);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!in_dev) PA_CUDA(cudaMemcpyAsync(const_cast<void*>(d_in), a, n * kb, cudaMemcpyHostToDevice, stream));
  PA_CUDA(launch_select(d_in, n, k, kb, cand, cand_cap, work, d_out, ws->err, stream));
  if (!out_dev) PA_CUDA(cudaMemcpyAsync(out, d_out, kb, cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && in_dev && out_dev);
}

// ---------------------------------------------------------------------------
// Sum
// ---------------------------------------------------------------------------
int sum_impl(const void* a, size_t n, int elem_kind, uint64_t* out, const pa_opts* opts, size_t chunk = 0,
             uint64_t* chunk_sums = nullptr) {
  if (int rc = check_opts(opts)) return rc;
  const int kb = sum_elem_bytes(elem_kind);
  if (kb == 0) return set_error(PA_ERR_ARG, "unknown element kind %d", elem_kind);
  if (!out) return set_error(PA_ERR_ARG, "out is NULL");
  if (n && !a) return set_error(PA_ERR_ARG, "input is NULL");
  if (chunk_sums && chunk == 0) return set_error(PA_ERR_ARG, "chunk is 0");
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool in_dev = is_device_ptr(a);
  const bool out_dev = is_device_ptr(out);
  const size_t nchunks = chunk_sums ? ceil_div(n, chunk) : 0;
  const bool sums_dev = chunk_sums && is_device_ptr(chunk_sums);
  const void* d_in = nullptr;
  unsigned long long* partials = nullptr;
  uint32_t* ticket = nullptr;
  unsigned long long* d_out = nullptr;
  unsigned long long* d_sums = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? a : c.take<char>(n * kb);
    partials = c.take<unsigned long long>(sum_partials_needed());
    ticket = c.take<uint32_t>(1);
    d_out = out_dev ? reinterpret_cast<unsigned long long*>(out) : c.take<unsigned long long>(1);
    if (chunk_sums)
      d_sums = sums_dev ? reinterpret_cast<unsigned long long*>(chunk_sums) : c.take<unsigned long long>(nchunks);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!in_dev && n) PA_CUDA(cudaMemcpyAsync(const_cast<void*>(d_in), a, n * kb, cudaMemcpyHostToDevice, stream));
  if (chunk_sums) {
    // per-chunk sums (the reference's caller-provided sum_array) and their total
    PA_CUDA(cudaMemsetAsync(d_out, 0, sizeof(uint64_t), stream));
    PA_CUDA(launch_sum_chunks(d_in, n, elem_kind, chunk, d_sums, d_out, stream));
    if (!sums_dev && nchunks)
      PA_CUDA(cudaMemcpyAsync(chunk_sums, d_sums, nchunks * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  } else {
    PA_CUDA(cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream));
    PA_CUDA(launch_sum(d_in, n, elem_kind, partials, ticket, d_out, ws->err, stream));
  }
  if (!out_dev) PA_CUDA(cudaMemcpyAsync(out, d_out, sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && in_dev && out_dev && (!chunk_sums || sums_dev));
}

}  // namespace

size_t sort_scratch_bytes(size_t n, int kb, bool has_vals, int radix_bits) {
  SortScratch s{};
  return sort_scratch_layout(nullptr, n, kb, has_vals, &s, radix_bits);
}

size_t sort_scratch_layout(char* base, size_t n, int kb, bool has_vals, SortScratch* s, int radix_bits) {
  const int passes = sort_passes(kb, radix_bits);
  const size_t bins = (size_t)1 << radix_bits;
  const size_t tile_keys = onesweep_tile_keys(kb, has_vals, radix_bits);
  const size_t tiles = ceil_div(n, tile_keys);
  const size_t sb = onesweep_status_bytes(n);
  // the first pass's prepared offsets (launch_tile_counts)
  const bool prepared = kb == 4 && !has_vals && radix_bits == 8 && n < ((size_t)1 << 30) && tiles >= 2 &&
                        tile_counts_supported(tile_keys);
  Carve c{base};
  s->radix_bits = radix_bits;
  s->passes = passes;
  s->counts = c.take<unsigned long long>((size_t)passes * bins);
  s->zero_begin = reinterpret_cast<char*>(s->counts);
  s->tile_ctr = c.take<uint32_t>((size_t)passes + 1);
  s->tc_ticket = s->tile_ctr + passes;
  s->status = c.take<char>((size_t)passes * tiles * bins * sb);
  s->zero_bytes = (size_t)(base + c.off - s->zero_begin);
  s->bin_start = c.take<unsigned long long>((size_t)passes * bins);
  s->ctrl = c.take<SortCtrl>(1);
  s->tiles = tiles;
  s->status_bytes = sb;
  s->tile_prefix = prepared ? c.take<uint32_t>(tiles * 256) : nullptr;
  s->chunk_tot = prepared ? c.take<uint32_t>((size_t)kTileCountMaxChunks * 256) : nullptr;
  s->chunk_excl = prepared ? c.take<uint32_t>((size_t)kTileCountMaxChunks * 256) : nullptr;
  return c.off;
}

cudaError_t enqueue_sort(const SortScratch& s, void* d_keys, void* d_tmp, uint32_t* d_vals, uint32_t* d_tvals,
                         size_t n, int kb, bool is_float, uint32_t* err, cudaStream_t stream,
                         const std::function<cudaError_t()>& mark) {
  const int rb = s.radix_bits;
  const int passes = s.passes;
  const size_t bins = (size_t)1 << rb;
  const bool has_vals = d_vals != nullptr;
  auto m = [&]() { return mark ? mark() : cudaSuccess; };
  if (n <= small_sort_max_keys(kb, has_vals)) {  // one CTA, one launch
    (void)d_tmp;
    (void)d_tvals;
    (void)err;
    cudaError_t e = m();
    if (e == cudaSuccess) e = launch_small_sort(d_keys, d_vals, n, kb, is_float, stream);
    if (e == cudaSuccess) e = m();
    return e;
  }
  cudaError_t e = cudaMemsetAsync(s.zero_begin, 0, s.zero_bytes, stream);
  if (e == cudaSuccess) e = m();
  // With the tables (and 16-byte aligned keys) the histogram also prepares
  // the first pass's tile offsets.
  const bool prepared = s.tile_prefix && kb == 4 && rb == 8 && !has_vals && n < ((size_t)1 << 30) &&
                        (reinterpret_cast<uintptr_t>(d_keys) & 15u) == 0;
  uint32_t tpc = 0;
  if (e == cudaSuccess)
    e = prepared ? launch_tile_counts(static_cast<const uint32_t*>(d_keys), n, onesweep_tile_keys(kb, false, rb),
                                      is_float, s.counts, s.tile_prefix, s.chunk_tot, s.chunk_excl, s.tc_ticket, &tpc,
                                      stream)
                 : launch_digit_counts(d_keys, n, kb, passes, rb, 0, (uint32_t)rb, is_float, s.counts, stream);
  if (e == cudaSuccess) e = m();
  if (e == cudaSuccess) e = launch_scan_digits(s.counts, passes, rb, n, is_float, true, s.bin_start, s.ctrl, stream);
  if (e == cudaSuccess) e = m();
  for (int p = 0; p < passes && e == cudaSuccess; ++p) {
    OnesweepArgs a{};
    a.keys_a = d_keys;
    a.keys_b = d_tmp;
    a.vals_a = d_vals;
    a.vals_b = d_tvals;
    a.n = n;
    a.shift = (uint32_t)(rb * p);
    a.pass = p;
    a.is_float = is_float ? 1 : 0;
    a.radix_bits = rb;
    a.bin_start = s.bin_start + (size_t)p * bins;
    a.status = s.status + (size_t)p * s.tiles * bins * s.status_bytes;
    a.tile_counter = s.tile_ctr + p;
    a.ctrl = s.ctrl;
    a.err = err;
    if (prepared && p == 0) {  // pass 0, when it runs, reads the keys the histogram read
      a.tile_prefix = s.tile_prefix;
      a.chunk_excl = s.chunk_excl;
      a.tiles_per_chunk = tpc;
    }
    e = launch_onesweep_pass(a, kb, has_vals, stream);
    if (e == cudaSuccess) e = m();
  }
  if (e == cudaSuccess) e = launch_final_copy(d_keys, d_tmp, d_vals, d_tvals, n, kb, s.ctrl, stream);
  if (e == cudaSuccess) e = m();
  return e;
}

int record_error(int status, const char* message) { return set_error(status, "%s", message); }

const DeviceInfo& device_info() {
  static DeviceInfo infos[64];
  static std::mutex mu;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::lock_guard<std::mutex> lk(mu);  // launches come from callers' threads and the server's thread
  DeviceInfo& d = infos[dev];
  if (d.device != dev) {
    int sms = 0, smem = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    d.sm_count = sms > 0 ? sms : 1;
    d.max_smem_optin = (size_t)smem;
    d.device = dev;
  }
  return d;
}

cudaError_t ensure_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::set<std::tuple<int, const void*, size_t>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_tuple(dev, func, bytes);
  if (done.count(key)) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done.insert(key);
  return e;
}

}  // namespace pa

using namespace pa;

extern "C" {

const char* pa_status_string(int status) {
  switch (status) {
    case PA_OK: return "PA_OK";
    case PA_ERR_ARG: return "PA_ERR_ARG";
    case PA_ERR_OOM: return "PA_ERR_OOM";
    case PA_ERR_CUDA: return "PA_ERR_CUDA";
    case PA_ERR_TIMEOUT: return "PA_ERR_TIMEOUT";
    case PA_ERR_NO_DEVICE: return "PA_ERR_NO_DEVICE";
    default: return "PA_ERR_UNKNOWN";
  }
}

const char* pa_last_error_message(void) { return g_last_error.c_str(); }

int pa_device_available(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count > 0 ? 1 : 0;
}

int pa_stream_check(void* stream) {
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(static_cast<cudaStream_t>(stream), &ws)) return rc;
  return finish(ws, static_cast<cudaStream_t>(stream), false);
}

int pa_release_workspaces(void) {
  if (!pa_device_available()) return PA_OK;
  std::lock_guard<std::mutex> lock(g_mu);
  int dev0 = 0;
  cudaGetDevice(&dev0);
  for (auto& kv : g_ws) {
    cudaSetDevice(kv.first.first);
    cudaStreamSynchronize(kv.first.second);
    if (kv.second.dev) cudaFree(kv.second.dev);
    if (kv.second.err) cudaFree(kv.second.err);
    if (kv.second.err_host) cudaFreeHost(kv.second.err_host);
  }
  g_ws.clear();
  cudaSetDevice(dev0);
  return PA_OK;
}

int pa_sort_u32(uint32_t* keys, uint32_t* tmp, size_t n, const pa_opts* opts) {
  return sort_impl(keys, tmp, nullptr, nullptr, n, 4, false, opts);
}
int pa_sort_u32_inplace(uint32_t* keys, size_t n, size_t scratch_keys, const pa_opts* opts) {
  return inplace_impl(keys, n, scratch_keys, opts);
}
int pa_sort_timed(int key_kind, void* keys, void* tmp, uint32_t* vals, uint32_t* tmp_vals, size_t n,
                  float* phase_ms, int phase_cap, const pa_opts* opts) {
  if (!phase_ms || phase_cap <= 0) return set_error(PA_ERR_ARG, "phase_ms is required");
  switch (key_kind) {
    case PA_KEY_U32: return sort_impl(keys, tmp, vals, tmp_vals, n, 4, false, opts, phase_ms, phase_cap);
    case PA_KEY_U64: return sort_impl(keys, tmp, vals, tmp_vals, n, 8, false, opts, phase_ms, phase_cap);
    case PA_KEY_F32: return sort_impl(keys, tmp, vals, tmp_vals, n, 4, true, opts, phase_ms, phase_cap);
    default: return set_error(PA_ERR_ARG, "unknown key kind %d", key_kind);
  }
}

int pa_sort_u64(uint64_t* keys, uint64_t* tmp, size_t n, const pa_opts* opts) {
  return sort_impl(keys, tmp, nullptr, nullptr, n, 8, false, opts);
}
int pa_sort_f32(float* keys, float* tmp, size_t n, const pa_opts* opts) {
  return sort_impl(keys, tmp, nullptr, nullptr, n, 4, true, opts);
}
int pa_sort_kv_u32(uint32_t* keys, uint32_t* vals, uint32_t* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts) {
  if (n && !vals) return set_error(PA_ERR_ARG, "vals is NULL");
  return sort_impl(keys, tmp_keys, vals, tmp_vals, n, 4, false, opts);
}
int pa_sort_kv_u64(uint64_t* keys, uint32_t* vals, uint64_t* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts) {
  if (n && !vals) return set_error(PA_ERR_ARG, "vals is NULL");
  return sort_impl(keys, tmp_keys, vals, tmp_vals, n, 8, false, opts);
}
int pa_sort_kv_f32(float* keys, uint32_t* vals, float* tmp_keys, uint32_t* tmp_vals, size_t n,
                   const pa_opts* opts) {
  if (n && !vals) return set_error(PA_ERR_ARG, "vals is NULL");
  return sort_impl(keys, tmp_keys, vals, tmp_vals, n, 4, true, opts);
}

int pa_sort_two_phase_u32(uint32_t* a, uint32_t* b, size_t n, const pa_opts* opts) {
  if (n && !b) return set_error(PA_ERR_ARG, "b is NULL");
  int rc = sort_impl(a, b, nullptr, nullptr, n, 4, false, opts);
  if (rc != PA_OK || n == 0) return rc;
  cudaStream_t stream = stream_of(opts);
  PA_CUDA(cudaMemcpyAsync(b, a, n * sizeof(uint32_t), cudaMemcpyDefault, stream));
  PA_CUDA(cudaStreamSynchronize(stream));
  return PA_OK;
}

int pa_hist_byte_components_u32(const uint32_t* a, size_t n, uint64_t* out, const pa_opts* opts) {
  return hist_impl(a, n, 4, 4, 0, 8, out, opts);
}

int pa_hist_one_byte_u32(const uint32_t* a, size_t n, unsigned shift, uint64_t* out, const pa_opts* opts) {
  if (shift >= 32) return set_error(PA_ERR_ARG, "shift %u is not below 32", shift);
  return hist_impl(a, n, 4, 1, shift, 0, out, opts);
}

int pa_hist_one_byte_u64(const uint64_t* a, size_t n, unsigned shift, uint64_t* out, const pa_opts* opts) {
  if (shift >= 64) return set_error(PA_ERR_ARG, "shift %u is not below 64", shift);
  return hist_impl(a, n, 8, 1, shift, 0, out, opts);
}

int pa_hist_u8(const uint8_t* a, size_t n, uint64_t* out, const pa_opts* opts) {
  return hist_impl(a, n, 1, 1, 0, 0, out, opts);
}

int pa_counting_sort_u8(uint8_t* a, size_t n, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (n == 0) return PA_OK;
  if (!a) return set_error(PA_ERR_ARG, "a is NULL");
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool dev = is_device_ptr(a);
  uint8_t* d_a = nullptr;
  unsigned long long* counts = nullptr;
  auto layout = [&](Carve& c) {
    counts = c.take<unsigned long long>(256);
    d_a = dev ? a : c.take<uint8_t>(n);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!dev) PA_CUDA(cudaMemcpyAsync(d_a, a, n, cudaMemcpyHostToDevice, stream));
  PA_CUDA(cudaMemsetAsync(counts, 0, 256 * sizeof(unsigned long long), stream));
  PA_CUDA(launch_digit_counts(d_a, n, 1, 1, 8, 0, 0, false, counts, stream));
  PA_CUDA(launch_counting_fill(d_a, n, counts, stream));
  if (!dev) PA_CUDA(cudaMemcpyAsync(a, d_a, n, cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && dev);
}

int pa_sort_copy_u32(uint32_t* src, uint32_t* dst, size_t n, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (n == 0) return PA_OK;
  if (!src || !dst) return set_error(PA_ERR_ARG, "NULL buffer");
  if (src == dst) return pa_sort_u32(dst, nullptr, n, opts);
  if (int rc = device_ready()) return rc;
  if (!is_device_ptr(src) && !is_device_ptr(dst)) {
    std::memcpy(dst, src, n * sizeof(uint32_t));
  } else {
    cudaStream_t stream = stream_of(opts);
    PA_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(uint32_t), cudaMemcpyDefault, stream));
    if (!is_device_ptr(dst) || !is_device_ptr(src)) PA_CUDA(cudaStreamSynchronize(stream));
  }
  return pa_sort_u32(dst, src, n, opts);  // src is the scratch, as in the reference
}

int pa_partition_radix_u32(uint32_t* a, size_t n, const size_t* k, size_t k_len, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (k_len == 0 || n == 0) return PA_OK;
  if (!a || !k) return set_error(PA_ERR_ARG, "NULL buffer");
  for (size_t i = 0; i < k_len; ++i) {
    if (k[i] >= n) return set_error(PA_ERR_ARG, "k[%zu] = %zu is not below n = %zu", i, k[i], n);
    if (i && k[i] < k[i - 1]) return set_error(PA_ERR_ARG, "k[] must be ascending (k[%zu] < k[%zu])", i, i - 1);
  }
  // Many k: a sorted array is partitioned around every k at once (each
  // a[k[i]] is the k[i]-th smallest, nothing before it is larger, nothing
  // after it is smaller), so the partition is one GPU sort.
  if (k_len > kPartitionSelectMax) return pa_sort_u32(a, nullptr, n, opts);
  // A few k: one select per k gives the pivot values, then one pass puts
  // every key in its bucket among them (pa_partition.cu), about
  // (20 + 4 k_len) bytes per key against the sort's 36.
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool dev = is_device_ptr(a);
  const size_t cand_cap = n / 4 + 1024;
  uint32_t *d_a = nullptr, *tmp = nullptr, *piv = nullptr;
  void *cand = nullptr, *work = nullptr;
  unsigned long long* counts = nullptr;
  auto layout = [&](Carve& c) {
    d_a = dev ? a : c.take<uint32_t>(n);
    tmp = c.take<uint32_t>(n);
    cand = c.take<char>(cand_cap * 4);
    work = c.take<char>(select_state_bytes());
    piv = c.take<uint32_t>(kPartitionMaxPivots);
    counts = c.take<unsigned long long>(partition_scratch_words(n, (int)k_len));
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!dev) PA_CUDA(cudaMemcpyAsync(d_a, a, n * 4, cudaMemcpyHostToDevice, stream));
  for (size_t i = 0; i < k_len; ++i)
    PA_CUDA(launch_select(d_a, n, k[i], 4, cand, cand_cap, work, piv + i, ws->err, stream));
  PA_CUDA(launch_partition(d_a, tmp, n, piv, (int)k_len, counts, stream));
  PA_CUDA(cudaMemcpyAsync(a, tmp, n * 4, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, dev && opts && opts->async_device);
}

int pa_hist_quanta_u32(const uint32_t* a, size_t l, size_t r, size_t work_quanta, size_t quanta,
                       unsigned which_byte, uint64_t* out, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (!out || (quanta && !a)) return set_error(PA_ERR_ARG, "NULL buffer");
  if (which_byte > 3) return set_error(PA_ERR_ARG, "which_byte %u is not below 4", which_byte);
  if (work_quanta == 0) return set_error(PA_ERR_ARG, "work_quanta is 0");
  if (l <= r && r / work_quanta >= quanta)
    return set_error(PA_ERR_ARG, "index %zu falls in quantum %zu, beyond quanta = %zu", r, r / work_quanta, quanta);
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const size_t len = l <= r ? r - l + 1 : 0;
  const bool in_dev = is_device_ptr(a);
  const bool out_dev = is_device_ptr(out);
  const uint32_t* d_in = nullptr;
  unsigned long long* d_out = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? a + l : c.take<uint32_t>(len);
    d_out = out_dev ? reinterpret_cast<unsigned long long*>(out) : c.take<unsigned long long>(quanta * 256);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve rr{ws->dev};
  layout(rr);
  if (!in_dev && len)
    PA_CUDA(cudaMemcpyAsync(const_cast<uint32_t*>(d_in), a + l, len * 4, cudaMemcpyHostToDevice, stream));
  PA_CUDA(cudaMemsetAsync(d_out, 0, quanta * 256 * sizeof(uint64_t), stream));
  if (len) PA_CUDA(launch_quanta_counts(d_in, l, l + len, work_quanta, which_byte, d_out, stream));
  if (!out_dev) PA_CUDA(cudaMemcpyAsync(out, d_out, quanta * 256 * sizeof(uint64_t), cudaMemcpyDeviceToHost, stream));
  return finish(ws, stream, opts && opts->async_device && in_dev && out_dev);
}

int pa_start_of_bins_u32(const uint32_t* a, size_t n, size_t work_quanta, size_t quanta, unsigned digit,
                         uint64_t* out, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (!out || (n && !a)) return set_error(PA_ERR_ARG, "NULL buffer");
  if (digit > 3) return set_error(PA_ERR_ARG, "digit %u is not below 4", digit);
  if (work_quanta == 0) return set_error(PA_ERR_ARG, "work_quanta is 0");
  if (n && (n - 1) / work_quanta >= quanta)
    return set_error(PA_ERR_ARG, "n = %zu needs more than quanta = %zu", n, quanta);
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  const bool in_dev = is_device_ptr(a);
  const bool out_dev = is_device_ptr(out);
  const uint32_t* d_in = nullptr;
  unsigned long long *counts = nullptr, *sob = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? a : c.take<uint32_t>(n);
    counts = c.take<unsigned long long>(quanta * 256);
    sob = c.take<unsigned long long>(quanta * 256 + 256);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve rr{ws->dev};
  layout(rr);
  if (!in_dev && n) PA_CUDA(cudaMemcpyAsync(const_cast<uint32_t*>(d_in), a, n * 4, cudaMemcpyHostToDevice, stream));
  PA_CUDA(cudaMemsetAsync(counts, 0, quanta * 256 * sizeof(uint64_t), stream));
  if (n) PA_CUDA(launch_quanta_counts(d_in, 0, n, work_quanta, digit, counts, stream));
  PA_CUDA(launch_quanta_start_of_bins(counts, quanta, sob, stream));
  PA_CUDA(cudaMemcpyAsync(out, sob, quanta * 256 * sizeof(uint64_t), out_dev ? cudaMemcpyDeviceToDevice
                                                                             : cudaMemcpyDeviceToHost,
                          stream));
  return finish(ws, stream, opts && opts->async_device && in_dev && out_dev);
}

int pa_select_u32(const uint32_t* a, size_t n, size_t k, uint32_t* out, const pa_opts* opts) {
  return select_impl(a, n, k, 4, out, opts);
}
int pa_select_u64(const uint64_t* a, size_t n, size_t k, uint64_t* out, const pa_opts* opts) {
  return select_impl(a, n, k, 8, out, opts);
}

int pa_select_radix_u32(uint32_t* a, size_t start, size_t length, size_t k, uint32_t* out, const pa_opts* opts) {
  if (int rc = check_opts(opts)) return rc;
  if (!a || !out) return set_error(PA_ERR_ARG, "NULL buffer");
  if (length == 0 || k < start || k - start >= length)
    return set_error(PA_ERR_ARG, "k = %zu is outside [start, start + length) = [%zu, %zu)", k, start, start + length);
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = stream_of(opts);
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  uint32_t* base = a + start;
  const size_t n = length, kk = k - start;
  const bool in_dev = is_device_ptr(base);
  const bool out_dev = is_device_ptr(out);
  const size_t cand_cap = n / 4 + 1024;
  uint32_t* d_in = nullptr;
  void *cand = nullptr, *work = nullptr;
  uint32_t* d_val = nullptr;
  unsigned long long* d_idx = nullptr;
  auto layout = [&](Carve& c) {
    d_in = in_dev ? base : c.take<uint32_t>(n);
    cand = c.take<char>(cand_cap * 4);
    work = c.take<char>(select_state_bytes());
    d_val = c.take<uint32_t>(2);
    d_idx = c.take<unsigned long long>(1);
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  if (!in_dev) PA_CUDA(cudaMemcpyAsync(d_in, base, n * 4, cudaMemcpyHostToDevice, stream));
  PA_CUDA(launch_select(d_in, n, kk, 4, cand, cand_cap, work, d_val, ws->err, stream));
  // The reference rearranges the range and leaves the answer at a[k]; here
  // the answer is swapped with a[k] from the first place that holds it, so
  // the range stays a permutation of its input.
  PA_CUDA(launch_find_key(d_in, n, kk, d_val, d_idx, stream));
  if (in_dev) PA_CUDA(launch_swap_key(d_in, n, kk, d_idx, stream));
  PA_CUDA(cudaMemcpyAsync(out, d_val, 4, out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream));
  unsigned long long idx = n;
  if (!in_dev) PA_CUDA(cudaMemcpyAsync(&idx, d_idx, sizeof(idx), cudaMemcpyDeviceToHost, stream));
  const int rc = finish(ws, stream, in_dev && out_dev && opts && opts->async_device);
  if (rc != PA_OK) return rc;
  if (!in_dev && idx < n && idx != kk) std::swap(base[idx], base[kk]);
  return PA_OK;
}

int pa_selftest_wait_expiry(unsigned spin_limit) {
  if (spin_limit == 0) return set_error(PA_ERR_ARG, "spin_limit must be positive");
  if (int rc = device_ready()) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t stream = 0;
  Workspace* ws = nullptr;
  if (int rc = get_workspace(stream, &ws)) return rc;
  // Two tiles of keys; the one CTA launched takes ticket 1, so its look-back
  // polls tile 0's status word, which no CTA ever publishes.
  const size_t n = 2 * onesweep_tile_keys(4, false);
  uint32_t *keys = nullptr, *tmp = nullptr, *ticket = nullptr;
  unsigned long long* bin_start = nullptr;
  char* status = nullptr;
  SortCtrl* ctrl = nullptr;
  auto layout = [&](Carve& c) {
    keys = c.take<uint32_t>(n);
    tmp = c.take<uint32_t>(n);
    bin_start = c.take<unsigned long long>(256);
    status = c.take<char>(2 * 256 * onesweep_status_bytes(n));
    ticket = c.take<uint32_t>(1);
    ctrl = c.take<SortCtrl>(1);  // all zero: pass 0 runs, keys -> tmp
  };
  Carve m{nullptr};
  layout(m);
  if (int rc = ensure_dev(ws, stream, m.off)) return rc;
  Carve r{ws->dev};
  layout(r);
  static const uint32_t kTicket = 1;
  PA_CUDA(cudaMemsetAsync(ws->dev, 0, r.off, stream));
  PA_CUDA(cudaMemcpyAsync(ticket, &kTicket, sizeof(kTicket), cudaMemcpyHostToDevice, stream));
  OnesweepArgs a{};
  a.keys_a = keys;
  a.keys_b = tmp;
  a.n = n;
  a.bin_start = bin_start;
  a.status = status;
  a.tile_counter = ticket;
  a.ctrl = ctrl;
  a.err = ws->err;
  a.spin_limit = spin_limit;
  a.max_ctas = 1;
  PA_CUDA(launch_onesweep_pass(a, 4, false, stream));
  return finish(ws, stream, false);
}

int pa_sum_u32(const uint32_t* a, size_t n, uint64_t* out, const pa_opts* opts) {
  return sum_impl(a, n, kElemU32, out, opts);
}
int pa_sum_u64(const uint64_t* a, size_t n, uint64_t* out, const pa_opts* opts) {
  return sum_impl(a, n, kElemU64, out, opts);
}
int pa_sum_typed(const void* a, size_t n, int elem_kind, uint64_t* out, const pa_opts* opts) {
  return sum_impl(a, n, elem_kind, out, opts);
}
int pa_sum_chunked(const void* a, size_t n, int elem_kind, size_t chunk, uint64_t* chunk_sums, uint64_t* out,
                   const pa_opts* opts) {
  if (n && !chunk_sums) return set_error(PA_ERR_ARG, "chunk_sums is NULL");
  if (n == 0) {
    if (!out) return set_error(PA_ERR_ARG, "out is NULL");
    const uint64_t zero = 0;
    PA_CUDA(cudaMemcpy(out, &zero, sizeof(zero), cudaMemcpyDefault));
    return PA_OK;
  }
  return sum_impl(a, n, elem_kind, out, opts, chunk, chunk_sums);
}

}  // extern "C"
