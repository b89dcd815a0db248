// Serving loop: sort / select / histogram requests arrive on any thread, are
// admitted against an HBM budget, run with their data device-resident, and
// complete asynchronously.  Waiting requests of one kind share a unit:
// 32-bit sorts one batched launch (the persistent segmented-sort kernel),
// histograms one launch over all their arrays, 64-bit sorts and selects one
// allocation, stream and completion event.  Scheduling policy:
// pa_serve_core.h; this file is its CUDA backend and the C ABI.
//
// No reference counterpart (the reference has no serving path; its nearest
// idea is choosing an algorithm by free physical memory, RadixSortLSD.h:
// 799-892 with MemoryUsage.cpp:20-87, which here becomes admission by free
// HBM against a configured budget).
//
// Each admitted unit runs on the least busy of several streams: host->device
// copies of its keys, its kernels, device->host copies of its results, all in
// one stream-ordered allocation from the server's own memory pool (so
// admission never synchronises the device), then an event the scheduler
// polls.  Units on different streams overlap: copies of one with kernels of
// another.  The pool does not let a unit reuse memory that a unit on another
// stream freed but whose work is still running (that reuse would make the
// runtime chain the two streams and serialise the units); it reuses memory
// once the freeing unit's work has completed, and keeps what it has mapped
// until the server is destroyed.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "pa_common.cuh"
#include "pa_gpu.h"
#include "pa_kernels.cuh"
#include "pa_segmented.cuh"
#include "pa_serve_core.h"

namespace pa {
namespace serve {
namespace {

struct UnitState {
  int lane = 0;
  cudaEvent_t ev = nullptr;
  char* dmem = nullptr;
  uint32_t* err_host = nullptr;  // pinned word the unit's device error word is copied to
  void* staging = nullptr;       // pinned image of a batched unit's plan tables
  void* result_host = nullptr;   // pinned landing place of a select / histogram result
  cudaError_t launch_error = cudaSuccess;
  std::unique_ptr<seg::HostPlan> plan;
};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

pa_request* user_of(const Request* r) { return static_cast<pa_request*>(r->user); }

bool is_dev(const void* p) {
  cudaPointerAttributes at;
  if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Streams outlive servers: a server takes its streams from a process-wide
// free list (per device) and returns them when it is destroyed.  Measured on
// GB300: with a fresh set of 32 streams created and destroyed per server, the
// host-buffer makespan of the same request stream grew from ~40 ms to ~100 ms
// over twenty servers created one after another in one process, while the
// same stream on device-resident keys (no host copies) and single-stream
// copies stayed flat.
std::mutex g_stream_mu;
std::vector<std::pair<int, cudaStream_t>> g_free_streams;

cudaStream_t take_stream(int device) {
  {
    std::lock_guard<std::mutex> lk(g_stream_mu);
    for (size_t i = 0; i < g_free_streams.size(); ++i)
      if (g_free_streams[i].first == device) {
        const cudaStream_t s = g_free_streams[i].second;
        g_free_streams.erase(g_free_streams.begin() + (long)i);
        return s;
      }
  }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return s;
}

void give_stream(int device, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(g_stream_mu);
  g_free_streams.emplace_back(device, s);
}

class GpuBackend {
 public:
  explicit GpuBackend(int lanes) {
    cudaGetDevice(&device_);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device_;
    if (cudaMemPoolCreate(&pool_, &props) == cudaSuccess) {
      uint64_t keep = ~0ull;
      int no = 0, yes = 1;
      cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep);
      cudaMemPoolSetAttribute(pool_, cudaMemPoolReuseAllowInternalDependencies, &no);
      cudaMemPoolSetAttribute(pool_, cudaMemPoolReuseAllowOpportunistic, &yes);
      cudaMemPoolSetAttribute(pool_, cudaMemPoolReuseFollowEventDependencies, &yes);
    } else {
      pool_ = nullptr;
    }
    cudaGetLastError();
    for (int i = 0; i < lanes; ++i) {
      const cudaStream_t s = take_stream(device_);
      if (!s) break;
      streams_.push_back(s);
      lane_units_.push_back(0);
    }
  }
  ~GpuBackend() {
    for (auto s : streams_) {
      cudaStreamSynchronize(s);
      give_stream(device_, s);
    }
    if (pool_) cudaMemPoolDestroy(pool_);
    for (const auto& b : pinned_) cudaFreeHost(b.first);
  }
  bool ok() const { return pool_ != nullptr && !streams_.empty(); }

  // Maps `bytes` into the pool now (one allocation, freed at once; the pool
  // keeps what it mapped), so later admissions reuse it instead of waiting
  // for the driver to map memory.
  cudaError_t reserve(size_t bytes) {
    if (!bytes) return cudaSuccess;
    void* p = nullptr;
    cudaStream_t s = streams_[0];
    cudaError_t e = cudaMallocFromPoolAsync(&p, bytes, pool_, s);
    if (e == cudaSuccess) e = cudaFreeAsync(p, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) cudaGetLastError();
    return e;
  }
  int device() const { return device_; }

  // Device memory free to the driver plus what the server's pool holds mapped
  // but unused (it keeps memory of finished units for reuse).
  size_t free_bytes() {
    size_t f = 0, t = 0;
    if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    uint64_t reserved = 0, used = 0;
    if (pool_ && cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(pool_, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      f += (size_t)(reserved - used);
    cudaGetLastError();
    return f;
  }

  // 32-bit sorts of a shared unit run as one segmented-sort launch.
  static bool segmented(const Unit& u) {
    return u.batched && u.reqs[0]->op == OP_SORT && u.reqs[0]->key_bytes == 4;
  }
  // Bytes of one request's result slot: the select's key (8, zero-extended)
  // or the histogram's 256 counts.
  static size_t result_slot(int op) { return op == OP_SELECT ? 8 : op == OP_HIST ? 256 * 8 : 0; }

  size_t unit_bytes(const Unit& u) {
    if (segmented(u)) {
      size_t total = 0;
      for (const Request* r : u.reqs) total += r->n;
      // keys + tmp, plus the plan block (under 1 byte per key for 8192-key tiles)
      return 1024 + align256(total * 4) * 2 + total + ((size_t)8 << 20);
    }
    return group_layout(u, nullptr, nullptr);
  }
  void launch(Unit& u) {
    auto* st = new UnitState();
    u.state = st;
    // the lane with the fewest units in flight; ties go round robin
    const int lanes = (int)streams_.size();
    st->lane = next_lane_;
    for (int i = 1; i < lanes; ++i) {
      const int c = (next_lane_ + i) % lanes;
      if (lane_units_[c] < lane_units_[st->lane]) st->lane = c;
    }
    next_lane_ = (st->lane + 1) % (int)streams_.size();
    ++lane_units_[st->lane];
    u.lane = st->lane;
    cudaStream_t s = streams_[st->lane];
    st->err_host = static_cast<uint32_t*>(take_pinned(64));
    if (!st->err_host) {
      st->launch_error = cudaErrorMemoryAllocation;
      return;
    }
    *st->err_host = 0;
    cudaError_t e = cudaEventCreateWithFlags(&st->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&st->dmem), u.bytes, pool_, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(st->dmem, 0, 256, s);  // error word + result slot
    if (e == cudaSuccess) e = segmented(u) ? launch_batch(u, st, s) : launch_group(u, st, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st->err_host, st->dmem, 4, cudaMemcpyDeviceToHost, s);
    if (st->dmem) {
      const cudaError_t f = cudaFreeAsync(st->dmem, s);
      if (e == cudaSuccess) e = f;
    }
    if (e == cudaSuccess) e = cudaEventRecord(st->ev, s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      st->launch_error = e;
    }
  }

  bool finished(Unit& u) {
    auto* st = static_cast<UnitState*>(u.state);
    if (st->launch_error != cudaSuccess) return true;
    const cudaError_t q = cudaEventQuery(st->ev);
    if (q == cudaErrorNotReady) return false;
    if (q != cudaSuccess) {
      cudaGetLastError();
      st->launch_error = q;
    }
    return true;
  }

  void finish(Unit& u) {
    auto* st = static_cast<UnitState*>(u.state);
    int status = PA_OK;
    // after a failed launch, copies enqueued before the failure may still
    // read the request's buffers or the staging block: let them finish
    if (st->launch_error != cudaSuccess) {
      cudaStreamSynchronize(streams_[st->lane]);
      cudaGetLastError();
    }
    if (st->launch_error != cudaSuccess)
      status = st->launch_error == cudaErrorMemoryAllocation ? PA_ERR_OOM : PA_ERR_CUDA;
    else if (*st->err_host)
      status = PA_ERR_TIMEOUT;
    // results land in page-locked memory first (a device-to-host copy into the
    // caller's pageable array would make the launching thread wait for the
    // unit's work); they move to the caller's array now that the work is done
    if (status == PA_OK && st->result_host) {
      const size_t slot = result_slot(u.reqs[0]->op);
      for (size_t i = 0; i < u.reqs.size(); ++i)
        std::memcpy(user_of(u.reqs[i])->result, static_cast<char*>(st->result_host) + i * slot, slot);
    }
    for (Request* r : u.reqs) r->status = status;
    if (st->ev) cudaEventDestroy(st->ev);
    --lane_units_[st->lane];
    give_pinned(st->err_host);
    give_pinned(st->staging);
    give_pinned(st->result_host);
    delete st;
    u.state = nullptr;
  }

  double now() { return now_s(); }

 private:
  // A unit of requests of one kind (one request, or a shared unit of 64-bit
  // sorts, selects or histograms), laid out in one device block:
  //   [error word 256][result slots][histogram job table][per request: keys
  //   (host buffers only), then tmp + sort scratch, or the select's
  //   candidates + state].
  // Measures the block (dmem == nullptr, returns its bytes) or enqueues the
  // unit's copies and kernels on `s` with that layout.  Requests of a unit
  // run one after another on its stream; the histograms of a unit are counted
  // by one launch over all of their arrays.
  size_t group_layout(const Unit& u, UnitState* st, cudaStream_t s, cudaError_t* err_out = nullptr) {
    const Request* h = u.reqs[0];
    const int op = h->op;
    const size_t kb = (size_t)h->key_bytes;
    const size_t cnt = u.reqs.size();
    const size_t slot = result_slot(op);
    char* base = st ? st->dmem : nullptr;
    const bool run = base != nullptr;
    cudaError_t e = cudaSuccess;
    uint32_t* err = reinterpret_cast<uint32_t*>(base);
    size_t off = 256;
    char* results = base + off;
    off += align256(slot * cnt);
    HistJob* jobs = reinterpret_cast<HistJob*>(base + off);
    if (op == OP_HIST) off += align256(sizeof(HistJob) * cnt);
    std::vector<HistJob> hj;
    uint32_t chunks = 0;
    if (run && slot) {
      st->result_host = take_pinned(slot * cnt);
      if (!st->result_host) e = cudaErrorMemoryAllocation;
      if (e == cudaSuccess) e = cudaMemsetAsync(results, 0, slot * cnt, s);
    }
    for (size_t i = 0; i < cnt && e == cudaSuccess; ++i) {
      const Request* r = u.reqs[i];
      pa_request* q = user_of(r);
      const bool host = !q->internal_device;
      void* keys = q->keys;
      if (host) {
        keys = base + off;
        off += align256(r->n * kb);
        if (run) e = cudaMemcpyAsync(keys, q->keys, r->n * kb, cudaMemcpyHostToDevice, s);
      }
      if (op == OP_SORT) {
        void* tmp = base + off;
        off += align256(r->n * kb);
        char* scratch = base + off;
        off += align256(sort_scratch_bytes(r->n, (int)kb, false));
        if (run && e == cudaSuccess) {
          SortScratch sc{};
          sort_scratch_layout(scratch, r->n, (int)kb, false, &sc);
          e = enqueue_sort(sc, keys, tmp, nullptr, nullptr, r->n, (int)kb, false, err, s);
          if (e == cudaSuccess && host) e = cudaMemcpyAsync(q->keys, keys, r->n * kb, cudaMemcpyDeviceToHost, s);
        }
      } else if (op == OP_SELECT) {
        const size_t cap = r->n / 4 + 1024;
        void* cand = base + off;
        off += align256(cap * kb);
        void* work = base + off;
        off += align256(select_state_bytes());
        if (run && e == cudaSuccess) e = launch_select(keys, r->n, q->k, (int)kb, cand, cap, work, results + i * slot, err, s);
      } else {
        hj.push_back({keys, (unsigned long long)r->n, reinterpret_cast<unsigned long long*>(results + i * slot),
                      q->shift, chunks});
        chunks += (uint32_t)((r->n + kHistJobChunk - 1) / kHistJobChunk);
      }
    }
    if (run && e == cudaSuccess && op == OP_HIST) {
      // the job table goes up from page-locked memory (see launch_batch)
      st->staging = take_pinned(sizeof(HistJob) * cnt);
      if (!st->staging) e = cudaErrorMemoryAllocation;
      if (e == cudaSuccess) {
        std::memcpy(st->staging, hj.data(), sizeof(HistJob) * cnt);
        e = cudaMemcpyAsync(jobs, st->staging, sizeof(HistJob) * cnt, cudaMemcpyHostToDevice, s);
      }
      if (e == cudaSuccess) e = launch_digit_counts_multi(jobs, (int)cnt, chunks, (int)kb, s);
    }
    if (run && e == cudaSuccess && slot)
      e = cudaMemcpyAsync(st->result_host, results, slot * cnt, cudaMemcpyDeviceToHost, s);
    if (err_out) *err_out = e;
    return off + 1024;
  }

  cudaError_t launch_group(Unit& u, UnitState* st, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    group_layout(u, st, s, &e);
    return e;
  }

  // Coalesced 32-bit sorts: keys back to back, one persistent segmented-sort
  // launch over them, results copied back per request.
  cudaError_t launch_batch(Unit& u, UnitState* st, cudaStream_t s) {
    std::vector<uint64_t> off(u.reqs.size() + 1, 0);
    for (size_t i = 0; i < u.reqs.size(); ++i) off[i + 1] = off[i] + u.reqs[i]->n;
    const size_t total = off.back();
    st->plan.reset(new seg::HostPlan());
    pa_segsort_config cfg{};
    if (seg::build_host_plan(off.data(), u.reqs.size(), &cfg, st->plan.get()) != PA_OK) return cudaErrorInvalidValue;
    // the plan tables go up from page-locked memory: a copy from pageable
    // memory would make this thread wait for the stream's earlier copies
    st->staging = take_pinned(seg::plan_image_bytes(*st->plan));
    if (!st->staging) return cudaErrorMemoryAllocation;
    char* base = st->dmem;
    uint32_t* keys = reinterpret_cast<uint32_t*>(base + 256);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(base + 256 + align256(total * 4));
    char* plan = base + 256 + 2 * align256(total * 4);
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < u.reqs.size() && e == cudaSuccess; ++i) {
      pa_request* q = user_of(u.reqs[i]);
      e = cudaMemcpyAsync(keys + off[i], q->keys, u.reqs[i]->n * 4, cudaMemcpyDefault, s);
    }
    if (e == cudaSuccess) e = seg::upload_plan(*st->plan, plan, s, st->staging);
    if (e == cudaSuccess) {
      seg::PlanDev pd = seg::device_view(*st->plan, plan, keys, tmp);
      pd.err = reinterpret_cast<uint32_t*>(base);  // the unit's error word
      e = seg::launch_plan(*st->plan, pd, plan, seg::plan_grid(*st->plan), s);
    }
    for (size_t i = 0; i < u.reqs.size() && e == cudaSuccess; ++i) {
      pa_request* q = user_of(u.reqs[i]);
      e = cudaMemcpyAsync(q->keys, keys + off[i], u.reqs[i]->n * 4, cudaMemcpyDefault, s);
    }
    return e;
  }

  // Page-locked host blocks in power-of-two size classes, kept for reuse
  // until the server is destroyed (freeing page-locked memory synchronises
  // the device).  Returns nullptr if the allocation fails.
  static int size_class(size_t bytes) {
    int c = 6;
    while (((size_t)1 << c) < bytes) ++c;
    return c;
  }
  void* take_pinned(size_t bytes) {
    const int c = size_class(bytes);
    std::lock_guard<std::mutex> lk(mu_);
    auto& fl = free_pinned_[c];
    if (!fl.empty()) {
      void* p = fl.back();
      fl.pop_back();
      return p;
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, (size_t)1 << c) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    pinned_.push_back({p, c});
    return p;
  }
  void give_pinned(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    for (const auto& b : pinned_)
      if (b.first == p) {
        free_pinned_[b.second].push_back(p);
        return;
      }
  }

  int device_ = 0;
  cudaMemPool_t pool_ = nullptr;
  std::vector<cudaStream_t> streams_;
  std::vector<int> lane_units_;
  int next_lane_ = 0;
  std::mutex mu_;
  std::vector<std::pair<void*, int>> pinned_;
  std::vector<void*> free_pinned_[64];
};

}  // namespace
}  // namespace serve
}  // namespace pa

using namespace pa;
using namespace pa::serve;

struct pa_server {
  std::unique_ptr<GpuBackend> backend;
  std::unique_ptr<Scheduler<GpuBackend>> sched;
  std::thread worker;
  std::atomic<bool> stop{false};
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::atomic<size_t> outstanding{0};
};

namespace {

void on_done(pa_server* s, Request* r) {
  pa_request* q = static_cast<pa_request*>(r->user);
  q->t_submit = r->t_submit;
  q->t_admit = r->t_admit;
  q->t_done = r->t_done;
  q->unit_size = r->unit_size;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    q->status = r->status;  // published last: waiters key on it
    s->outstanding--;
  }
  delete r;
  s->done_cv.notify_all();
}

void worker_loop(pa_server* s, int device) {
  cudaSetDevice(device);
  while (!s->stop.load() || !s->sched->idle()) {
    if (!s->sched->step()) {
      std::unique_lock<std::mutex> lk(s->mu);
      s->work_cv.wait_for(lk, std::chrono::microseconds(50));
    }
  }
}

}  // namespace

extern "C" {

int pa_server_create(const pa_serve_config* cfg, pa_server** out) {
  if (!out) return record_error(PA_ERR_ARG, "out is NULL");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return record_error(PA_ERR_NO_DEVICE, "no CUDA device");
  }
  pa_serve_config c{};
  if (cfg) c = *cfg;
  for (int r : c.reserved)
    if (r) return record_error(PA_ERR_ARG, "pa_serve_config.reserved must be zero");
  if (c.reserve_mib < 0) return record_error(PA_ERR_ARG, "pa_serve_config.reserve_mib is negative");
  Config sc;
  if (c.hbm_budget_bytes) sc.budget_bytes = c.hbm_budget_bytes;
  if (c.max_inflight > 0) sc.max_inflight = c.max_inflight;
  if (c.max_batch_requests > 0) sc.max_batch_requests = c.max_batch_requests;
  if (c.join_max_keys_log2 < 0 || c.join_max_keys_log2 > 40 || c.unit_max_keys_log2 < 0 ||
      c.unit_max_keys_log2 > 40)
    return record_error(PA_ERR_ARG, "pa_serve_config: key limits are powers of two up to 2^40");
  if (c.join_max_keys_log2 > 0) sc.max_join_keys = (size_t)1 << c.join_max_keys_log2;
  if (c.unit_max_keys_log2 > 0) sc.max_batch_keys = sc.max_group_keys = (size_t)1 << c.unit_max_keys_log2;
  sc.coalesce = c.no_coalesce == 0;
  const int lanes = c.num_streams > 0 ? c.num_streams : 4;
  auto* s = new pa_server();
  s->backend.reset(new GpuBackend(lanes));
  if (!s->backend->ok()) {
    delete s;
    return record_error(PA_ERR_CUDA, "could not create the server's memory pool or streams");
  }
  if (c.reserve_mib > 0) {
    const size_t want = std::min((size_t)c.reserve_mib << 20, sc.budget_bytes);
    if (s->backend->reserve(want) != cudaSuccess) {
      delete s;
      return record_error(PA_ERR_OOM, "could not map reserve_mib of device memory into the server's pool");
    }
  }
  s->sched.reset(new Scheduler<GpuBackend>(*s->backend, sc, [s](Request* r) { on_done(s, r); }));
  s->worker = std::thread(worker_loop, s, s->backend->device());
  *out = s;
  return PA_OK;
}

int pa_server_submit(pa_server* s, pa_request* q) {
  if (!s || !q) return record_error(PA_ERR_ARG, "NULL server or request");
  if (q->op < PA_REQ_SORT || q->op > PA_REQ_HISTOGRAM) return record_error(PA_ERR_ARG, "unknown request op");
  if (q->key_kind != PA_KEY_U32 && q->key_kind != PA_KEY_U64)
    return record_error(PA_ERR_ARG, "key_kind must be PA_KEY_U32 or PA_KEY_U64");
  if (q->n && !q->keys) return record_error(PA_ERR_ARG, "keys is NULL");
  if (q->op == PA_REQ_SELECT && q->k >= q->n) return record_error(PA_ERR_ARG, "select k is not below n");
  if (q->op == PA_REQ_HISTOGRAM && q->shift >= (q->key_kind == PA_KEY_U32 ? 32u : 64u))
    return record_error(PA_ERR_ARG, "histogram shift too large");
  if (q->op != PA_REQ_SORT && !q->result) return record_error(PA_ERR_ARG, "result is NULL");
  q->internal_device = is_dev(q->keys) ? 1 : 0;
  q->unit_size = 0;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    q->status = -1;
    s->outstanding++;
  }
  if (q->n == 0 || (q->op == PA_REQ_SORT && q->n == 1)) {  // nothing to do on the device
    std::lock_guard<std::mutex> lk(s->mu);
    q->t_submit = q->t_admit = q->t_done = now_s();
    q->unit_size = 1;
    q->status = PA_OK;
    s->outstanding--;
    s->done_cv.notify_all();
    return PA_OK;
  }
  auto* r = new Request();
  r->op = q->op == PA_REQ_SORT ? OP_SORT : q->op == PA_REQ_SELECT ? OP_SELECT : OP_HIST;
  r->key_bytes = q->key_kind == PA_KEY_U32 ? 4 : 8;
  r->n = q->n;
  r->user = q;
  s->sched->submit(r);
  s->work_cv.notify_one();
  return PA_OK;
}

int pa_server_wait(pa_server* s, pa_request* q) {
  if (!s || !q) return record_error(PA_ERR_ARG, "NULL server or request");
  std::unique_lock<std::mutex> lk(s->mu);
  s->done_cv.wait(lk, [q] { return q->status != -1; });
  return q->status;
}

int pa_server_drain(pa_server* s) {
  if (!s) return record_error(PA_ERR_ARG, "NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  s->done_cv.wait(lk, [s] { return s->outstanding.load() == 0; });
  return PA_OK;
}

int pa_server_stats(pa_server* s, uint64_t* out, int count) {
  if (!s || !out) return record_error(PA_ERR_ARG, "NULL argument");
  const Stats st = s->sched->stats();
  const uint64_t v[9] = {st.submitted, st.completed, st.rejected, st.units, st.batched_units, st.coalesced_requests,
                         st.peak_bytes, (uint64_t)(st.launch_s * 1e6), (uint64_t)(st.finish_s * 1e6)};
  for (int i = 0; i < count && i < 9; ++i) out[i] = v[i];
  return PA_OK;
}

int pa_server_destroy(pa_server* s) {
  if (!s) return PA_OK;
  pa_server_drain(s);
  s->stop = true;
  s->work_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  delete s;
  return PA_OK;
}

}  // extern "C"
