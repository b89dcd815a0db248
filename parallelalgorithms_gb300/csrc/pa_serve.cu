// Serving loop: sort / select / histogram requests arrive on any thread, are
// admitted against an HBM budget, run with their data device-resident, and
// complete asynchronously, with waiting 32-bit sorts coalesced into one
// batched launch (the persistent segmented-sort kernel).  Scheduling policy:
// pa_serve_core.h; this file is its CUDA backend and the C ABI.
//
// No reference counterpart (the reference has no serving path; its nearest
// idea is choosing an algorithm by free physical memory, RadixSortLSD.h:
// 799-892 with MemoryUsage.cpp:20-87, which here becomes admission by free
// HBM against a configured budget).
//
// Each admitted unit runs on one of several streams: host->device copies of
// its keys, its kernels, device->host copies of its results, all in one
// stream-ordered allocation (cudaMallocAsync / cudaFreeAsync, so admission
// never synchronises the device), then an event the scheduler polls.
// Units on different streams overlap: copies of one with kernels of another.
#include <cuda_runtime.h>

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

class GpuBackend {
 public:
  GpuBackend(int lanes) {
    cudaGetDevice(&device_);
    // Keep memory freed by finished units in the process's stream-ordered pool
    // instead of returning it to the driver at every synchronisation.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device_) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
    for (int i = 0; i < lanes; ++i) {
      cudaStream_t s;
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
      streams_.push_back(s);
    }
  }
  ~GpuBackend() {
    for (auto s : streams_) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    for (auto* w : pinned_words_) cudaFreeHost(w);
  }
  int device() const { return device_; }

  size_t free_bytes() {
    size_t f = 0, t = 0;
    if (cudaMemGetInfo(&f, &t) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return f;
  }

  size_t unit_bytes(const Unit& u) {
    size_t b = 1024;  // error word + result slots
    if (u.batched) {
      size_t total = 0;
      for (const Request* r : u.reqs) total += r->n;
      // keys + tmp, plus the plan block (under 1 byte per key for 8192-key tiles)
      return b + align256(total * 4) * 2 + total + ((size_t)8 << 20);
    }
    const Request* r = u.reqs[0];
    const pa_request* q = user_of(r);
    const size_t kb = (size_t)r->key_bytes;
    const bool host = !q->internal_device;
    if (host) b += align256(r->n * kb);
    switch (r->op) {
      case OP_SORT: b += align256(r->n * kb) + align256(sort_scratch_bytes(r->n, (int)kb, false)); break;
      case OP_SELECT: b += align256((r->n / 4 + 1024) * kb) + align256(select_state_bytes()); break;
      default: b += 256 * 8; break;
    }
    return b;
  }

  void launch(Unit& u) {
    auto* st = new UnitState();
    u.state = st;
    st->lane = next_lane_++ % (int)streams_.size();
    u.lane = st->lane;
    cudaStream_t s = streams_[st->lane];
    st->err_host = take_word();
    *st->err_host = 0;
    cudaError_t e = cudaEventCreateWithFlags(&st->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&st->dmem), u.bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(st->dmem, 0, 256, s);  // error word + result slot
    if (e == cudaSuccess) e = u.batched ? launch_batch(u, st, s) : launch_single(u, st, s);
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
    if (st->launch_error != cudaSuccess)
      status = st->launch_error == cudaErrorMemoryAllocation ? PA_ERR_OOM : PA_ERR_CUDA;
    else if (*st->err_host)
      status = PA_ERR_TIMEOUT;
    for (Request* r : u.reqs) r->status = status;
    if (st->ev) cudaEventDestroy(st->ev);
    give_word(st->err_host);
    delete st;
    u.state = nullptr;
  }

  double now() { return now_s(); }

 private:
  // Layout of a single-request unit: [err+result 256][keys][tmp / cand][scratch]
  cudaError_t launch_single(Unit& u, UnitState* st, cudaStream_t s) {
    Request* r = u.reqs[0];
    pa_request* q = user_of(r);
    const size_t kb = (size_t)r->key_bytes;
    char* base = st->dmem;
    uint32_t* err = reinterpret_cast<uint32_t*>(base);
    void* result = base + 8;  // 8-byte select result
    size_t off = 256;
    void* keys = q->keys;
    const bool host = !q->internal_device;
    cudaError_t e = cudaSuccess;
    if (host) {
      keys = base + off;
      off += align256(r->n * kb);
      e = cudaMemcpyAsync(keys, q->keys, r->n * kb, cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess) return e;
    if (r->op == OP_SORT) {
      void* tmp = base + off;
      off += align256(r->n * kb);
      SortScratch sc{};
      sort_scratch_layout(base + off, r->n, (int)kb, false, &sc);
      e = enqueue_sort(sc, keys, tmp, nullptr, nullptr, r->n, (int)kb, false, err, s);
      if (e == cudaSuccess && host) e = cudaMemcpyAsync(q->keys, keys, r->n * kb, cudaMemcpyDeviceToHost, s);
    } else if (r->op == OP_SELECT) {
      const size_t cap = r->n / 4 + 1024;
      void* cand = base + off;
      off += align256(cap * kb);
      void* work = base + off;
      e = launch_select(keys, r->n, q->k, (int)kb, cand, cap, work, result, err, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(q->result, result, 8, cudaMemcpyDeviceToHost, s);
    } else {
      auto* counts = reinterpret_cast<unsigned long long*>(base + off);
      e = cudaMemsetAsync(counts, 0, 256 * 8, s);
      if (e == cudaSuccess) e = launch_digit_counts(keys, r->n, (int)kb, 1, 8, q->shift, 0, false, counts, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(q->result, counts, 256 * 8, cudaMemcpyDeviceToHost, s);
    }
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
    char* base = st->dmem;
    uint32_t* keys = reinterpret_cast<uint32_t*>(base + 256);
    uint32_t* tmp = reinterpret_cast<uint32_t*>(base + 256 + align256(total * 4));
    char* plan = base + 256 + 2 * align256(total * 4);
    cudaError_t e = cudaSuccess;
    for (size_t i = 0; i < u.reqs.size() && e == cudaSuccess; ++i) {
      pa_request* q = user_of(u.reqs[i]);
      e = cudaMemcpyAsync(keys + off[i], q->keys, u.reqs[i]->n * 4, cudaMemcpyDefault, s);
    }
    if (e == cudaSuccess) e = seg::upload_plan(*st->plan, plan, s);
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

  uint32_t* take_word() {
    std::lock_guard<std::mutex> lk(mu_);
    if (free_words_.empty()) {
      uint32_t* w = nullptr;
      if (cudaMallocHost(&w, 64) != cudaSuccess) {
        cudaGetLastError();
        static uint32_t fallback;
        return &fallback;
      }
      pinned_words_.push_back(w);
      return w;
    }
    uint32_t* w = free_words_.back();
    free_words_.pop_back();
    return w;
  }
  void give_word(uint32_t* w) {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto* p : pinned_words_)
      if (p == w) {
        free_words_.push_back(w);
        return;
      }
  }

  int device_ = 0;
  std::vector<cudaStream_t> streams_;
  int next_lane_ = 0;
  std::mutex mu_;
  std::vector<uint32_t*> pinned_words_, free_words_;
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
  Config sc;
  if (c.hbm_budget_bytes) sc.budget_bytes = c.hbm_budget_bytes;
  if (c.max_inflight > 0) sc.max_inflight = c.max_inflight;
  if (c.max_batch_requests > 0) sc.max_batch_requests = c.max_batch_requests;
  sc.coalesce = c.no_coalesce == 0;
  const int lanes = c.num_streams > 0 ? c.num_streams : 4;
  auto* s = new pa_server();
  s->backend.reset(new GpuBackend(lanes));
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
  const uint64_t v[7] = {st.submitted, st.completed, st.rejected, st.units, st.batched_units, st.coalesced_requests,
                         st.peak_bytes};
  for (int i = 0; i < count && i < 7; ++i) out[i] = v[i];
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
