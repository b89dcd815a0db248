// Scheduling core of the serving loop: requests arrive on any thread, wait in
// FIFO order, are admitted while their device memory fits the configured HBM
// budget (and the memory the device reports free), are grouped into units --
// the head request and the waiting requests of the same kind (operation and
// key width) share one unit: 32-bit sorts one persistent segmented-sort
// launch, histograms one multi-array histogram launch, 64-bit sorts and
// selects one allocation, stream and completion event -- and retire when
// their unit's device work has finished.
//
// Header-only and free of CUDA: the device side is a Backend with
//   size_t free_bytes();                  device memory free right now
//   size_t unit_bytes(const Unit&);       device memory a unit needs
//   void   launch(Unit&);                 enqueue the unit's copies + kernels
//   bool   finished(Unit&);               has its device work completed?
//   void   finish(Unit&);                 collect results, release memory
//   double now();                         seconds on a monotonic clock
// so the policy is tested on the CPU with a fake backend
// (tests/cpp/serve_core_test.cpp) and run on the GPU by pa_serve.cu.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <deque>
#include <functional>
#include <list>
#include <mutex>
#include <vector>

namespace pa {
namespace serve {

enum Op : int { OP_SORT = 0, OP_SELECT = 1, OP_HIST = 2 };

// Status codes written into Request::status (the C ABI's pa_status values).
enum : int { ST_PENDING = -1, ST_OK = 0, ST_ERR_OOM = 2 };

struct Request {
  int op = OP_SORT;
  int key_bytes = 4;
  size_t n = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int status = ST_PENDING;
  int unit_size = 0;  // requests in the unit that served it (1 = alone)
  void* user = nullptr;
};

struct Unit {
  std::vector<Request*> reqs;  // all of one kind (operation and key width)
  bool batched = false;        // more than one request
  size_t bytes = 0;
  int lane = -1;         // backend stream slot
  void* state = nullptr;
};

struct Config {
  size_t budget_bytes = (size_t)64 << 30;
  int max_inflight = 4;             // units on the device at once
  int max_batch_requests = 256;     // requests coalesced into one launch
  // Only requests of at most max_join_keys keys share units: for them the
  // fixed cost of a unit (allocation, copies, launches, event) is a large
  // part of the time.  Larger requests run alone, so that their copies and
  // kernels overlap those of the units on the other streams.
  size_t max_join_keys = (size_t)1 << 20;
  size_t max_batch_keys = (size_t)1 << 22;   // keys of a segmented (32-bit sort) unit
  size_t max_group_keys = (size_t)1 << 22;   // keys of any other shared unit
  size_t window = 1024;             // waiting requests scanned for coalescing
  bool coalesce = true;
};

struct Stats {
  size_t submitted = 0, completed = 0, rejected = 0, units = 0, batched_units = 0, coalesced_requests = 0;
  size_t peak_bytes = 0;
  double launch_s = 0, finish_s = 0;  // scheduler-thread time spent enqueueing units / completing them
};

template <class Backend>
class Scheduler {
 public:
  using DoneFn = std::function<void(Request*)>;

  Scheduler(Backend& b, const Config& c, DoneFn done = {}) : b_(b), cfg_(c), done_(std::move(done)) {}

  // Thread-safe.
  void submit(Request* r) {
    r->status = ST_PENDING;
    r->t_submit = b_.now();
    std::lock_guard<std::mutex> lk(mu_);
    incoming_.push_back(r);
    ++stats_.submitted;
  }

  // One scheduling round (scheduler thread only): retire finished units,
  // then admit waiting requests.  Returns true if anything changed.
  bool step() {
    bool progress = false;
    {
      std::lock_guard<std::mutex> lk(mu_);
      while (!incoming_.empty()) {
        waiting_.push_back(incoming_.front());
        incoming_.pop_front();
        progress = true;
      }
    }
    for (auto it = inflight_.begin(); it != inflight_.end();) {
      if (b_.finished(*it)) {
        const double f0 = b_.now();
        b_.finish(*it);
        stats_.finish_s += b_.now() - f0;
        in_use_ -= it->bytes;
        const double t = b_.now();
        for (Request* r : it->reqs) {
          r->t_done = t;
          if (r->status == ST_PENDING) r->status = ST_OK;
          complete(r);
        }
        it = inflight_.erase(it);
        progress = true;
      } else {
        ++it;
      }
    }
    while (!waiting_.empty() && (int)inflight_.size() < cfg_.max_inflight) {
      Unit u = next_unit();
      // shrink a batch that does not fit; a single request that can never
      // fit the budget is rejected; one that fits later waits (FIFO)
      for (;;) {
        u.bytes = b_.unit_bytes(u);
        if (fits(u.bytes)) break;
        if (u.reqs.size() > 1) {
          u.reqs.pop_back();
          u.batched = u.reqs.size() > 1;
          continue;
        }
        break;
      }
      if (!fits(u.bytes)) {
        if (u.reqs.size() == 1 && u.bytes > cfg_.budget_bytes) {
          Request* r = u.reqs[0];
          remove_waiting(u);
          r->status = ST_ERR_OOM;
          r->t_done = b_.now();
          ++stats_.rejected;
          complete(r);
          progress = true;
          continue;
        }
        break;  // wait for memory to come back
      }
      remove_waiting(u);
      const double t = b_.now();
      for (Request* r : u.reqs) {
        r->t_admit = t;
        r->unit_size = (int)u.reqs.size();
      }
      in_use_ += u.bytes;
      stats_.peak_bytes = std::max(stats_.peak_bytes, in_use_);
      ++stats_.units;
      if (u.batched) {
        ++stats_.batched_units;
        stats_.coalesced_requests += u.reqs.size();
      }
      inflight_.push_back(std::move(u));
      const double l0 = b_.now();
      b_.launch(inflight_.back());
      stats_.launch_s += b_.now() - l0;
      progress = true;
    }
    return progress;
  }

  bool idle() {
    std::lock_guard<std::mutex> lk(mu_);
    return incoming_.empty() && waiting_.empty() && inflight_.empty();
  }
  size_t in_use() const { return in_use_; }
  size_t inflight_units() const { return inflight_.size(); }
  size_t waiting() const { return waiting_.size(); }
  Stats stats() {
    std::lock_guard<std::mutex> lk(mu_);
    return stats_;
  }

 private:
  // 32-bit sorts share one persistent segmented-sort launch; other kinds
  // share an allocation, a stream and (histograms) one launch.
  static bool segmented(const Request* r) { return r->op == OP_SORT && r->key_bytes == 4; }
  static bool same_kind(const Request* a, const Request* b) { return a->op == b->op && a->key_bytes == b->key_bytes; }

  bool fits(size_t bytes) {
    if (in_use_ + bytes > cfg_.budget_bytes) return false;
    return bytes <= b_.free_bytes();
  }

  // The head request, plus the requests of its kind found among the next
  // `window` waiting ones, in arrival order, up to the unit's key limit.
  Unit next_unit() {
    Unit u;
    Request* head = waiting_.front();
    u.reqs.push_back(head);
    const size_t limit = segmented(head) ? cfg_.max_batch_keys : cfg_.max_group_keys;
    if (cfg_.coalesce && head->n <= cfg_.max_join_keys && head->n < limit) {
      size_t keys = head->n;
      size_t scanned = 0;
      for (auto it = std::next(waiting_.begin()); it != waiting_.end() && scanned < cfg_.window; ++it, ++scanned) {
        if ((int)u.reqs.size() >= cfg_.max_batch_requests) break;
        if (!same_kind(head, *it)) continue;
        if ((*it)->n > cfg_.max_join_keys || keys + (*it)->n > limit) continue;
        keys += (*it)->n;
        u.reqs.push_back(*it);
      }
    }
    u.batched = u.reqs.size() > 1;
    return u;
  }

  void remove_waiting(const Unit& u) {
    for (Request* r : u.reqs) {
      auto it = std::find(waiting_.begin(), waiting_.end(), r);
      if (it != waiting_.end()) waiting_.erase(it);
    }
  }

  void complete(Request* r) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      ++stats_.completed;
    }
    if (done_) done_(r);
  }

  Backend& b_;
  Config cfg_;
  DoneFn done_;
  std::mutex mu_;
  std::deque<Request*> incoming_;
  std::deque<Request*> waiting_;
  std::list<Unit> inflight_;
  size_t in_use_ = 0;
  Stats stats_;
};

}  // namespace serve
}  // namespace pa
