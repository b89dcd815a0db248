// Project-written stand-in for the subset of Intel oneTBB that the reference
// headers use on Linux (Configuration.h:18-22, RadixSortLsdParallel.h:8-9):
//   task_group{run,wait}, parallel_invoke, parallel_reduce + blocked_range +
//   split, parallel_for(first,last,f), global_control, tick_count.
//
// Test infrastructure only: it exists so that the reference's own CPU code can
// be compiled unchanged and used as the parity checker and as the timed CPU
// baseline.  It is a fixed-size thread pool (one worker per hardware thread
// minus the caller); a thread blocked in task_group::wait() executes queued
// tasks instead of sleeping, so the reference's nested parallel_invoke
// recursion cannot deadlock.  The pool size can be capped with the
// environment variable PA_REF_THREADS.
#ifndef PA_TBB_SHIM_TBB_H
#define PA_TBB_SHIM_TBB_H

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdlib>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

namespace tbb {
namespace detail_shim {

class pool {
 public:
  static pool& instance() {
    static pool p;
    return p;
  }
  unsigned concurrency() const { return nthreads_ + 1; }

  void submit(std::function<void()> fn) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      queue_.push_back(std::move(fn));
    }
    cv_.notify_one();
  }

  // Runs one queued task on the calling thread (newest first, which is
  // usually a child of the task the caller is waiting on).
  bool help_one() {
    std::function<void()> fn;
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (queue_.empty()) return false;
      fn = std::move(queue_.back());
      queue_.pop_back();
    }
    fn();
    return true;
  }

  ~pool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  pool() {
    unsigned hw = std::thread::hardware_concurrency();
    if (hw == 0) hw = 1;
    if (const char* env = std::getenv("PA_REF_THREADS")) {
      long v = std::strtol(env, nullptr, 10);
      if (v >= 1) hw = (unsigned)v;
    }
    nthreads_ = hw - 1;
    for (unsigned i = 0; i < nthreads_; ++i)
      workers_.emplace_back([this] { worker_loop(); });
  }

  void worker_loop() {
    for (;;) {
      std::function<void()> fn;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return stop_ || !queue_.empty(); });
        if (stop_ && queue_.empty()) return;
        fn = std::move(queue_.front());  // oldest first: the largest subtrees
        queue_.pop_front();
      }
      fn();
    }
  }

  unsigned nthreads_ = 0;
  std::vector<std::thread> workers_;
  std::deque<std::function<void()>> queue_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool stop_ = false;
};

}  // namespace detail_shim

class task_group {
 public:
  task_group() : pending_(std::make_shared<std::atomic<long>>(0)) {}
  ~task_group() { wait(); }

  template <class F>
  void run(F&& f) {
    pending_->fetch_add(1, std::memory_order_relaxed);
    auto pending = pending_;
    std::function<void()> body(std::forward<F>(f));
    detail_shim::pool::instance().submit([pending, body]() {
      body();
      pending->fetch_sub(1, std::memory_order_release);
    });
  }

  void wait() {
    while (pending_->load(std::memory_order_acquire) != 0) {
      if (!detail_shim::pool::instance().help_one()) std::this_thread::yield();
    }
  }

 private:
  std::shared_ptr<std::atomic<long>> pending_;
};

template <class F0>
inline void parallel_invoke(F0&& f0) {
  f0();
}

template <class F0, class... Fs>
inline void parallel_invoke(F0&& f0, Fs&&... fs) {
  task_group g;
  (g.run(std::forward<Fs>(fs)), ...);
  f0();
  g.wait();
}

class split {};

template <class T>
class blocked_range {
 public:
  blocked_range(T b, T e, std::size_t grain = 1) : begin_(b), end_(e), grain_(grain) {}
  T begin() const { return begin_; }
  T end() const { return end_; }
  std::size_t size() const { return (std::size_t)(end_ - begin_); }
  bool empty() const { return !(begin_ < end_); }
  std::size_t grainsize() const { return grain_; }

 private:
  T begin_, end_;
  std::size_t grain_;
};

namespace detail_shim {
template <class T, class Body>
void reduce_rec(const blocked_range<T>& r, Body& body, std::size_t leaf) {
  if (r.size() <= leaf) {
    body(r);
    return;
  }
  T mid = r.begin() + (T)(r.size() / 2);
  Body right(body, split());
  parallel_invoke([&] { reduce_rec(blocked_range<T>(r.begin(), mid, r.grainsize()), body, leaf); },
                  [&] { reduce_rec(blocked_range<T>(mid, r.end(), r.grainsize()), right, leaf); });
  body.join(right);
}
}  // namespace detail_shim

template <class T, class Body>
inline void parallel_reduce(const blocked_range<T>& range, Body& body) {
  std::size_t parts = 4 * (std::size_t)detail_shim::pool::instance().concurrency();
  std::size_t leaf = range.size() / parts;
  if (leaf < range.grainsize()) leaf = range.grainsize();
  if (leaf < 1) leaf = 1;
  detail_shim::reduce_rec(range, body, leaf);
}

template <class Index, class F>
inline void parallel_for(Index first, Index last, const F& f) {
  if (!(first < last)) return;
  std::size_t n = (std::size_t)(last - first);
  std::size_t parts = (std::size_t)detail_shim::pool::instance().concurrency();
  std::size_t chunk = (n + parts - 1) / parts;
  task_group g;
  for (std::size_t s = 0; s < n; s += chunk) {
    std::size_t e = s + chunk < n ? s + chunk : n;
    g.run([=, &f] {
      for (std::size_t i = s; i < e; ++i) f((Index)(first + (Index)i));
    });
  }
  g.wait();
}

class global_control {
 public:
  enum parameter { max_allowed_parallelism, thread_stack_size };
  global_control(parameter, std::size_t) {}
};

class tick_count {
 public:
  class interval_t {
   public:
    explicit interval_t(double s) : s_(s) {}
    double seconds() const { return s_; }

   private:
    double s_;
  };
  static tick_count now() {
    tick_count t;
    t.t_ = std::chrono::steady_clock::now();
    return t;
  }
  friend interval_t operator-(const tick_count& a, const tick_count& b) {
    return interval_t(std::chrono::duration<double>(a.t_ - b.t_).count());
  }

 private:
  std::chrono::steady_clock::time_point t_;
};

namespace info {
inline int default_concurrency() { return (int)detail_shim::pool::instance().concurrency(); }
}  // namespace info

}  // namespace tbb

#endif  // PA_TBB_SHIM_TBB_H
