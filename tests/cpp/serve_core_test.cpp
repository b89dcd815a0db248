// Scheduling policy of the serving loop (pa_serve_core.h) driven by a fake
// device backend on the CPU: no GPU, no CUDA.  Exits non-zero on the first
// failed check.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <set>
#include <thread>
#include <vector>

#include "pa_serve_core.h"

using namespace pa::serve;

#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);     \
      std::exit(1);                                                \
    }                                                              \
  } while (0)

// A unit "runs" for `polls` calls of finished(); memory is n * key bytes * 2.
struct FakeBackend {
  size_t free = (size_t)1 << 40;
  int polls = 3;
  double clock = 0;
  int launched = 0, finished_units = 0, max_seen_inflight = 0, inflight = 0;
  std::vector<std::vector<Request*>> units;
  size_t free_bytes() { return free; }
  size_t unit_bytes(const Unit& u) {
    size_t b = 0;
    for (const Request* r : u.reqs) b += r->n * (size_t)r->key_bytes * 2;
    return b;
  }
  void launch(Unit& u) {
    u.state = new int(polls);
    ++launched;
    ++inflight;
    max_seen_inflight = std::max(max_seen_inflight, inflight);
    units.push_back(u.reqs);
  }
  bool finished(Unit& u) { return --*static_cast<int*>(u.state) <= 0; }
  void finish(Unit& u) {
    delete static_cast<int*>(u.state);
    ++finished_units;
    --inflight;
  }
  double now() { return clock += 1.0; }
};

static Request make(int op, int kb, size_t n) {
  Request r;
  r.op = op;
  r.key_bytes = kb;
  r.n = n;
  return r;
}

static void run_to_idle(Scheduler<FakeBackend>& s) {
  for (int i = 0; i < 100000 && !s.idle(); ++i) s.step();
  CHECK(s.idle());
}

int main() {
  // 1. coalescing: waiting requests of the head's kind (operation and key
  // width) share its unit, in arrival order; kinds never mix; FIFO heads
  {
    FakeBackend b;
    Config c;
    c.max_inflight = 8;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs;
    rs.push_back(make(OP_SORT, 4, 100));   // 0
    rs.push_back(make(OP_SELECT, 4, 50));  // 1
    rs.push_back(make(OP_SORT, 8, 70));    // 2
    rs.push_back(make(OP_SORT, 4, 30));    // 3
    rs.push_back(make(OP_HIST, 8, 10));    // 4
    rs.push_back(make(OP_SORT, 4, 20));    // 5
    rs.push_back(make(OP_SELECT, 4, 40));  // 6
    rs.push_back(make(OP_SELECT, 8, 40));  // 7
    rs.push_back(make(OP_HIST, 8, 12));    // 8
    rs.push_back(make(OP_SORT, 8, 60));    // 9
    for (auto& r : rs) s.submit(&r);
    run_to_idle(s);
    CHECK(b.units.size() == 5);
    CHECK(b.units[0].size() == 3);  // the three 32-bit sorts, arrival order
    CHECK(b.units[0][0] == &rs[0] && b.units[0][1] == &rs[3] && b.units[0][2] == &rs[5]);
    CHECK(b.units[1].size() == 2 && b.units[1][0] == &rs[1] && b.units[1][1] == &rs[6]);  // 32-bit selects
    CHECK(b.units[2].size() == 2 && b.units[2][0] == &rs[2] && b.units[2][1] == &rs[9]);  // 64-bit sorts
    CHECK(b.units[3].size() == 2 && b.units[3][0] == &rs[4] && b.units[3][1] == &rs[8]);  // 64-bit histograms
    CHECK(b.units[4].size() == 1 && b.units[4][0] == &rs[7]);                             // the one 64-bit select
    for (auto& r : rs) {
      CHECK(r.status == ST_OK);
      CHECK(r.t_submit <= r.t_admit && r.t_admit < r.t_done);
    }
    CHECK(rs[0].unit_size == 3 && rs[1].unit_size == 2 && rs[7].unit_size == 1);
    const Stats st = s.stats();
    CHECK(st.submitted == 10 && st.completed == 10 && st.units == 5 && st.batched_units == 4);
    CHECK(st.coalesced_requests == 9);
  }
  // 1b. a shared unit of a kind other than 32-bit sorts stops at max_group_keys
  {
    FakeBackend b;
    Config c;
    c.max_inflight = 8;
    c.max_group_keys = 100;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs;
    rs.push_back(make(OP_SORT, 8, 60));
    rs.push_back(make(OP_SORT, 8, 50));   // would exceed 100 keys with the head: next unit
    rs.push_back(make(OP_SORT, 8, 30));   // fits with the head
    rs.push_back(make(OP_SORT, 8, 150));  // larger than the limit: alone
    for (auto& r : rs) s.submit(&r);
    run_to_idle(s);
    CHECK(b.units.size() == 3);
    CHECK(b.units[0].size() == 2 && b.units[0][0] == &rs[0] && b.units[0][1] == &rs[2]);
    CHECK(b.units[1].size() == 1 && b.units[1][0] == &rs[1]);
    CHECK(b.units[2].size() == 1 && b.units[2][0] == &rs[3]);
  }
  // 1c. requests above max_join_keys run alone, as the head or among waiting ones
  {
    FakeBackend b;
    Config c;
    c.max_inflight = 8;
    c.max_join_keys = 40;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs;
    rs.push_back(make(OP_SORT, 4, 50));  // head above the join limit: alone
    rs.push_back(make(OP_SORT, 4, 10));
    rs.push_back(make(OP_SORT, 4, 41));  // above the limit: skipped by the group
    rs.push_back(make(OP_SORT, 4, 40));  // at the limit: joins
    for (auto& r : rs) s.submit(&r);
    run_to_idle(s);
    CHECK(b.units.size() == 3);
    CHECK(b.units[0].size() == 1 && b.units[0][0] == &rs[0]);
    CHECK(b.units[1].size() == 2 && b.units[1][0] == &rs[1] && b.units[1][1] == &rs[3]);
    CHECK(b.units[2].size() == 1 && b.units[2][0] == &rs[2]);
  }
  // 2. coalescing off: every request alone
  {
    FakeBackend b;
    Config c;
    c.coalesce = false;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs(5, make(OP_SORT, 4, 10));
    for (auto& r : rs) s.submit(&r);
    run_to_idle(s);
    CHECK(b.units.size() == 5);
  }
  // 3. HBM budget: units wait for memory; a request that can never fit is rejected
  {
    FakeBackend b;
    Config c;
    c.budget_bytes = 1000;
    c.coalesce = false;
    c.max_inflight = 16;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs;
    for (int i = 0; i < 6; ++i) rs.push_back(make(OP_SORT, 8, 30));  // 480 bytes each
    rs.push_back(make(OP_SORT, 8, 100));                               // 1600 bytes: never fits
    rs.push_back(make(OP_SORT, 8, 30));
    for (auto& r : rs) s.submit(&r);
    size_t peak = 0;
    for (int i = 0; i < 100000 && !s.idle(); ++i) {
      s.step();
      peak = std::max(peak, s.in_use());
      CHECK(s.in_use() <= 1000);
    }
    CHECK(s.idle());
    CHECK(peak == 960);  // two units at a time
    CHECK(rs[6].status == ST_ERR_OOM);
    for (int i = 0; i < 8; ++i)
      if (i != 6) CHECK(rs[i].status == ST_OK);
    CHECK(s.stats().rejected == 1);
  }
  // 4. a batch that does not fit is shrunk, not refused
  {
    FakeBackend b;
    Config c;
    c.budget_bytes = 1000;
    Scheduler<FakeBackend> s(b, c);
    std::vector<Request> rs(4, make(OP_SORT, 4, 100));  // 800 bytes each; two never fit together
    for (auto& r : rs) s.submit(&r);
    run_to_idle(s);
    CHECK(b.units.size() == 4);
    for (auto& u : b.units) CHECK(u.size() == 1);
  }
  // 5. device free memory also gates admission
  {
    FakeBackend b;
    b.free = 500;
    Config c;
    Scheduler<FakeBackend> s(b, c);
    Request r = make(OP_SORT, 8, 100);
    s.submit(&r);
    for (int i = 0; i < 50; ++i) s.step();
    CHECK(r.status == ST_PENDING && s.waiting() == 1);
    b.free = 1 << 20;
    run_to_idle(s);
    CHECK(r.status == ST_OK);
  }
  // 6. max_inflight, and submissions from several threads while it runs
  {
    FakeBackend b;
    b.polls = 5;
    Config c;
    c.max_inflight = 3;
    c.max_batch_requests = 4;
    std::atomic<int> done{0};
    Scheduler<FakeBackend> s(b, c, [&](Request*) { done++; });
    const int kThreads = 4, kPer = 500;
    std::vector<std::unique_ptr<Request>> rs;
    for (int i = 0; i < kThreads * kPer; ++i)
      rs.emplace_back(new Request(make(i % 5 == 0 ? OP_SELECT : OP_SORT, i % 3 == 0 ? 8 : 4, 1 + i % 97)));
    std::atomic<bool> go{false};
    std::vector<std::thread> ts;
    for (int t = 0; t < kThreads; ++t)
      ts.emplace_back([&, t] {
        while (!go) {
        }
        for (int i = 0; i < kPer; ++i) s.submit(rs[t * kPer + i].get());
      });
    go = true;
    int steps = 0;
    while (done.load() < kThreads * kPer && steps < 10000000) {
      s.step();
      ++steps;
    }
    for (auto& t : ts) t.join();
    run_to_idle(s);
    CHECK(done.load() == kThreads * kPer);
    CHECK(b.max_seen_inflight <= 3);
    std::set<Request*> seen;
    for (auto& u : b.units) {
      CHECK(u.size() <= 4);
      for (Request* r : u) CHECK(seen.insert(r).second);  // each request in exactly one unit
    }
    CHECK(seen.size() == (size_t)kThreads * kPer);
    for (auto& r : rs) CHECK(r->status == ST_OK);
  }
  std::printf("OK\n");
  return 0;
}
