// Checks of the commit's host threads (gpu_inscy_gb300/csrc/host_threads.h),
// built with g++ by tests/test_host_threads.py.  Prints "ok" and exits 0, or
// names the failed check and exits 1.
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_threads.h"

static int failures = 0;
#define CHECK(c)                                              \
  do {                                                        \
    if (!(c)) {                                               \
      std::printf("FAILED %s (line %d)\n", #c, __LINE__);     \
      ++failures;                                             \
    }                                                         \
  } while (0)

static void pool_runs_every_task() {
  for (int workers : {0, 1, 3, 7}) {
    inscy::HostPool pool(workers);
    CHECK(pool.workers() == workers);
    for (int tasks : {0, 1, 2, 5, 64, 1000}) {
      std::vector<std::atomic<int>> hits(tasks > 0 ? tasks : 1);
      for (auto& h : hits) h = 0;
      pool.run(tasks, [&](int i) { hits[i].fetch_add(1); });
      for (int i = 0; i < tasks; ++i) CHECK(hits[i].load() == 1);
    }
  }
}

// a throwing task: the others still run, run() returns only after all have
// ended and rethrows the first exception; the pool stays usable
static void pool_rethrows_after_all_tasks() {
  inscy::HostPool pool(4);
  for (int rep = 0; rep < 20; ++rep) {
    const int tasks = 200;
    std::vector<std::atomic<int>> hits(tasks);
    for (auto& h : hits) h = 0;
    std::atomic<int> running{0};
    bool threw = false;
    std::string what;
    try {
      pool.run(tasks, [&](int i) {
        running.fetch_add(1);
        hits[i].fetch_add(1);
        if (i % 37 == 5) {
          running.fetch_sub(1);
          throw std::runtime_error("task " + std::to_string(i));
        }
        volatile double x = 0;
        for (int k = 0; k < 2000; ++k) x = x + k;
        running.fetch_sub(1);
      });
    } catch (const std::runtime_error& e) {
      threw = true;
      what = e.what();
    }
    CHECK(threw);
    CHECK(what.rfind("task ", 0) == 0);
    CHECK(running.load() == 0);  // no task still runs when run() has returned
    for (int i = 0; i < tasks; ++i) CHECK(hits[i].load() == 1);
    std::atomic<int> after{0};
    pool.run(16, [&](int) { after.fetch_add(1); });
    CHECK(after.load() == 16);
  }
}

static bool all_minus_one(const int* b, size_t w) {
  for (size_t i = 0; i < w; ++i)
    if (b[i] != -1) return false;
  return true;
}

static void filler_blocks() {
  inscy::BlockFiller f;
  f.start(1000);
  for (int i = 0; i < 10; ++i) {
    auto b = f.take();
    CHECK(b != nullptr);
    CHECK(all_minus_one(b.get(), 1000));
    b[0] = 7;  // a taken block is the caller's
  }
  // a new size: blocks of the old size are not handed out
  f.start(333);
  for (int i = 0; i < 5; ++i) {
    auto b = f.take();
    CHECK(all_minus_one(b.get(), 333));
  }
  f.start(333);  // same size: the spare stays
  auto b = f.take();
  CHECK(all_minus_one(b.get(), 333));
  f.start(0);
  auto z = f.take();
  CHECK(z != nullptr);
}

int main() {
  pool_runs_every_task();
  pool_rethrows_after_all_tasks();
  filler_blocks();
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
