// Host threads of the engine's commit: a task pool for its data-parallel
// loops and a helper that prepares label blocks ahead of it.  Plain C++17
// (no CUDA), so the CPU tests build and exercise them on their own.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

namespace inscy {

// Host threads for the data-parallel loops of the commit.  run(tasks, fn)
// calls fn(i) for every i in [0, tasks) on the workers and the calling
// thread and returns when all are done.  Only as many workers as there are
// tasks beyond the caller's are woken, and the caller waits for the tasks,
// not for every worker to check in (a late worker finds the run's counter
// exhausted and calls nothing).  A task that throws does not stop the
// others; run() rethrows the first exception once every task has ended.
class HostPool {
 public:
  explicit HostPool(int workers) {
    for (int i = 0; i < workers; ++i) th_.emplace_back([this] { loop(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : th_) t.join();
  }
  int workers() const { return (int)th_.size(); }
  void run(int tasks, const std::function<void(int)>& fn) {
    if (tasks <= 0) return;
    auto job = std::make_shared<Job>();
    job->fn = &fn;
    job->tasks = tasks;
    const int wake = std::min(tasks - 1, (int)th_.size());
    if (wake > 0) {
      {
        std::lock_guard<std::mutex> g(m_);
        cur_ = job;
        ++gen_;
      }
      if (wake == (int)th_.size())
        cv_.notify_all();
      else
        for (int i = 0; i < wake; ++i) cv_.notify_one();
    }
    work(*job);
    if (job->done.load(std::memory_order_acquire) < tasks) {
      std::unique_lock<std::mutex> lk(m_);
      done_.wait(lk, [&] { return job->done.load(std::memory_order_acquire) >= tasks; });
    }
    {
      std::lock_guard<std::mutex> g(m_);
      if (cur_ == job) cur_.reset();
    }
    // every task has ended (none still uses fn): the first failure goes to
    // the caller
    if (job->err) std::rethrow_exception(job->err);
  }

 private:
  struct Job {
    const std::function<void(int)>* fn = nullptr;
    int tasks = 0;
    std::atomic<int> next{0}, done{0};
    std::mutex err_m;
    std::exception_ptr err;  // the first exception a task threw
  };
  void work(Job& j) {
    for (;;) {
      const int i = j.next.fetch_add(1);
      if (i >= j.tasks) break;
      try {
        (*j.fn)(i);
      } catch (...) {
        std::lock_guard<std::mutex> g(j.err_m);
        if (!j.err) j.err = std::current_exception();
      }
      if (j.done.fetch_add(1, std::memory_order_acq_rel) + 1 == j.tasks) {
        std::lock_guard<std::mutex> g(m_);
        done_.notify_all();
      }
    }
  }
  void loop() {
    long long seen = 0;
    for (;;) {
      std::shared_ptr<Job> job;
      {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
        job = cur_;
      }
      if (job) work(*job);
    }
  }
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_, done_;
  std::shared_ptr<Job> cur_;
  long long gen_ = 0;
  bool stop_ = false;
};

// Label blocks are filled with -1 by a helper thread one block ahead of the
// commit, which then takes rows that need no initialisation (the fill of
// fresh memory, about 100 KB a row at n = 25,000, is off its critical path).
class BlockFiller {
 public:
  BlockFiller() : th_([this] { loop(); }) {}
  ~BlockFiller() {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_ = true;
    }
    cv_.notify_all();
    th_.join();
  }
  // blocks of `words` ints from now on; one is filled at once (a spare of
  // that size left from the previous run is kept)
  void start(size_t words) {
    std::lock_guard<std::mutex> lk(m_);
    if (words == words_) return;
    ++gen_;
    words_ = words;
    spare_.reset();
    want_ = words > 0;
    cv_.notify_all();
  }
  // a block of -1s (filled here when the helper has not finished one)
  std::unique_ptr<int[]> take() {
    std::unique_lock<std::mutex> lk(m_);
    std::unique_ptr<int[]> b;
    if (spare_) {
      b = std::move(spare_);
    } else if (!busy_) {
      const size_t w = words_;
      lk.unlock();
      b.reset(new int[w]);
      std::fill(b.get(), b.get() + w, -1);
      lk.lock();
    } else {
      cv_.wait(lk, [&] { return spare_ != nullptr || !busy_; });
      if (spare_) {
        b = std::move(spare_);
      } else {
        const size_t w = words_;
        lk.unlock();
        b.reset(new int[w]);
        std::fill(b.get(), b.get() + w, -1);
        lk.lock();
      }
    }
    want_ = true;
    cv_.notify_all();
    return b;
  }

 private:
  void loop() {
    std::unique_lock<std::mutex> lk(m_);
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || (want_ && !spare_); });
      if (stop_) return;
      want_ = false;
      busy_ = true;
      const size_t w = words_;
      const long long g = gen_;
      lk.unlock();
      // an allocation failure leaves no spare: take() then allocates (and
      // reports the failure) on the caller's thread
      std::unique_ptr<int[]> b(new (std::nothrow) int[w]);
      if (b) std::fill(b.get(), b.get() + w, -1);
      lk.lock();
      busy_ = false;
      if (b && g == gen_ && !spare_) spare_ = std::move(b);
      cv_.notify_all();
    }
  }
  std::mutex m_;
  std::condition_variable cv_;
  std::unique_ptr<int[]> spare_;
  size_t words_ = 0;
  long long gen_ = 0;
  bool want_ = false, busy_ = false, stop_ = false;
  std::thread th_;
};

}  // namespace inscy
