// Host worker threads for the library's FP64 set-up loops (model
// coefficients, validity checks, copies).
//
// Starting a std::thread costs tens of microseconds on the Grace host, so a
// parallel loop that spawned 16 threads spent about 1 ms on that alone; the
// set-up of a 1040 x 540 electromag2 model runs five such loops.  The pool
// starts its workers once per process and wakes them per loop.
//
// One loop runs at a time (callers from several host threads take turns);
// a task must not start a loop of its own.  A process forked after the
// workers started gets a fresh pool on its first loop.
#pragma once

#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace sfd {

class HostPool {
 public:
  static constexpr unsigned kMaxThreads = 16;

  // The process's pool (created on first use, or anew in a forked child).
  static HostPool& get() {
    static std::mutex create_m;
    static HostPool* pool = nullptr;
    std::lock_guard<std::mutex> g(create_m);
    if (!pool || pool->pid_ != getpid()) pool = new HostPool();  // a forked child's copy is left unused
    return *pool;
  }

  // Threads that run(): the workers plus the caller.
  unsigned size() const { return (unsigned)workers_.size() + 1; }

  // task(0) .. task(ntasks - 1), on the workers and the calling thread.
  void run(int ntasks, const std::function<void(int)>& task) {
    std::lock_guard<std::mutex> one_at_a_time(run_m_);
    {
      std::lock_guard<std::mutex> lk(m_);
      task_ = &task;
      ntasks_ = ntasks;
      next_.store(0);
      ++gen_;
    }
    cv_work_.notify_all();
    for (int i; (i = next_.fetch_add(1)) < ntasks;) task(i);
    std::unique_lock<std::mutex> lk(m_);
    cv_done_.wait(lk, [&] { return active_ == 0; });
    task_ = nullptr;  // a worker that wakes later finds no loop to join
  }

 private:
  HostPool() : pid_(getpid()) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned n = std::min(kMaxThreads, hw) - 1;
    for (unsigned t = 0; t < n; ++t) workers_.emplace_back([this] { work(); });
    for (auto& w : workers_) w.detach();  // the pool lives until the process exits
  }

  void work() {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(m_);
    for (;;) {
      cv_work_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      if (!task_) continue;
      const std::function<void(int)>* task = task_;
      const int n = ntasks_;
      ++active_;
      lk.unlock();
      for (int i; (i = next_.fetch_add(1)) < n;) (*task)(i);
      lk.lock();
      if (--active_ == 0) cv_done_.notify_all();
    }
  }

  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex run_m_, m_;
  std::condition_variable cv_work_, cv_done_;
  const std::function<void(int)>* task_ = nullptr;
  int ntasks_ = 0;
  std::atomic<int> next_{0};
  int active_ = 0;
  uint64_t gen_ = 0;
};

}  // namespace sfd
