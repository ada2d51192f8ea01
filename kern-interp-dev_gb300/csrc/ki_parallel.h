// Host-side parallel loop over contiguous index ranges: a persistent pool of
// worker threads (one job at a time; a second concurrent caller, or a caller
// in a forked child, starts its own std::threads instead).
#pragma once

#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace ki {

class WorkerPool {
 public:
  static constexpr int kMaxWorkers = 15;

  static WorkerPool& get() {
    static WorkerPool pool;
    return pool;
  }

  // task(1), ..., task(n_tasks) on the workers while the caller runs task(0);
  // false (nothing run) when the pool is busy or belongs to another process.
  // Workers poll for a new job for about 200 microseconds after each one
  // (host phases issue jobs back to back), then sleep on a condition variable.
  bool run(int n_tasks, const std::function<void(int)>& task) {
    if (n_tasks > (int)workers_.size() || getpid() != pid_) return false;
    std::unique_lock<std::mutex> busy(job_mutex_, std::try_to_lock);
    if (!busy.owns_lock()) return false;
    task_ = &task;
    done_.store(0, std::memory_order_relaxed);
    {
      // the job's generation and task count in one word: a worker that skips
      // the job reads nothing else, so the next job cannot be seen half-set
      std::lock_guard<std::mutex> g(m_);
      const long long next = ((gen_.load(std::memory_order_relaxed) >> 8) + 1) << 8;
      gen_.store(next | n_tasks, std::memory_order_release);
    }
    cv_.notify_all();
    task(0);
    for (int spin = 0; done_.load(std::memory_order_acquire) != n_tasks; spin++)
      if (spin > 4096) std::this_thread::yield();
    return true;
  }

  ~WorkerPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      gen_.store(((gen_.load(std::memory_order_relaxed) >> 8) + 1) << 8, std::memory_order_release);
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  WorkerPool() : pid_(getpid()) {
    const int hw = (int)std::thread::hardware_concurrency();
    const int nw = std::max(0, std::min(kMaxWorkers, hw - 1));
    for (int w = 0; w < nw; w++) workers_.emplace_back([this, w] { loop(w); });
  }

  void loop(int w) {
    long long seen = 0;
    for (;;) {
      long long g = gen_.load(std::memory_order_acquire);
      if (g == seen) {
        const auto t0 = std::chrono::steady_clock::now();
        for (int spin = 1; g == seen; spin++) {
          if ((spin & 255) == 0 &&
              std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(200)) {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [&] { return gen_.load(std::memory_order_acquire) != seen; });
          }
          g = gen_.load(std::memory_order_acquire);
        }
      }
      seen = g;
      if (stop_) return;
      if (w >= (int)(g & 255)) continue;
      (*task_)(w + 1);
      done_.fetch_add(1, std::memory_order_acq_rel);
    }
  }

  const pid_t pid_;
  std::vector<std::thread> workers_;
  std::mutex job_mutex_, m_;
  std::condition_variable cv_;
  const std::function<void(int)>* task_ = nullptr;
  std::atomic<int> done_{0};
  std::atomic<long long> gen_{0};
  bool stop_ = false;
};

// fn(part, lo, hi) over [0, n) split into contiguous ranges, in part order,
// on up to 16 threads (one part on the caller's thread below `min_items`
// items).  Returns the number of parts.  fn must only write state owned by
// its part.
inline int parallel_part_count(int n, int min_items = 4096) {
  const int hw = (int)std::thread::hardware_concurrency();
  return (n < min_items) ? 1 : std::max(1, std::min(16, hw));
}

template <typename Fn>
int parallel_parts(int n, Fn fn, int min_items = 4096) {
  const int T = parallel_part_count(n, min_items);
  if (T == 1) {
    fn(0, 0, n);
    return 1;
  }
  const int chunk = (n + T - 1) / T;
  const std::function<void(int)> task = [&](int t) {
    const int lo = std::min(n, t * chunk), hi = std::min(n, lo + chunk);
    fn(t, lo, hi);
  };
  if (WorkerPool::get().run(T - 1, task)) return T;
  std::vector<std::thread> th;
  for (int t = 1; t < T; t++) {
    const int lo = std::min(n, t * chunk), hi = std::min(n, lo + chunk);
    th.emplace_back(fn, t, lo, hi);
  }
  fn(0, 0, std::min(n, chunk));
  for (auto& x : th) x.join();
  return T;
}

// fn(lo, hi) over the same ranges.
template <typename Fn>
void parallel_ranges(int n, Fn fn, int min_items = 4096) {
  parallel_parts(n, [&](int, int lo, int hi) { fn(lo, hi); }, min_items);
}

}  // namespace ki
