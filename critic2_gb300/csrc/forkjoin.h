// A fork-join pool for the host side of the lockstep path tracers: the
// per-batch state-machine work over thousands of independent rays is split
// into contiguous chunks, one per thread.  Workers spin on a generation
// counter (yielding) between jobs, which keeps a fork-join to a few
// microseconds; the calling thread takes chunk 0.  An exception thrown by a
// chunk is rethrown to the caller after every chunk has finished.
#pragma once

#include <algorithm>
#include <atomic>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace c2g {

class ForkJoin {
 public:
  explicit ForkJoin(int nthreads) : n_(std::max(1, nthreads)) {
    for (int t = 1; t < n_; t++) workers_.emplace_back([this, t] { loop(t); });
  }
  ~ForkJoin() {
    stop_.store(true, std::memory_order_release);
    gen_.fetch_add(1, std::memory_order_acq_rel);
    for (std::thread &w : workers_) w.join();
  }
  ForkJoin(const ForkJoin &) = delete;
  ForkJoin &operator=(const ForkJoin &) = delete;

  int threads() const { return n_; }

  // f(begin, end) over [0, count) in n_ contiguous chunks.
  void run(long count, const std::function<void(long, long)> &f) {
    if (n_ == 1 || count < 2 * n_) {
      f(0, count);
      return;
    }
    job_ = &f;
    count_ = count;
    err_ = nullptr;
    left_.store(n_ - 1, std::memory_order_release);
    gen_.fetch_add(1, std::memory_order_acq_rel);
    chunk(0);
    while (left_.load(std::memory_order_acquire) > 0) std::this_thread::yield();
    job_ = nullptr;
    if (err_) std::rethrow_exception(err_);
  }

 private:
  void chunk(int t) {
    const long b = count_ * t / n_, e = count_ * (t + 1) / n_;
    try {
      (*job_)(b, e);
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu_);
      if (!err_) err_ = std::current_exception();
    }
  }
  void loop(int t) {
    // generation 0 is the pool's state at construction: a worker that starts
    // after the first job was posted still sees that job as new
    unsigned long seen = 0;
    for (;;) {
      unsigned long g;
      while ((g = gen_.load(std::memory_order_acquire)) == seen) std::this_thread::yield();
      seen = g;
      if (stop_.load(std::memory_order_acquire)) return;
      chunk(t);
      left_.fetch_sub(1, std::memory_order_acq_rel);
    }
  }

  int n_;
  std::vector<std::thread> workers_;
  std::atomic<unsigned long> gen_{0};
  std::atomic<int> left_{0};
  std::atomic<bool> stop_{false};
  const std::function<void(long, long)> *job_ = nullptr;
  long count_ = 0;
  std::exception_ptr err_;
  std::mutex mu_;
};

}  // namespace c2g
