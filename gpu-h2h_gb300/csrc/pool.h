// pool.h -- a fixed set of worker threads with a blocking parallel_for, used
// by the host phases (elimination fill-in merges, sparse table, label
// allocation).  The reference spawns fresh std::threads per level instead.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace gh {

class Pool {
 public:
  explicit Pool(int threads) : nthreads_(std::max(1, threads)) {
    for (int i = 1; i < nthreads_; i++) workers_.emplace_back([this, i] { loop(i); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> l(mu_);
      stop_ = true;
      gen_++;
    }
    cv_.notify_all();
    for (auto &t : workers_) t.join();
  }
  int size() const { return nthreads_; }

  // Calls fn(begin, end, worker) over [0, n) in chunks; returns when all are done.
  void parallel_for(int64_t n, int64_t grain, const std::function<void(int64_t, int64_t, int)> &fn) {
    if (n <= 0) return;
    if (nthreads_ == 1 || n <= grain) {
      fn(0, n, 0);
      return;
    }
    {
      std::lock_guard<std::mutex> l(mu_);
      fn_ = &fn;
      n_ = n;
      grain_ = std::max<int64_t>(1, grain);
      next_.store(0);
      pending_ = nthreads_ - 1;
      gen_++;
    }
    cv_.notify_all();
    work(0);
    std::unique_lock<std::mutex> l(mu_);
    done_cv_.wait(l, [this] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  void work(int id) {
    for (;;) {
      int64_t b = next_.fetch_add(grain_);
      if (b >= n_) break;
      (*fn_)(b, std::min(n_, b + grain_), id);
    }
  }
  void loop(int id) {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
      }
      work(id);
      {
        std::lock_guard<std::mutex> l(mu_);
        if (--pending_ == 0) done_cv_.notify_all();
      }
    }
  }
  int nthreads_;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int64_t, int64_t, int)> *fn_ = nullptr;
  int64_t n_ = 0, grain_ = 1;
  std::atomic<int64_t> next_{0};
  int pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

}  // namespace gh
