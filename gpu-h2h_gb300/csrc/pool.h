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
#include <memory>
#include <thread>
#include <utility>
#include <vector>

namespace gh {

// An allocator whose element construction without arguments leaves the
// value uninitialised: std::vector<T, NoInit<T>> v(n) skips the zero fill
// of buffers that are written in full right after.
template <class T>
struct NoInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInit<U>;
  };
  NoInit() = default;
  template <class U>
  NoInit(const NoInit<U> &) {}
  template <class U, class... Args>
  void construct(U *p, Args &&...args) {
    if constexpr (sizeof...(Args) == 0)
      ::new ((void *)p) U;
    else
      ::new ((void *)p) U(std::forward<Args>(args)...);
  }
};

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

// out[0] = 0, out[i + 1] = out[i] + f(i) for i in [0, n), in two passes over
// chunks of the range on the pool (chunk sums, then the prefix inside each).
template <class F>
void parallel_prefix(Pool &pool, int64_t n, int64_t *out, const F &f) {
  const int64_t grain = int64_t(1) << 16;
  const int64_t nch = (n + grain - 1) / grain;
  std::vector<int64_t> part(nch + 1, 0);
  pool.parallel_for(nch, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t c = lo; c < hi; c++) {
      int64_t s = 0;
      for (int64_t i = c * grain, e = std::min(n, i + grain); i < e; i++) s += f(i);
      part[c + 1] = s;
    }
  });
  for (int64_t c = 0; c < nch; c++) part[c + 1] += part[c];
  out[0] = 0;
  pool.parallel_for(nch, 1, [&](int64_t lo, int64_t hi, int) {
    for (int64_t c = lo; c < hi; c++) {
      int64_t s = part[c];
      for (int64_t i = c * grain, e = std::min(n, i + grain); i < e; i++) {
        s += f(i);
        out[i + 1] = s;
      }
    }
  });
}

}  // namespace gh
