// ys_pool.h -- a small pool of host threads (see BuildPool).
#pragma once

#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace ys {

// A few host threads a collider keeps for its per-step host work (the cloth
// tree's build, the zone projections of the response); creating threads
// each time would cost what they save.
// run(n, f) calls f(0) ... f(n - 1) on the pool's threads and the caller's
// and returns when all have returned.
class BuildPool {
 public:
  explicit BuildPool(int threads) {
    for (int i = 0; i + 1 < threads; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~BuildPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (std::thread& t : workers_) t.join();
  }
  int size() const { return (int)workers_.size() + 1; }
  void run(int n, const std::function<void(int)>& f) {
    {
      std::lock_guard<std::mutex> g(mu_);
      job_ = &f;
      njob_ = n;
      next_ = 0;
      left_ = n;
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> l(mu_);
    done_.wait(l, [this] { return left_ == 0; });
    job_ = nullptr;
  }

 private:
  void work() {
    for (;;) {
      int i;
      const std::function<void(int)>* f;
      {
        std::lock_guard<std::mutex> g(mu_);
        if (!job_ || next_ >= njob_) return;
        i = next_++;
        f = job_;
      }
      (*f)(i);
      std::lock_guard<std::mutex> g(mu_);
      if (--left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      work();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* job_ = nullptr;
  int njob_ = 0, next_ = 0, left_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

}  // namespace ys
