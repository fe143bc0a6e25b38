// host_pool.h -- the context's host thread pool.
#pragma once

#include <atomic>
#include <condition_variable>
#include <exception>
#include <functional>
#include <mutex>
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <thread>
#include <vector>

namespace gpb {

// A fixed set of host threads for the host work between device phases (the
// 32 x 32 eigenproblems of the block solver, the OWT-UCM host stages):
// run(n, f) calls f(0..n-1) on the workers and the calling thread and
// returns when all are done.  The first exception that an f(i) throws is
// thrown again by run once all are done.  With n <= 1, f runs inline and
// may itself call run; an f that runs on the workers must not.
class HostPool {
 public:
  explicit HostPool(unsigned nthreads) {
    for (unsigned t = 1; t < nthreads; t++) th_.emplace_back([this] { work(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (std::thread& t : th_) t.join();
  }
  void run(int n, const std::function<void(int)>& f) {
    if (th_.empty() || n <= 1) {
      for (int i = 0; i < n; i++) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      f_ = &f;
      n_ = n;
      next_ = 0;
      busy_ = (int)th_.size();
      gen_++;
    }
    cv_.notify_all();
    drain();
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [this] { return busy_ == 0; });
    f_ = nullptr;
    if (err_) {
      std::exception_ptr e = err_;
      err_ = nullptr;
      lk.unlock();
      std::rethrow_exception(e);
    }
  }

 private:
  void drain() {
    for (int i; (i = next_.fetch_add(1)) < n_;) {
      try {
        (*f_)(i);
      } catch (...) {
        std::lock_guard<std::mutex> lk(err_mu_);
        if (!err_) err_ = std::current_exception();
      }
    }
  }
  void work() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
        if (quit_) return;
        seen = gen_;
      }
      drain();
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_.notify_one();
    }
  }
  std::vector<std::thread> th_;
  std::mutex mu_, err_mu_;
  std::exception_ptr err_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* f_ = nullptr;
  std::atomic<int> next_{0};
  int n_ = 0, busy_ = 0;
  uint64_t gen_ = 0;
  bool quit_ = false;
};

// One host copy of `bytes` bytes from src to dst.
struct CopyJob {
  void* dst;
  const void* src;
  size_t bytes;
};

// Runs the copies on the pool, cut into pieces of at most `piece` bytes so
// that a few large copies spread over the workers too.
inline void parallel_copy(HostPool& pool, const std::vector<CopyJob>& jobs, size_t piece = (size_t)1 << 20) {
  std::vector<CopyJob> parts;
  for (const CopyJob& j : jobs)
    for (size_t off = 0; off < j.bytes; off += piece)
      parts.push_back({(char*)j.dst + off, (const char*)j.src + off, std::min(piece, j.bytes - off)});
  pool.run((int)parts.size(), [&](int i) { memcpy(parts[i].dst, parts[i].src, parts[i].bytes); });
}

}  // namespace gpb
